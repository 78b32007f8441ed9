// errors.h — exception types the C ABI maps to status codes
// (AMCA_ERR_CUDA, AMCA_ERR_DEVICE, AMCA_ERR_STATE; anything else is
// AMCA_ERR_ARG).
#pragma once

#include <stdexcept>
#include <string>

namespace amca {

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string &m) : std::runtime_error(m) {}
};
struct DeviceError : std::runtime_error {
  explicit DeviceError(const std::string &m) : std::runtime_error(m) {}
};
struct StateError : std::runtime_error {
  explicit StateError(const std::string &m) : std::runtime_error(m) {}
};

}  // namespace amca
