// writers.cpp — see writers.h. The text layout (separators, line breaks,
// counters carried between sections, default ostream number formatting) is
// the reference's, so files diff clean against a reference run.
#include "writers.h"

#include <errno.h>
#include <sys/stat.h>
#include <unistd.h>

#include <string.h>

#include <algorithm>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace amca {

namespace {

const char *W2 = "  ";
const char *W3 = "    ";
const char *W4 = "      ";
const char *W5 = "        ";
const char *W6 = "          ";

std::string padded(int width, int number) {
  if (width <= 0) return "";
  std::string s = std::to_string(number);
  return std::string(width > (int)s.size() ? width - s.size() : 0, '0') + s;
}

void make_dir(const std::string &path) {
  if (mkdir(path.c_str(), 0755) != 0 && errno != EEXIST)
    throw std::runtime_error("cannot create directory " + path);
}

// VtkManager::create_path: mkdir of everything before the last '/'
void create_path(const std::string &file) { make_dir(file.substr(0, file.find_last_of('/'))); }

std::string cwd() {
  char buf[4096];
  if (!getcwd(buf, sizeof buf)) return ".";
  return buf;
}

static_assert(__BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__, "appended VTR pieces are written in host byte order");

// One array of an appended piece: its XML attributes, bytes per cell (0 for
// a coordinate array) and how to fill one k-plane of interior cells.
struct AppendedArray {
  std::string attrs;
  size_t bytes;
};

// The .vtr piece with the arrays of the ASCII piece (same names, types and
// order) as raw little-endian binary in one appended block (VTK XML,
// header_type UInt64: each array is preceded by its byte count). Values are
// those the ASCII piece prints: grain ids through the VTR shuffle, cell
// temperatures through an int, melted flags (1 in the plain realm); Euler
// angles and coordinates keep full FP64 precision where the text has six
// significant digits. Written one k-plane at a time.
void write_piece_appended(const OutputView &v, const std::vector<int> &vars, const std::string &path) {
  const int nxg = v.nx + 2, nyg = v.ny + 2, nzg = v.nz + 2;
  const int64_t nxyg = (int64_t)nxg * nyg;
  const int64_t plane = (int64_t)v.nx * v.ny, ncell = plane * v.nz;
  std::vector<int> used;
  std::vector<AppendedArray> arrays;
  for (int var : vars) {
    if (var == 0 && v.temperature) {
      arrays.push_back({"type=\"Float64\" Name=\"cell_temperature\"", 8});
    } else if (var == 2) {
      arrays.push_back({"type=\"Int64\" Name=\"grain_id\"", 8});
    } else if (var == 3) {
      arrays.push_back({"type=\"Float64\" Name=\"grain_orientation\" NumberOfComponents=\"3\"", 24});
    } else if (var == 6) {
      arrays.push_back({"type=\"Int8\" Name=\"melted_flag\"", 1});
    } else {
      continue;
    }
    used.push_back(var);
  }
  std::ofstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot write " + path);
  uint64_t offset = 0;
  f << "<?xml version=\"1.0\"?>\n";
  f << "<VTKFile type=\"RectilinearGrid\" version=\"0.1\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n";
  f << W2 << "<RectilinearGrid WholeExtent=\"0 " << v.nx << " 0 " << v.ny << " 0 " << v.nz << "\">\n";
  f << W3 << "<Piece Extent=\"0 " << v.nx << " 0 " << v.ny << " 0 " << v.nz << "\">\n";
  f << W4 << "<CellData Scalars=\"grain_id\">\n";
  for (const AppendedArray &a : arrays) {
    f << W5 << "<DataArray " << a.attrs << " format=\"appended\" offset=\"" << offset << "\"/>\n";
    offset += 8 + a.bytes * (uint64_t)ncell;
  }
  f << W4 << "</CellData>\n";
  f << W4 << "<Coordinates>\n";
  const char *nm[3] = {"X_Coordinates", "Y_Coordinates", "Z_Coordinates"};
  const int npts[3] = {v.nx + 1, v.ny + 1, v.nz + 1};
  for (int a = 0; a < 3; a++) {
    f << W5 << "<DataArray type=\"Float64\" Name=\"" << nm[a] << "\" format=\"appended\" offset=\"" << offset
      << "\"/>\n";
    offset += 8 + 8 * (uint64_t)npts[a];
  }
  f << W4 << "</Coordinates>\n";
  f << W3 << "</Piece>\n";
  f << W2 << "</RectilinearGrid>\n";
  f << W2 << "<AppendedData encoding=\"raw\">\n" << W3 << "_";
  std::vector<char> buf;
  for (size_t q = 0; q < used.size(); ++q) {
    const int var = used[q];
    const uint64_t nbytes = arrays[q].bytes * (uint64_t)ncell;
    f.write((const char *)&nbytes, 8);
    buf.resize((size_t)(arrays[q].bytes * plane));
    for (int k = 1; k < nzg - 1; k++) {
      char *o = buf.data();
      for (int j = 1; j < nyg - 1; j++)
        for (int i = 1; i < nxg - 1; i++) {
          const int64_t c = k * nxyg + (int64_t)j * nxg + i;
          if (var == 0) {
            const double t = (double)(int)v.temperature[c];
            memcpy(o, &t, 8);
            o += 8;
          } else if (var == 2) {
            int val = v.orient[c];
            if (val >= 0 && v.mapped_vtr) val = (*v.mapped_vtr)[val];
            const int64_t w = val;
            memcpy(o, &w, 8);
            o += 8;
          } else if (var == 3) {
            const int val = v.orient[c];
            double e[3] = {0.0, 0.0, 0.0};
            if (val >= 0)
              for (int a = 0; a < 3; a++) e[a] = v.euler[3 * (int64_t)val + a];
            memcpy(o, e, 24);
            o += 24;
          } else {
            *o++ = (char)(v.melted ? (int8_t)v.melted[c] : (int8_t)1);
          }
        }
      f.write(buf.data(), (std::streamsize)buf.size());
    }
  }
  const double org[3] = {v.x0, v.y0, v.z0};
  for (int a = 0; a < 3; a++) {
    std::vector<double> x((size_t)npts[a]);
    for (int i = 0; i < npts[a]; i++) x[i] = org[a] + i * v.h;
    const uint64_t nbytes = 8 * (uint64_t)npts[a];
    f.write((const char *)&nbytes, 8);
    f.write((const char *)x.data(), (std::streamsize)nbytes);
  }
  f << "\n" << W2 << "</AppendedData>\n";
  f << "</VTKFile>\n";
  if (!f) throw std::runtime_error("cannot write " + path);
}

}  // namespace

void VtrSeries::configure(const OutputConfig &o, const std::string &workdir) {
  cfg_ = o;
  by_freq_ = o.frequency >= 1;
  threshold_ = 1.0e8;
  if (o.time_interval_set && o.time_interval > 0) threshold_ = 0.0;
  // VtrManager::initialize: directory part and pvd name of output_data_base_name
  const std::string &base = o.base;
  const size_t slash = base.find_last_of('/');
  const size_t dot = base.find_last_of('.');
  const std::string dir = base.substr(0, slash);
  if (dot) pvd_name_ = base.substr(slash + 1, dot);
  else pvd_name_ = base.substr(slash + 1);
  const std::string root = workdir.empty() ? cwd() : workdir;
  pvd_path_ = (!dir.empty() && dir[0] == '/') ? dir : root + "/" + dir;
}

bool VtrSeries::due(int step, double time) {
  if (by_freq_) return step % cfg_.frequency == 0;
  if (time >= threshold_) {
    threshold_ += cfg_.time_interval;
    threshold_ = std::max(int(time / cfg_.time_interval + 1) * cfg_.time_interval, threshold_);
    return true;
  }
  return false;
}

void VtrSeries::make_dirs() const {
  if (cfg_.frequency == 0) return;
  create_path(pvd_path_ + "/Dummy");
  create_path(pvd_path_ + "/grainsTimeStates/Dummy");
}

void VtrSeries::write(const OutputView &v, double time) {
  const std::string step_dir = pvd_path_ + "/grainsTimeStates/timeStep_" + padded(5, num_output_);
  create_path(step_dir + "/" + pvd_name_);
  times_.emplace_back(num_output_, time);
  const int nxg = v.nx + 2, nyg = v.ny + 2, nzg = v.nz + 2, nxyg = nxg * nyg;
  if (cfg_.appended) {
    write_piece_appended(v, cfg_.variables, step_dir + "/" + pvd_name_ + padded(5, 0) + ".vtr");
  } else {
    std::ofstream f(step_dir + "/" + pvd_name_ + padded(5, 0) + ".vtr");
    if (!f) throw std::runtime_error("cannot write " + step_dir);
    f << "<?xml version=\"1.0\"?>\n";
    f << "<VTKFile type=\"RectilinearGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
    f << W2 << "<RectilinearGrid WholeExtent=\"" << 0 << " " << v.nx << " " << 0 << " " << v.ny << " " << 0 << " "
      << v.nz << "\">\n";
    f << W3 << "<Piece Extent=\"" << 0 << " " << v.nx << " " << 0 << " " << v.ny << " " << 0 << " " << v.nz
      << "\">\n";
    f << W4 << "<CellData Scalars=\"grain_id\">\n";
    for (int var : cfg_.variables) {
      if (var == 0 && v.temperature) {  // temperature, written through an int (VtrManager.cpp:231-245)
        f << W5 << "<DataArray type=\"Float64\" Name=\"cell_temperature\" format=\"ascii\">\n";
        for (int k = 1; k < nzg - 1; k++)
          for (int j = 1; j < nyg - 1; j++) {
            f << W6;
            for (int i = 1; i < nxg - 1; i++) {
              const int val = (int)v.temperature[k * nxyg + j * nxg + i];
              f << val << " ";
            }
            f << std::endl;
          }
        f << "\n";
        f << W5 << "</DataArray>" << std::endl;
      } else if (var == 2) {  // grain_ID
        f << W5 << "<DataArray type=\"Int64\" Name=\"grain_id\" format=\"ascii\">\n";
        for (int k = 1; k < nzg - 1; k++)
          for (int j = 1; j < nyg - 1; j++) {
            f << W6;
            for (int i = 1; i < nxg - 1; i++) {
              int val = v.orient[k * nxyg + j * nxg + i];
              if (val >= 0 && v.mapped_vtr) val = (*v.mapped_vtr)[val];
              f << val << " ";
            }
            f << "\n";
          }
        f << "\n";
        f << W5 << "</DataArray>" << std::endl;
      } else if (var == 3) {  // grain_orientation
        f << W5 << "<DataArray type=\"Float64\" Name=\"grain_orientation\" NumberOfComponents=\"3\" format=\"ascii\">\n";
        for (int k = 1; k < nzg - 1; k++)
          for (int j = 1; j < nyg - 1; j++) {
            f << W6;
            for (int i = 1; i < nxg - 1; i++) {
              const int val = v.orient[k * nxyg + j * nxg + i];
              if (val >= 0) {
                for (int a = 0; a < 3; a++) f << v.euler[3 * (int64_t)val + a] << " ";
              } else {
                f << "0" << " " << "0" << " " << "0" << " ";
              }
            }
            f << "\n";
          }
        f << "\n";
        f << W5 << "</DataArray>" << std::endl;
      } else if (var == 6) {  // melted_flag: a plain realm has no melt history; cells count as melted
        f << W5 << "<DataArray type=\"Int8\" Name=\"melted_flag\" format=\"ascii\">\n";
        for (int k = 1; k < nzg - 1; k++)
          for (int j = 1; j < nyg - 1; j++) {
            f << W6;
            for (int i = 1; i < nxg - 1; i++) f << (v.melted ? (int)v.melted[k * nxyg + j * nxg + i] : 1) << " ";
            f << "\n";
          }
        f << "\n";
        f << W5 << "</DataArray>" << std::endl;
      }
    }
    f << W4 << "</CellData>\n";
    f << W4 << "<Coordinates>\n";
    const double off[3] = {v.h * 0 + v.x0, v.h * 0 + v.y0, v.h * 0 + v.z0};
    const int ng[3] = {nxg, nyg, nzg};
    const char *nm[3] = {"X_Coordinates", "Y_Coordinates", "Z_Coordinates"};
    for (int a = 0; a < 3; a++) {
      f << W5 << "<DataArray type=\"Float64\" name=\"" << nm[a] << "\" format=\"ascii\">\n";
      f << W6;
      for (int i = 0; i < ng[a] - 1; i++) f << off[a] + i * v.h << " ";
      f << W5 << "</DataArray>\n";
    }
    f << W4 << "</Coordinates>\n\n";
    f << W3 << "</Piece>\n";
    f << W2 << "</RectilinearGrid>\n";
    f << "</VTKFile>\n";
  }
  {
    std::ofstream f(step_dir + "/" + pvd_name_ + padded(5, pvtk_num_) + ".pvtr");
    f << "<?xml version=\"1.0\"?>\n";
    f << "<VTKFile type=\"PRectilinearGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
    f << W2 << "<PRectilinearGrid  WholeExtent=\"" << 0 << " " << v.nx << " " << 0 << " " << v.ny << " " << 0 << " "
      << v.nz << "\" \n";
    f << "                  " << "GhostLevel = \"0\">\n";
    f << W3 << "<PCellData Scalars=\"grain_id\">\n";
    for (int var : cfg_.variables) {
      switch (var) {
        case 0: f << W4 << "<PDataArray type=\"Float64\" Name=\"cell_temperature\"  format=\"ascii\"/>\n"; break;
        case 2: f << W4 << "<PDataArray type=\"Int64\" Name=\"grain_id\" format=\"ascii\"/>\n"; break;
        case 3:
          f << W4 << "<PDataArray type=\"Float64\" Name=\"grain_orientation\" NumberOfComponents=\"3\" format=\"ascii\"/>\n";
          break;
        case 6: f << W4 << "<PDataArray type=\"Int8\" Name=\"melted_flag\" format=\"ascii\"/>\n"; break;
        case 11:
          f << W4 << "<PDataArray type=\"Int8\" Name=\"growth_flag\"  format=\"ascii\"/>\n";
          f << W4 << "<PDataArray type=\"Float64\" Name=\"cooling\"  format=\"ascii\"/>\n";
          break;
        case 12:
          f << W4 << "<PDataArray type=\"Float64\" Name=\"p\"  format=\"ascii\"/>\n";
          f << W4 << "<PDataArray type=\"Float64\" Name=\"tMCS\"  format=\"ascii\"/>\n";
          f << W4 << "<PDataArray type=\"Float64\" Name=\"vf_a\"  format=\"ascii\"/>\n";
          f << W4 << "<PDataArray type=\"Float64\" Name=\"vf_b\"  format=\"ascii\"/>\n";
          f << W4 << "<PDataArray type=\"Float64\" Name=\"Hardness\"  format=\"ascii\"/>\n";
          break;
        default: break;
      }
    }
    f << W3 << "</PCellData>\n";
    f << W3 << "<PCoordinates>\n";
    for (int a = 0; a < 3; a++) f << W4 << "<PDataArray type=\"Float64\" format=\"ascii\"/>\n";
    f << W3 << "</PCoordinates>\n";
    f << W3 << "<Piece Extent=\"" << 0 << " " << v.nx << " " << 0 << " " << v.ny << " " << 0 << " " << v.nz
      << "\"\n";
    f << W3 << "      " << "Source=\"" << pvd_name_ << padded(5, 0) << ".vtr\" />\n";
    f << W2 << "</PRectilinearGrid>\n";
    f << "</VTKFile>\n";
  }
  ++pvtk_num_;
  {
    std::ofstream f(pvd_path_ + "/" + pvd_name_ + ".pvd");
    f << "<?xml version=\"1.0\"?>\n";
    f << "<VTKFile type=\"Collection\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
    f << W2 << "<Collection>\n";
    int counter = 0;
    for (const auto &tp : times_) {
      f.setf(std::ios::fixed);
      f.precision(8);
      f.fill('0');
      f << W3 << "<DataSet timestep=\"" << std::left << tp.second << "\" group=\"\" part=\"0\" file=\""
        << "./grainsTimeStates" << "/timeStep_" << padded(5, tp.first) << "/" << pvd_name_ << padded(5, counter)
        << ".pvtr" << "\"/>\n";
      ++counter;
    }
    f << W2 << "</Collection>\n";
    f << "</VTKFile>\n";
  }
  ++num_output_;
}

void write_final_grains(const OutputView &v, const std::string &vtk_path, const std::string &pvd_path) {
  const int nx = v.nx + 2, ny = v.ny + 2, nz = v.nz + 2, nxy = nx * ny;
  const int32_t *u = v.orient;
  std::ofstream vtk(vtk_path.c_str());
  std::ofstream one((pvd_path + "/finalResult.txt").c_str());
  int count = 0;
  const int per_line = 10;
  vtk << "# vtk DataFile Version 2.0" << std::endl;
  vtk << "Test Data" << std::endl;
  vtk << "ASCII" << std::endl;
  vtk << "DATASET RECTILINEAR_GRID" << std::endl;
  int maxVal = -1;
  for (int k = 1; k < nz - 1; ++k)
    for (int j = 1; j < ny - 1; ++j)
      for (int i = 1; i < nx - 1; ++i) maxVal = std::max(maxVal, (int)u[k * nxy + j * nx + i]);
  vtk << "DIMENSIONS " << v.nx + 1 << " " << v.ny + 1 << " " << v.nz + 1 << std::endl;
  const double org[3] = {v.x0, v.y0, v.z0};
  const int n[3] = {v.nx, v.ny, v.nz};
  const char *name[3] = {"X_COORDINATES ", "Y_COORDINATES ", "Z_COORDINATES "};
  for (int a = 0; a < 3; a++) {
    vtk << name[a] << n[a] + 1 << " double" << std::endl;
    vtk << org[a] << " ";
    for (int i = 0; i < n[a]; ++i) {
      vtk << org[a] + (i + 1) * v.h << " ";
      count++;
      if (count % per_line == 0) {
        vtk << std::endl;
        count = 0;
      }
    }
    if (count != 0) {
      vtk << std::endl;
      if (a == 2) count = 0;  // only the Z block resets the carried counter
    }
    vtk << std::endl;
  }
  auto mapped = [&](int val) {
    if (v.shuffle_vtk) {
      if (val >= 0 && v.mapped_vtk) val = (*v.mapped_vtk)[val];
    } else if (v.mapped_vtr) {
      if (val >= 0) val = (*v.mapped_vtr)[val];
    }
    return val;
  };
  vtk << "CELL_DATA " << v.nx * v.ny * v.nz << std::endl;
  vtk << "SCALARS grain_id double 1" << std::endl;
  vtk << "LOOKUP_TABLE default" << std::endl;
  for (int k = 1; k < nz - 1; ++k)
    for (int j = 1; j < ny - 1; ++j)
      for (int i = 1; i < nx - 1; ++i) {
        vtk << mapped(u[k * nxy + j * nx + i]) << " ";
        count++;
        if (count % per_line == 0) {
          vtk << std::endl;
          count = 0;
        }
      }
  if (count != 0) vtk << std::endl;
  vtk << "SCALARS number_cells int 1" << std::endl;
  vtk << "LOOKUP_TABLE default" << std::endl;
  std::vector<int> numCells((size_t)(maxVal + 1), 0);
  for (int k = 1; k < nz - 1; ++k)
    for (int j = 1; j < ny - 1; ++j)
      for (int i = 1; i < nx - 1; ++i) {
        const int val = u[k * nxy + j * nx + i];
        if (val >= 0) numCells[val]++;
      }
  for (int k = 1; k < nz - 1; ++k)
    for (int j = 1; j < ny - 1; ++j)
      for (int i = 1; i < nx - 1; ++i) {
        int val = u[k * nxy + j * nx + i];
        if (val >= 0) val = numCells[val];
        vtk << val << " ";
        count++;
        if (count % 10 == 0) {
          vtk << std::endl;
          count = 0;
        }
      }
  if (count != 0) vtk << std::endl;
  vtk << "SCALARS melted_flag int 1" << std::endl;
  vtk << "LOOKUP_TABLE default" << std::endl;
  for (int k = 1; k < nz - 1; ++k)
    for (int j = 1; j < ny - 1; ++j)
      for (int i = 1; i < nx - 1; ++i) {
        vtk << (v.melted ? (int)v.melted[k * nxy + j * nx + i] : 1) << " ";  // plain realm: 1 (outputToFile)
        count++;
        if (count % 10 == 0) {
          vtk << std::endl;
          count = 0;
        }
      }
  if (count != 0) vtk << std::endl;
  vtk << "VECTORS EulerAngle float" << std::endl;
  for (int k = 1; k < nz - 1; ++k)
    for (int j = 1; j < ny - 1; ++j)
      for (int i = 1; i < nx - 1; ++i) {
        const int val = u[k * nxy + j * nx + i];
        if (val >= 0) {
          const double *e = v.euler + 3 * (int64_t)val;
          vtk << e[0] << " " << e[1] << " " << e[2] << " ";
          count++;
          if (count % 10 == 0) {
            vtk << std::endl;
            count = 0;
          }
        } else {
          vtk << 0.0 << " " << 0.0 << " " << 0.0 << " ";
        }
      }
  vtk << std::endl;
  vtk.close();

  one << "X0" << "  " << "Y0" << "  " << "Z0" << "  " << " Dcell" << "  " << "nx_cell" << "  " << "ny_cell" << "  "
      << "nz_cell" << std::endl;
  one << v.x0 << " " << v.y0 << " " << v.z0 << " " << v.h << " " << v.nx << " " << v.ny << " " << v.nz << std::endl;
  one << "grain_ID" << "  " << "number_cells" << "  " << "melted_flag" << "  " << "EulerAngle1" << " "
      << "EulerAngle2" << " " << "EulerAngle3" << std::endl;
  for (int k = 1; k < nz - 1; ++k)
    for (int j = 1; j < ny - 1; ++j)
      for (int i = 1; i < nx - 1; ++i) {
        int val = u[k * nxy + j * nx + i];
        one << mapped(val) << " ";
        val = u[k * nxy + j * nx + i];
        if (val >= 0) val = numCells[val];
        one << val << " ";
        one << (v.melted ? (int)v.melted[k * nxy + j * nx + i] : 1) << " ";
        val = u[k * nxy + j * nx + i];
        if (val >= 0) {
          const double *e = v.euler + 3 * (int64_t)val;
          one << e[0] << " " << e[1] << " " << e[2] << " ";
        } else {
          one << 0.0 << " " << 0.0 << " " << 0.0 << " ";
        }
        one << std::endl;
      }
}

void write_grain_info(const OutputView &v, const std::string &file_name) {
  const size_t dot = file_name.find_last_of('.');
  const std::string path = file_name.substr(0, dot) + "0.txt";
  std::ofstream f(path.c_str());
  if (!f) throw std::runtime_error("cannot write " + path);
  const int nxg = v.nx + 2, nyg = v.ny + 2, nzg = v.nz + 2;
  const int64_t ncells = (int64_t)nxg * nyg * nzg;
  f << "numCell; numOrientation; numLocalGrain; numGlobalExpectedGrain; start Point X; Y; Z; number Point nx; ny; nz; dCell"
    << "\n";
  f << ncells << "  " << v.n_orient << "  " << v.n_grains << "  " << v.expected_grains << "  " << v.x0 << "  " << v.y0
    << "  " << v.z0 << "  " << nxg << "  " << nyg << "  " << nzg << "  " << v.h << std::endl;
  f << "Cell informatin: ID; grainID; orientationID; hasBeenMelted; undercooling of seed" << std::endl;
  for (int64_t c = 0; c < ncells; ++c) {
    const bool melted = v.melted ? v.melted[c] != 0 : false;
    f << c << "  " << v.grain[c] << "  " << v.orient[c] << "  " << melted << "  " << v.site_dtc[c];
    f << std::endl;
  }
  f << "Orientation informatin: ID; EularAngle" << std::endl;
  for (int64_t o = 0; o < v.n_orient; ++o) {
    f << o << "  ";
    for (int a = 0; a < 3; a++) f << v.euler[3 * o + a] << "  ";
    f << std::endl;
  }
  f << "Grain information: ID; cellID; grainCenter; orientationID" << std::endl;
  for (int64_t g = 0; g < v.n_grains; ++g) {
    f << g << "  " << v.gcell[g] << "  " << v.gx[g] << "  " << v.gy[g] << "  " << v.gz[g] << "  ";
    f << v.gori[g] << "   " << std::endl;
  }
}

}  // namespace amca
