"""FP64 restatement of the thermal model's forward and backward passes
(test infrastructure: only tests/ and bench.py's checks use it).

The network is the library's (amca3d_gb300/csrc/surrogate.h): Fourier
features of five normalised inputs, four SiLU layers of 256 and an FP32 head
giving mu and s (log of the error scale). The GPU rounds to bf16 at fixed
points: the features, every layer's weights, the stored pre-activations and
activations of the hidden layers, and the stored gradients of the
pre-activations. With ``bf16_points=True`` this restatement rounds the same
values at the same points and computes everything else in FP64, so the
GPU's results differ from it only by FP32 accumulation order (and the rare
bf16 rounding that this flips). With ``bf16_points=False`` it is plain FP64
throughout, which the finite-difference check uses.

Loss (per batch of n): sum over samples of 0.5 (mu - y)^2 / n for mu, and
lambda_s (0.5 exp(-2 s) (mu - y)^2 + s) / n for s with mu held fixed;
s is clamped to [-12, 4].

The FE field (``scan_field``) is the Rosenthal quasi-steady solution of the
current pass of a raster scan, in the operation order of the library's
thermal_field.cuh and of amca3d_gb300.decks.Rosenthal.field.
"""
from __future__ import annotations

import math

import numpy as np

N_IN, N_FREQ, N_ENC, N_HID, N_LAYERS, N_OUT = 5, 64, 128, 256, 4, 2
LAMBDA_S = 0.1
S_MIN, S_MAX = -12.0, 4.0


def in_dim(layer: int) -> int:
    return N_ENC if layer == 0 else N_HID


def layout() -> dict:
    """Blocks of the parameter vector (amca_thermal_get_params order): name ->
    (offset, shape)."""
    off, o = {}, 0
    for layer in range(N_LAYERS):
        off[f"W{layer}"] = (o, (N_HID, in_dim(layer)))
        o += N_HID * in_dim(layer)
        off[f"b{layer}"] = (o, (N_HID,))
        o += N_HID
    off["Wh"] = (o, (N_OUT, N_HID))
    o += N_OUT * N_HID
    off["bh"] = (o, (N_OUT,))
    return off


def param_total() -> int:
    o, s = layout()["bh"]
    return o + int(np.prod(s))


def unpack(p: np.ndarray) -> dict:
    return {k: p[o:o + int(np.prod(s))].reshape(s).astype(np.float64) for k, (o, s) in layout().items()}


def pack(d: dict) -> np.ndarray:
    out = np.zeros(param_total(), np.float64)
    for k, (o, s) in layout().items():
        out[o:o + int(np.prod(s))] = np.asarray(d[k], np.float64).ravel()
    return out


def bf16(x) -> np.ndarray:
    """Round to the nearest bf16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, np.float64).astype(np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def features(raw: np.ndarray, fourier: np.ndarray, shift: np.ndarray, scale: np.ndarray) -> np.ndarray:
    """[n x 128] features: phases in FP32 in the kernel's order, sin / cos in FP64."""
    raw = np.asarray(raw, np.float32)
    u = (raw - np.asarray(shift, np.float32)) * np.asarray(scale, np.float32)
    B = np.asarray(fourier, np.float32).reshape(N_FREQ, N_IN)
    f = np.zeros((raw.shape[0], N_FREQ), np.float32)
    for i in range(N_IN):  # f = fl(f + fl(B u)), i ascending
        f = f + B[:, i][None, :] * u[:, i][:, None]
    ang = 2.0 * math.pi * f.astype(np.float64)
    return np.concatenate([np.sin(ang), np.cos(ang)], axis=1)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward_backward(params: np.ndarray, raw: np.ndarray, target: np.ndarray, enc: dict, bf16_points: bool = True):
    """Returns (grad vector, mu, s, loss per sample). enc: fourier, in_shift, in_scale."""
    r = bf16 if bf16_points else (lambda x: np.asarray(x, np.float64))
    P = unpack(np.asarray(params, np.float64))
    n = raw.shape[0]
    y = np.asarray(target, np.float64)
    E = r(features(raw, enc["fourier"], enc["in_shift"], enc["in_scale"]))
    acts = [E]  # inputs of the layers, as the GEMMs read them
    Zs = []     # pre-activations
    h = E
    for layer in range(N_LAYERS):
        W = r(P[f"W{layer}"])
        z = h @ W.T + P[f"b{layer}"]
        Zs.append(z)
        if layer < N_LAYERS - 1:
            h = r(silu(z))
            acts.append(h)
    h4 = silu(Zs[-1])  # FP32 head input (not rounded)
    mu = h4 @ P["Wh"][0] + P["bh"][0]
    s = np.clip(h4 @ P["Wh"][1] + P["bh"][1], S_MIN, S_MAX)
    res = mu - y
    dmu = res / n
    ds = LAMBDA_S * (1.0 - np.exp(-2.0 * s) * res * res) / n
    g = {}
    h4r = r(h4)
    g["Wh"] = np.stack([dmu @ h4r, ds @ h4r])
    g["bh"] = np.array([dmu.sum(), ds.sum()])
    dh = dmu[:, None] * P["Wh"][0][None, :] + ds[:, None] * P["Wh"][1][None, :]
    dz = r(dh * silu_grad(Zs[-1]))
    for layer in range(N_LAYERS - 1, -1, -1):
        g[f"b{layer}"] = dz.sum(axis=0)
        g[f"W{layer}"] = dz.T @ acts[layer]
        if layer > 0:
            dh = dz @ r(P[f"W{layer}"])
            dz = r(dh * silu_grad(r(Zs[layer - 1])))
    return pack(g), mu, s, 0.5 * res * res


def predict(params: np.ndarray, raw: np.ndarray, enc: dict, bf16_points: bool = True):
    """(T, error estimate) in K, as amca_thermal_eval reports them (output
    map T = t_shift + t_scale mu, or t_shift + t_scale exp(mu) with log_output)."""
    _, mu, s, _ = forward_backward(params, raw, np.zeros(raw.shape[0]), enc, bf16_points)
    if enc.get("log_output"):
        T = enc["t_shift"] + enc["t_scale"] * np.exp(mu)
        return T, 2.0 * (T - enc["t_shift"]) * np.exp(s)
    return enc["t_shift"] + enc["t_scale"] * mu, 2.0 * enc["t_scale"] * np.exp(s)


def target_of(T, enc: dict):
    """Normalised training target of temperatures T (K)."""
    y = (np.asarray(T, np.float64) - enc["t_shift"]) / enc["t_scale"]
    return np.log(y) if enc.get("log_output") else y


def loss_total(params: np.ndarray, raw, target, enc, mu_fixed) -> float:
    """FP64 scalar whose gradient forward_backward(bf16_points=False)
    returns at the parameters where mu == mu_fixed: the mu loss plus the s
    loss with mu held at mu_fixed (the stop-gradient of the error head)."""
    _, mu, s, _ = forward_backward(params, raw, target, enc, bf16_points=False)
    n = raw.shape[0]
    y = np.asarray(target, np.float64)
    res, res0 = mu - y, np.asarray(mu_fixed, np.float64) - y
    return float(np.sum(0.5 * res * res) / n + LAMBDA_S * np.sum(0.5 * np.exp(-2.0 * s) * res0 * res0 + s) / n)


# ---------------------------------------------------------------------------
# FE field of a raster scan (thermal_field.cuh)
# ---------------------------------------------------------------------------
LN2 = 0.6931471805599453
INV_LN2 = 1.4426950408889634
EXP_TAYLOR = [1.0 / math.factorial(k) for k in range(14)]


def field_exp(a):
    a = np.maximum(np.asarray(a, np.float64), -700.0)
    k = np.rint(a * INV_LN2)
    rr = a - k * LN2
    p = np.full_like(rr, EXP_TAYLOR[13])
    for j in range(12, -1, -1):
        p = p * rr + EXP_TAYLOR[j]
    return np.ldexp(p, k.astype(np.int64))


def scan_position(scan: dict, t: float):
    k, tl = 0, t
    if scan["ntracks"] > 1 and scan["track_time"] > 0:
        k = min(max(int(t / scan["track_time"]), 0), scan["ntracks"] - 1)
        tl = t - k * scan["track_time"]
    direction = -1.0 if k & 1 else 1.0
    xl = scan["x_turn"] - scan["speed"] * tl if k & 1 else scan["x_start"] + scan["speed"] * tl
    return xl, scan["y_line"] + k * scan["hatch"], direction


def scan_field(scan: dict, x, y, z, t: float):
    xl, yl, d = scan_position(scan, t)
    xi = (np.asarray(x, np.float64) - xl) * d
    dy = np.asarray(y, np.float64) - yl
    dz = np.asarray(z, np.float64) - scan["z_top"]
    rad = np.maximum(np.sqrt((xi * xi + dy * dy) + dz * dz), 1e-9)
    q = (scan["absorptivity"] * scan["power"]) / ((2.0 * math.pi * scan["conductivity"]) * rad)
    T = scan["t0"] + q * field_exp(-(scan["speed"] * (rad + xi)) / (2.0 * scan["diffusivity"]))
    return np.minimum(T, scan["t_cap"])
