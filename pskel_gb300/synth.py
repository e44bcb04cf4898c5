"""Seeded synthetic inputs for the stencil workloads.

Every value comes from a counter-based generator: the 64-bit SplitMix64
finaliser (Steele, Lea, Flood, "Fast splittable pseudorandom number
generators", OOPSLA 2014) applied to ``base(seed, stream) + (i + 1) * golden``,
so any element can be produced independently of the others and the same seed
always yields the same bits. Uniforms take the top 24 bits (exact in fp32),
normals use fp64 Box-Muller rounded once to fp32.

Workloads (grid shapes, value distributions and masks of the reference
benchmark applications' configurations):
  * jacobi2d  -- 5-point Jacobi, 4 neighbours of weight 0.25 in N,S,W,E order,
                 interior U[0,1), ring 0;
  * life      -- Game of Life, uint8 Bernoulli(0.3) cells everywhere, Moore mask;
  * advect2d  -- advection-diffusion, U[0,1) noise plus 16 Gaussian blobs,
                 winds u,v ~ N(0, 0.1), ring 0;
  * heat3d    -- 7-point heat/Jacobi, U[0,1), halo value 0,
                 centre weight 1-6a and neighbours a = 1/8.
"""
from __future__ import annotations

import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_STREAM = np.uint64(0xD1B54A32D192ED03)


def _mix64(z: np.ndarray) -> np.ndarray:
    z = z.astype(np.uint64, copy=True)
    z ^= z >> np.uint64(30)
    z *= _M1
    z ^= z >> np.uint64(27)
    z *= _M2
    z ^= z >> np.uint64(31)
    return z


def u64(seed: int, stream: int, n: int) -> np.ndarray:
    """n raw 64-bit values of stream ``stream`` under ``seed``."""
    with np.errstate(over="ignore"):
        key = np.array([(seed & (2**64 - 1))], dtype=np.uint64) * GOLDEN
        key ^= np.array([stream & (2**64 - 1)], dtype=np.uint64) * _STREAM
        base = _mix64(key)[0]
        idx = np.arange(1, n + 1, dtype=np.uint64)
        return _mix64(base + idx * GOLDEN)


def uniform_f32(seed: int, stream: int, shape) -> np.ndarray:
    n = int(np.prod(shape))
    x = u64(seed, stream, n) >> np.uint64(40)
    return (x.astype(np.float32) * np.float32(2.0**-24)).reshape(shape)


def bernoulli_u8(seed: int, stream: int, shape, p: float) -> np.ndarray:
    n = int(np.prod(shape))
    x = u64(seed, stream, n) >> np.uint64(40)
    return (x < np.uint64(round(p * 2**24))).astype(np.uint8).reshape(shape)


def normal_f32(seed: int, stream: int, shape, sigma: float) -> np.ndarray:
    n = int(np.prod(shape))
    a = (u64(seed, stream, n) >> np.uint64(11)).astype(np.float64)
    b = (u64(seed, stream + 1, n) >> np.uint64(11)).astype(np.float64)
    u1 = (a + 1.0) * 2.0**-53
    u2 = b * 2.0**-53
    z = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
    return (sigma * z).astype(np.float32).reshape(shape)


def f32_to_bf16(x: np.ndarray) -> np.ndarray:
    """Round fp32 to bf16 bit patterns (uint16), nearest even, NaN kept quiet."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    nan = ((u & 0x7F800000) == 0x7F800000) & ((u & 0x007FFFFF) != 0)
    with np.errstate(over="ignore"):
        r = (u + np.uint32(0x7FFF) + ((u >> 16) & 1)) >> 16
    r = np.where(nan, (u >> 16) | 0x40, r)
    return r.astype(np.uint16)


def bf16_to_f32(b: np.ndarray) -> np.ndarray:
    return (np.asarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


# ------------------------------------------------------------------ masks

# Offsets (dh, dw) and weights, in the order the functor sums them.
JACOBI4_OFFSETS = [(-1, 0), (1, 0), (0, -1), (0, 1)]
JACOBI4_WEIGHTS = [0.25, 0.25, 0.25, 0.25]
MOORE8_OFFSETS = [(-1, -1), (-1, 0), (-1, 1), (0, -1), (0, 1), (1, -1), (1, 0), (1, 1)]
HEAT7_ALPHA = 0.125
HEAT7_OFFSETS = [(0, 0, 0), (-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)]
HEAT7_WEIGHTS = [1.0 - 6 * HEAT7_ALPHA] + [HEAT7_ALPHA] * 6

# Stream ids, one per field, so fields never share random bits.
S_GRID, S_WIND_U, S_WIND_V, S_BLOBS, S_BATCH = 1, 3, 5, 7, 9


def jacobi2d(W: int, H: int, seed: int = 1):
    """(in, out) for the Jacobi workload: interior U[0,1), ring 0 in both."""
    a = uniform_f32(seed, S_GRID, (H, W))
    a[0, :] = 0
    a[-1, :] = 0
    a[:, 0] = 0
    a[:, -1] = 0
    return a, a.copy()


def batch_shapes(n: int, seed: int = 1, smin: int = 64, smax: int = 2048, imin: int = 10, imax: int = 500):
    """[(W, H, iterations)] of a batched workload: sides log-uniform in
    [smin, smax], iterations uniform in [imin, imax]."""
    u = (u64(seed, S_BATCH, 3 * n) >> np.uint64(11)).astype(np.float64) * 2.0**-53
    u = u.reshape(n, 3)
    lo, hi = np.log(smin), np.log(smax)
    W = np.minimum(smax, np.floor(np.exp(lo + (hi - lo) * u[:, 0]))).astype(int)
    H = np.minimum(smax, np.floor(np.exp(lo + (hi - lo) * u[:, 1]))).astype(int)
    it = np.minimum(imax, imin + np.floor((imax - imin + 1) * u[:, 2])).astype(int)
    return [(int(w), int(h), int(i)) for w, h, i in zip(W, H, it)]


def life(W: int, H: int, seed: int = 1, p: float = 0.3):
    """(in, out) for Game of Life: Bernoulli(p) everywhere, both arrays equal."""
    a = bernoulli_u8(seed, S_GRID, (H, W), p)
    return a, a.copy()


def advect2d(W: int, H: int, seed: int = 1, blobs: int = 16, sigma_wind: float = 0.1):
    """(phi_in, phi_out, u, v) for advection-diffusion."""
    phi = uniform_f32(seed, S_GRID, (H, W)).astype(np.float64)
    prm = uniform_f32(seed, S_BLOBS, (blobs, 3)).astype(np.float64)
    hh = np.arange(H, dtype=np.float64)[:, None]
    ww = np.arange(W, dtype=np.float64)[None, :]
    for k in range(blobs):
        ch, cw = prm[k, 0] * H, prm[k, 1] * W
        sig = W / 64.0 + prm[k, 2] * (W / 16.0 - W / 64.0)
        phi += np.exp(-((hh - ch) ** 2 + (ww - cw) ** 2) / (2.0 * sig * sig))
    phi = phi.astype(np.float32)
    phi[0, :] = 0
    phi[-1, :] = 0
    phi[:, 0] = 0
    phi[:, -1] = 0
    u = normal_f32(seed, S_WIND_U, (H, W), sigma_wind)
    v = normal_f32(seed, S_WIND_V, (H, W), sigma_wind)
    return phi, phi.copy(), u, v


ADVECT_K, ADVECT_DT, ADVECT_INV_DX = 0.1, 0.2, 10.0


def heat3d(W: int, H: int, D: int, seed: int = 1):
    """(in, out) for the 3D heat workload, layout [h][w][d]."""
    a = uniform_f32(seed, S_GRID, (H, W, D))
    return a, a.copy()
