"""Seeded synthetic right-hand sides for the solver workloads.

The reference publishes no datasets; its driver builds one right-hand side
(``MPI_REAL/system.c:452-468``).  These generators produce the seeded inputs
of the five measured workloads, all in the reference's x-fastest layout
(flat index ``i + j*nx + k*nx*ny``), returned as ``(nz, ny, nx)`` arrays.

* ``uniform_rhs``  — i.i.d. U[-0.5, 0.5] from ``numpy.random.default_rng(seed)``,
  mean subtracted (48^3 seed 0; 256^3 seed 1).
* ``blob_rhs``     — sum of 64 periodic Gaussian blobs of width 0.02 with
  U[0,1)^3 centres and +-1 amplitudes, mean subtracted (384^3 mixed precision).
* ``helmholtz_batch`` — 48 complex shifted-Helmholtz problems on cubic grids
  with sides from {32, 48, 64, 96, 128, 160}.
* ``differentiable_batch`` — 16 real shifted problems at 128^3 with targets.
"""
from __future__ import annotations

import numpy as np


def uniform_rhs(n, seed: int, dtype=np.float64) -> np.ndarray:
    nx, ny, nz = (n, n, n) if np.isscalar(n) else tuple(n)
    rng = np.random.default_rng(seed)
    b = rng.uniform(-0.5, 0.5, size=nx * ny * nz)
    b -= b.mean()
    return b.reshape(nz, ny, nx).astype(dtype, copy=False)


def _periodic_gauss_1d(n: int, centres: np.ndarray, width: float) -> np.ndarray:
    """(K, n) table exp(-d^2 / (2 w^2)) with d the periodic minimum-image distance."""
    x = np.arange(n) / n
    d = np.abs(x[None, :] - centres[:, None])
    d = np.minimum(d, 1.0 - d)
    return np.exp(-d * d / (2.0 * width * width))


def blob_rhs(n: int, seed: int, blobs: int = 64, width: float = 0.02) -> np.ndarray:
    """Sum of periodic Gaussian blobs on the unit cube, mean subtracted.

    The Gaussian of a per-axis minimum-image distance factorises over the
    axes, so the field is a sum of ``blobs`` rank-1 tensors and is built as one
    (n x K) @ (K x n^2) product.
    """
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, 1.0, size=(blobs, 3))
    amps = rng.choice(np.array([-1.0, 1.0]), size=blobs)
    gx = _periodic_gauss_1d(n, centres[:, 0], width)
    gy = _periodic_gauss_1d(n, centres[:, 1], width)
    gz = _periodic_gauss_1d(n, centres[:, 2], width) * amps[:, None]
    yx = (gy[:, :, None] * gx[:, None, :]).reshape(blobs, n * n)
    b = (gz.T @ yx).reshape(n, n, n)
    b -= b.mean()
    return b


def helmholtz_batch(seed: int = 4, count: int = 48, sides=(32, 48, 64, 96, 128, 160)):
    """48 complex problems: side n, sigma = sr + i si (sr~U[0,50], si~U[1,50]), complex b."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.choice(np.asarray(sides)))
        sigma = complex(rng.uniform(0.0, 50.0), rng.uniform(1.0, 50.0))
        b = (rng.uniform(-0.5, 0.5, n ** 3) + 1j * rng.uniform(-0.5, 0.5, n ** 3)).reshape(n, n, n)
        out.append((n, sigma, b))
    return out


def differentiable_batch(seed: int = 5, count: int = 16, n: int = 128):
    """16 real problems at n^3: sigma~U[0.1,10], zero-mean uniform b, x* ~ N(0,1)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        sigma = float(rng.uniform(0.1, 10.0))
        b = rng.uniform(-0.5, 0.5, n ** 3)
        b -= b.mean()
        xstar = rng.standard_normal(n ** 3)
        out.append((sigma, b.reshape(n, n, n), xstar.reshape(n, n, n)))
    return out
