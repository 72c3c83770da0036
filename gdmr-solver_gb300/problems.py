"""Synthetic linear systems for the deflated minimal residual (DMR) solver.

The reference ships no datasets and no benchmark inputs (its only driver,
progDMR.c:117-181, draws a random dense tridiagonal system with rand()), so
every workload here is generated from a fixed seed:

* random numbers: SplitMix64 (Steele, Lea & Flood 2014) used as a counter
  stream, output k of seed s is mix(s + (k+1)*0x9E3779B97F4A7C15);
* Gaussians: Box-Muller (1958) on pairs of outputs; a complex Gaussian has
  real and imaginary parts i.i.d. N(0, 1/2);
* unknowns are numbered lexicographically, i + Nx*(j + Ny*l);
* operators are CSR with int32 row pointers and int32 column indices, rows
  sorted by column.

Everything is vectorised numpy so a 128^3 operator (14.6M non-zeros) builds in
a few seconds.  Values are complex128; the complex64 forms are plain casts.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Outputs offset..offset+count-1 of the SplitMix64 stream started at `seed`."""
    with np.errstate(over="ignore"):
        k = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + k * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Doubles in [0, 1) from the top 53 bits of each SplitMix64 output."""
    return (splitmix64(seed, count, offset) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def complex_gaussian(seed: int, n: int) -> np.ndarray:
    """n complex normals, re and im i.i.d. N(0, 1/2), by Box-Muller on output pairs."""
    u = uniform01(seed, 2 * n)
    u1 = 1.0 - u[0::2]          # (0, 1]: log is finite
    u2 = u[1::2]
    r = np.sqrt(-np.log(u1))    # sqrt(-2 ln u1) / sqrt(2)
    th = 2.0 * np.pi * u2
    return (r * np.cos(th) + 1j * r * np.sin(th)).astype(np.complex128)


@dataclass
class CSR:
    """Square complex CSR matrix (int32 row pointers and column indices)."""
    n: int
    indptr: np.ndarray
    indices: np.ndarray
    data: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def nnz(self) -> int:
        return int(self.indptr[-1])

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.data, self.indices, self.indptr), shape=(self.n, self.n))

    def astype(self, dtype) -> "CSR":
        return CSR(self.n, self.indptr, self.indices, self.data.astype(dtype), dict(self.meta))


def _assemble(n: int, rows: list, cols: list, vals: list) -> CSR:
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    v = np.concatenate(vals)
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    counts = np.bincount(r, minlength=n)
    indptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=indptr[1:])
    if indptr[-1] >= 2 ** 31:
        raise ValueError("nnz needs int64 row pointers; not supported by this generator")
    return CSR(n, indptr.astype(np.int32), c.astype(np.int32), v.astype(np.complex128))


def helmholtz(shape: tuple, kappa: float, damping: float) -> CSR:
    """(1/h^2)-scaled 5-point (2D) or 7-point (3D) Dirichlet Laplacian minus kappa^2 (1 + i*damping).

    h = 1/(N+1) on every axis (the grids here are cubic/square), boundary
    neighbours are dropped, diagonal 2d/h^2 - kappa^2 (1 + i damping) and
    off-diagonals -1/h^2.
    """
    dims = len(shape)
    if dims not in (2, 3):
        raise ValueError("2D or 3D grids only")
    n = int(np.prod(shape))
    idx = np.arange(n, dtype=np.int64)
    coords = []
    rem = idx.copy()
    for ax in range(dims):
        coords.append(rem % shape[ax])
        rem //= shape[ax]
    strides = [int(np.prod(shape[:ax])) for ax in range(dims)]
    inv_h2 = [(shape[ax] + 1) ** 2 for ax in range(dims)]
    shift = kappa * kappa * complex(1.0, damping)
    rows, cols, vals = [idx], [idx], [np.full(n, sum(2.0 * s for s in inv_h2) - shift, dtype=np.complex128)]
    for ax in range(dims):
        for d in (-1, 1):
            ok = (coords[ax] + d >= 0) & (coords[ax] + d < shape[ax])
            r = idx[ok]
            rows.append(r)
            cols.append(r + d * strides[ax])
            vals.append(np.full(r.size, -float(inv_h2[ax]), dtype=np.complex128))
    A = _assemble(n, rows, cols, vals)
    A.meta = {"kind": "helmholtz", "shape": tuple(shape), "kappa": kappa, "damping": damping}
    return A


def helmholtz_stencil(shape: tuple, kappa: float, damping: float) -> tuple:
    """(d, wx, wy, wz) of the matrix-free form of helmholtz(shape, kappa, damping)."""
    inv_h2 = [(L + 1) ** 2 for L in shape]
    d = sum(2.0 * s for s in inv_h2) - kappa * kappa * complex(1.0, damping)
    w = [-float(s) for s in inv_h2] + [0.0] * (3 - len(shape))
    return complex(d), complex(w[0]), complex(w[1]), complex(w[2])


def variable_helmholtz(shape: tuple, kappa: float, damping: float, seed: int, block: int = 8) -> CSR:
    """3D 7-point -div(a grad u) - kappa^2 (1 + i damping) u with piecewise-constant a.

    a is constant on block^3 cells: Re a ~ U[1,4], Im a ~ U[0,0.2]; a face
    coefficient is the mean of its two cells, a boundary face uses the
    cell's own a; h_axis = 1/(L_axis + 1).
    """
    Lx, Ly, Lz = shape
    n = Lx * Ly * Lz
    idx = np.arange(n, dtype=np.int64)
    x, y, z = idx % Lx, (idx // Lx) % Ly, idx // (Lx * Ly)
    bx, by, bz = -(-Lx // block), -(-Ly // block), -(-Lz // block)
    nb = bx * by * bz
    u = uniform01(seed, 2 * nb)
    a_blocks = (1.0 + 3.0 * u[0::2]) + 1j * (0.2 * u[1::2])
    a = a_blocks[(x // block) + bx * ((y // block) + by * (z // block))]
    strides = (1, Lx, Lx * Ly)
    coords = (x, y, z)
    inv_h2 = [(L + 1) ** 2 for L in shape]
    diag = np.full(n, -kappa * kappa * complex(1.0, damping), dtype=np.complex128)
    rows, cols, vals = [], [], []
    for ax in range(3):
        for d in (-1, 1):
            ok = (coords[ax] + d >= 0) & (coords[ax] + d < shape[ax])
            nbr = idx + d * strides[ax]
            face = np.where(ok, 0.5 * (a + a[np.where(ok, nbr, idx)]), a)
            diag += face * inv_h2[ax]
            r = idx[ok]
            rows.append(r)
            cols.append(nbr[ok])
            vals.append(-face[ok] * inv_h2[ax])
    rows.append(idx)
    cols.append(idx)
    vals.append(diag)
    A = _assemble(n, rows, cols, vals)
    A.meta = {"kind": "variable_helmholtz", "shape": tuple(shape), "kappa": kappa,
              "damping": damping, "seed": seed}
    return A


def unit_gaussian_rhs(n: int, seed: int) -> np.ndarray:
    b = complex_gaussian(seed, n)
    return b / np.linalg.norm(b)


def drifting_sequence(n: int, count: int, seed: int, drift: float = 0.05) -> list:
    """b_1 unit complex Gaussian; b_{j+1} = b_j + drift*||b_j|| g_j/||g_j||."""
    b = unit_gaussian_rhs(n, seed)
    out = [b]
    for j in range(1, count):
        g = complex_gaussian(seed + 1000 * j, n)
        b = b + drift * np.linalg.norm(b) * g / np.linalg.norm(g)
        out.append(b)
    return out


def gaussian_source_rhs(shape: tuple, seed: int, sigma: float = 3.0, noise: float = 0.01) -> np.ndarray:
    """exp(-|p - p_r|^2 / (2 sigma^2)) (cell units) at a seeded uniform position, plus
    complex Gaussian noise eta with ||eta|| = noise * ||source||."""
    dims = len(shape)
    n = int(np.prod(shape))
    u = uniform01(seed, dims)
    centre = [u[ax] * (shape[ax] - 1) for ax in range(dims)]
    idx = np.arange(n, dtype=np.int64)
    r2 = np.zeros(n)
    rem = idx.copy()
    for ax in range(dims):
        c = rem % shape[ax]
        rem //= shape[ax]
        r2 += (c - centre[ax]) ** 2
    s = np.exp(-r2 / (2.0 * sigma * sigma)).astype(np.complex128)
    eta = complex_gaussian(seed ^ 0x5DEECE66D, n)
    s = s + noise * np.linalg.norm(s) * eta / np.linalg.norm(eta)
    return s


# ---------------------------------------------------------------------------
# The named workloads.  Seeds are fixed and reported with every result.
# ---------------------------------------------------------------------------

def config_2d64():
    """2D 5-point Helmholtz 64x64, kappa=20, damping 0.05; 8 unit Gaussian RHS (seeds 1..8);
    m=40, k=10, tol 1e-10, at most 2000 matrix-vector products."""
    A = helmholtz((64, 64), 20.0, 0.05)
    rhs = [unit_gaussian_rhs(A.n, s) for s in range(1, 9)]
    return A, rhs, dict(m=40, k=10, tol=1e-10, max_matvecs=2000)


def config_3d128():
    """3D 7-point Helmholtz 128^3, kappa=30, damping 0.1; 32 drifting RHS; m=60, k=20, tol 1e-10."""
    A = helmholtz((128, 128, 128), 30.0, 0.1)
    return A, (lambda count=32: drifting_sequence(A.n, count, seed=11)), dict(m=60, k=20, tol=1e-10)


def shard_seeds(nrhs: int, rank: int) -> list:
    """Seeds of the right-hand sides a rank solves when independent systems shard across
    ranks (weak scaling): rank r gets 100 + 1000 r + [0, nrhs)."""
    return [100 + 1000 * rank + r for r in range(nrhs)]


def config_3d96_batch(count: int = 64):
    """3D 7-point Helmholtz 96^3, kappa=24, damping 0.1; `count` Gaussian-source RHS; m=48, k=24."""
    shape = (96, 96, 96)
    A = helmholtz(shape, 24.0, 0.1)
    rhs = [gaussian_source_rhs(shape, 100 + r) for r in range(count)]
    return A, rhs, dict(m=48, k=24, tol=1e-10)
