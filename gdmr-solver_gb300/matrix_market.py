"""MatrixMarket coordinate files <-> the CSR form the library takes (gdmr_system_create,
impCsrLS, impCsrLS_z).  The reference accepts only a dense operator (impOptLS,
testLS.cu:288-307); this is the loader the sparse plugins need.

Supported: `%%MatrixMarket matrix coordinate {real|complex|integer} {general|symmetric|
hermitian|skew-symmetric}`, 1-based indices, square matrices.  Duplicate entries are summed.
"""
from __future__ import annotations

import numpy as np

from problems import CSR


def read(path: str) -> CSR:
    with open(path, "r") as f:
        header = f.readline().strip().split()
        if len(header) < 5 or header[0].lower() != "%%matrixmarket" or header[1].lower() != "matrix":
            raise ValueError("not a MatrixMarket matrix file")
        fmt, field, sym = header[2].lower(), header[3].lower(), header[4].lower()
        if fmt != "coordinate":
            raise ValueError("only the coordinate format is supported")
        if field not in ("real", "complex", "integer"):
            raise ValueError(f"unsupported field {field}")
        line = f.readline()
        while line.startswith("%"):
            line = f.readline()
        nr, nc, nnz = (int(t) for t in line.split())
        if nr != nc:
            raise ValueError("the operator must be square")
        data = np.loadtxt(f, ndmin=2) if nnz else np.zeros((0, 4 if field == "complex" else 3))
    if data.shape[0] != nnz:
        raise ValueError(f"expected {nnz} entries, found {data.shape[0]}")
    r = data[:, 0].astype(np.int64) - 1
    c = data[:, 1].astype(np.int64) - 1
    v = data[:, 2] + (1j * data[:, 3] if field == "complex" else 0)
    if r.size and (r.min() < 0 or c.min() < 0 or r.max() >= nr or c.max() >= nr):
        raise ValueError("index out of range")
    if sym != "general":
        off = r != c
        if sym == "symmetric":
            mirror = v[off]
        elif sym == "hermitian":
            mirror = np.conj(v[off])
        elif sym == "skew-symmetric":
            mirror = -v[off]
        else:
            raise ValueError(f"unsupported symmetry {sym}")
        r, c, v = np.concatenate([r, c[off]]), np.concatenate([c, r[off]]), np.concatenate([v, mirror])
    import scipy.sparse as sp
    S = sp.coo_matrix((v.astype(np.complex128), (r, c)), shape=(nr, nr)).tocsr()
    S.sum_duplicates()
    S.sort_indices()
    return CSR(nr, S.indptr.astype(np.int32), S.indices.astype(np.int32), S.data.astype(np.complex128),
               {"kind": "matrix_market", "path": path})


def write(path: str, A: CSR, comment: str = "") -> None:
    rows = np.repeat(np.arange(A.n), np.diff(A.indptr))
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate complex general\n")
        if comment:
            for ln in comment.splitlines():
                f.write(f"% {ln}\n")
        f.write(f"{A.n} {A.n} {A.nnz}\n")
        for r, c, v in zip(rows, A.indices, A.data):
            f.write(f"{r + 1} {c + 1} {v.real:.17g} {v.imag:.17g}\n")
