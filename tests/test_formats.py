"""Operator and deflation-space file formats (CPU)."""
import os

import numpy as np
import pytest

import gdmr
import matrix_market
import problems


def test_matrix_market_roundtrip(tmp_path):
    A = problems.helmholtz((7, 5), 3.0, 0.1)
    p = str(tmp_path / "a.mtx")
    matrix_market.write(p, A, comment="7x5 Helmholtz")
    B = matrix_market.read(p)
    assert B.n == A.n and B.nnz == A.nnz
    assert np.array_equal(B.indptr, A.indptr) and np.array_equal(B.indices, A.indices)
    assert np.array_equal(B.data, A.data)


def test_matrix_market_symmetric_and_real(tmp_path):
    p = str(tmp_path / "s.mtx")
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real symmetric\n% test\n3 3 4\n1 1 2\n2 1 -1\n2 2 2\n3 3 5\n")
    A = matrix_market.read(p)
    D = A.to_scipy().toarray()
    assert np.array_equal(D, np.array([[2, -1, 0], [-1, 2, 0], [0, 0, 5]], dtype=complex))


def test_matrix_market_rejects_bad_files(tmp_path):
    p = str(tmp_path / "bad.mtx")
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    with pytest.raises(ValueError):
        matrix_market.read(p)


def test_deflation_file_roundtrip_and_integrity(tmp_path, lib):
    rng = np.random.default_rng(0)
    Z = rng.standard_normal((3, 17)) + 1j * rng.standard_normal((3, 17))
    p = str(tmp_path / "z.gdmr")
    gdmr.write_deflation(p, Z)
    assert np.array_equal(gdmr.read_deflation(p, 3, 17), Z)
    raw = bytearray(open(p, "rb").read())
    assert raw[:8] == b"GDMRDEFL" and int.from_bytes(raw[8:12], "little") == 1
    with pytest.raises(gdmr.GDMRError):
        gdmr.read_deflation(p, 4, 17)           # wrong k
    raw[40] ^= 0xFF                              # corrupt the payload
    open(p, "wb").write(bytes(raw))
    with pytest.raises(gdmr.GDMRError) as e:
        gdmr.read_deflation(p, 3, 17)
    assert "checksum" in str(e.value)
    with pytest.raises(gdmr.GDMRError):
        gdmr.read_deflation(str(tmp_path / "missing.gdmr"), 3, 17)
