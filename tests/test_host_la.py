"""The library's host linear algebra (csrc/hostla.cpp), on the CPU:

- the band reduction that gives the Lanczos T eigenvalues (dsbev('N') in
  diagmat_banded, block_lanczos.f90:2006-2052) against dense numpy eigvalsh;
- the dense eigensolver (Householder tridiagonalisation + implicit
  symmetric QR) against numpy, eigenvectors included;
- the heapsort that selects the Davidson guess vectors (dsortindxa1,
  initvec_ondiag block_davidson.f90:463-532) against the oracle's
  restatement, including the order of ties.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    nvcc = shutil.which("nvcc")
    cuda_home = os.environ.get("CUDA_HOME") or (os.path.dirname(os.path.dirname(nvcc)) if nvcc else "")
    cuda_inc = os.path.join(cuda_home, "include")
    if not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("CUDA headers not found")
    out = str(tmp_path_factory.mktemp("hostla") / "hostla_driver")
    cmd = [gxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "adc_ottawa_gb300", "csrc"), "-I", cuda_inc,
           os.path.join(ROOT, "tests", "host", "hostla_driver.cpp"),
           os.path.join(ROOT, "adc_ottawa_gb300", "csrc", "hostla.cpp"), "-o", out]
    subprocess.run(cmd, check=True)
    return out


def run(driver, mode, header, data, tmp_path, out_dtype, n):
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(fin, "wb") as f:
        f.write(np.array(header, np.int32).tobytes())
        f.write(np.ascontiguousarray(data, np.float64).tobytes(order="F"))
    subprocess.run([driver, mode, fin, fout], check=True)
    return np.fromfile(fout, out_dtype, n)


@pytest.mark.parametrize("n,kd", [(1, 0), (7, 1), (50, 3), (300, 10), (640, 10)])
def test_band_eigenvalues(driver, tmp_path, n, kd):
    rs = np.random.RandomState(n + kd)
    A = np.zeros((n, n))
    for d in range(kd + 1):
        v = rs.standard_normal(n - d)
        A[np.arange(d, n), np.arange(n - d)] = v
        A[np.arange(n - d), np.arange(d, n)] = v
    w = run(driver, "sbev", [n, kd], np.asfortranarray(A), tmp_path, np.float64, n)
    ref = np.linalg.eigvalsh(A)
    assert np.abs(w - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


def test_dense_eigenvalues(driver, tmp_path):
    rs = np.random.RandomState(3)
    B = rs.standard_normal((120, 120))
    A = B + B.T
    w = run(driver, "syev", [120], np.asfortranarray(A), tmp_path, np.float64, 120)
    assert np.abs(w - np.linalg.eigvalsh(A)).max() <= 1e-12 * np.abs(A).max() * 10


@pytest.mark.parametrize("n,kind", [(1, "rand"), (2, "rand"), (3, "rand"), (37, "rand"), (160, "rand"),
                                    (50, "degenerate"), (64, "diagonal"), (40, "graded")])
def test_dense_eigenvectors(driver, tmp_path, n, kind):
    """dsyev('V') stand-in: ascending eigenvalues within 1e-12 of numpy and
    orthonormal eigenvectors with A V = V diag(w), also for repeated
    eigenvalues, an already diagonal matrix and a widely graded spectrum."""
    rs = np.random.RandomState(n)
    if kind == "rand":
        B = rs.standard_normal((n, n))
        A = B + B.T
    elif kind == "degenerate":
        Q, _ = np.linalg.qr(rs.standard_normal((n, n)))
        w0 = np.repeat([-1.0, 0.5, 2.0, 7.0, 7.0], n // 5)
        A = (Q * w0) @ Q.T
        A = 0.5 * (A + A.T)
    elif kind == "diagonal":
        A = np.diag(rs.standard_normal(n))
    else:
        Q, _ = np.linalg.qr(rs.standard_normal((n, n)))
        A = (Q * np.logspace(-8, 4, n)) @ Q.T
        A = 0.5 * (A + A.T)
    out = run(driver, "syevv", [n], np.asfortranarray(A), tmp_path, np.float64, n + n * n)
    w, V = out[:n], out[n:].reshape((n, n), order="F")
    scale = max(np.abs(A).max(), 1e-300)
    assert np.all(np.diff(w) >= 0)
    assert np.abs(w - np.linalg.eigvalsh(A)).max() <= 1e-12 * scale * max(1, n / 10)
    assert np.abs(V.T @ V - np.eye(n)).max() <= 1e-12 * max(1, n / 10)
    assert np.abs(A @ V - V * w).max() <= 1e-12 * scale * max(1, n / 10)


@pytest.mark.parametrize("n", [1, 6, 1000, 65537])
def test_heapsort_matches_reference_order(built, driver, tmp_path, n):
    rs = np.random.RandomState(n)
    arr = np.round(rs.uniform(0.0, 3.0, n) * 4) / 4          # many ties
    idx = run(driver, "heap", [n], arr, tmp_path, np.int64, n)
    assert np.array_equal(idx, oracle.heapsort_index(arr).astype(np.int64))


@pytest.mark.parametrize("n", [2, 9, 800, 5000])
def test_descending_heapsort_is_ascending_on_negated_keys(built, driver, tmp_path, n):
    """init_vec_singlesubspace sorts hii with dsortindxa1('D'); the library
    runs its ascending heapsort on -hii.  Both comparisons flip, so the
    permutation, ties included, is the reference's."""
    rs = np.random.RandomState(n + 1)
    arr = np.round(rs.uniform(-1.0, 3.0, n) * 4) / 4          # many ties, both signs
    idx = run(driver, "heap", [n], -arr, tmp_path, np.int64, n)
    assert np.array_equal(idx, oracle.heapsort_index_desc(arr).astype(np.int64))
    assert np.array_equal(oracle.heapsort_index(-arr), oracle.heapsort_index_desc(arr))
