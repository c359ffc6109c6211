"""CPU test of the host subspace eigensolvers (tincr_gb300/csrc/eigen_host.cpp) against LAPACK
(numpy.linalg.eigh): the full decomposition and the lowest-k solver (Householder, multisection,
inverse iteration) on random, nearly degenerate, exactly degenerate, diagonal and block-diagonal
symmetric matrices, on one thread (n < 128) and on several."""

import ctypes
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tincr_gb300", "csrc", "eigen_host.cpp")

WRAP = r'''
#include "%s"
extern "C" int test_eigh_lowest(int n, const double *a, int k, double *w, double *y) {
    return tincr::eigh_lowest_upper(n, a, k, w, y) ? 1 : 0;
}
extern "C" int test_eigh_full(int n, const double *a, double *w, double *z) {
    return tincr::eigh_upper(n, a, w, z) ? 1 : 0;
}
'''


@pytest.fixture(scope="module")
def lib():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    d = tempfile.mkdtemp()
    src = os.path.join(d, "wrap.cpp")
    open(src, "w").write(WRAP % SRC)
    so = os.path.join(d, "libeig.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-fopenmp", "-shared", "-fPIC", src, "-o", so], check=True)
    L = ctypes.CDLL(so)
    dp = ctypes.POINTER(ctypes.c_double)
    L.test_eigh_lowest.argtypes = [ctypes.c_int, dp, ctypes.c_int, dp, dp]
    L.test_eigh_full.argtypes = [ctypes.c_int, dp, dp, dp]
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _cases(rng, n):
    b = rng.standard_normal((n, n))
    yield b + b.T
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    ev = np.sort(rng.uniform(0.5, 2.0, n))
    ev[:min(n, 4)] = 0.7 + 1e-12 * np.arange(min(n, 4))
    yield (q * ev) @ q.T
    ev = np.repeat(np.sort(rng.uniform(0.3, 1.5, (n + 1) // 2)), 2)[:n]
    yield (q * ev) @ q.T
    yield np.diag(np.sort(rng.uniform(0.2, 1.5, n))) + 1e-3 * (b + b.T)
    # reflections with nothing to reflect: a diagonal matrix (every column), and two decoupled
    # blocks (the column at the block edge), which the threaded reduction takes without an update
    yield np.diag(rng.uniform(0.2, 1.5, n))
    h = n // 2
    c = b + b.T
    c[:h, h:] = 0.0
    c[h:, :h] = 0.0
    yield c


@pytest.mark.parametrize("n", [1, 2, 3, 17, 60, 150, 300])
def test_lowest_pairs_match_lapack(lib, n):
    rng = np.random.default_rng(n)
    k = min(n, 20)
    for a in _cases(rng, n):
        a = np.ascontiguousarray(0.5 * (a + a.T))
        up = np.triu(a) + np.tril(np.full_like(a, 7.0), -1)    # only the upper triangle may be read
        w = np.zeros(k)
        y = np.zeros((k, n))
        assert lib.test_eigh_lowest(n, _p(np.ascontiguousarray(up)), k, _p(w), _p(y)) == 1
        ref = np.linalg.eigvalsh(a)[:k]
        scale = max(1.0, np.abs(a).max())
        assert np.abs(w - ref).max() < 1e-13 * scale * n
        for r in range(k):
            assert np.linalg.norm(a @ y[r] - w[r] * y[r]) < 1e-12 * scale * n
        assert np.abs(y @ y.T - np.eye(k)).max() < 1e-12


@pytest.mark.parametrize("n", [5, 80])
def test_full_decomposition_matches_lapack(lib, n):
    rng = np.random.default_rng(100 + n)
    b = rng.standard_normal((n, n))
    a = np.ascontiguousarray(b + b.T)
    w = np.zeros(n)
    z = np.zeros((n, n))
    assert lib.test_eigh_full(n, _p(a), _p(w), _p(z)) == 1
    assert np.abs(w - np.linalg.eigvalsh(a)).max() < 1e-12 * np.abs(a).max() * n
