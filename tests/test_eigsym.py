"""The host symmetric eigensolver of the namelist driver's readhess
(pimd-tunneling_gb300/host/eigsym.hpp, cyclic Jacobi), compiled on its own:
eigenvalues and eigenvectors of random symmetric and polymer-Hessian-like
banded matrices against numpy's eigh."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = r'''
#include <cstdio>
#include <vector>
#include "eigsym.hpp"
int main() {
    int n;
    if (std::scanf("%d", &n) != 1) return 2;
    std::vector<double> a((size_t)n * n), w, v;
    for (auto &x : a)
        if (std::scanf("%lf", &x) != 1) return 2;
    const int sweeps = pgh::eigsym_jacobi(n, a, w, v);
    std::printf("%d\n", sweeps);
    for (int j = 0; j < n; j++) std::printf("%.17g\n", w[j]);
    for (size_t k = 0; k < v.size(); k++) std::printf("%.17g\n", v[k]);
    return 0;
}
'''


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("eig")
    src = d / "harness.cpp"
    src.write_text(HARNESS)
    exe = d / "harness"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "pimd-tunneling_gb300", "host"), str(src),
                    "-o", str(exe)], check=True)
    return str(exe)


def _solve(exe, A):
    n = A.shape[0]
    text = "%d\n" % n + "\n".join("%.17g" % x for x in A.ravel())
    out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True).stdout.split()
    sweeps = int(out[0])
    w = np.array(out[1:1 + n], dtype=float)
    v = np.array(out[1 + n:], dtype=float).reshape(n, n)
    return sweeps, w, v


def _check(A, sweeps, w, v):
    assert sweeps >= 0
    wn, vn = np.linalg.eigh(A)
    scale = np.max(np.abs(wn))
    np.testing.assert_allclose(w, wn, rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(v.T @ v, np.eye(A.shape[0]), atol=1e-12)
    np.testing.assert_allclose(A @ v, v * w, atol=1e-11 * scale)


def test_random_symmetric(harness):
    rs = np.random.RandomState(2)
    for n in (1, 2, 7, 40):
        B = rs.randn(n, n)
        A = B + B.T
        _check(A, *_solve(harness, A))


def test_banded_polymer_like(harness):
    """A fixed-end polymer Hessian: springs on the tridiagonal of each dof, a
    dense bead block, one negative mode; the eigenvalues span several decades."""
    rs = np.random.RandomState(4)
    P, nd = 12, 3
    n = P * nd
    A = np.zeros((n, n))
    for b in range(P):
        K = rs.randn(nd, nd) * 1e-3
        A[b * nd:(b + 1) * nd, b * nd:(b + 1) * nd] = K + K.T + np.eye(nd) * 2.0
        if b + 1 < P:
            A[b * nd:(b + 1) * nd, (b + 1) * nd:(b + 2) * nd] = -np.eye(nd)
            A[(b + 1) * nd:(b + 2) * nd, b * nd:(b + 1) * nd] = -np.eye(nd)
    A[0, 0] -= 3.0
    _check(A, *_solve(harness, A))
