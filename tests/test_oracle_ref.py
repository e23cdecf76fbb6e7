"""The oracle pinned against the reference's own CPU code (no GPU).

oracle/build.py compiles three of the reference's source files where they
lie - src/cosma/local_multiply.cpp (the naive local_multiply_cpu loop and the
CPU build's local_multiply -> cosma::gemm), src/cosma/blas.cpp and
src/cosma/scalapack.cpp (numroc) - into oracle/_ref/libcosma_ref.so, with
stand-in headers for MPI / BLACS / COSTA and a CBLAS over scipy's OpenBLAS.
Where the reference's sources are absent these tests skip.
"""
import ctypes as C
import glob
import os

import numpy as np
import pytest

import oracle
from oracle import build as ob

from test_oracle import _load


@pytest.fixture(scope="module")
def ref():
    path = ob.build_ref()
    if path is None:
        pytest.skip("the reference's sources are not present here (oracle/_ref not built)")
    import scipy
    libs = glob.glob(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs", "libscipy_openblas*.so"))
    if not libs:
        pytest.skip("scipy's bundled OpenBLAS not found")
    os.environ.setdefault("COSMA_REF_OPENBLAS", os.path.abspath(libs[0]))
    lib = C.CDLL(str(path))
    vp, i32, dbl = C.c_void_p, C.c_int, C.c_double
    lib.ref_local_multiply_cpu_d.argtypes = [vp, vp, vp, i32, i32, i32, dbl, dbl]
    lib.ref_local_multiply_d.argtypes = [vp, vp, vp, i32, i32, i32, dbl, dbl]
    lib.ref_gemm_z.argtypes = [i32, i32, i32, vp, vp, i32, vp, i32, vp, vp, i32]
    lib.ref_numroc.argtypes = [i32] * 5
    lib.ref_numroc.restype = i32
    for f in (lib.ref_local_multiply_cpu_d, lib.ref_local_multiply_d, lib.ref_gemm_z):
        f.restype = None
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _ops(c):
    A = np.asfortranarray(c["A"] if c["ta"] == "N" else c["A"].T)
    B = np.asfortranarray(c["B"] if c["tb"] == "N" else c["B"].T)
    return A, B


@pytest.mark.parametrize("m,n,k", [(4, 4, 4), (3, 4, 5), (17, 9, 33), (1, 1, 1), (40, 3, 70)])
def test_local_multiply_cpu_restatement_is_bitwise_the_reference(ref, m, n, k):
    """oracle.local_multiply_cpu restates local_multiply.cpp:278-297; same loop, same bits."""
    rng = np.random.default_rng(m * 1000 + n * 10 + k)
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    for alpha, beta in ((1.0, 1.0), (1.5, -0.25), (-2.0, 0.0)):
        mine = C0.copy(order="F")
        oracle.local_multiply_cpu(A, B, mine, alpha, beta)
        theirs = C0.copy(order="F")
        ref.ref_local_multiply_cpu_d(_p(A), _p(B), _p(theirs), m, n, k, alpha, beta)
        np.testing.assert_array_equal(mine, theirs)


def test_numroc_restatement_is_the_reference(ref):
    """oracle.numroc restates scalapack.cpp:49-88 on every small case."""
    for n in range(0, 41):
        for nb in range(1, 8):
            for nprocs in range(1, 6):
                for isrc in range(nprocs):
                    for iproc in range(nprocs):
                        assert oracle.numroc(n, nb, iproc, isrc, nprocs) == ref.ref_numroc(n, nb, iproc, isrc, nprocs)


def test_block_cyclic_fixture_sizes_are_the_references(ref):
    """tests/golden/block_cyclic.npz local sizes come out of the reference's numroc."""
    for c in _load("block_cyclic.npz")["cases"]:
        G = c["G"]
        assert c["lr"] == ref.ref_numroc(G.shape[0], c["mb"], c["myrow"], c["rsrc"], c["prow"])
        assert c["lc"] == ref.ref_numroc(G.shape[1], c["nb"], c["mycol"], c["csrc"], c["pcol"])


@pytest.mark.parametrize("idx", range(8))
def test_exact_fixtures_against_the_references_cpu_path(ref, idx):
    """The golden GEMM fixtures against the reference's two CPU paths: the
    CPU build's local_multiply (cosma::gemm -> cblas_dgemm) and the naive
    checker loop, each within the sequential-accumulation bound."""
    c = _load("gemm_exact.npz")["cases"][idx]
    A, B = _ops(c)
    m, k = A.shape
    n = B.shape[1]
    bound = (k + 2) * 2.0 ** -53 * (abs(c["alpha"]) * np.abs(A) @ np.abs(B) + abs(c["beta"]) * np.abs(c["C"])) + 1e-300
    for fn in (ref.ref_local_multiply_d, ref.ref_local_multiply_cpu_d):
        Cm = np.asfortranarray(c["C"].copy())
        fn(_p(A), _p(B), _p(Cm), m, n, k, c["alpha"], c["beta"])
        assert np.all(np.abs(Cm - c["expected"]) <= bound)
    # and the oracle's BLAS-semantics gemm agrees with the reference's cosma::gemm
    mine = np.asfortranarray(c["C"].copy())
    oracle.gemm("N", "N", c["alpha"], A, B, c["beta"], mine)
    theirs = np.asfortranarray(c["C"].copy())
    ref.ref_local_multiply_d(_p(A), _p(B), _p(theirs), m, n, k, c["alpha"], c["beta"])
    assert np.all(np.abs(mine - theirs) <= 2 * bound)


def test_complex_gemm_against_the_references_cosma_gemm(ref):
    m, n, k = 9, 7, 11
    A = oracle.uniform((m, k), 1, dtype=np.complex128)
    B = oracle.uniform((k, n), 2, dtype=np.complex128)
    C0 = oracle.uniform((m, n), 3, dtype=np.complex128)
    al, be = 1.0 - 0.5j, 0.25 + 1j
    mine = C0.copy(order="F")
    oracle.gemm("N", "N", al, A, B, be, mine)
    theirs = C0.copy(order="F")
    a2 = np.array([al.real, al.imag])
    b2 = np.array([be.real, be.imag])
    ref.ref_gemm_z(m, n, k, _p(a2), _p(A), m, _p(B), k, _p(b2), _p(theirs), m)
    assert np.max(np.abs(mine - theirs)) < 1e-13
