"""CPU checks of the oracle (the FP64 restatement of the reference path).

The reference cannot run here (Fortran, no compiler) and ships no vectors
for this path, so the oracle is pinned by independent mathematics:
dense eigendecomposition of the assembled matrix, exact propagation, the
closed-form structure of the coupling block, and the reference's own
heapsort tie order.
"""
import numpy as np
import pytest

import oracle
from tests.conftest import system


@pytest.fixture(scope="module")
def cfg1(built):
    no, nv = 5, 19
    e, eri = system(no, nv, 1234)
    M = oracle.Matrix.build(no, nv, e, eri)
    return no, nv, e, eri, M


def structural_nnz(no, nv):
    n1 = no * nv
    pv, po = nv * (nv - 1) // 2, no * (no - 1) // 2
    return (n1 * (n1 - 1) // 2 + no * nv * (no + nv - 1) + pv * no * (2 * no + nv - 2)
            + po * nv * (no + 2 * nv - 2) + 2 * po * pv * (2 * no + 2 * nv - 4))


def test_config1_dimensions(cfg1):
    no, nv, e, eri, M = cfg1
    assert M.ndim == 4655
    # every structural element is far above minc for this seed
    assert M.nnz == structural_nnz(no, nv) == 188005


def test_kpq_layout(built):
    kpq = oracle.select(3, 5)
    n1 = 15
    assert tuple(kpq[0, :5]) == (15, 15, 30, 15, 30)
    # first single (a=4, j=1), first class-1 double (a=b=4, i=j=1)
    assert tuple(kpq[1]) == (1, 1, 1, -1, 4, -1, 0)
    assert tuple(kpq[n1 + 1]) == (2, 1, 1, 1, 4, 4, 1)
    # 4II block is the 4I block with spin 12 and type 5
    c4 = 30
    s4 = 1 + n1 + 15 + 30 + 15
    a = kpq[s4:s4 + c4].copy()
    b = kpq[s4 + c4:s4 + 2 * c4].copy()
    assert np.all(a[:, 1] == 11) and np.all(b[:, 1] == 12) and np.all(b[:, 6] == 5)
    a[:, [1, 6]] = 0
    b[:, [1, 6]] = 0
    assert np.array_equal(a, b)


def test_coincidence_structure(cfg1):
    """Every kept ph-2p2h element satisfies a in {a',b'} or k in {k',l'}."""
    no, nv, e, eri, M = cfg1
    kpq = oracle.select(no, nv)
    d, h, oi, oj = M.coo()
    cp = oj > no * nv
    s, t = kpq[oi[cp]], kpq[oj[cp]]
    a, k = s[:, 4], s[:, 2]
    ok = (a == t[:, 4]) | (a == t[:, 5]) | (k == t[:, 2]) | (k == t[:, 3])
    assert ok.all()
    assert np.all(oi < oj)
    assert np.all(np.abs(h) > 1e-12)


def test_davidson_matches_dense(cfg1):
    no, nv, e, eri, M = cfg1
    w = np.linalg.eigh(M.dense())[0]
    for precon in (1, 2):
        for deflate in (True, False):
            st, ev, _, info = M.davidson(6, 1e-8, precon=precon, deflate=deflate)
            assert st == 0
            assert np.abs(ev - w[:6]).max() < 1e-10, (precon, deflate, ev - w[:6])


def test_davidson_subdiag_guess(cfg1):
    no, nv, e, eri, M = cfg1
    w = np.linalg.eigh(M.dense())[0]
    st, ev, vecs, info = M.davidson(6, 1e-8, subdiag=True, guessdim=200, want_vectors=True)
    assert st == 0 and np.abs(ev - w[:6]).max() < 1e-10
    H = M.dense()
    r = H @ vecs - vecs * ev
    assert np.linalg.norm(r, axis=0).max() < 1e-7


def test_lanczos_moments_match_dense(cfg1):
    no, nv, e, eri, M = cfg1
    H = M.dense()
    b, ncyc = 3, 8
    q0 = np.random.RandomState(3).rand(M.ndim, b)
    T, ev = M.block_lanczos(q0, ncyc, orthotype=0)
    Q = np.linalg.qr(q0)[0]
    Tk = np.eye(T.shape[0])[:, :b]
    Hk = Q.copy()
    for k in range(1, 2 * ncyc):
        Tk = T @ Tk
        Hk = H @ Hk
        mT, mH = np.trace(Tk[:b]), np.trace(Q.T @ Hk)
        assert abs(mT - mH) <= 1e-11 * abs(mH)
    # extreme Ritz values bound the spectrum
    w = np.linalg.eigvalsh(H)
    assert ev[0] >= w[0] - 1e-10 and ev[-1] <= w[-1] + 1e-10


def test_lanczos_pro_keeps_orthogonality(cfg1):
    no, nv, e, eri, M = cfg1
    q0 = np.random.RandomState(5).rand(M.ndim, 2)
    T0, ev0 = M.block_lanczos(q0, 40, orthotype=0)
    T1, ev1 = M.block_lanczos(q0, 40, orthotype=1)
    w = np.linalg.eigvalsh(M.dense())
    # with PRO the lowest Ritz value converges to the true lowest eigenvalue
    assert abs(ev1[0] - w[0]) < 1e-6


def test_sil_autocorrelation_exact(cfg1):
    no, nv, e, eri, M = cfg1
    H = M.dense()
    w, V = np.linalg.eigh(H)
    f = np.random.RandomState(2).rand(M.ndim)
    st, a, nmult = M.autocorr(f, tout=0.5, tfinal=10.0, kdim=12, tol=1e-10)
    assert st == 0 and len(a) == 41
    c = V.T @ f
    ts = np.arange(len(a)) * 0.5
    ex = np.array([np.sum(c * c * np.exp(-1j * w * t)) for t in ts])
    assert np.abs(a - ex).max() <= 1e-8 * np.abs(ex).max()


def test_heapsort_tie_order(built):
    # ties resolve in heap order (NR heapsort), not stably
    idx = oracle.heapsort_index(np.array([2.0, 1.0, 2.0, 1.0, 2.0, 1.0]))
    assert sorted(idx[:3]) == [2, 4, 6]
    assert list(idx) == list(oracle.heapsort_index(np.array([2.0, 1.0, 2.0, 1.0, 2.0, 1.0])))
