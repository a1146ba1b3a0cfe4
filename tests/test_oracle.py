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


def _cheb_exact(w, c, bounds, nk):
    """sum_j c_j T_k(x_j), x = the eigenvalues mapped by matxvec_chebyshev."""
    dE = bounds[1] - bounds[0]
    x = (2.0 / dE) * w - (2.0 * (bounds[0] / dE) + 1.0)
    T = np.zeros((nk, len(w)))
    T[0] = 1.0
    if nk > 1:
        T[1] = x
    for k in range(2, nk):
        T[k] = 2.0 * x * T[k - 1] - T[k - 2]
    return T @ c, T


@pytest.mark.parametrize("chebyord", [40, 41])
def test_chebyshev_auto_exact(cfg1, chebyord):
    """C_k of chebyshev_auto (direct for k <= ord, doubling formulas above)
    against sum_j <v_j|q0>^2 T_k(x_j) from a dense eigendecomposition; an odd
    order is rounded down to even as chebyshev_initialise does."""
    no, nv, e, eri, M = cfg1
    w, V = np.linalg.eigh(M.dense())
    bounds = np.array([w[0] - 0.2, 1.1 * w[-1]])
    q0 = np.random.RandomState(3).uniform(size=M.ndim)
    a, q1 = M.chebyshev_auto(q0, bounds, chebyord, n1=no * nv)
    assert len(a) == 81 and q1.shape == (no * nv, 41)
    ex, _ = _cheb_exact(w, (V.T @ q0) ** 2, bounds, len(a))
    assert np.abs(a - ex).max() <= 1e-12 * a[0]
    assert np.array_equal(q1[:, 0], q0[: no * nv])
    # q_1 = H_norm q_0
    dE = bounds[1] - bounds[0]
    q1_ref = (2.0 / dE) * M.matvec(q0)[:, 0] - (2.0 * (bounds[0] / dE) + 1.0) * q0
    assert np.abs(q1[:, 1] - q1_ref[: no * nv]).max() <= 1e-13 * np.abs(q1_ref).max()


def test_chebyshev_project_exact(cfg1):
    """project_psi0 equals V diag(sum_k f_k g_k T_k(x_j)) V^T q0."""
    no, nv, e, eri, M = cfg1
    w, V = np.linalg.eigh(M.dense())
    bounds = np.array([w[0] - 0.2, 1.1 * w[-1]])
    ord_, projen = 60, 0.5 * (w[0] + w[-1])
    q0 = np.random.RandomState(4).uniform(size=M.ndim)
    pq = M.chebyshev_project(q0, bounds, ord_, projen)
    dE = bounds[1] - bounds[0]
    es = 2.0 * ((projen - (0.5 * dE + bounds[0])) / dE)
    al = np.pi / (ord_ + 2)
    k = np.arange(ord_ + 1)
    gk = ((1 - k / (ord_ + 2)) * np.sin(al) * np.cos(k * al) + np.cos(al) * np.sin(k * al) / (ord_ + 2)) / np.sin(al)
    fk = np.empty(ord_ + 1)
    fk[0] = 1 - np.arccos(es) / np.pi
    fk[1:] = -2 * np.sin(k[1:] * np.arccos(es)) / (k[1:] * np.pi)
    _, T = _cheb_exact(w, np.zeros(len(w)), bounds, ord_ + 1)
    filt = (fk * gk) @ T
    ref = V @ (filt * (V.T @ q0))
    assert np.abs(pq - ref).max() <= 1e-11 * np.abs(ref).max()
    # the filter passes the lower half of the spectrum (step at projen)
    assert filt[w < projen - 3.0].min() > 0.95 and np.abs(filt[w > projen + 3.0]).max() < 0.05


def test_spectral_bounds_match_dense(cfg1):
    """spectral_bounds_davlanc: Davidson lowest and Lanczos highest eigenvalue."""
    no, nv, e, eri, M = cfg1
    w = np.linalg.eigvalsh(M.dense())
    st, b = M.spectral_bounds()
    assert st == 0
    assert abs(b[0] - w[0]) <= 1e-10 and abs(b[1] - w[-1]) <= 1e-9


def test_singlesubspace_block(cfg1):
    """init_vec_singlesubspace: orthonormal columns supported on the 800
    configurations of largest hii."""
    no, nv, e, eri, M = cfg1
    q = M.singlesubspace_block(2)
    diag = M.coo()[0]
    thr = np.sort(diag)[::-1][799]
    support = np.flatnonzero(np.abs(q).sum(1))
    assert 400 <= len(support) and np.all(diag[support] >= thr - 1e-4)
    assert np.allclose(q.T @ q, np.eye(2), atol=1e-12)


def test_adc1_guess_oracle():
    """initvec_adc1 (block_davidson.f90:246-289): the ADC(1) singles matrix
    (K_ph_ph + C1_ph_ph, get_matrix.f90:17-82) is symmetric, its diagonal is
    e_a - e_k + 2(ak|ak) - (aa|kk), and a Davidson started from its lowest
    eigenvectors converges to the same roots as the on-diagonal guess."""
    from adc_ottawa_gb300 import synth_system

    no, nv = 4, 9
    e, eri = synth_system(no, nv, 7)
    A = oracle.adc1_matrix(no, nv, e, eri)
    assert np.array_equal(A, A.T)
    M = oracle.Matrix.build(no, nv, e, eri)
    G = oracle.adc1_guess(no, nv, e, eri, M.ndim, 9)
    assert np.abs(G.T @ G - np.eye(9)).max() < 1e-12 and not G[no * nv:].any()
    st, ev, _, _ = M.davidson(4, 1e-9, guess=G)
    st2, ev2, _, _ = M.davidson(4, 1e-9)
    assert st == 0 and st2 == 0
    assert np.abs(ev - ev2).max() < 1e-10


def test_direct_path_matrix_equals_stored():
    """The direct (matvec) path's ph-ph formulas Ca1/Cb1/Cc1/Cc2
    (adc_ph.f90:98-303) are algebraically the stored path's CA/CB/CC
    (DC = (x+y)/(2xy) = (1/x + 1/y)/2): the oracle's direct matrix has the
    same coupling block bit for bit, its ph-ph block agrees to roundoff, and
    the spectra agree."""
    from adc_ottawa_gb300 import synth_system

    no, nv = 4, 9
    e, eri = synth_system(no, nv, 7)
    Hs = oracle.Matrix.build(no, nv, e, eri).dense()
    Hd = oracle.Matrix.build_direct(no, nv, e, eri).dense()
    n1 = no * nv
    assert np.array_equal(Hs[:n1, n1:], Hd[:n1, n1:]) and np.array_equal(Hs[n1:, n1:], Hd[n1:, n1:])
    assert np.abs(Hs[:n1, :n1] - Hd[:n1, :n1]).max() <= 1e-13 * np.abs(Hs[:n1, :n1]).max()
    ws, wd = np.linalg.eigvalsh(Hs), np.linalg.eigvalsh(Hd)
    assert np.abs(ws - wd).max() <= 1e-12 * np.abs(ws).max()
