"""The ADC(2) f-vector (get_modifiedtm_adc2, get_moment.f90:153-442) on CPU.

The oracle restates the reference's loops term by term (oracle/fvector.cpp).
The GPU computes the 1h1p block as dense contractions over pair matrices
(adc_ottawa_gb300/csrc/fvec.cu).  fvec_factored below is a numpy statement
of exactly those contractions; agreeing with the oracle to rounding checks
the regrouping of every F/tau term before any GPU runs it.
"""
import numpy as np
import pytest

import oracle


def full_eri(nbas, eri):
    idx = np.arange(nbas)
    P = np.maximum.outer(idx, idx)
    Q = np.minimum.outer(idx, idx)
    pq = (P * (P + 1) // 2 + Q).ravel()
    A = np.maximum.outer(pq, pq)
    B = np.minimum.outer(pq, pq)
    return eri[A * (A + 1) // 2 + B].reshape(nbas, nbas, nbas, nbas)


def fvec_factored(no, nv, e, eri, dpl):
    """The 1h1p f-vector through the pair-matrix contractions of fvec.cu."""
    nb = no + nv
    V = full_eri(nb, eri)
    o, v = slice(0, no), slice(no, nb)
    eo, ev = e[:no], e[no:]
    dvo, dov, dvv, doo = dpl[v, o], dpl[o, v], dpl[v, v], dpl[o, o]
    vovo, vvoo, ooov, vvov = V[v, o, v, o], V[v, v, o, o], V[o, o, o, v], V[v, v, o, v]
    vvvv, oooo = V[v, v, v, v], V[o, o, o, o]
    n1 = no * nv
    M = lambda X: X.reshape(n1, n1)  # noqa: E731
    D = eo[None, :, None, None] + eo[None, None, None, :] - ev[:, None, None, None] - ev[None, None, :, None]
    T = (2 * vovo - vovo.transpose(0, 3, 2, 1)) / D
    Km = 2 * vovo - vvoo.transpose(0, 2, 1, 3)
    X2 = vvoo.transpose(0, 2, 1, 3)
    Tsw = T.transpose(0, 3, 2, 1)
    A1 = vovo / D
    L2 = vovo.transpose(0, 3, 2, 1) / D
    J = 2 * np.einsum("bakl->akbl", vvoo) - vovo
    Z = (M(Km) @ M(T) + M(T) @ M(Km)).reshape(nv, no, nv, no)
    Y = (M(vovo) @ M(T) + M(X2) @ M(Tsw) + M(A1) @ M(Km) + M(L2) @ M(J)).reshape(nv, no, nv, no)
    R = dov.T[None, None, :, :] / D            # d(l,b) / D(ak,bl) as [a,k,b,l]
    f2526 = (Z * R).sum(axis=(2, 3))
    f2728 = -np.einsum("albk,akbl->ak", Y, R)
    Dmn = eo[:, None, None, None] + eo[None, :, None, None] - ev[None, None, :, None] - ev[None, None, None, :]
    W = np.einsum("acbd,ckdl->abkl", vvvv, T)
    W += np.einsum("ambn,mnab,mnkl->abkl", vovo, 1.0 / Dmn,
                   2 * oooo.transpose(0, 2, 1, 3) - oooo.transpose(0, 2, 3, 1))
    f29 = np.einsum("abkl,akbl->ak", W, R)
    f0 = np.einsum("akbl,bl->ak", T, dvo)
    fc = np.einsum("akbl,bl->ak", T, 0.5 * f0)
    tauA = -0.5 * np.einsum("clbm,albm->ca", T, A1)
    tauB = -0.5 * np.einsum("bmcl,bkcl->mk", T, A1)
    G21 = 2 * np.einsum("aclb->albc", vvov) - np.einsum("ablc->albc", vvov)
    tau21 = -np.einsum("blcm,albc->am", A1, G21) / (eo[None, :] - ev[:, None])
    tau22 = np.einsum("mnlb,blam->an", ooov, T) / (eo[None, :] - ev[:, None])
    tau23 = -np.einsum("blcm,lkmc->bk", A1, 2 * ooov - ooov.transpose(2, 1, 0, 3)) / (eo[None, :] - ev[:, None])
    tau24 = np.einsum("bkcl,dblc->dk", A1, 2 * vvov - np.einsum("dclb->dblc", vvov)) / (eo[None, :] - ev[:, None])
    tot = (dvo + f0 + f2526 + f2728 + f29 + np.einsum("ca,ck->ak", tauA, dvo) + dvo @ tauB + fc
           + tau21 @ doo + tau22 @ doo + dvv @ tau23 + dvv @ tau24)
    return -np.sqrt(2.0) * tot.reshape(-1)


@pytest.mark.parametrize("no,nv,seed", [(3, 7, 5), (5, 19, 11), (6, 23, 2)])
def test_factored_singles_match_reference_loops(no, nv, seed):
    e, eri = oracle.synth_system(no, nv, seed)
    dpl = oracle.synth_dipole(no + nv, seed + 1)
    ref = oracle.modified_tm_adc2(no, nv, e, eri, dpl, sections=1)[: no * nv]
    got = fvec_factored(no, nv, e, eri, dpl)
    # FP64 regrouping only: 1e-13 of the largest entry
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def test_oracle_sections_are_independent():
    no, nv = 4, 11
    e, eri = oracle.synth_system(no, nv, 7)
    dpl = oracle.synth_dipole(no + nv, 8)
    both = oracle.modified_tm_adc2(no, nv, e, eri, dpl, 3)
    s1 = oracle.modified_tm_adc2(no, nv, e, eri, dpl, 1)
    s2 = oracle.modified_tm_adc2(no, nv, e, eri, dpl, 2)
    n1 = no * nv
    assert np.array_equal(both[:n1], s1[:n1]) and np.all(s1[n1:] == 0)
    assert np.array_equal(both[n1:], s2[n1:]) and np.all(s2[:n1] == 0)
    # class IV2 = sqrt(3) (antisymmetric combination), IV1 symmetric: both present
    assert np.count_nonzero(both[n1:]) > 0.9 * (len(both) - n1)


def test_oracle_doubles_by_hand():
    """One entry of each 2h2p class recomputed from the dipole_ph.f90 formulas."""
    no, nv = 3, 5
    e, eri = oracle.synth_system(no, nv, 3)
    dpl = oracle.synth_dipole(no + nv, 4)
    V = full_eri(no + nv, eri)
    mtm = oracle.modified_tm_adc2(no, nv, e, eri, dpl, 2)
    kpq = oracle.select(no, nv)
    seen = set()
    for col in range(no * nv + 1, len(kpq)):
        k, j, a, b, typ = kpq[col, 2] - 1, kpq[col, 3] - 1, kpq[col, 4] - 1, kpq[col, 5] - 1, kpq[col, 6]
        if typ in seen:
            continue
        seen.add(typ)
        d = dpl
        if typ == 1:
            f = sum(-d[m, k] / (e[m] + e[k] - 2 * e[a]) * V[a, k, a, m] for m in range(no))
            f += sum(d[a, c] / (2 * e[k] - e[a] - e[c]) * V[c, k, a, k] for c in range(no, no + nv))
            f *= 2
        elif typ == 2:
            f = sum(-d[m, k] / (e[m] + e[k] - e[a] - e[b]) * (V[a, m, b, k] + V[a, k, b, m]) for m in range(no))
            f += sum(d[a, c] / (2 * e[k] - e[b] - e[c]) * V[c, k, b, k] + d[b, c] / (2 * e[k] - e[a] - e[c]) * V[c, k, a, k]
                     for c in range(no, no + nv))
            f *= np.sqrt(2)
        elif typ == 3:
            l = j  # noqa: E741
            f = sum(d[m, k] / (e[m] + e[l] - 2 * e[a]) * V[a, m, a, l] + d[m, l] / (e[k] + e[m] - 2 * e[a]) * V[a, k, a, m]
                    for m in range(no))
            f -= sum(d[a, c] / (e[k] + e[l] - e[a] - e[c]) * (V[c, k, a, l] + V[c, l, a, k]) for c in range(no, no + nv))
            f *= np.sqrt(2)
        else:
            l = j  # noqa: E741
            s = 1.0 if typ == 4 else -1.0
            f = sum(d[m, k] / (e[m] + e[l] - e[a] - e[b]) * (V[a, m, b, l] + s * V[a, l, m, b])
                    + d[m, l] / (e[k] + e[m] - e[a] - e[b]) * (V[a, k, m, b] + s * V[a, m, b, k]) for m in range(no))
            f -= sum(d[a, c] / (e[k] + e[l] - e[b] - e[c]) * (V[c, k, b, l] + s * V[c, l, b, k])
                     + d[b, c] / (e[k] + e[l] - e[a] - e[c]) * (V[c, l, a, k] + s * V[c, k, a, l]) for c in range(no, no + nv))
            if typ == 5:
                f *= np.sqrt(3)
        assert abs(f - mtm[col - 1]) <= 1e-14 * max(1.0, abs(f))
    assert seen == {1, 2, 3, 4, 5}


def test_synth_dipole_shared_and_symmetric(built):
    import adc_ottawa_gb300 as ag

    a = ag.synth_dipole(24, 9)
    b = oracle.synth_dipole(24, 9)
    assert np.array_equal(a, b)
    assert np.array_equal(a, a.T)
    assert 0.2 < np.abs(np.diag(a)).mean() < 0.8


def test_fill_stvc_order(built):
    import adc_ottawa_gb300 as ag

    rng = np.random.default_rng(0)
    v = rng.normal(size=200)
    v[17] = v[3] = 5.0       # a tie in v^2
    got = ag.fill_stvc(v, 12)
    ref = oracle.heapsort_index_desc(v * v)[:12]
    assert np.array_equal(got, ref)
    assert sorted(np.abs(v[got - 1])) == sorted(np.sort(np.abs(v))[-12:])
    Q = ag.lanczos_guess_vecs(v, 120, 4, lancguess=3)
    assert np.allclose(np.linalg.norm(Q, axis=0), 1.0)
    assert np.count_nonzero(Q[:120]) == 4 and np.count_nonzero(Q[120:]) == 4
