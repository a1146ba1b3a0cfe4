"""The ADC(2) f-vector on the GPU (adcgpu_modified_tm_adc2, replacing
get_modifiedtm_adc2, get_moment.f90:153-442) against the oracle's
reference-order restatement, and its use as the start vector of the
final-space Lanczos (lanczos_guess_vecs, adc2_opa.f90:380-520) and of the
wavepacket propagation (init_wavepacket, fvecprop.f90:338-357)."""
import numpy as np
import pytest

import oracle
from tests.conftest import system

pytestmark = pytest.mark.gpu

# The 2h2p entries follow the reference's expression order under --fmad=false:
# bit-exact.  The 1h1p entries are regrouped into FP64 contractions:
# within 1e-12 of the largest entry.
SINGLES_RTOL = 1e-12


def _ctx(no, nv, seed, complex_eri=False):
    from adc_ottawa_gb300 import AdcGpu, synth_dipole

    e, eri = system(no, nv, seed)
    g = AdcGpu(0)
    g.set_orbitals(no, nv, e)
    if complex_eri:
        nb = no + nv
        full = np.zeros((nb, nb, nb, nb), order="F")
        idx = np.arange(nb)
        P, Q = np.maximum.outer(idx, idx), np.minimum.outer(idx, idx)
        pq = (P * (P + 1) // 2 + Q)
        for r in range(nb):
            for s in range(nb):
                a = np.maximum(pq[r, s], pq)
                b = np.minimum(pq[r, s], pq)
                full[r, s] = eri[a * (a + 1) // 2 + b]
        buf = np.zeros((nb, nb, nb, nb), np.complex128, order="F")
        buf.real[...] = full
        g.set_eri_mo_complex(buf)
    else:
        g.set_eri_packed(eri)
    dpl = synth_dipole(no + nv, seed + 1)
    g.set_dipole(dpl)
    return g, e, eri, dpl


@pytest.mark.parametrize("no,nv,seed", [(5, 19, 1234), (8, 40, 3), (3, 60, 7)])
def test_fvector_matches_oracle(gpu, no, nv, seed):
    g, e, eri, dpl = _ctx(no, nv, seed)
    got = g.get_modifiedtm_adc2()
    ref = oracle.modified_tm_adc2(no, nv, e, eri, dpl)
    n1 = no * nv
    assert np.array_equal(got[n1:], ref[n1:])
    assert np.abs(got[:n1] - ref[:n1]).max() <= SINGLES_RTOL * np.abs(ref[:n1]).max()
    g.close()


def test_fvector_complex_layout_and_errors(gpu):
    """The reference ERI layout gives the same f-vector bit for bit; a
    missing dipole matrix and a foreign kpq are refused."""
    from adc_ottawa_gb300 import AdcGpu, AdcGpuError, select_adc2s

    no, nv, seed = 4, 13, 21
    g1, _, _, _ = _ctx(no, nv, seed)
    g2, _, _, _ = _ctx(no, nv, seed, complex_eri=True)
    a = g1.get_modifiedtm_adc2()
    kpq = select_adc2s(no, nv)
    assert np.array_equal(a, g2.get_modifiedtm_adc2(kpq))
    bad = kpq.copy()
    bad[no * nv + 1, 4] += 1
    with pytest.raises(AdcGpuError) as ei:
        g1.get_modifiedtm_adc2(bad)
    assert ei.value.code == 16
    e, eri = system(no, nv, seed)
    h = AdcGpu(0)
    h.set_orbitals(no, nv, e)
    h.set_eri_packed(eri)
    with pytest.raises(AdcGpuError) as ei:
        h.get_modifiedtm_adc2()
    assert ei.value.code == 12
    for x in (g1, g2, h):
        x.close()


def test_fvector_starts_lanczos_and_propagation(gpu):
    """lancguess = 1 start block from the GPU f-vector: the Lanczos T matrix
    equals the oracle's from the oracle f-vector's block (first cycles); the
    wavepacket autocorrelation from the f-vector equals the oracle's."""
    from adc_ottawa_gb300 import ADCGPU_FP64, lanczos_guess_vecs

    no, nv, seed = 5, 19, 1234
    g, e, eri, dpl = _ctx(no, nv, seed)
    g.write_fspace_adc2_1(None, precision=ADCGPU_FP64)
    f = g.get_modifiedtm_adc2()
    f_ref = oracle.modified_tm_adc2(no, nv, e, eri, dpl)
    n1, lmain, ncyc = no * nv, 4, 6
    Q = lanczos_guess_vecs(f, n1, lmain, lancguess=1)
    assert np.array_equal(Q, lanczos_guess_vecs(f_ref, n1, lmain, lancguess=1))
    T, ev, _ = g.lancdiag_block(Q, ncyc)
    M = oracle.Matrix.build(no, nv, e, eri)
    T_ref, ev_ref = M.block_lanczos(Q, ncyc)
    # T equals the oracle's up to a block-diagonal sign similarity (the QR
    # sign conventions): compare eigenvalues and first-block moments
    assert np.abs(ev - ev_ref).max() <= 1e-9 * np.abs(ev_ref).max()
    Tk, Trk = np.eye(lmain * ncyc)[:, :lmain], np.eye(lmain * ncyc)[:, :lmain]
    for _ in range(1, 2 * ncyc):
        Tk, Trk = T @ Tk, T_ref @ Trk
        assert np.abs(Tk[:lmain] - Trk[:lmain]).max() <= 1e-10 * np.abs(Trk[:lmain]).max()
    a, _ = g.propagate_fvec(f, 0.5, 4.0, 12, 1e-9)
    st, a_ref, _ = M.autocorr(f_ref, 0.5, 4.0, 12, 1e-9)
    assert st == 0 and a.shape[1] == len(a_ref)
    assert np.abs(a[0] - a_ref).max() <= 1e-7 * np.abs(a_ref).max()
    g.close()
