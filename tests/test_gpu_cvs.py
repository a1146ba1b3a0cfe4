"""The CVS ADC(2)-s matrix on the GPU (adcgpu_build_adc2s_cvs, replacing
write_fspace_adc2_1_cvs, fspacetrial.f90:566-596) against the oracle's
restatement of get_offdiag_adc2_save_cvs_omp (get_matrix.f90:1323-1726):
diagonal and kept elements bit for bit, the FP64 sigma product, Davidson,
block Lanczos from the CVS f-vector, and the SCRATCH files."""
import os

import numpy as np
import pytest

import oracle
from tests.conftest import sorted_coo, system

pytestmark = pytest.mark.gpu

CASES = [(5, 19, [1, 2], 1234), (8, 40, [1], 3), (6, 30, [2, 5], 11)]


def _cvs(no, nv, core, seed):
    from adc_ottawa_gb300 import AdcGpu

    e, eri = system(no, nv, seed)
    g = AdcGpu(0)
    g.set_orbitals(no, nv, e)
    g.set_eri_packed(eri)
    noffd = g.write_fspace_adc2_1_cvs(core)
    return g, e, eri, noffd


@pytest.mark.parametrize("no,nv,core,seed", CASES)
def test_cvs_build_matches_oracle(gpu, no, nv, core, seed):
    g, e, eri, noffd = _cvs(no, nv, core, seed)
    ref = oracle.Matrix.build_cvs(no, nv, e, eri, core)
    d_ref, h_ref, i_ref, j_ref = ref.coo()
    assert g.ndim == ref.ndim
    assert np.array_equal(g.get_diag(), d_ref)
    assert noffd == ref.nnz
    h, oi, oj = g.export_coo()
    a = sorted_coo(h, oi, oj)
    b = sorted_coo(h_ref, i_ref, j_ref)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert np.array_equal(a[0], b[0])
    x = np.random.RandomState(no).rand(g.ndim, 21)      # a group of 16, then 4 and 1
    y = g.sigma(x)
    assert np.abs(y - ref.matvec(x)).max() <= 1e-13 * np.abs(y).max()
    g.close()


def test_cvs_davidson_and_refusals(gpu):
    from adc_ottawa_gb300 import ADCGPU_MIXED, PRECON_FOLD, AdcGpuError

    no, nv, core, seed = 6, 30, [2, 5], 11
    g, e, eri, _ = _cvs(no, nv, core, seed)
    res = g.davdiag_block(6, 1e-8)
    st, ev, _, _ = oracle.Matrix.build_cvs(no, nv, e, eri, core).davidson(6, 1e-8)
    assert res.status == 0 and st == 0
    assert np.abs(res.evals - ev).max() < 1e-8
    for kw in ({"precision": ADCGPU_MIXED}, {"precon": PRECON_FOLD}, {"lsubdiag": 1}):
        with pytest.raises(AdcGpuError) as ei:
            g.davdiag_block(6, 1e-8, **kw)
        assert ei.value.code == 16
    g.close()


def test_cvs_fvector_lanczos_and_files(gpu, tmp_path):
    """The CVS f-vector (get_modifiedtm_adc2 with lcvs) against the oracle,
    the block Lanczos started from it (lancguess = 1), and hmlt files with
    the reference's record layout."""
    from adc_ottawa_gb300 import lanczos_guess_vecs, select_adc2s_cvs, synth_dipole

    no, nv, core, seed = 5, 19, [1, 2], 1234
    g, e, eri, noffd = _cvs(no, nv, core, seed)
    dpl = synth_dipole(no + nv, seed + 1)
    g.set_dipole(dpl)
    kpq = select_adc2s_cvs(no, nv, core)
    f = g.get_modifiedtm_adc2(kpq)
    f_ref = oracle.modified_tm_adc2(no, nv, e, eri, dpl, kpq=kpq)
    n1 = len(core) * nv
    assert np.array_equal(f[n1:], f_ref[n1:])
    assert np.abs(f[:n1] - f_ref[:n1]).max() <= 1e-12 * np.abs(f_ref[:n1]).max()
    Q = lanczos_guess_vecs(f, n1, 4, lancguess=1)
    _, ev, _ = g.lancdiag_block(Q, 8)
    _, ev_ref = oracle.Matrix.build_cvs(no, nv, e, eri, core).block_lanczos(Q, 8)
    assert np.abs(ev - ev_ref).max() <= 1e-9 * np.abs(ev_ref).max()
    g.write_hmlt_files(str(tmp_path), "c")
    off = os.path.getsize(tmp_path / "hmlt.offc")
    rec = 8 + 655360 * 16 + 4
    assert off == rec * (noffd // 655360 + 1)
    assert os.path.getsize(tmp_path / "hmlt.diac") == (8 + 8) + (8 + 8 * g.ndim)
    g.close()
