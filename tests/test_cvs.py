"""CVS configuration list and the oracle's CVS builder, on CPU.

select_atom_is_cvs / select_atom_d_cvs (select_fano.f90:112-142, 903-1027)
and write_fspace_adc2_1_cvs (fspacetrial.f90:566-596).  The CVS matrix uses
the ADC(2)-s formulas on a subset of the configurations, so it is the
principal submatrix of the ADC(2)-s matrix on those configurations; the
oracle's two builders agreeing on it checks both loop structures."""
import numpy as np
import pytest

import oracle


def test_select_cvs_matches_oracle(built):
    import adc_ottawa_gb300 as ag

    for no, nv, core in [(5, 19, [1, 2]), (6, 11, [3]), (4, 9, [1, 2, 4])]:
        a = ag.select_adc2s_cvs(no, nv, core)
        b = oracle.select_cvs(no, nv, core)
        assert np.array_equal(a, b)
        n1 = len(core) * nv
        assert a[0, 0] == n1 and a[0, 1] == 0 and a[0, 2] == 0
        holes = a[1:, 2:4]
        d = a[n1 + 1:]
        incore = np.isin(d[:, 2], core).astype(int) + np.isin(d[:, 3], core).astype(int)
        assert np.all(incore == 1)                       # exactly one core hole per double
        assert set(holes[:n1, 0]) == set(core)
        assert np.all(d[:, 6] >= 3)                      # no i=j classes


def test_select_cvs_rejects_bad_core(built):
    import adc_ottawa_gb300 as ag

    for core in ([], [0], [6], [2, 2], [1, 2, 3, 4, 5]):
        with pytest.raises(ag.AdcGpuError):
            ag.select_adc2s_cvs(5, 10, core)


@pytest.mark.parametrize("no,nv,core,seed", [(5, 19, [1, 2], 3), (6, 13, [2], 8)])
def test_cvs_matrix_is_principal_submatrix(no, nv, core, seed):
    e, eri = oracle.synth_system(no, nv, seed)
    full = oracle.Matrix.build(no, nv, e, eri).dense()
    cvs = oracle.Matrix.build_cvs(no, nv, e, eri, core)
    H = cvs.dense()
    kf = oracle.select(no, nv)
    kc = oracle.select_cvs(no, nv, core)
    pos = {tuple(r): i for i, r in enumerate(kf[1:])}
    idx = np.array([pos[tuple(r)] for r in kc[1:]])
    sub = full[np.ix_(idx, idx)]
    assert np.abs(H - sub).max() <= 1e-14 * np.abs(sub).max()
    d, _, _, _ = cvs.coo()
    assert np.array_equal(d, np.diag(full)[idx])
