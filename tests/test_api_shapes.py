"""Shape checks of the host-side wrappers (api.AdcGpu), on the CPU.  Arrays
cross the C ABI as bare pointers, so a wrong length must be refused before
the library is called; a wrapper object with no context stands in for a
built one (the checks run before any library call)."""
import numpy as np
import pytest


@pytest.fixture
def fake():
    from adc_ottawa_gb300.api import AdcGpu

    g = AdcGpu.__new__(AdcGpu)          # no device context: only the checks can run
    g._h = None
    g.nocc, g.nvirt, g.ndim, g.noffd = 2, 3, 20, 0
    return g


@pytest.mark.parametrize("call", [
    lambda g: g.sigma(np.zeros(19)),
    lambda g: g.sigma(np.zeros((21, 2))),
    lambda g: g.lancdiag_block(np.zeros((19, 2)), 3),
    lambda g: g.lancdiag_block(np.zeros(20), 3),
    lambda g: g.silstep(np.zeros(20, complex), np.zeros(19, complex), 0.1, 5, 1e-8),
    lambda g: g.propagate_fvec(np.zeros((20, 0)), 0.1, 0.2, 5, 1e-8),
    lambda g: g.chebyshev_auto(np.zeros(21), [0.0, 1.0], 4),
    lambda g: g.chebyshev_auto(np.zeros(20), [0.0, 1.0, 2.0], 4),
    lambda g: g.project_psi0(np.zeros((20, 2)), [0.0], 4, 0.5),
])
def test_wrong_shapes_are_refused(built, fake, call):
    from adc_ottawa_gb300 import AdcGpuError

    with pytest.raises(AdcGpuError) as ei:
        call(fake)
    assert ei.value.code == 12


def test_batch_schedule_largest_first():
    """The batch driver submits systems largest first (by the stored values a
    sigma product streams) and returns results in the caller's order."""
    from adc_ottawa_gb300 import batch

    systems = batch.seeded_systems(64)
    order = batch.schedule(systems, 8)
    assert sorted(order) == list(range(64))
    w = [batch.work_estimate(systems[i][0], systems[i][1]) for i in order]
    assert all(a >= b for a, b in zip(w, w[1:]))
    # the smallest system's work is a small fraction of the largest's
    assert w[-1] < 0.05 * w[0]
