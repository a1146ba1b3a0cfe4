"""Host logic of chebyshev_auto_order_domain (chebyspec.f90:25-116) on the
CPU: chebyshev_auto_order_domain runs against a stand-in for the device context whose three
calls are answered by the oracle, so the widening of the bounds (:84-85), the
optional projection (:90), the even-order rounding and the output files are
checked without a GPU."""
import numpy as np
import pytest

import oracle
from tests.conftest import system


class OracleContext:
    """The three AdcGpu calls chebyshev_auto_order_domain makes, answered by the oracle."""

    def __init__(self, M, n1):
        self.M, self.n1, self.calls = M, n1, []

    def spectral_bounds(self, precon=2):
        self.calls.append(("bounds", precon))
        st, b = self.M.spectral_bounds(precon=precon)
        assert st == 0
        return b

    def project_psi0(self, q, b, chebyord, projen, df=False):
        self.calls.append(("project", chebyord, projen))
        q = np.asfortranarray(q).reshape(self.M.ndim, -1)
        return np.column_stack([self.M.chebyshev_project(q[:, p], b, chebyord, projen) for p in range(q.shape[1])])

    def chebyshev_auto(self, q, b, chebyord, save1h1p=False, df=False):
        self.calls.append(("auto", chebyord))
        q = np.asfortranarray(q).reshape(self.M.ndim, -1)
        res = [self.M.chebyshev_auto(q[:, p], b, chebyord, n1=self.n1 if save1h1p else 0) for p in range(q.shape[1])]
        auto = np.stack([r[0] for r in res])
        q1 = np.stack([r[1].T for r in res]) if save1h1p else None
        return auto, q1


@pytest.fixture(scope="module")
def ctx(built):
    no, nv = 5, 19
    e, eri = system(no, nv, 1234)
    return OracleContext(oracle.Matrix.build(no, nv, e, eri), no * nv)


def test_driver_estimates_and_widens(ctx, tmp_path):
    from adc_ottawa_gb300 import chebyshev_auto_order_domain

    q0 = np.random.RandomState(5).uniform(size=ctx.M.ndim)
    ctx.calls.clear()
    auto, q1, b = chebyshev_auto_order_domain(ctx, q0, 15, save1h1p=True, outdir=str(tmp_path))
    raw = ctx.M.spectral_bounds()[1]       # threaded oracle: equal to roundoff
    assert [c[0] for c in ctx.calls] == ["bounds", "auto"] and ctx.calls[1][1] == 15
    assert np.allclose(b, [0.9 * raw[0], 1.1 * raw[1]], rtol=1e-12, atol=0)
    assert auto.shape == (1, 29) and q1.shape == (1, 15, ctx.n1)       # order 15 -> 14
    lines = (tmp_path / "chebyauto").read_text().split("\n")
    assert lines[0].startswith("#    Spectral bounds:") and len(lines) == 3 + 29 + 1
    assert float(lines[3].split()[1].replace("E", "e")) == pytest.approx(auto[0, 0], rel=1e-13)
    raw_bytes = (tmp_path / "cheby1h1p").read_bytes()
    assert len(raw_bytes) == 15 * (8 * ctx.n1 + 8)
    first = np.frombuffer(raw_bytes[4:4 + 8 * ctx.n1], np.float64)
    assert np.array_equal(first, q0[: ctx.n1])


def test_driver_projects_first(ctx):
    from adc_ottawa_gb300 import chebyshev_auto_order_domain

    w = np.linalg.eigvalsh(ctx.M.dense())
    q0 = np.random.RandomState(6).uniform(size=ctx.M.ndim)
    given = np.array([w[0] - 0.5, w[-1]])
    projen = 0.5 * (w[0] + w[-1])
    ctx.calls.clear()
    auto, _, b = chebyshev_auto_order_domain(ctx, q0, 20, bounds=given, lprojpsi0=True, projen=projen)
    assert [c[0] for c in ctx.calls] == ["project", "auto"]
    pq = ctx.M.chebyshev_project(q0, b, 20, projen)
    ref, _ = ctx.M.chebyshev_auto(pq, b, 20)
    assert np.array_equal(auto[0], ref)
    # the filtered state keeps less weight than the unfiltered one
    assert auto[0, 0] < ctx.M.chebyshev_auto(q0, b, 20)[0][0]


@pytest.mark.parametrize("chebyord", [0, 1, 2, 3])
def test_low_orders(ctx, chebyord):
    """ord = chebyord rounded down to even; C_0 = |q0|^2, C_k = <q0|q_k> up to
    ord, and for ord = 2 the doubling formulas give C_3 = 2<q_1|q_2> - C_1 and
    C_4 = 2|q_2|^2 - C_0."""
    w = np.linalg.eigvalsh(ctx.M.dense())
    b = np.array([w[0] - 0.2, 1.1 * w[-1]])
    q0 = np.random.RandomState(7).uniform(size=ctx.M.ndim)
    a, _ = ctx.M.chebyshev_auto(q0, b, chebyord)
    o = chebyord - chebyord % 2
    assert len(a) == 2 * o + 1
    assert a[0] == pytest.approx(q0 @ q0, rel=1e-14)
    if o >= 2:
        dE = b[1] - b[0]
        q1 = (2.0 / dE) * ctx.M.matvec(q0)[:, 0] - (2.0 * (b[0] / dE) + 1.0) * q0
        q2 = 2.0 * ((2.0 / dE) * ctx.M.matvec(q1)[:, 0] - (2.0 * (b[0] / dE) + 1.0) * q1) - q0
        assert a[1] == pytest.approx(q0 @ q1, rel=1e-12)
        assert a[2] == pytest.approx(q0 @ q2, rel=1e-12)
        assert a[3] == pytest.approx(2 * (q1 @ q2) - a[1], rel=1e-12)
        assert a[4] == pytest.approx(2 * (q2 @ q2) - a[0], rel=1e-12)
