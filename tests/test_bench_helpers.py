"""Host-side helpers of bench.py (no GPU): the per-value-store roofline
summary, the traffic model's keys, and the recorded sigma-column count of
the reference algorithm for the benchmarked workload."""
import importlib.util
import os

from tests.conftest import ROOT


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_by_store_roofline_and_traffic_keys():
    b = _bench()
    stats = {"bf16": {"calls": 10, "ms": 45.0, "alg_bytes": 1.0e11, "columns": 400},
             "fp32": {"calls": 0, "ms": 0.0, "alg_bytes": 0.0, "columns": 0},
             "fp64": {"calls": 5, "ms": 580.0, "alg_bytes": 6.0e10, "columns": 150}}
    out = b.by_store_roofline(stats, 6787.9)
    assert set(out) == {"bf16", "fp64"}
    assert abs(out["bf16"]["achieved_gbs"] - 1.0e11 / 45e-3 / 1e9) < 1e-6
    assert abs(out["bf16"]["share_of_sigma_ms"] + out["fp64"]["share_of_sigma_ms"] - 1.0) < 1e-12
    assert set(b.TRAFFIC_PER_ALG_BYTE) == {"bf16", "fp32", "fp64"}


def test_reference_column_count_fixture():
    b = _bench()
    rc = b.reference_columns(b.NO, b.NV)
    assert rc is not None and rc["nmult_reference"] > 0 and rc["iterations"] > 0
    assert b.reference_columns(10, 110) is None
