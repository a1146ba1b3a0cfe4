"""GPU builder and sigma product against the oracle (bit-exact structure)."""
import numpy as np
import pytest

import oracle
from tests.conftest import sorted_coo, system

pytestmark = pytest.mark.gpu

CASES = [(5, 19, 1234), (4, 9, 7), (6, 30, 11), (2, 3, 5)]


def make(no, nv, seed, precision=0):
    from adc_ottawa_gb300 import AdcGpu, select_adc2s

    e, eri = system(no, nv, seed)
    g = AdcGpu(0)
    g.set_orbitals(no, nv, e)
    g.set_eri_packed(eri)
    g.write_fspace_adc2_1(select_adc2s(no, nv), precision=precision)
    return g, e, eri


@pytest.mark.parametrize("no,nv,seed", CASES)
def test_build_bit_exact(gpu, no, nv, seed):
    g, e, eri = make(no, nv, seed)
    ref = oracle.Matrix.build(no, nv, e, eri)
    assert g.noffd == ref.nnz
    d_ref, h_ref, oi_ref, oj_ref = ref.coo()
    assert np.array_equal(g.get_diag(), d_ref)
    h, oi, oj = g.export_coo()
    a = sorted_coo(h, oi, oj)
    b = sorted_coo(h_ref, oi_ref, oj_ref)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert np.array_equal(a[0], b[0])            # values bit-identical
    g.close()


def test_threshold_edge(gpu):
    """A system scaled so that many elements straddle minc = 1e-12: the kept
    set still matches bit for bit."""
    from adc_ottawa_gb300 import AdcGpu, select_adc2s

    no, nv = 4, 10
    e, eri = system(no, nv, 3)
    eri = eri * 3e-12
    g = AdcGpu(0)
    g.set_orbitals(no, nv, e)
    g.set_eri_packed(eri)
    g.write_fspace_adc2_1(select_adc2s(no, nv))
    ref = oracle.Matrix.build(no, nv, e, eri)
    d_ref, h_ref, oi_ref, oj_ref = ref.coo()
    assert 0 < ref.nnz < 0.9 * (no * nv * (no * nv - 1) // 2 + 200 * 40)
    assert g.noffd == ref.nnz
    h, oi, oj = g.export_coo()
    a, b = sorted_coo(h, oi, oj), sorted_coo(h_ref, oi_ref, oj_ref)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    g.close()


def test_mo_complex_layout_matches_packed(gpu):
    """The reference's complex nmo^4 buffer_real layout gives the same matrix."""
    from adc_ottawa_gb300 import AdcGpu, select_adc2s

    no, nv = 3, 6
    e, eri = system(no, nv, 21)
    n = no + nv
    full = np.zeros((n, n, n, n), dtype=np.complex128, order="F")
    idx = 0
    pq = [(p, q) for p in range(n) for q in range(p + 1)]
    for PQ in range(len(pq)):
        p, q = pq[PQ]
        for RS in range(PQ + 1):
            r, s = pq[RS]
            v = eri[idx]
            idx += 1
            for (a, b, c, d) in [(p, q, r, s), (q, p, r, s), (p, q, s, r), (q, p, s, r),
                                 (r, s, p, q), (s, r, p, q), (r, s, q, p), (s, r, q, p)]:
                full[a, b, c, d] = v
    g1 = AdcGpu(0)
    g1.set_orbitals(no, nv, e)
    g1.set_eri_mo_complex(full)
    g1.write_fspace_adc2_1(select_adc2s(no, nv))
    g2, _, _ = make(no, nv, 21)
    assert g1.noffd == g2.noffd
    assert np.array_equal(g1.get_diag(), g2.get_diag())
    a, b = sorted_coo(*g1.export_coo()), sorted_coo(*g2.export_coo())
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_rejects_foreign_kpq(gpu):
    from adc_ottawa_gb300 import AdcGpu, AdcGpuError, select_adc2s

    no, nv = 3, 5
    e, eri = system(no, nv, 1)
    g = AdcGpu(0)
    g.set_orbitals(no, nv, e)
    g.set_eri_packed(eri)
    kpq = select_adc2s(no, nv)
    kpq[5, 4] += 1
    with pytest.raises(AdcGpuError) as ei:
        g.write_fspace_adc2_1(kpq)
    assert ei.value.code == 16


@pytest.mark.parametrize("no,nv,seed", CASES[:3])
@pytest.mark.parametrize("m", [1, 3, 11])
def test_sigma_matches_oracle(gpu, no, nv, seed, m):
    g, e, eri = make(no, nv, seed)
    ref = oracle.Matrix.build(no, nv, e, eri)
    x = np.random.RandomState(m).standard_normal((g.ndim, m))
    y = g.sigma(x)
    y_ref = ref.matvec(x)
    assert np.abs(y - y_ref).max() <= 1e-13 * np.abs(y_ref).max()
    g.close()


def test_sigma_symmetric_full_size(gpu):
    """Size-independent property at a larger size: x.(Hy) == y.(Hx)."""
    g, e, eri = make(10, 60, 4)
    rs = np.random.RandomState(1)
    x, y = rs.standard_normal(g.ndim), rs.standard_normal(g.ndim)
    hx, hy = g.sigma(x), g.sigma(y)
    assert abs(x @ hy - y @ hx) <= 1e-12 * np.linalg.norm(x) * np.linalg.norm(hy)
    # linearity
    h2 = g.sigma(np.stack([x, y, 2 * x - 3 * y], axis=1))
    assert np.allclose(h2[:, 2], 2 * hx - 3 * hy, rtol=0, atol=1e-11 * np.abs(hx).max())


def test_hmlt_files_roundtrip(gpu, tmp_path):
    """SCRATCH file layout of filetools.f90 (wrtdg / wrtoffdg records)."""
    g, e, eri = make(4, 9, 7)
    g.write_hmlt_files(str(tmp_path), "i")
    raw = np.fromfile(tmp_path / "hmlt.diai", dtype=np.uint8)
    n = int(np.frombuffer(raw[0:4], np.int32)[0])
    assert n == 8
    maxbl, nbuf = np.frombuffer(raw[4:12], np.int32)
    assert maxbl == 655360 and nbuf == 1
    n2 = int(np.frombuffer(raw[16:20], np.int32)[0])
    diag = np.frombuffer(raw[20:20 + n2], np.float64)
    assert np.array_equal(diag, g.get_diag())
    off = np.fromfile(tmp_path / "hmlt.offi", dtype=np.uint8)
    B = 655360
    rec = int(np.frombuffer(off[0:4], np.int32)[0])
    assert rec == 16 * B + 4
    body = off[4:4 + rec]
    nlim = int(np.frombuffer(body[16 * B:16 * B + 4], np.int32)[0])
    assert nlim == g.noffd
    h = np.frombuffer(body[:8 * B], np.float64)[:nlim]
    oi = np.frombuffer(body[8 * B:12 * B], np.int32)[:nlim]
    oj = np.frombuffer(body[12 * B:16 * B], np.int32)[:nlim]
    a, b = sorted_coo(h, oi, oj), sorted_coo(*g.export_coo())
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.slow
def test_config2_full_size_golden(gpu):
    """nocc=10, nvirt=110 (N=606,650): kept structure, diagonal and values
    bit-identical to the oracle's committed fingerprint."""
    import hashlib
    import json
    import os

    from tests.conftest import ROOT

    gold = json.load(open(os.path.join(ROOT, "tests", "golden", "config2.json")))
    g, e, eri = make(gold["nocc"], gold["nvirt"], gold["seed"])
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    assert sha(e) == gold["e_sha"] and sha(eri) == gold["eri_sha"]
    assert g.noffd == gold["nnz"]
    assert sha(g.get_diag()) == gold["diag_sha"]
    h, oi, oj = g.export_coo()
    assert [str(x) for x in oracle.structure_hash(oi, oj)] == gold["structure_hash"]
    k = np.lexsort((oj, oi))
    assert sha(h[k]) == gold["values_sorted_sha"]
    g.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_sigma_launch_shapes_agree(gpu, prec, tmp_path):
    """Every launch shape the autotuner may pick gives the same product, and
    the tuned shape is cached and re-applied."""
    import ctypes as C

    from adc_ottawa_gb300 import autotune
    from adc_ottawa_gb300._native import lib

    g, e, eri = make(6, 30, 11, precision=prec)
    x = np.random.RandomState(3).standard_normal((g.ndim, 5))
    ref = g.sigma(x)
    tol = 1e-12 if prec == 0 else 5e-3
    for chunk in (16, 64, 256):
        for mc in (1, 2, 4):
            for staged in (0, 8):
                assert lib().adcgpu_sigma_set_shape(g._h, chunk, mc | staged, mc | staged) == 0
                y = g.sigma(x)
                assert np.abs(y - ref).max() <= tol * np.abs(ref).max(), (chunk, mc, staged)
    cache = str(tmp_path / "tune.json")
    r1 = autotune.tune(g, 5, prec, cache=cache)
    r2 = autotune.tune(g, 5, prec, cache=cache)
    assert not r1["cached"] and r2["cached"] and r1["chunk"] == r2["chunk"]
    y = g.sigma(x)
    assert np.abs(y - ref).max() <= tol * np.abs(ref).max()
    g.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_sigma_tiled_passes_agree(gpu, prec):
    """20 columns (a 16-column tile pass and 4 more): the tiled pass 1 (tensor
    cores for BF16 values, CUDA cores otherwise) and the CUDA-core tile agree
    with the per-warp pass 1.  FP64: to roundoff.  BF16 values: the tensor-core
    pass carries the vectors as BF16 hi + lo pairs (~2^-17 relative)."""
    from adc_ottawa_gb300._native import lib

    g, e, eri = make(6, 30, 11, precision=prec)
    x = np.random.RandomState(5).standard_normal((g.ndim, 20))
    assert lib().adcgpu_sigma_set_shape(g._h, 64, 2 | 16, 4 | 16) == 0     # per-warp
    ref = g.sigma(x)
    scale = np.abs(ref).max()
    for bits, tol in ((32, 1e-12 if prec == 0 else 1e-5), (0, 1e-12 if prec == 0 else 2e-4)):
        assert lib().adcgpu_sigma_set_shape(g._h, 64, 2 | bits, 4 | bits) == 0
        y = g.sigma(x)
        assert np.abs(y - ref).max() <= tol * scale, (bits, np.abs(y - ref).max() / scale)
    g.close()
