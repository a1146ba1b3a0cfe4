"""Batched execution of independent ADC(2)-s problems on one GPU.

Many seeded systems of uneven size (and many SIL wavepackets) are solved
concurrently: every system owns a context with its own CUDA stream, the host
drives them from a thread pool (the C ABI releases the GIL), so builds,
sigma products and dense kernels of different systems overlap on the device.
Wavepackets on one matrix share every sigma product (adcgpu_autocorr runs
them as one block of 2P real columns).
"""
from __future__ import annotations

import concurrent.futures as cf
import time

import numpy as np

from . import api


def seeded_systems(n: int = 64, seed: int = 4242, nocc=(4, 12), nvirt=(30, 120)):
    """n systems with nocc ~ U{nocc}, nvirt ~ U{nvirt} and seeds seed + i."""
    rs = np.random.RandomState(seed)
    return [(int(rs.randint(nocc[0], nocc[1] + 1)), int(rs.randint(nvirt[0], nvirt[1] + 1)), seed + i)
            for i in range(n)]


def _solve_one(args):
    no, nv, seed, nroots, tol, precision, precon = args
    t0 = time.perf_counter()
    e, eri = api.synth_system(no, nv, seed, nthreads=2)
    g = api.AdcGpu(0)
    g.set_orbitals(no, nv, e)
    g.set_eri_packed(eri)
    g.write_fspace_adc2_1(None, precision=precision)
    r = g.davdiag_block(nroots, tol, precision=precision, precon=precon, want_vectors=False,
                        raise_on_nonconv=False)
    g.close()
    return {"nocc": no, "nvirt": nv, "seed": seed, "N": int(api.adc2s_dim(no, nv)[0]), "status": r.status,
            "iterations": r.iterations, "evals": r.evals.tolist(), "seconds": time.perf_counter() - t0}


def work_estimate(no: int, nv: int) -> float:
    """Relative cost of one system: the stored coupling values a sigma
    product streams, about N (2 nocc + 2 nvirt) for N configurations."""
    return float(api.adc2s_dim(no, nv)[0]) * (2 * no + 2 * nv)


def schedule(systems, workers: int):
    """Longest-processing-time-first order for a pool of `workers` streams:
    the systems sorted by decreasing work estimate (stable for equal ones),
    so the large systems start first and the small ones fill the tail.
    Returns the indices into `systems` in submission order."""
    del workers   # the greedy pool assigns each next job to the first free worker
    return sorted(range(len(systems)), key=lambda i: -work_estimate(systems[i][0], systems[i][1]))


def solve_many(systems, nroots: int = 8, tol: float = 1e-6, precision: int = api.ADCGPU_MIXED,
               precon: int = api.PRECON_DPR, workers: int = 8):
    """Solves all systems concurrently, largest first (`schedule`); returns
    the per-system results in the order of `systems` and the wall time of
    the whole batch."""
    t = time.perf_counter()
    order = schedule(systems, workers)
    jobs = {i: (*systems[i], nroots, tol, precision, precon) for i in order}
    res = [None] * len(systems)
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        futs = {ex.submit(_solve_one, jobs[i]): i for i in order}
        for f in cf.as_completed(futs):
            res[futs[f]] = f.result()
    return res, time.perf_counter() - t


def wavepackets(g: api.AdcGpu, npackets: int, seed: int = 77) -> np.ndarray:
    """Seeded positive 'dipole-like' start vectors (ndim x npackets)."""
    return api.synth_uniform_block(g.ndim, npackets, seed)
