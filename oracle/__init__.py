"""ORACLE -- test infrastructure only.

CPU FP64 restatement of mschuurman/ADC_ottawa's ADC(2)-s path (oracle.cpp),
loaded through ctypes.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may use this module, and only as the checker;
the product package never imports it.

Parity status: unpinned against the reference's own outputs (the reference is
Fortran, no Fortran compiler is available, and the reference ships no test
vectors for this path).  It is pinned by independent checks instead: dense
eigendecomposition of the assembled matrix, exact propagation, and structural
rules (tests/test_oracle.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)


def build(force: bool = False) -> str:
    """Compile oracle.cpp and the shared synthetic generator with the
    committed Makefile (strict IEEE flags; make decides what is stale)."""
    if force:
        subprocess.run(["make", "-s", "-C", _HERE, "clean"], check=True)
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.orc_select.argtypes = [C.c_int, C.c_int, _ip]
        L.orc_select.restype = C.c_int
        L.orc_build.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_int]
        L.orc_build.restype = C.c_void_p
        L.orc_build_direct.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_int]
        L.orc_build_direct.restype = C.c_void_p
        L.orc_matrix_ndim.argtypes = [C.c_void_p]
        L.orc_matrix_ndim.restype = C.c_int64
        L.orc_matrix_nnz.argtypes = [C.c_void_p]
        L.orc_matrix_nnz.restype = C.c_int64
        L.orc_matrix_copy.argtypes = [C.c_void_p, _dp, _dp, _ip, _ip]
        L.orc_matrix_from_coo.argtypes = [C.c_int64, _dp, C.c_int64, _dp, _ip, _ip]
        L.orc_matrix_from_coo.restype = C.c_void_p
        L.orc_matrix_free.argtypes = [C.c_void_p]
        L.orc_structure_hash.argtypes = [C.c_int64, _ip, _ip, C.POINTER(C.c_uint64)]
        L.orc_matvec.argtypes = [C.c_void_p, C.c_int, _dp, _dp, C.c_int]
        L.orc_eigh.argtypes = [C.c_int, _dp, _dp, _dp]
        L.orc_heapsort_index.argtypes = [C.c_int, _dp, _ip]
        L.orc_heapsort_index_desc.argtypes = [C.c_int, _dp, _ip]
        L.orc_davidson.argtypes = [C.c_void_p, _ip, C.c_double, C.c_int, _dp, _dp, _ip]
        L.orc_davidson.restype = C.c_int
        L.orc_davidson_guess.argtypes = [C.c_void_p, _ip, C.c_double, C.c_int, _dp, _dp, _dp, _ip]
        L.orc_davidson_guess.restype = C.c_int
        L.orc_adc1_matrix.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_adc1_matrix.restype = C.c_int
        L.orc_block_lanczos.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp, C.c_int, _dp, _dp]
        L.orc_block_lanczos.restype = C.c_int
        L.orc_autocorr.argtypes = [C.c_void_p, _dp, C.c_double, C.c_double, C.c_int, C.c_double,
                                   _dp, C.POINTER(C.c_int), _i64p]
        L.orc_autocorr.restype = C.c_int
        L.orc_chebyshev_auto.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _dp, _dp, C.c_int64]
        L.orc_chebyshev_auto.restype = C.c_int
        L.orc_chebyshev_project.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_double]
        L.orc_chebyshev_project.restype = C.c_int
        L.orc_synth_orbitals.argtypes = [C.c_int, C.c_int, C.c_uint64, _dp]
        L.orc_synth_orbitals.restype = C.c_int
        L.orc_eri_packed_size.argtypes = [C.c_int]
        L.orc_eri_packed_size.restype = C.c_int64
        L.orc_synth_eri_packed.argtypes = [C.c_int, C.c_uint64, _dp, C.c_int]
        L.orc_synth_eri_packed.restype = C.c_int
        L.orc_synth_uniform_block.argtypes = [C.c_int64, C.c_int, C.c_uint64, _dp]
        L.orc_synth_uniform_block.restype = C.c_int
        L.orc_adc2s_dim.argtypes = [C.c_int, C.c_int, _ip]
        L.orc_adc2s_dim.restype = C.c_int64
        L.orc_build_cvs.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_int, _ip, C.c_int]
        L.orc_build_cvs.restype = C.c_void_p
        L.orc_cvs_dim.argtypes = [C.c_int, C.c_int, C.c_int, _ip, _ip]
        L.orc_cvs_dim.restype = C.c_int64
        L.orc_select_adc2s_cvs.argtypes = [C.c_int, C.c_int, C.c_int, _ip, _ip]
        L.orc_select_adc2s_cvs.restype = C.c_int
        L.orc_synth_dipole.argtypes = [C.c_int, C.c_uint64, _dp]
        L.orc_synth_dipole.restype = C.c_int
        L.orc_modified_tm_adc2.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, C.c_int64, _ip, _dp, C.c_int]
        L.orc_modified_tm_adc2.restype = C.c_int
        _lib = L
    return _lib


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def synth_system(no: int, nv: int, seed: int, nthreads: int = 0):
    """The seeded synthetic system (orbital energies, packed ERIs) from the
    generator compiled into the oracle library: the same source and bits as
    adc_ottawa_gb300.synth_system, without loading the product library."""
    e = np.empty(no + nv)
    assert lib().orc_synth_orbitals(no, nv, seed, _p(e)) == 0
    eri = np.empty(lib().orc_eri_packed_size(no + nv))
    assert lib().orc_synth_eri_packed(no + nv, seed, _p(eri), nthreads) == 0
    return e, eri


def synth_uniform_block(nrow: int, ncol: int, seed: int) -> np.ndarray:
    out = np.empty((nrow, ncol), order="F")
    assert lib().orc_synth_uniform_block(nrow, ncol, seed, _p(out)) == 0
    return out


def synth_dipole(nbas: int, seed: int) -> np.ndarray:
    """The seeded synthetic dipole matrix dpl (nbas x nbas, symmetric)."""
    d = np.empty((nbas, nbas), order="F")
    assert lib().orc_synth_dipole(nbas, seed, _p(d)) == 0
    return d


def select_cvs(no: int, nv: int, core) -> np.ndarray:
    """The CVS kpq (select_atom_is_cvs / select_atom_d_cvs) as (ndim+1, 7) int32."""
    core = np.ascontiguousarray(core, np.int32)
    cnt = np.zeros(5, np.int32)
    ndim = int(lib().orc_cvs_dim(no, nv, len(core), _p(core, _ip), _p(cnt, _ip)))
    assert ndim > 0
    kpq = np.zeros((ndim + 1, 7), np.int32)
    assert lib().orc_select_adc2s_cvs(no, nv, len(core), _p(core, _ip), _p(kpq, _ip)) == 0
    return kpq


def modified_tm_adc2(no: int, nv: int, e, eri, dpl, sections: int = 3, kpq=None) -> np.ndarray:
    """get_modifiedtm_adc2's f-vector over a configuration list (the ADC(2)-s
    list by default; a CVS list skips the i=j classes as lcvs does),
    get_moment.f90:153-442, FP64 in the reference's loop and expression
    order.  sections: 1 = singles only, 2 = doubles only, 3 = both."""
    if kpq is None:
        kpq = select(no, nv)
    kpq = np.ascontiguousarray(kpq, np.int32)
    ndim = kpq.shape[0] - 1
    e = np.ascontiguousarray(e, np.float64)
    eri = np.ascontiguousarray(eri, np.float64)
    dpl = np.asfortranarray(dpl, np.float64)
    mtm = np.zeros(ndim)
    assert lib().orc_modified_tm_adc2(no, nv, _p(e), _p(eri), _p(dpl), ndim, _p(kpq, _ip), _p(mtm), sections) == 0
    return mtm


def adc2s_dim(no: int, nv: int) -> int:
    cnt = np.zeros(5, np.int32)
    return int(lib().orc_adc2s_dim(no, nv, _p(cnt, _ip)))


def adc1_matrix(no: int, nv: int, e, eri) -> np.ndarray:
    """The ADC(1) singles matrix (get_diag/offdiag_tda_direct), n1 x n1."""
    e = np.ascontiguousarray(e, np.float64)
    eri = np.ascontiguousarray(eri, np.float64)
    M = np.zeros((no * nv, no * nv), order="F")
    assert lib().orc_adc1_matrix(no, nv, _p(e), _p(eri), _p(M)) == no * nv
    return M


def adc1_guess(no: int, nv: int, e, eri, ndim: int, blocksize: int) -> np.ndarray:
    """initvec_adc1's start block: the blocksize lowest ADC(1) eigenvectors
    (numpy's LAPACK, ascending) in the singles rows of an ndim x blocksize
    block."""
    _, U = np.linalg.eigh(adc1_matrix(no, nv, e, eri))
    G = np.zeros((ndim, blocksize), order="F")
    G[: no * nv] = U[:, :blocksize]
    return G


def select(no: int, nv: int) -> np.ndarray:
    """kpq(7, 0:ndim) as a (ndim+1, 7) int32 array (row c = Fortran column c)."""
    n1 = no * nv
    ndim = n1 + n1 + nv * (nv - 1) // 2 * no + no * (no - 1) // 2 * nv + 2 * (no * (no - 1) // 2) * (nv * (nv - 1) // 2)
    kpq = np.zeros((ndim + 1, 7), dtype=np.int32)
    got = lib().orc_select(no, nv, _p(kpq, _ip))
    assert got == ndim
    return kpq


class Matrix:
    """The stored ADC(2)-s matrix: diagonal + upper-triangle COO (1-based)."""

    def __init__(self, handle):
        self.h = handle

    @classmethod
    def build(cls, no, nv, e, eri, nthreads=0):
        e = np.ascontiguousarray(e, dtype=np.float64)
        eri = np.ascontiguousarray(eri, dtype=np.float64)
        return cls(lib().orc_build(no, nv, _p(e), _p(eri), nthreads))

    @classmethod
    def build_cvs(cls, no, nv, e, eri, core, nthreads=0):
        """write_fspace_adc2_1_cvs: the CVS ADC(2)-s matrix for the core
        orbitals core (1-based occupied indices)."""
        e = np.ascontiguousarray(e, np.float64)
        eri = np.ascontiguousarray(eri, np.float64)
        core = np.ascontiguousarray(core, np.int32)
        h = lib().orc_build_cvs(no, nv, _p(e), _p(eri), len(core), _p(core, _ip), nthreads)
        assert h
        return cls(h)

    @classmethod
    def build_direct(cls, no, nv, e, eri, nthreads=0):
        """The matrix of the direct (matvec) path: ph-ph block from
        Ca1/Cb1/Cc1/Cc2 (adc_ph.f90:98-303), coupling and 2p2h diagonal as
        in the stored path."""
        e = np.ascontiguousarray(e, dtype=np.float64)
        eri = np.ascontiguousarray(eri, dtype=np.float64)
        return cls(lib().orc_build_direct(no, nv, _p(e), _p(eri), nthreads))

    @classmethod
    def from_coo(cls, diag, h, oi, oj):
        diag = np.ascontiguousarray(diag, np.float64)
        h = np.ascontiguousarray(h, np.float64)
        oi = np.ascontiguousarray(oi, np.int32)
        oj = np.ascontiguousarray(oj, np.int32)
        return cls(lib().orc_matrix_from_coo(len(diag), _p(diag), len(h), _p(h), _p(oi, _ip), _p(oj, _ip)))

    @property
    def ndim(self):
        return lib().orc_matrix_ndim(self.h)

    @property
    def nnz(self):
        return lib().orc_matrix_nnz(self.h)

    def coo(self):
        n, z = self.ndim, self.nnz
        diag = np.empty(n)
        h = np.empty(z)
        oi = np.empty(z, np.int32)
        oj = np.empty(z, np.int32)
        lib().orc_matrix_copy(self.h, _p(diag), _p(h), _p(oi, _ip), _p(oj, _ip))
        return diag, h, oi, oj

    def dense(self):
        diag, h, oi, oj = self.coo()
        H = np.diag(diag)
        H[oi - 1, oj - 1] = h
        H[oj - 1, oi - 1] = h
        return H

    def matvec(self, V, nthreads=0):
        V = np.asfortranarray(V, dtype=np.float64)
        if V.ndim == 1:
            V = V.reshape(-1, 1, order="F")
        W = np.empty_like(V, order="F")
        lib().orc_matvec(self.h, V.shape[1], _p(V), _p(W), nthreads)
        return W

    def davidson(self, nstates, tol, blocksize=0, maxvec=-1, niter=100, precon=1, deflate=True,
                 subdiag=False, guessdim=800, nthreads=0, want_vectors=False, guess=None):
        """guess: ndim x blocksize start vectors (initvec_adc1 places the
        ADC(1) eigenvectors this way); otherwise initvec_subdiag/_ondiag."""
        ip = np.array([nstates, blocksize, maxvec, niter, precon, int(deflate), int(subdiag), guessdim],
                      dtype=np.int32)
        ev = np.empty(nstates)
        vecs = np.empty((self.ndim, nstates), order="F") if want_vectors else None
        iout = np.zeros(3, np.int32)
        if guess is not None:
            bs = blocksize if blocksize > 0 else max(nstates + 5, 2 * nstates)
            G = np.asfortranarray(guess, np.float64)
            assert G.shape == (self.ndim, bs), (G.shape, bs)
            st = lib().orc_davidson_guess(self.h, _p(ip, _ip), tol, nthreads, _p(G), _p(ev),
                                          _p(vecs) if want_vectors else None, _p(iout, _ip))
        else:
            st = lib().orc_davidson(self.h, _p(ip, _ip), tol, nthreads, _p(ev),
                                    _p(vecs) if want_vectors else None, _p(iout, _ip))
        return st, ev, vecs, dict(iterations=int(iout[0]), nmult=int(iout[1]), nconv=int(iout[2]))

    def block_lanczos(self, q0, ncycles, orthotype=0, nthreads=0):
        q0 = np.asfortranarray(q0, dtype=np.float64)
        b = q0.shape[1]
        nvec = b * ncycles
        T = np.empty((nvec, nvec), order="F")
        ev = np.empty(nvec)
        lib().orc_block_lanczos(self.h, b, ncycles, orthotype, _p(q0), nthreads, _p(T), _p(ev))
        return T, ev

    def autocorr(self, f, tout, tfinal, kdim, tol):
        f = np.ascontiguousarray(f, np.float64)
        nt = int(tfinal / (0.5 * tout)) + 1
        out = np.zeros(2 * nt)
        ntimes = C.c_int(0)
        nmult = C.c_int64(0)
        st = lib().orc_autocorr(self.h, _p(f), tout, tfinal, kdim, tol, _p(out), C.byref(ntimes), C.byref(nmult))
        a = out[0::2] + 1j * out[1::2]
        return st, a[: ntimes.value], nmult.value

    def chebyshev_auto(self, q0, bounds, chebyord, n1=0):
        """C_0..C_2ord of chebyshev_auto (chebyspec.f90:246-330); with n1 > 0
        also the first n1 elements of q_0..q_ord (the save1h1p array)."""
        q0 = np.ascontiguousarray(q0, np.float64)
        bounds = np.ascontiguousarray(bounds, np.float64)
        out = np.zeros(2 * chebyord + 1)
        q1 = np.zeros((n1, chebyord + 1), order="F") if n1 else None
        o = lib().orc_chebyshev_auto(self.h, _p(q0), _p(bounds), chebyord, _p(out),
                                     _p(q1) if n1 else None, n1)
        return out[: 2 * o + 1], (q1[:, : o + 1] if n1 else None)

    def chebyshev_project(self, q0, bounds, chebyord, projen):
        """project_psi0 (chebyspec.f90:398-470) on a copy of q0."""
        q = np.array(q0, np.float64)
        bounds = np.ascontiguousarray(bounds, np.float64)
        lib().orc_chebyshev_project(self.h, _p(q), _p(bounds), chebyord, projen)
        return q

    def singlesubspace_block(self, blocksize, subdim=800):
        """init_vec_singlesubspace (block_lanczos.f90:748-923): the lowest
        blocksize eigenvectors of H restricted to the subdim configurations of
        largest hii (extended past near-degeneracies < 1e-6), scattered into an
        N x blocksize block.  The descending heapsort dsortindxa1('D') is the
        ascending one on negated keys (the same comparisons).  dsyev is
        numpy's LAPACK here (eigenvector signs are free; the Lanczos
        eigenvalues do not depend on them)."""
        diag, h, oi, oj = self.coo()
        n = len(diag)
        indx = heapsort_index(-diag)                  # 1-based, descending hii
        subdim = min(subdim, n)
        while subdim < n and abs(diag[indx[subdim - 1] - 1] - diag[indx[subdim] - 1]) < 1e-6:
            subdim += 1
        sub2full = indx[:subdim] - 1
        full2sub = np.full(n, -1, np.int64)
        full2sub[sub2full] = np.arange(subdim)
        hsub = np.diag(diag[sub2full])
        keep = (full2sub[oi - 1] >= 0) & (full2sub[oj - 1] >= 0)
        i1, j1 = full2sub[oi[keep] - 1], full2sub[oj[keep] - 1]
        hsub[i1, j1] = h[keep]
        hsub[j1, i1] = h[keep]
        _, V = np.linalg.eigh(hsub)
        q = np.zeros((n, blocksize), order="F")
        q[sub2full, :] = V[:, :blocksize]
        return q

    def spectral_bounds(self, precon=2, nthreads=0):
        """spectral_bounds_davlanc (specbounds.f90:121-205): the lowest
        eigenvalue from a 1-root block Davidson (block 5, subspace 20, tol 1e-8,
        subspace-diagonalisation guess), the highest from a block Lanczos
        (block 2, 100 cycles, PRO) started from init_vec_singlesubspace."""
        st, ev, _, _ = self.davidson(1, 1e-8, blocksize=5, maxvec=20, niter=100, precon=precon, deflate=True,
                                     subdiag=True, guessdim=800, nthreads=nthreads)
        q0 = self.singlesubspace_block(2)
        _, evl = self.block_lanczos(q0, 100, orthotype=1, nthreads=nthreads)
        return st, np.array([ev[0], evl[-1]])

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_matrix_free(self.h)
            self.h = None


def structure_hash(oi, oj):
    oi = np.ascontiguousarray(oi, np.int32)
    oj = np.ascontiguousarray(oj, np.int32)
    out = np.zeros(3, np.uint64)
    lib().orc_structure_hash(len(oi), _p(oi, _ip), _p(oj, _ip), out.ctypes.data_as(C.POINTER(C.c_uint64)))
    return tuple(int(x) for x in out)


def heapsort_index(arr):
    arr = np.ascontiguousarray(arr, np.float64)
    out = np.empty(len(arr), np.int32)
    lib().orc_heapsort_index(len(arr), _p(arr), _p(out, _ip))
    return out


def heapsort_index_desc(arr):
    """dsortindxa1('D', ...): descending, ties in heap order (1-based)."""
    arr = np.ascontiguousarray(arr, np.float64)
    out = np.empty(len(arr), np.int32)
    lib().orc_heapsort_index_desc(len(arr), _p(arr), _p(out, _ip))
    return out


def eigh(A):
    A = np.asfortranarray(A, np.float64)
    n = A.shape[0]
    w = np.empty(n)
    V = np.empty((n, n), order="F")
    lib().orc_eigh(n, _p(A), _p(w), _p(V))
    return w, V
