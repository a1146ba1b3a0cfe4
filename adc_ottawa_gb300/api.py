"""Host-side mirror of the reference's interfaces for the ADC(2)-s hot path.

Each method wraps one C-ABI entry point of libadcgpu.so and keeps the name
and argument meaning of the Fortran routine it replaces:

  write_fspace_adc2_1  source/adclib/fspacetrial.f90:533-564
  davdiag_block        source/eigen/block_davidson.f90:33-145
  lancdiag_block       source/eigen/block_lanczos.f90:28-81
  silstep              source/propagation/sillib.f90:108-393
  propagate_fvec       source/propagation/fvecprop.f90:27-105 (autocorrelation)
  chebyshev_auto       source/propagation/chebyspec.f90:246-330
  project_psi0         source/propagation/chebyspec.f90:398-470
  spectral_bounds      source/propagation/specbounds.f90:121-205

Failures raise AdcGpuError carrying the library status code; the reference
calls error_control/STOP in the same places (iomod.f90:94-112).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._native import DavInfo, DavParams, SilState, lib, ptr

ADCGPU_FP64 = 0
ADCGPU_MIXED = 1
ADCGPU_DIRECT = 2   # FP64, coupling block recomputed in every sigma product (the matvec path)
PRECON_DPR, PRECON_OLSEN, PRECON_MLP, PRECON_FOLD = 1, 2, 3, 4

STATUS = {
    0: "ok", 1: "Illegal integration order", 2: "Stepsize underflow", 3: "Diagonalisation failed",
    4: "Illegal initial stepsize", 10: "Not all vectors have converged", 11: "out of device memory",
    12: "bad input", 13: "CUDA error", 14: "device wait timed out", 15: "no matrix built",
    16: "unsupported", 17: "eigensolver failed",
}


class AdcGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {STATUS.get(code, 'error')}: {msg}")
        self.code = code


_ip = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)


def synth_orbitals(nocc: int, nvirt: int, seed: int) -> np.ndarray:
    e = np.empty(nocc + nvirt)
    st = lib().adcgpu_synth_orbitals(nocc, nvirt, seed, ptr(e))
    if st:
        raise AdcGpuError(st, "synth_orbitals")
    return e


def eri_packed_size(nbas: int) -> int:
    return int(lib().adcgpu_eri_packed_size(nbas))


def synth_eri_packed(nbas: int, seed: int, nthreads: int = 0) -> np.ndarray:
    eri = np.empty(eri_packed_size(nbas))
    st = lib().adcgpu_synth_eri_packed(nbas, seed, ptr(eri), nthreads)
    if st:
        raise AdcGpuError(st, "synth_eri_packed")
    return eri


def synth_system(nocc: int, nvirt: int, seed: int, nthreads: int = 0):
    """Seeded synthetic closed-shell system: (e, packed ERIs)."""
    return synth_orbitals(nocc, nvirt, seed), synth_eri_packed(nocc + nvirt, seed, nthreads)


def synth_uniform_block(nrow: int, ncol: int, seed: int) -> np.ndarray:
    out = np.empty((nrow, ncol), order="F")
    st = lib().adcgpu_synth_uniform_block(nrow, ncol, seed, ptr(out))
    if st:
        raise AdcGpuError(st, "synth_uniform_block")
    return out


def cvs_dim(nocc: int, nvirt: int, core) -> int:
    """Dimension of the CVS space of the core orbitals (1-based occupied indices)."""
    core = np.ascontiguousarray(core, np.int32)
    n = int(lib().adcgpu_cvs_dim(nocc, nvirt, len(core), ptr(core, _ip), None))
    if n <= 0:
        raise AdcGpuError(12, "cvs_dim: 0 < ncore < nocc distinct occupied orbitals")
    return n


def select_adc2s_cvs(nocc: int, nvirt: int, core) -> np.ndarray:
    """select_atom_is_cvs + select_atom_d_cvs: the CVS kpq as (ndim+1, 7) int32."""
    core = np.ascontiguousarray(core, np.int32)
    kpq = np.zeros((cvs_dim(nocc, nvirt, core) + 1, 7), np.int32)
    st = lib().adcgpu_select_adc2s_cvs(nocc, nvirt, len(core), ptr(core, _ip), ptr(kpq, _ip))
    if st:
        raise AdcGpuError(st, "select_adc2s_cvs")
    return kpq


def synth_dipole(nbas: int, seed: int) -> np.ndarray:
    """Seeded synthetic dipole matrix dpl (nbas x nbas, symmetric, column-major)."""
    d = np.empty((nbas, nbas), order="F")
    st = lib().adcgpu_synth_dipole(nbas, seed, ptr(d))
    if st:
        raise AdcGpuError(st, "synth_dipole")
    return d


def fill_stvc(vctr: np.ndarray, lmain: int) -> np.ndarray:
    """fill_stvc (fspacetrial.f90:1255-1270): 1-based indices of the lmain
    largest vctr**2, in dsortindxa1('D') order."""
    v = np.ascontiguousarray(vctr, np.float64)
    out = np.zeros(lmain, np.int32)
    st = lib().adcgpu_fill_stvc(len(v), ptr(v), lmain, ptr(out, _ip))
    if st:
        raise AdcGpuError(st, "fill_stvc")
    return out


def lanczos_guess_vecs(mtm: np.ndarray, n1: int, lmain: int, lancguess: int = 1) -> np.ndarray:
    """The final-space Lanczos start block from the f-vector
    (lanczos_guess_vecs, adc2_opa.f90:380-520, and init_vec_unit /
    init_vec_1h1p2h2p, block_lanczos.f90:201-289), ADC(2)-s:

    - lancguess 1: unit vectors on the lmain singles with the largest f^2;
    - lancguess 3: (e_k1 +- e_k2)/sqrt(2) pairing the i-th largest single k1
      with the i-th largest double k2, '+' when f(k1) > 0 and f(k2) > 0.
    """
    mtm = np.asarray(mtm, np.float64)
    ndim = len(mtm)
    Q = np.zeros((ndim, lmain), order="F")
    if lancguess == 1:
        for i, k in enumerate(fill_stvc(mtm[:n1], lmain)):
            Q[k - 1, i] = 1.0
    elif lancguess == 3:
        i1 = fill_stvc(mtm[:n1], lmain)
        i2 = n1 + fill_stvc(mtm[n1:], lmain)
        fac = 1.0 / np.sqrt(2.0)
        for i in range(lmain):
            k1, k2 = int(i1[i]), int(i2[i])
            Q[k1 - 1, i] = fac
            Q[k2 - 1, i] = fac if (mtm[k1 - 1] > 0 and mtm[k2 - 1] > 0) else -fac
    else:
        raise AdcGpuError(12, "lanczos_guess_vecs: lancguess 1 or 3 (ADC(2)-s)")
    return Q


def adc2s_dim(nocc: int, nvirt: int):
    cnt = np.zeros(5, np.int32)
    n = lib().adcgpu_adc2s_dim(nocc, nvirt, ptr(cnt, _ip))
    return int(n), cnt


def select_adc2s(nocc: int, nvirt: int) -> np.ndarray:
    """kpq(7, 0:ndim) as an (ndim+1, 7) int32 array: row c is Fortran column c."""
    ndim, _ = adc2s_dim(nocc, nvirt)
    kpq = np.zeros((ndim + 1, 7), np.int32)
    st = lib().adcgpu_select_adc2s(nocc, nvirt, ptr(kpq, _ip))
    if st:
        raise AdcGpuError(st, "select_adc2s")
    return kpq


@dataclass
class DavidsonResult:
    evals: np.ndarray
    evecs: np.ndarray | None
    status: int
    iterations: int
    nmult: int
    nconv: int
    seconds: float
    sigma_seconds: float
    max_residual: float = 0.0
    iters_bf16: int = 0
    iters_fp32: int = 0
    iters_fp64: int = 0
    nmult_reference: int = 0


class AdcGpu:
    """One device-resident ADC(2)-s problem (an adcgpu_ctx)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        st = lib().adcgpu_ctx_create(device, C.byref(h))
        if st:
            raise AdcGpuError(st, "adcgpu_ctx_create (is a GPU visible?)")
        self._h = h
        self.nocc = self.nvirt = 0
        self.ndim = 0
        self.noffd = 0

    def _check(self, st: int, what: str):
        if st:
            msg = lib().adcgpu_last_error(self._h)
            raise AdcGpuError(st, f"{what}: {msg.decode() if msg else ''}")

    def _rows(self, a: np.ndarray, what: str) -> None:
        """Host arrays cross the C ABI as bare pointers, so their shape is
        checked here: ndim rows and at least one column."""
        if a.ndim != 2 or a.shape[0] != self.ndim or a.shape[1] < 1:
            raise AdcGpuError(12, f"{what}: expected {self.ndim} rows, got shape {a.shape}")

    @staticmethod
    def _bounds(bounds) -> np.ndarray:
        b = np.ascontiguousarray(bounds, np.float64).reshape(-1)
        if b.shape != (2,):
            raise AdcGpuError(12, f"bounds must be [Emin, Emax], got {b.shape[0]} values")
        return b

    def close(self):
        if getattr(self, "_h", None):
            lib().adcgpu_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- inputs ---------------------------------------------------------------
    def set_orbitals(self, nocc: int, nvirt: int, e: np.ndarray):
        e = np.ascontiguousarray(e, np.float64)
        self._check(lib().adcgpu_set_orbitals(self._h, nocc, nvirt, ptr(e)), "set_orbitals")
        self.nocc, self.nvirt = nocc, nvirt
        self.ndim = adc2s_dim(nocc, nvirt)[0]

    def set_eri_packed(self, eri: np.ndarray):
        eri = np.ascontiguousarray(eri, np.float64)
        self._check(lib().adcgpu_set_eri_packed(self._h, ptr(eri)), "set_eri_packed")

    def set_eri_mo_complex(self, buffer_real: np.ndarray):
        """moIntegrals%buffer_real: complex (nmo,nmo,nmo,nmo), Fortran order."""
        b = np.asarray(buffer_real, dtype=np.complex128)
        flat = np.ascontiguousarray(b.reshape(-1, order="F")).view(np.float64)
        self._check(lib().adcgpu_set_eri_mo_complex(self._h, ptr(flat)), "set_eri_mo_complex")

    # -- builder --------------------------------------------------------------
    def write_fspace_adc2_1(self, kpq: np.ndarray | None = None, chr: str = "i", precision: int = ADCGPU_FP64) -> int:
        """Build H on the device; returns noffdel (kept off-diagonal count)."""
        self.ndim = adc2s_dim(self.nocc, self.nvirt)[0]
        noff = C.c_int64(0)
        kp = None if kpq is None else ptr(np.ascontiguousarray(kpq, np.int32), _ip)
        self._check(lib().adcgpu_build_adc2s(self._h, self.ndim, kp, C.byref(noff), chr.encode(), precision),
                    "write_fspace_adc2_1")
        self.noffd = int(noff.value)
        return self.noffd

    def write_fspace_adc2_1_cvs(self, core, kpq: np.ndarray | None = None, chr: str = "i") -> int:
        """write_fspace_adc2_1_cvs (fspacetrial.f90:566-596): build the CVS
        matrix of the core orbitals (1-based occupied indices) on the device,
        FP64; returns noffdel.  The solvers then work in the CVS space
        (self.ndim becomes its dimension)."""
        core = np.ascontiguousarray(core, np.int32)
        ndim = cvs_dim(self.nocc, self.nvirt, core)
        noff = C.c_int64(0)
        kp = None if kpq is None else np.ascontiguousarray(kpq, np.int32)
        self._check(lib().adcgpu_build_adc2s_cvs(self._h, ndim, None if kp is None else ptr(kp, _ip), len(core),
                                                 ptr(core, _ip), C.byref(noff), chr.encode()),
                    "write_fspace_adc2_1_cvs")
        self.ndim = ndim
        self.noffd = int(noff.value)
        return self.noffd

    def get_diag(self) -> np.ndarray:
        d = np.empty(self.ndim)
        self._check(lib().adcgpu_get_diag(self._h, ptr(d)), "get_diag")
        return d

    def export_coo(self):
        n = self.noffd
        h = np.empty(n)
        oi = np.empty(n, np.int32)
        oj = np.empty(n, np.int32)
        self._check(lib().adcgpu_export_coo(self._h, n, ptr(h), ptr(oi, _ip), ptr(oj, _ip)), "export_coo")
        return h, oi, oj

    def write_hmlt_files(self, directory: str, flag: str = "i"):
        self._check(lib().adcgpu_write_hmlt_files(self._h, directory.encode(), flag.encode()), "write_hmlt_files")

    # -- sigma ----------------------------------------------------------------
    def sigma(self, V: np.ndarray) -> np.ndarray:
        V = np.asfortranarray(V, dtype=np.float64)
        one = V.ndim == 1
        if one:
            V = V.reshape(-1, 1, order="F")
        self._rows(V, "sigma")
        W = np.empty_like(V, order="F")
        self._check(lib().adcgpu_sigma(self._h, V.shape[1], ptr(V), ptr(W)), "sigma")
        return W[:, 0] if one else W

    def sigma_device(self, m: int, dv: int, dw: int, ld: int):
        self._check(lib().adcgpu_sigma_device(self._h, m, C.c_void_p(dv), C.c_void_p(dw), ld), "sigma_device")

    def last_sigma_ms(self) -> float:
        return float(lib().adcgpu_last_sigma_ms(self._h))

    def sigma_stats(self, reset: bool = False) -> dict:
        out = np.zeros(4)
        self._check(lib().adcgpu_sigma_stats(self._h, ptr(out), int(reset)), "sigma_stats")
        return {"calls": int(out[0]), "ms": float(out[1]), "alg_bytes": float(out[2]), "columns": int(out[3])}

    def sigma_stats_by_store(self, reset: bool = False) -> dict:
        """sigma_stats split by the value store the calls read (the mixed
        ladder's BF16, FP32 and FP64 phases)."""
        out = np.zeros(12)
        self._check(lib().adcgpu_sigma_stats_by_store(self._h, ptr(out), int(reset)), "sigma_stats_by_store")
        return {name: {"calls": int(out[4 * k]), "ms": float(out[4 * k + 1]), "alg_bytes": float(out[4 * k + 2]),
                       "columns": int(out[4 * k + 3])}
                for k, name in enumerate(("bf16", "fp32", "fp64"))}

    def device_bytes(self) -> int:
        return int(lib().adcgpu_device_bytes(self._h))

    def set_fp64_arith(self, mode: int):
        """0: FP64 fused multiply-adds (default); 1: double-float arithmetic
        on the FP32 pipe for FP64 block products of 16 or more columns."""
        self._check(lib().adcgpu_set_fp64_arith(self._h, int(mode)), "set_fp64_arith")

    # -- solvers --------------------------------------------------------------
    def davdiag_block(self, davstates: int, davtol: float, dmain: int = 0, maxsubdim: int = -1, maxiter: int = 100,
                      precon: int = PRECON_DPR, ldfl: bool = True, lsubdiag: bool = False, guessdim: int = 800,
                      precision: int = ADCGPU_FP64, refine: int = 0, tol_bf16: float = 0.0,
                      tol_fp32: float = 0.0, want_vectors: bool = True,
                      raise_on_nonconv: bool = True, refine_block: int = 0,
                      ladc1guess: bool = False) -> DavidsonResult:
        """ladc1guess: initvec_adc1 (the ADC(1) eigenvectors) as the guess,
        ahead of lsubdiag, as davdiag_block's lrdadc1 (block_davidson.f90:94-117)."""
        p = DavParams(davstates=davstates, dmain=dmain, maxsubdim=maxsubdim, maxiter=maxiter, precon=precon,
                      ldfl=int(ldfl), lsubdiag=2 if ladc1guess else int(lsubdiag), guessdim=guessdim, davtol=davtol,
                      precision=precision, refine=refine, tol_bf16=tol_bf16, tol_fp32=tol_fp32,
                      refine_block=refine_block)
        ev = np.empty(davstates)
        vec = np.empty((self.ndim, davstates), order="F") if want_vectors else None
        info = DavInfo()
        st = lib().adcgpu_davidson(self._h, C.byref(p), ptr(ev), ptr(vec), C.byref(info))
        if st and not (st == 10 and not raise_on_nonconv):
            self._check(st, "davdiag_block")
        return DavidsonResult(ev, vec, st, info.iterations, info.nmult, info.nconv, info.seconds, info.sigma_seconds,
                              info.max_residual, info.iters_bf16, info.iters_fp32, info.iters_fp64,
                              info.nmult_reference)

    # -- dipole start vectors --------------------------------------------------------
    def set_dipole(self, dpl: np.ndarray):
        """The dipole matrix dpl (nbas x nbas) of one component in the MO basis."""
        d = np.asfortranarray(dpl, np.float64)
        nb = self.nocc + self.nvirt
        if d.shape != (nb, nb):
            raise AdcGpuError(12, f"set_dipole: dpl must be {nb} x {nb}")
        self._check(lib().adcgpu_set_dipole(self._h, ptr(d)), "set_dipole")

    def get_modifiedtm_adc2(self, kpq: np.ndarray | None = None) -> np.ndarray:
        """get_modifiedtm_adc2 (get_moment.f90:153-442): the f-vector
        <Psi_J|D|Psi_0> over the ADC(2)-s intermediate states, or over the
        CVS states of a CVS kpq."""
        ndim = adc2s_dim(self.nocc, self.nvirt)[0] if kpq is None else len(kpq) - 1
        kp = None if kpq is None else np.ascontiguousarray(kpq, np.int32)
        mtm = np.empty(ndim)
        self._check(lib().adcgpu_modified_tm_adc2(self._h, ndim, None if kp is None else ptr(kp, _ip), ptr(mtm)),
                    "get_modifiedtm_adc2")
        return mtm

    def lancdiag_block(self, q0: np.ndarray, ncycles: int, orthotype: int = 0, want_tmat: bool = True,
                       want_evals: bool = True, want_ritz: bool = False):
        q0 = np.asfortranarray(q0, np.float64)
        self._rows(q0, "lancdiag_block")
        b = q0.shape[1]
        nvec = b * ncycles
        T = np.empty((nvec, nvec), order="F") if want_tmat else None
        ev = np.empty(nvec) if want_evals else None
        R = np.empty((self.ndim, nvec), order="F") if want_ritz else None
        self._check(lib().adcgpu_block_lanczos(self._h, b, ncycles, orthotype, ptr(q0), ptr(T), ptr(ev), ptr(R)),
                    "lancdiag_block")
        return T, ev, R

    def silstep(self, psi: np.ndarray, dtpsi: np.ndarray, intperiod: float, intorder: int, tol: float,
                relax: bool = False, restart: bool = True, stdform: bool = True):
        psi = np.ascontiguousarray(psi, np.complex128)
        dtpsi = np.ascontiguousarray(dtpsi, np.complex128)
        if psi.shape != (self.ndim,) or dtpsi.shape != (self.ndim,):
            raise AdcGpuError(12, f"silstep: psi and dtpsi must hold {self.ndim} values")
        step = C.c_double(0.0)
        order = C.c_int(0)
        state = SilState()
        st = lib().adcgpu_silstep(self._h, ptr(psi.view(np.float64)), ptr(dtpsi.view(np.float64)), len(psi),
                                  intperiod, intorder, tol, int(relax), int(restart), int(stdform), C.byref(step),
                                  C.byref(order), C.byref(state))
        self._check(st, "silstep")
        return psi, dtpsi, step.value, order.value, state

    def propagate_fvec(self, fvecs: np.ndarray, tout: float, tfinal: float, kdim: int, autotol: float):
        """Autocorrelation a(t) of each column of fvecs (t = 0, tout, 2 tout, ...)."""
        f = np.asfortranarray(fvecs, np.float64)
        if f.ndim == 1:
            f = f.reshape(-1, 1, order="F")
        self._rows(f, "propagate_fvec")
        nwp = f.shape[1]
        nt = int(tfinal / (0.5 * tout)) + 1
        out = np.zeros((nwp, nt, 2))
        ntimes = C.c_int(0)
        nmult = C.c_int64(0)
        self._check(lib().adcgpu_autocorr(self._h, nwp, ptr(f), tout, tfinal, kdim, autotol, ptr(out),
                                          C.byref(ntimes), C.byref(nmult)), "propagate_fvec")
        a = out[..., 0] + 1j * out[..., 1]
        return a[:, : ntimes.value], int(nmult.value)

    # -- Chebyshev order-domain autocorrelation ------------------------------------
    def spectral_bounds(self, precon: int = PRECON_OLSEN, maxiter: int = 100, ldfl: bool = True,
                        guessdim: int = 800) -> np.ndarray:
        """spectral_bounds(bounds,'c','davlanc',...) (specbounds.f90:121-205):
        the unwidened [Emin, Emax] estimate.  precon, maxiter, ldfl and
        guessdim are the final-space Davidson settings the reference leaves
        to the user (precon_f, maxiter_f, ldfl_f, guessdim_f)."""
        p = DavParams(maxiter=maxiter, precon=precon, ldfl=int(ldfl), guessdim=guessdim)
        b = np.zeros(2)
        self._check(lib().adcgpu_spectral_bounds(self._h, C.byref(p), ptr(b)), "spectral_bounds")
        return b

    def chebyshev_auto(self, q0: np.ndarray, bounds, chebyord: int, save1h1p: bool = False, df: bool = False):
        """C_k, k = 0..2 ord, of chebyshev_auto (chebyspec.f90:246-330) for each
        column of q0 (ord = chebyord rounded down to even).  df: double-float
        sigma arithmetic for blocks of >= 16 vectors.  Returns
        (auto[nvec, 2 ord + 1], q1h1p[nvec, ord + 1, n1] or None)."""
        q = np.asfortranarray(q0, np.float64)
        if q.ndim == 1:
            q = q.reshape(-1, 1, order="F")
        self._rows(q, "chebyshev_auto")
        nvec = q.shape[1]
        b = self._bounds(bounds)
        ordr = max(chebyord, 0) - max(chebyord, 0) % 2     # the library's rounded order sets the strides
        out = np.zeros((nvec, 2 * ordr + 1))
        h1 = np.zeros((nvec, ordr + 1, self.nocc * self.nvirt)) if save1h1p else None
        o = C.c_int(0)
        self._check(lib().adcgpu_chebyshev_auto(self._h, nvec, ptr(q), ptr(b), chebyord, int(df), ptr(out),
                                                ptr(h1), C.byref(o)), "chebyshev_auto")
        if o.value != ordr:
            raise AdcGpuError(12, f"chebyshev_auto: order {o.value}, expected {ordr}")
        return out, h1

    def project_psi0(self, q0: np.ndarray, bounds, chebyord: int, projen: float, df: bool = False) -> np.ndarray:
        """project_psi0 (chebyspec.f90:398-470) on a copy of q0 (columns)."""
        q = np.array(q0, np.float64, order="F", copy=True)
        one = q.ndim == 1
        if one:
            q = q.reshape(-1, 1, order="F")
        self._rows(q, "project_psi0")
        b = self._bounds(bounds)
        self._check(lib().adcgpu_chebyshev_project(self._h, q.shape[1], ptr(q), ptr(b), chebyord, projen,
                                                   int(df)), "project_psi0")
        return q[:, 0] if one else q


def write_davidson_file(path: str, evals: np.ndarray, evecs: np.ndarray) -> None:
    """The davname eigenpair file of wreigenpairs (block_davidson.f90:1469-1532):
    one Fortran unformatted sequential record (i, E_i, x_i) per root, roots in
    the given (ascending) order; readdavvc (adc_common.f90:999-1052) reads it."""
    ev = np.ascontiguousarray(evals, np.float64).reshape(-1)
    X = np.asfortranarray(evecs, np.float64)
    if X.ndim != 2 or X.shape[1] != ev.shape[0]:
        raise AdcGpuError(12, f"write_davidson_file: {ev.shape[0]} values but vectors of shape {X.shape}")
    st = lib().adcgpu_write_davidson_file(path.encode(), X.shape[0], X.shape[1], ptr(ev), ptr(X))
    if st:
        raise AdcGpuError(st, f"write_davidson_file {path}")


def read_davidson_file(path: str, ndim: int):
    """Records (i, E_i, x_i) of a davname file, as readdavvc reads them."""
    idx, ev, vecs = [], [], []
    with open(path, "rb") as f:
        while True:
            head = f.read(4)
            if not head:
                break
            n = int(np.frombuffer(head, np.int32)[0])
            body = f.read(n)
            tail = int(np.frombuffer(f.read(4), np.int32)[0])
            if n != tail or n != 12 + 8 * ndim:
                raise AdcGpuError(12, f"{path}: record of {n} bytes (trailer {tail}), expected {12 + 8 * ndim}")
            idx.append(int(np.frombuffer(body[:4], np.int32)[0]))
            ev.append(float(np.frombuffer(body[4:12], np.float64)[0]))
            vecs.append(np.frombuffer(body[12:], np.float64).copy())
    return np.array(idx), np.array(ev), np.array(vecs).T


def fortran_e(x: float, w: int = 21, d: int = 14) -> str:
    """Fortran Ew.d edit descriptor (0.ddddE+xx form, as gfortran writes it)."""
    x = float(x)
    if x == 0.0:
        body = "0." + "0" * d + "E+00"
    else:
        m, e = f"{abs(x):.{d - 1}e}".split("e")
        digits = m.replace(".", "")
        ex = int(e) + 1
        body = "0." + digits + (f"E{ex:+03d}" if abs(ex) <= 99 else f"{ex:+04d}")
    if x < 0.0 or (x == 0.0 and np.signbit(x)):
        body = "-" + body
    return body.rjust(w)


def write_chebyshev_auto(path: str, bounds, auto) -> None:
    """The 'chebyauto' file of write_chebyshev_auto (chebyspec.f90:334-368)."""
    with open(path, "w") as f:
        f.write("#    Spectral bounds:" + "".join("  " + fortran_e(b) for b in bounds) + "\n\n")
        f.write("#    Order [k]    C_k\n")
        for k, c in enumerate(auto):
            f.write(f"{k:6d}" + " " * 11 + fortran_e(c) + "\n")


def write_cheby1h1p(path: str, q1h1p) -> None:
    """The 'cheby1h1p' file of write_1h1p (chebyspec.f90:372-394): one Fortran
    unformatted sequential record per order k = 0..ord."""
    with open(path, "wb") as f:
        for col in np.asarray(q1h1p, np.float64):
            rec = np.ascontiguousarray(col).tobytes()
            mark = np.int32(len(rec)).tobytes()
            f.write(mark + rec + mark)


def chebyshev_auto_order_domain(g: "AdcGpu", q0: np.ndarray, chebyord: int, bounds=None, lprojpsi0: bool = False,
                                projen: float = 0.0, save1h1p: bool = False, outdir: str | None = None,
                                precon: int = PRECON_OLSEN, df: bool = False):
    """chebyshev_auto_order_domain (chebyspec.f90:25-116) for the columns of q0:
    spectral bounds (estimated by spectral_bounds when not given) widened to
    [0.9 Emin, 1.1 Emax] (:84-85), optional projection onto an energy window
    (:90), the order-domain autocorrelation, and, with outdir, the files
    'chebyauto' (and 'cheby1h1p') of the first column.
    Returns (auto, q1h1p, widened bounds)."""
    import os

    b = g.spectral_bounds(precon) if bounds is None else np.asarray(bounds, np.float64)
    b = np.array([0.9 * b[0], 1.1 * b[1]])
    q = np.asfortranarray(q0, np.float64)
    if lprojpsi0:
        q = g.project_psi0(q, b, chebyord, projen, df)
    auto, q1 = g.chebyshev_auto(q, b, chebyord, save1h1p, df)
    if outdir is not None:
        write_chebyshev_auto(os.path.join(outdir, "chebyauto"), b, auto[0])
        if save1h1p:
            write_cheby1h1p(os.path.join(outdir, "cheby1h1p"), q1[0])
    return auto, q1, b
