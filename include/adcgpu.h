/*
 * adcgpu.h -- C ABI of the GB300 (sm_103a) ADC(2)-s hot path.
 *
 * One shared library, libadcgpu.so, replaces four Fortran subsystems of
 * mschuurman/ADC_ottawa beneath the unchanged Fortran driver:
 *
 *   builder   write_fspace_adc2_1        source/adclib/fspacetrial.f90:533-564
 *             (get_offdiag_adc2_save_omp source/adclib/get_matrix.f90:705-1186,
 *              get_diag_adc2_save        source/adclib/get_matrix.f90:267-311)
 *   solvers   davdiag_block              source/eigen/block_davidson.f90:33-145
 *             lancdiag_block             source/eigen/block_lanczos.f90:28-81
 *   SIL       SILStep                    source/propagation/sillib.f90:108-393
 *             propagate_sillib           source/propagation/fvecprop.f90:365-564
 *   Chebyshev chebyshev_auto_order_domain source/propagation/chebyspec.f90:25-116
 *             spectral_bounds            source/propagation/specbounds.f90:24-205
 *
 * Conventions
 *   - Plain C types only.  Host arrays are owned by the caller; the library
 *     owns all device memory, held in an adcgpu_ctx.
 *   - Matrices and vector blocks are Fortran column-major (leading dimension
 *     = number of rows), exactly as the reference keeps vmat/wmat/qmat.
 *   - Orbital and configuration indices in kpq and in exported COO triples are
 *     1-based, as in the reference.
 *   - Every entry point returns an adcgpu_status; nothing calls exit()/abort().
 *     adcgpu_last_error() gives a one-line description of the last failure.
 *   - A context is used from one host thread; it owns one CUDA stream.
 */
#ifndef ADCGPU_H
#define ADCGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  1-4 are the SIL error codes of sillib.f90:84-89. */
enum adcgpu_status {
  ADCGPU_OK = 0,
  ADCGPU_SIL_BAD_ORDER = 1,       /* "Illegal integration order"  */
  ADCGPU_SIL_STEP_UNDERFLOW = 2,  /* "Stepsize underflow"         */
  ADCGPU_SIL_DIAG_FAILED = 3,     /* "Diagonalisation failed"     */
  ADCGPU_SIL_BAD_RESTART = 4,     /* "Illegal initial stepsize"   */
  ADCGPU_NOT_CONVERGED = 10,      /* block_davidson.f90:767-770   */
  ADCGPU_OUT_OF_MEMORY = 11,
  ADCGPU_BAD_INPUT = 12,
  ADCGPU_CUDA_ERROR = 13,
  ADCGPU_DEVICE_TIMEOUT = 14,     /* a bounded device wait gave up */
  ADCGPU_NO_MATRIX = 15,          /* solver called before the builder */
  ADCGPU_UNSUPPORTED = 16,        /* e.g. a kpq that is not C1 ADC(2)-s */
  ADCGPU_EIGEN_FAILED = 17        /* dsyev/dsbev/dsteqr equivalent failed */
};

/* Storage precision of the stored matrix used by the sigma-vector product. */
enum adcgpu_precision {
  ADCGPU_FP64 = 0,   /* FP64 values, FP64 vectors: the plain drop-in path      */
  ADCGPU_MIXED = 1,  /* BF16/FP32 values, FP32 vectors and subspace GEMMs,
                        FP64 Rayleigh-Ritz, Gram-Schmidt and residual norms    */
  ADCGPU_DIRECT = 2  /* FP64 as ADCGPU_FP64, but the coupling block is not
                        stored: every sigma product recomputes it from the
                        integrals, a chunk of slabs at a time (the matvec
                        path, get_matvec_adc2s_omp dmatvec_davidson.f90
                        :1031-1230; ph-ph block from Ca1/Cb1/Cc1/Cc2)        */
};

/* Preconditioners (parameters.f90 precon; block_davidson.f90:1119-1123). */
enum adcgpu_precon {
  ADCGPU_PRECON_DPR = 1,    /* dpr   block_davidson.f90:1288-1342 */
  ADCGPU_PRECON_OLSEN = 2,  /* olsen block_davidson.f90:1346-1419 */
  ADCGPU_PRECON_MLP = 3,    /* learned correction, DPR as fallback (and in
                               the FP64 refinement of ADCGPU_MIXED) */
  ADCGPU_PRECON_FOLD = 4    /* singles block with the doubles residual folded
                               in (no reference counterpart): t_d = DPR,
                               t_s = (lambda - Hss)^-1 (r_s + B^T t_d) by 8
                               MINRES steps; one extra sigma product of the
                               block per iteration.  Runs without deflation
                               (ldfl is ignored).  Not root-safe: like inverse
                               iteration it can converge to a state above a
                               missed one (measured: 1 of 12 seeded systems);
                               DPR and Olsen found the right set on all */
};

typedef struct adcgpu_ctx adcgpu_ctx;

/* ---------------------------------------------------------------------------
 * Seeded synthetic system (stands in for the GAMESS/MO-integral producer,
 * source/qclib/load_electronic_structure.f90:153-342).  Host only.
 * ------------------------------------------------------------------------- */

/* Orbital energies e[nocc+nvirt]: occupied ~ U(-1.4,-0.4) Ha first, then
   virtual ~ U(0.1,3.0) Ha, each block sorted ascending. */
int adcgpu_synth_orbitals(int nocc, int nvirt, uint64_t seed, double* e);

/* Number of doubles in the canonical 8-fold packed ERI array for nbas MOs. */
int64_t adcgpu_eri_packed_size(int nbas);

/* Real MO ERIs (pq|rs) with 8-fold symmetry, one draw per canonical
   quadruple p>=q, r>=s, pq>=rs (1-based):
   N(0,1) * 0.3 * exp(-0.15|p-r| - 0.15|q-s|).  nthreads<=0: all cores. */
int adcgpu_synth_eri_packed(int nbas, uint64_t seed, double* eri, int nthreads);

/* Seeded "dipole-like" start block: nrow x ncol uniform(0,1) values
   (the random_number draws of init_vecs_random, block_lanczos.f90:402-439). */
int adcgpu_synth_uniform_block(int64_t nrow, int ncol, uint64_t seed, double* out);

/* Dipole matrix dpl(p,q) of one Cartesian component in the MO basis (the
   reference reads it from the GAMESS dipole integrals into the global dpl,
   source/qclib/load_electronic_structure.f90): nbas x nbas, column-major,
   symmetric, one draw per p>=q (1-based):
   N(0,1) * 0.5 * exp(-0.1|p-q|). */
int adcgpu_synth_dipole(int nbas, uint64_t seed, double* dpl);

/* ---------------------------------------------------------------------------
 * Configuration list kpq (select_atom_is select_fano.f90:16-60 and
 * select_atom_d flag -1 select_fano.f90:539-718; C1 symmetry, no frozen core).
 * ------------------------------------------------------------------------- */

/* Returns ndim = n1 + n2; counts5 (may be NULL) receives kpq(1..5,0). */
int64_t adcgpu_adc2s_dim(int nocc, int nvirt, int32_t* counts5);

/* Fills kpq(7, 0:ndim), column-major int32, column 0 holding the counts. */
int adcgpu_select_adc2s(int nocc, int nvirt, int32_t* kpq);

/* CVS configuration list: select_atom_is_cvs (select_fano.f90:112-142) and
   select_atom_d_cvs (:903-1027), C1 symmetry, no frozen orbitals.  core[ncore]
   holds the core orbitals (the icore list, 1-based occupied indices,
   0 < ncore < nocc).  Singles (a, core hole); doubles of the classes a=b,i<j
   and a<b,i<j (spin I, then the spin II copy) whose hole pair holds exactly
   one core orbital.  adcgpu_cvs_dim returns ndim (-1 on bad input) and fills
   counts5 = kpq(1..5,0) (may be NULL). */
int64_t adcgpu_cvs_dim(int nocc, int nvirt, int ncore, const int32_t* core, int32_t* counts5);
int adcgpu_select_adc2s_cvs(int nocc, int nvirt, int ncore, const int32_t* core, int32_t* kpq);

/* ---------------------------------------------------------------------------
 * Context.
 * ------------------------------------------------------------------------- */
int adcgpu_ctx_create(int device, adcgpu_ctx** out);
int adcgpu_ctx_destroy(adcgpu_ctx* ctx);
const char* adcgpu_last_error(const adcgpu_ctx* ctx);

/* Orbital data (parameters.f90:21-32: e, nOcc, nVirt; occupied first). */
int adcgpu_set_orbitals(adcgpu_ctx* ctx, int nocc, int nvirt, const double* e);

/* ERIs as the canonical 8-fold packed real array (adcgpu_eri_packed_size). */
int adcgpu_set_eri_packed(adcgpu_ctx* ctx, const double* eri);

/* ERIs in the reference layout: moIntegrals%buffer_real, complex(8)
   (nmo,nmo,nmo,nmo) column-major, read through vpqrs (vpqrsmod.f90:13-27):
   the real part of element (r,s,u,v) is (rs|uv). */
int adcgpu_set_eri_mo_complex(adcgpu_ctx* ctx, const double* buffer_real);

/* ---------------------------------------------------------------------------
 * Builder: write_fspace_adc2_1(ndim,kpq,noffdel,chr), fspacetrial.f90:533-564.
 * Keeps H resident on the device.  kpq must be the ADC(2)-s list that
 * adcgpu_select_adc2s produces (checked; ADCGPU_UNSUPPORTED otherwise).
 * noffd_out = number of upper-triangle elements with |h| > minc = 1e-12
 * (the reference's count, get_matrix.f90:904,1059-1063).
 * precision: adcgpu_precision of the stored sigma-vector matrix.
 * ------------------------------------------------------------------------- */
int adcgpu_build_adc2s(adcgpu_ctx* ctx, int ndim, const int32_t* kpq,
                       int64_t* noffd_out, char flag, int precision);

/* CVS builder: write_fspace_adc2_1_cvs(ndim,kpq,noffdel,chr),
   fspacetrial.f90:566-596 (get_offdiag_adc2_save_cvs_omp get_matrix.f90
   :1323-1726 and get_diag_adc2_save :267-311).  core[ncore] is the icore
   list; kpq must be the list adcgpu_select_adc2s_cvs produces for it (checked;
   NULL = that list).  The matrix is held in FP64 (ph-ph block dense, coupling
   block as compressed rows) and replaces any matrix the context held; the
   sigma product, Davidson (ondiag guess, DPR or Olsen), block Lanczos, SIL,
   the COO export and the SCRATCH files then work on it.  The COO lists the
   ph-ph pairs as the reference's loop writes them (oi > oj), then the
   coupling entries (oi = single < oj = double). */
int adcgpu_build_adc2s_cvs(adcgpu_ctx* ctx, int ndim, const int32_t* kpq, int ncore,
                           const int32_t* core, int64_t* noffd_out, char flag);

/* Diagonal hii(ndim) (get_diag_adc2_save, get_matrix.f90:267-311). */
int adcgpu_get_diag(adcgpu_ctx* ctx, double* hii);

/* The kept off-diagonal elements as COO (h, oi<oj, 1-based), the content of
   SCRATCH/hmlt.off<flag>.  As in the reference, whose file order depends on
   the OpenMP schedule (get_matrix.f90:1059-1125), only the set is defined:
   the ph-ph block comes first (row-major), then the coupling block in the
   device's storage order.  cap must be >= noffd. */
int adcgpu_export_coo(adcgpu_ctx* ctx, int64_t cap, double* h, int32_t* oi,
                      int32_t* oj);

/* Writes SCRATCH-style files <dir>/hmlt.dia<flag> and <dir>/hmlt.off<flag>
   with the reference's Fortran unformatted sequential record layout
   (filetools.f90:24-44, buf_size = 655360). */
int adcgpu_write_hmlt_files(adcgpu_ctx* ctx, const char* dir, char flag);

/* ---------------------------------------------------------------------------
 * Dipole start vectors.
 * ------------------------------------------------------------------------- */

/* The dipole matrix dpl(p,q) of one component in the MO basis (the module
   array dpl that dipole_ph.f90 reads): nbas x nbas, column-major.  Held on
   the device until the orbitals change or the context is destroyed. */
int adcgpu_set_dipole(adcgpu_ctx* ctx, const double* dpl);

/* get_modifiedtm_adc2(ndim,kpq,mtm,ista), get_moment.f90:153-442: the
   ADC(2) f-vector mtm(J) = <Psi_J|D|Psi_0> over the ADC(2)-s intermediate
   states (kpq as for adcgpu_build_adc2s; NULL = that list), from the
   orbitals, ERIs and dipole matrix of the context.  It is the start vector
   of the final-space Lanczos (lanczos_guess_vecs, adc2_opa.f90:380-520),
   of the wavepacket propagation (init_wavepacket, fvecprop.f90:338-357)
   and of the Chebyshev autocorrelation (adc2_autospec.f90:162).  A CVS kpq
   (adcgpu_select_adc2s_cvs, ndim its dimension) gives the CVS f-vector (the
   i=j classes are absent, as lcvs skips them, :365-366).  FP64; mtm: host
   array of ndim doubles. */
int adcgpu_modified_tm_adc2(adcgpu_ctx* ctx, int ndim, const int32_t* kpq, double* mtm);

/* fill_stvc(ndim,vctr), fspacetrial.f90:1255-1270: the indices (1-based) of
   the lmain largest vctr(i)^2 in the order of dsortindxa1('D')
   (misc.f90:492+), the unit start vectors of lancguess = 1. */
int adcgpu_fill_stvc(int ndim, const double* vctr, int lmain, int32_t* stvc_lbl);

/* ---------------------------------------------------------------------------
 * Sigma-vector product W = H V for m columns (hxvec_incore,
 * block_davidson.f90:844-883; hxq_incore block_lanczos.f90:1325-1361).
 * Host arrays, ndim x m column-major.
 * ------------------------------------------------------------------------- */
int adcgpu_sigma(adcgpu_ctx* ctx, int m, const double* v, double* w);

/* Same on device buffers (leading dimension ld >= ndim), on the context's
   stream.  For ADCGPU_MIXED the device arrays are float. */
int adcgpu_sigma_device(adcgpu_ctx* ctx, int m, const void* dv, void* dw, int64_t ld);

/* ---------------------------------------------------------------------------
 * Block Davidson: davdiag_block(matdim,noffd), block_davidson.f90:33-145.
 * Parameters mirror the module globals read in davinitialise (:163-183).
 * ------------------------------------------------------------------------- */
typedef struct {
  int davstates;     /* nstates                                     */
  int dmain;         /* blocksize; 0 -> max(nstates+5, 2*nstates)   */
  int maxsubdim;     /* maxvec; <0 -> 4*blocksize                   */
  int maxiter;       /* niter                                       */
  int precon;        /* adcgpu_precon                               */
  int ldfl;          /* deflation of converged vectors (1/0); not
                        used with ADCGPU_PRECON_FOLD                */
  int lsubdiag;      /* 1: initvec_subdiag, 2: initvec_adc1 (the
                        reference's ladc1guess), 0: initvec_ondiag  */
  int guessdim;      /* subspace dimension for initvec_subdiag      */
  double davtol;     /* residual-norm tolerance                     */
  int precision;     /* adcgpu_precision for the iterations         */
  int refine;        /* MIXED: maxvec of the FP64 refinement, in blocks (0: 4) */
  double tol_bf16;   /* MIXED: residual at which the BF16-valued phase hands
                        over to the FP32-valued phase (0: 1e-2; <0: skip)    */
  double tol_fp32;   /* MIXED: residual at which the FP32 phase hands over to
                        the FP64 refinement (0: 1e-5 with ADCGPU_PRECON_FOLD,
                        5e-6 otherwise); the BF16 and FP32 phases also hand
                        over when their largest residual has not fallen by
                        10 % in 12 iterations (their precision floor)        */
  int refine_block;  /* MIXED: block size of the FP64 refinement, between
                        davstates and the solver's blocksize (0: min(blocksize,
                        max(davstates + 10, 1.5 davstates))); a block of
                        exactly davstates can miss a root                    */
} adcgpu_dav_params;

typedef struct {
  int iterations;    /* Davidson iterations performed (all phases) */
  int64_t nmult;     /* sigma-vector columns computed             */
  int nconv;         /* converged roots                           */
  double seconds;    /* wall time inside the solver               */
  double sigma_seconds;  /* time in the sigma-vector kernels      */
  double max_residual;   /* FP64 residual norm of the worst root  */
  int iters_bf16, iters_fp32, iters_fp64;   /* iterations per phase    */
  int64_t nmult_reference;  /* sigma columns the reference algorithm would
                               compute (it re-multiplies all currdim
                               columns every iteration)                 */
} adcgpu_dav_info;

/* evals[davstates] ascending; evecs ndim x davstates column-major (may be
   NULL).  Returns ADCGPU_NOT_CONVERGED when maxiter is exhausted (results are
   still written). */
int adcgpu_davidson(adcgpu_ctx* ctx, const adcgpu_dav_params* p, double* evals,
                    double* evecs, adcgpu_dav_info* info);

/* Writes the eigenpair records (i, E_i, x_i) like wreigenpairs
   (block_davidson.f90:1469-1532) to a Fortran unformatted sequential file. */
int adcgpu_write_davidson_file(const char* path, int ndim, int nstates,
                               const double* evals, const double* evecs);

/* ---------------------------------------------------------------------------
 * Block Lanczos: lancdiag_block(dimf,noff,flag), block_lanczos.f90:28-81.
 * q0: ndim x lmain start block of raw values; it is normalised and
 * orthonormalised by double MGS exactly as init_vecs_random (:402-439).
 * orthotype: 0 none, 1 PRO (:1474-1526).
 * tmat (nvec x nvec, nvec = lmain*ncycles) receives T as assembled at
 * :1197-1219; evals (nvec) the dsbev eigenvalues (calc_pseudospec :1941).
 * ritz (ndim x nvec, may be NULL): normalised Ritz vectors (:2237-2316).
 * ------------------------------------------------------------------------- */
int adcgpu_block_lanczos(adcgpu_ctx* ctx, int lmain, int ncycles, int orthotype,
                         const double* q0, double* tmat, double* evals,
                         double* ritz);

/* ---------------------------------------------------------------------------
 * SIL propagation.
 * ------------------------------------------------------------------------- */

/* The reference's SAVE variables of SILStep (sillib.f90:131-133) made
   explicit, one per wavepacket. */
typedef struct {
  int old_order;
  double old_error;
  double old_stepsize;
} adcgpu_sil_state;

/* One SILStep (sillib.f90:108-393) with Func = matxvec_treal
   (tdselib.f90:323-437, v2 = -i H v1) on the built matrix.
   psi, dtpsi: complex(8) arrays of length psidim (interleaved re,im) on the
   host; dtpsi must hold -iH psi on entry (as in fvecprop.f90:496).
   krylov: complex(8) psidim x (intorder-1) host work array (may be NULL:
   then the library keeps the Krylov vectors on the device; non-restart
   calls then need the same context).  Returns 0 or a SIL error code 1-4. */
int adcgpu_silstep(adcgpu_ctx* ctx, double* psi, double* dtpsi, int psidim,
                   double intperiod, int intorder, double tol, int relax,
                   int restart, int stdform, double* stepsize_out,
                   int* trueorder_out, adcgpu_sil_state* st);

/* propagate_sillib (fvecprop.f90:365-564) for nwp wavepackets at once.
   f: ndim x nwp real start vectors (f-vectors, normalised internally as in
   init_wavepacket :338-357).  Autocorrelation a(t) = sum_j psi_j(t/2)^2 *
   ||f||^2 at t = 0, tout, 2 tout, ... (ntimes = int(tfinal/(tout/2)) + 1
   values per wavepacket), written to auto_out as complex interleaved,
   layout [wavepacket][time].  nmult_out (may be NULL): matvecs per packet. */
int adcgpu_autocorr(adcgpu_ctx* ctx, int nwp, const double* f, double tout,
                    double tfinal, int kdim, double tol, double* auto_out,
                    int* ntimes_out, int64_t* nmult_out);

/* ---------------------------------------------------------------------------
 * Chebyshev order-domain autocorrelation (source/propagation/chebyspec.f90,
 * chebyshev_auto_order_domain :25-116), for nvec start vectors at once.
 * ------------------------------------------------------------------------- */

/* chebyshev_auto (chebyspec.f90:246-330) with chebyshev_recursion and
   matxvec_chebyshev_incore (tdselib.f90:1228-1398): q_k = T_k(H_norm) q_0,
   H_norm = (2/(Emax-Emin)) H - (2 Emin/(Emax-Emin) + 1).  bounds = {Emin, Emax}
   are used as given (the reference driver widens its estimate to
   {0.9 Emin, 1.1 Emax} first, :84-85).  chebyord is rounded down to even (ord,
   chebyshev_initialise :136; written to order_out, may be NULL).
   q0: ndim x nvec column-major.  auto_out: nvec x (2 ord + 1), layout
   [vector][k], C_k = <q_0|q_k> for k <= ord and the doubling formulas above.
   q1h1p (may be NULL, the save1h1p output): the first nocc*nvirt elements of
   q_0..q_ord, layout [vector][k][n1].
   df != 0: for nvec >= 16 the sigma product's tiled pass runs in double-float
   arithmetic on the FP32 pipe (a 48-bit significand, about 1e-14 relative
   per product) instead of native FP64, whose pipe GB300 runs at 1/64 of the
   FP32 rate; df = 0 is the plain FP64 path. */
int adcgpu_chebyshev_auto(adcgpu_ctx* ctx, int nvec, const double* q0,
                          const double* bounds, int chebyord, int df,
                          double* auto_out, double* q1h1p, int* order_out);

/* project_psi0 (chebyspec.f90:398-470): q0 <- sum_k f_k g_k T_k(H_norm) q0,
   the Jackson-damped Chebyshev expansion of the step function at projen, in
   place on the ndim x nvec block q0 (not normalised, as in the reference).
   ADCGPU_BAD_INPUT when projen lies outside bounds (the reference's acos
   would return NaN).  df as for adcgpu_chebyshev_auto. */
int adcgpu_chebyshev_project(adcgpu_ctx* ctx, int nvec, double* q0,
                             const double* bounds, int chebyord, double projen,
                             int df);

/* spectral_bounds_davlanc (specbounds.f90:121-205): bounds[0] from a one-root
   block Davidson with block 5, subspace 20, tol 1e-8 and the initvec_subdiag
   guess (the five settings specbounds makes), taking maxiter, precon, ldfl
   and guessdim from fp, the caller's final-space parameters (may be NULL:
   100, Olsen, deflation on, 800 -- the reference defaults, defaults.f90:84-94;
   a zero field also takes its default); the other fields of fp are ignored.
   bounds[1] is the highest Lanczos state energy of a block Lanczos (block 2,
   100 cycles, PRO) started from init_vec_singlesubspace
   (block_lanczos.f90:748-923).  Returns the bounds unwidened.
   Needs ndim >= 200. */
int adcgpu_spectral_bounds(adcgpu_ctx* ctx, const adcgpu_dav_params* fp,
                           double* bounds);

/* ---------------------------------------------------------------------------
 * Learned preconditioner (ADCGPU_PRECON_MLP).  No counterpart routine in the
 * reference: it replaces the diagonal preconditioner of dpr
 * (block_davidson.f90:1288-1342) by t = m * r / (lambda - h), m = MLP(features),
 * and falls back to dpr when no network is loaded.  The parameter vector is
 * W1[256][16], b1[256], W2[256][256], b2[256], w3[256], b3 (FP32).
 * ------------------------------------------------------------------------- */
int64_t adcgpu_mlp_num_params(void);
int adcgpu_mlp_set_params(adcgpu_ctx* ctx, const float* params, int64_t n);
int adcgpu_mlp_get_params(adcgpu_ctx* ctx, float* params, int64_t n);

/* One Adam step (lr > 0) or a gradient evaluation only (lr == 0) on G groups
   of S rows: features (G*S x 16), t0 = r / (lambda - h) and the target
   correction, from host arrays.  Loss = mean over groups of
   1 - cos^2(m * t0, target).  grad_out (may be NULL): the summed gradient. */
int adcgpu_mlp_train_step(adcgpu_ctx* ctx, int G, int S, const float* feats, const float* t0,
                          const float* target, float lr, float* loss_out, float* grad_out);

/* Fused inference on the built matrix for nb roots: m_out and t_out
   (N*nb, row q = i*N + j) for residuals R (N x nb, may be NULL) and Ritz
   values lam; feats_out (N*nb x 16, may be NULL) the features used. */
int adcgpu_mlp_infer(adcgpu_ctx* ctx, int nb, const double* lam, const double* R, float* m_out,
                     double* t_out, float* feats_out);

/* Davidson trace for training data: runs the FP64 Davidson of p and stores,
   every 'every' iterations, the residuals and Ritz vectors of the first
   davstates roots (N x davstates each) and their Ritz values, up to
   max_records iterations; converged eigenvectors go to evecs.
   *nrec receives the number of stored iterations. */
int adcgpu_davidson_trace(adcgpu_ctx* ctx, const adcgpu_dav_params* p, int every, int max_records,
                          double* R_out, double* X_out, double* lam_out, double* evals, double* evecs,
                          int* nrec);

/* ---------------------------------------------------------------------------
 * Timing helpers for benchmarks: device milliseconds of the last sigma
 * call as measured by CUDA events on the context's stream.
 * ------------------------------------------------------------------------- */
double adcgpu_last_sigma_ms(const adcgpu_ctx* ctx);

/* Device bytes held by the context (matrix, ERI blocks, work spaces). */
int64_t adcgpu_device_bytes(const adcgpu_ctx* ctx);

/* Arithmetic of the FP64 path's block products (no reference counterpart;
   the reference's FP64 arithmetic is MKL's): 0 (the default) FP64 fused
   multiply-adds; 1 double-float arithmetic on the FP32 pipe (hi + lo single
   precision pairs, about 1e-14 relative per product) for sigma products of
   16 or more columns and for the subspace GEMMs, which the GB300's FP64
   rate (1/64 of FP32) makes several times faster.  It applies to every
   solver that runs on the context (Davidson, Lanczos, SIL, Chebyshev); the
   mixed ladder's FP64 refinement always uses 1. */
int adcgpu_set_fp64_arith(adcgpu_ctx* ctx, int mode);

/* Number of CUDA kernels this library has launched in this process, over
   all contexts (a monotonic counter; differences give the launches of a
   region). */
uint64_t adcgpu_kernel_launches(void);

/* Sigma-product statistics accumulated since the last reset, measured with
   CUDA events on the context's stream around every sigma call (including
   those inside the solvers): out[0] calls, out[1] total device milliseconds,
   out[2] algorithmic bytes (per call: each kept coupling value once with a
   4-byte column index, the dense singles block as nocc^2 nvirt^2 values,
   nocc*nvirt+1 row pointers, the FP64 diagonal, the m vectors read and
   written once), out[3] columns multiplied.
   reset != 0 clears the counters after reading. */
int adcgpu_sigma_stats(adcgpu_ctx* ctx, double* out4, int reset);

/* The same four figures for each value store the calls read: out[0..3]
   BF16 values, out[4..7] FP32 values, out[8..11] FP64 values (the mixed
   ladder's three phases).  reset != 0 clears them (adcgpu_sigma_stats with
   reset clears them too). */
int adcgpu_sigma_stats_by_store(adcgpu_ctx* ctx, double* out12, int reset);

/* Allocation-free sigma product on device buffers, for callers that must
   not allocate device memory while they run: a host application whose
   device-memory budget is fixed in advance (the rest of the device belongs
   to another library or allocator), or a host thread that must not stall on
   cudaFree's device-wide wait.  No counterpart in the reference.  Same arguments and results as adcgpu_sigma_device for a matrix
   built with ADCGPU_MIXED (float buffers); instead of a context-owned,
   on-demand-allocated accumulator it uses a static device array of
   1,048,576 doubles (8 MiB, held by every device that loads the library
   until the process exits), so nocc*nvirt*m must not exceed 1,048,576
   (ADCGPU_BAD_INPUT otherwise).  The first call on a device looks up the
   array's device address; make that first call before any stream capture.
   All calls share the array: calls that overlap on the GPU race. */
int adcgpu_sigma_device_noalloc(adcgpu_ctx* ctx, int m, const void* dv, void* dw, int64_t ld);

/* Autotuner of the sigma kernels' launch shape: the tiled pass 1 against
   the per-warp pass 1 with its rows per work item (16..256), columns per
   pass (1, 2, 4) and staging, timed with CUDA events for m columns on the
   built matrix; the fastest shape is kept in the context and returned in
   the encoding of adcgpu_sigma_set_shape (the Python layer caches it in a
   JSON file). */
int adcgpu_sigma_autotune(adcgpu_ctx* ctx, int m, int* best_chunk, int* best_mc, double* best_ms);

/* Applies a launch shape (e.g. from the autotuner's cache).  In mc_fp64 /
   mc_fp32, bits 0-2 give the columns per pass, bit 3 selects the staged
   per-warp pass 1, bit 4 the per-warp pass 1 instead of the tiled one, bit
   5 the CUDA-core tiled pass 1 instead of the tensor-core one (BF16 values),
   bit 6 switches the tcgen05 sigma pass off, bit 7 runs segments A/B through
   the per-(slab, b') pass 2 and per-run pass 3 instead of the compact
   kernels, bit 8 makes a mixed-precision matrix's sigma product read the
   FP32 value store instead of the BF16 one, bit 9 keeps the FP32 Gram
   products (adcgpu_gram_f32 and the solvers' V^T W) on the CUDA cores, bit
   10 runs the FP32 values on two tcgen05 passes over their BF16 slices
   instead of the CUDA-core tile. */
int adcgpu_sigma_set_shape(adcgpu_ctx* ctx, int chunk, int mc_fp64, int mc_fp32);

/* The solvers' tall-skinny Gram product on device FP32 arrays: C(p x q,
   FP64, column-major, ldc) = A(N x p, lda)^T B(N x q, ldb), as calcrmat's
   dgemm (block_davidson.f90:954-967) and the projections of the block
   orthogonalisation (:1226-1284) form it on the mixed-precision phases.  For
   q <= 48 it runs on the tensor cores (each value split into three BF16
   slices, FP32-accurate products); otherwise on the CUDA cores. */
int adcgpu_gram_f32(adcgpu_ctx* ctx, int64_t N, int p, int q, const void* dA, int64_t lda, const void* dB,
                    int64_t ldb, double* dC, int ldc);

#ifdef __cplusplus
}
#endif

#endif /* ADCGPU_H */
