// Chebyshev order-domain autocorrelation on the GPU.
//
//   chebyshev_auto            chebyspec.f90:246-330
//   chebyshev_recursion       tdselib.f90:1228-1256
//   matxvec_chebyshev_incore  tdselib.f90:1300-1398
//   project_psi0              chebyspec.f90:398-470 (Jackson-damped filter)
//   spectral_bounds_davlanc   specbounds.f90:121-205
//   init_vec_singlesubspace   block_lanczos.f90:748-923
//
// P start vectors run together (column p of an N x P block).  Every order k is
// one FP64 sigma product of the block q_{k-1}, written into the buffer that
// will hold q_k, then one fused pass that turns it into q_k and accumulates
// the three inner products the autocorrelation needs, <q_0|q_k>, <q_k|q_k> and
// <q_{k-1}|q_k>, as per-block partial sums; a one-warp-per-sum kernel reduces
// those into the slot of order k on the device.  The expansion therefore runs
// with no host round trip: one copy brings the (ord+1) x P x 3 sums back at the
// end and C_k is assembled on the host as chebyshev_auto does it,
//   C_k      = <q_0|q_k>                     k = 0..ord
//   C_2k     = 2 <q_k|q_k> - C_0             k > ord/2
//   C_2k-1   = 2 <q_{k-1}|q_k> - C_1         k > ord/2.
// Three q buffers rotate (q_{k-2}, q_{k-1}, q_k); the sigma product never
// aliases its input.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

extern "C" int adcgpu_davidson(adcgpu_ctx* ctx, const adcgpu_dav_params* p, double* evals, double* evecs,
                               adcgpu_dav_info* info);
extern "C" int adcgpu_block_lanczos(adcgpu_ctx* ctx, int lmain, int ncycles, int orthotype, const double* q0,
                                    double* tmat, double* evals, double* ritz);

namespace adcgpu {

namespace {

// blocks of the fused pass: two per SM (c: the context in scope)
#define CHEB_BLK (c->nsm * 2)
constexpr int CHEB_THR = 256;

// Block partial sums of one pass, written to part[(blk*P + p)*3 + j].
__device__ __forceinline__ void block_sums3(double s0, double s1, double s2, int P, int p, double* __restrict__ part) {
  __shared__ double red[CHEB_THR / 32][3];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 16; o; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  if (lane == 0) { red[w][0] = s0; red[w][1] = s1; red[w][2] = s2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0, c = 0.0;
    for (int q = 0; q < CHEB_THR / 32; ++q) { a += red[q][0]; b += red[q][1]; c += red[q][2]; }
    double* d = part + ((int64_t)blockIdx.x * P + p) * 3;
    d[0] = a; d[1] = b; d[2] = c;
  }
  __syncthreads();
}

// <q_0|q_0> partials (slot 0 of the sums; the other two are zero).
__global__ void __launch_bounds__(CHEB_THR) k_cheb_norm0(int64_t N, int P, const double* __restrict__ Q0,
                                                         double* __restrict__ part) {
  for (int p = 0; p < P; ++p) {
    const double* q = Q0 + (int64_t)p * N;
    double s = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x)
      s = fma(q[r], q[r], s);
    block_sums3(s, 0.0, 0.0, P, p, part);
  }
}

// One order for P columns.  On entry Qk holds W = H q_{k-1}; on exit q_k:
//   q_k = a W - b q_{k-1}                  (k == 1)
//   q_k = 2 (a W - b q_{k-1}) - q_{k-2}    (k > 1, second != 0)
// a = 2/(Emax - Emin), b = 2 (Emin/(Emax - Emin)) + 1: the operations of
// matxvec_chebyshev_incore (:1380-1393) and chebyshev_recursion (:1240-1252)
// in the same order, each rounded separately (no contraction).
// acc (may be null): acc += ck q_k, the sum of project_psi0 (chebyspec.f90:446).
__global__ void __launch_bounds__(CHEB_THR) k_cheb_step(int64_t N, int P, double* __restrict__ Qk,
                                                        const double* __restrict__ Qkm1,
                                                        const double* __restrict__ Qkm2,
                                                        const double* __restrict__ Q0, double a, double b,
                                                        int second, double* __restrict__ acc, double ck,
                                                        double* __restrict__ part) {
  for (int p = 0; p < P; ++p) {
    const int64_t o = (int64_t)p * N;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
      const double v1 = Qkm1[o + r];
      double v = __dmul_rn(a, Qk[o + r]);
      v = __dsub_rn(v, __dmul_rn(b, v1));
      if (second) {
        v = __dmul_rn(2.0, v);
        v = __dsub_rn(v, Qkm2[o + r]);
      }
      Qk[o + r] = v;
      if (acc) acc[o + r] = __dadd_rn(acc[o + r], __dmul_rn(ck, v));
      s0 = fma(Q0[o + r], v, s0);
      s1 = fma(v, v, s1);
      s2 = fma(v1, v, s2);
    }
    block_sums3(s0, s1, s2, P, p, part);
  }
}

// sums[t] = sum over the nblk block partials of sum t = p*3 + j, in a fixed
// order (one warp per sum).
__global__ void k_cheb_reduce(int nblk, int P, const double* __restrict__ part, double* __restrict__ sums) {
  const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (t >= 3 * P) return;   // whole warps leave together
  double s = 0.0;
  for (int bl = lane; bl < nblk; bl += 32) s += part[(int64_t)bl * 3 * P + t];
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) sums[t] = s;
}

// acc = c q (the first term of project_psi0, :440)
__global__ void k_cheb_scale(int64_t n, double c, const double* __restrict__ q, double* __restrict__ acc) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    acc[r] = __dmul_rn(c, q[r]);
}

// V(rows[j0 + col], col) = 1 for col < m (V zeroed before): unit vectors of
// the subspace configurations.
__global__ void k_unit_cols(int64_t N, int m, const int64_t* __restrict__ rows, double* __restrict__ V) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col < m) V[(int64_t)col * N + rows[col]] = 1.0;
}

// S(i, col) = W(rows[i], col): the subspace rows of m columns of H.
__global__ void k_gather_rows(int64_t N, int sub, int m, const int64_t* __restrict__ rows,
                              const double* __restrict__ W, double* __restrict__ S) {
  const int64_t n = (int64_t)sub * m;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int col = (int)(t / sub), i = (int)(t - (int64_t)col * sub);
    S[t] = W[(int64_t)col * N + rows[i]];
  }
}

}  // namespace

struct ChebGPU {
  Ctx* c;
  int64_t N = 0;
  int P = 0, ord = 0;
  size_t blk_bytes = 0;
  double *Q0 = nullptr, *R[3] = {nullptr, nullptr, nullptr}, *acc = nullptr;
  double *part = nullptr, *sums = nullptr, *h1 = nullptr;
  size_t h1_bytes = 0, sums_bytes = 0;

  ~ChebGPU() {
    dfree(c, Q0, blk_bytes);
    for (double* r : R) dfree(c, r, blk_bytes);
    dfree(c, acc, blk_bytes);
    dfree(c, part, sizeof(double) * CHEB_BLK * 3 * (size_t)P);
    dfree(c, sums, sums_bytes);
    dfree(c, h1, h1_bytes);
  }

  int alloc(bool want_acc, int64_t n1, bool want_h1) {
    blk_bytes = sizeof(double) * (size_t)N * P;
    sums_bytes = sizeof(double) * 3 * (size_t)P * (ord + 1);
    ST(dmalloc(c, (void**)&Q0, blk_bytes));
    for (auto& r : R) ST(dmalloc(c, (void**)&r, blk_bytes));
    if (want_acc) ST(dmalloc(c, (void**)&acc, blk_bytes));
    ST(dmalloc(c, (void**)&part, sizeof(double) * CHEB_BLK * 3 * (size_t)P));
    ST(dmalloc(c, (void**)&sums, sums_bytes));
    if (want_h1) {
      h1_bytes = sizeof(double) * (size_t)n1 * (ord + 1) * P;
      ST(dmalloc(c, (void**)&h1, h1_bytes));
    }
    ADC_CUDA(c, cudaMemsetAsync(R[0], 0, blk_bytes, c->stream));
    return ADCGPU_OK;
  }

  int reduce_into(int k) {
    const int warps = 3 * P, wpb = CHEB_THR / 32;
    k_cheb_reduce<<<(warps + wpb - 1) / wpb, CHEB_THR, 0, c->stream>>>(CHEB_BLK, P, part, sums + (size_t)k * 3 * P);
    ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    return ADCGPU_OK;
  }

  // h1(:, k) of every column: the first n1 elements of q_k (save1h1p)
  int save_h1(int k, const double* q, int64_t n1) {
    if (!h1) return ADCGPU_OK;
    ADC_CUDA(c, cudaMemcpy2DAsync(h1 + (size_t)k * n1, sizeof(double) * (size_t)n1 * (ord + 1), q,
                                  sizeof(double) * (size_t)N, sizeof(double) * (size_t)n1, P,
                                  cudaMemcpyDeviceToDevice, c->stream));
    return ADCGPU_OK;
  }

  // Orders 1..ord from q_0 = Q0.  a, b: the scaling of matxvec_chebyshev;
  // coef (with acc): the projection coefficients f_k g_k.  df: the sigma
  // product's tiled pass in double-float arithmetic (restored on return).
  int expand(double a, double b, const std::vector<double>* coef, int64_t n1, int df) {
    struct DfScope {
      Ctx* c;
      int old;
      ~DfScope() { c->dense_df = old; }
    } scope{c, c->dense_df};
    c->dense_df = df ? 1 : 0;
    ADC_CUDA(c, cudaMemcpyAsync(R[1], Q0, blk_bytes, cudaMemcpyDeviceToDevice, c->stream));
    double *qkm2 = R[0], *qkm1 = R[1], *qk = R[2];
    for (int k = 1; k <= ord; ++k) {
      ST(sigma_fp64(c, P, qkm1, N, qk, N));
      k_cheb_step<<<CHEB_BLK, CHEB_THR, 0, c->stream>>>(N, P, qk, qkm1, qkm2, Q0, a, b, k > 1 ? 1 : 0,
                                                         coef ? acc : nullptr, coef ? (*coef)[k] : 0.0, part);
      ADC_COUNT_LAUNCH();
      ADC_CUDA(c, cudaGetLastError());
      if (!coef) ST(reduce_into(k));
      ST(save_h1(k, qk, n1));
      double* t = qkm2;
      qkm2 = qkm1;
      qkm1 = qk;
      qk = t;
    }
    return ADCGPU_OK;
  }
};

// The scaling of matxvec_chebyshev_incore (:1378-1393): a = 2/DeltaE and
// b = 2 (Emin/DeltaE) + 1.
static void cheb_scaling(const double* bounds, double& a, double& b) {
  const double DeltaE = bounds[1] - bounds[0], Emin = bounds[0];
  a = 2.0 / DeltaE;
  b = 2.0 * (Emin / DeltaE) + 1.0;
}

static int cheb_check(Ctx* c, int nvec, const void* q0, const double* bounds, int chebyord) {
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "build the matrix first");
  if (nvec <= 0 || !q0 || !bounds || chebyord < 0)
    return set_err(c, ADCGPU_BAD_INPUT, "nvec >= 1, q0, bounds and chebyord >= 0 required");
  if (!(bounds[1] > bounds[0])) return set_err(c, ADCGPU_BAD_INPUT, "spectral bounds must satisfy Emin < Emax");
  return ADCGPU_OK;
}

// init_vec_singlesubspace (block_lanczos.f90:748-923): the lowest b
// eigenvectors of H restricted to the 800 configurations of largest hii
// (extended while the next hii lies within 1e-6), scattered into an N x b
// block.  The subspace columns of H come from the sigma product of unit
// vectors, 64 at a time, so the stored matrix is never exported.
static int singlesubspace_block(Ctx* c, int b, std::vector<double>& q0) {
  const int64_t N = mat_dim(c);
  std::vector<double> hii(N), neg(N);
  ADC_CUDA(c, cudaMemcpyAsync(hii.data(), c->d_diag, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream));
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  // dsortindxa1('D') is the ascending heapsort with every comparison
  // reversed, i.e. the ascending one on negated keys
  for (int64_t i = 0; i < N; ++i) neg[i] = -hii[i];
  std::vector<int64_t> indx;
  host_heapsort_index(N, neg.data(), indx);
  int64_t sub = std::min<int64_t>(800, N);
  while (sub < N && std::fabs(hii[indx[sub - 1] - 1] - hii[indx[sub] - 1]) < 1e-6) ++sub;
  if (sub > 8192) return set_err(c, ADCGPU_UNSUPPORTED, "degenerate diagonal: subspace above 8192");
  std::vector<int64_t> rows(sub);
  for (int64_t i = 0; i < sub; ++i) rows[i] = indx[i] - 1;
  const int MC = 64;
  double *dV = nullptr, *dW = nullptr, *dS = nullptr;
  int64_t* drows = nullptr;
  const size_t vb = sizeof(double) * (size_t)N * MC, sb = sizeof(double) * (size_t)sub * MC;
  int st = dmalloc(c, (void**)&dV, vb);
  if (!st) st = dmalloc(c, (void**)&dW, vb);
  if (!st) st = dmalloc(c, (void**)&dS, sb);
  if (!st) st = dmalloc(c, (void**)&drows, sizeof(int64_t) * sub);
  std::vector<double> hsub((size_t)sub * sub);
  if (!st && cudaMemcpyAsync(drows, rows.data(), sizeof(int64_t) * sub, cudaMemcpyHostToDevice, c->stream) !=
                 cudaSuccess)
    st = set_err(c, ADCGPU_CUDA_ERROR, "copy of the subspace rows failed");
  for (int64_t j0 = 0; !st && j0 < sub; j0 += MC) {
    const int m = (int)std::min<int64_t>(MC, sub - j0);
    if (cudaMemsetAsync(dV, 0, sizeof(double) * (size_t)N * m, c->stream) != cudaSuccess) {
      st = set_err(c, ADCGPU_CUDA_ERROR, "memset failed");
      break;
    }
    k_unit_cols<<<1, MC, 0, c->stream>>>(N, m, drows + j0, dV); ADC_COUNT_LAUNCH();
    st = sigma_fp64(c, m, dV, N, dW, N);
    if (st) break;
    k_gather_rows<<<c->nsm, 256, 0, c->stream>>>(N, (int)sub, m, drows, dW, dS); ADC_COUNT_LAUNCH();
    if (cudaMemcpyAsync(hsub.data() + (size_t)j0 * sub, dS, sizeof(double) * (size_t)sub * m,
                        cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
      st = set_err(c, ADCGPU_CUDA_ERROR, std::string("subspace Hamiltonian: ") + cudaGetErrorString(cudaGetLastError()));
  }
  dfree(c, dV, vb);
  dfree(c, dW, vb);
  dfree(c, dS, sb);
  dfree(c, drows, sizeof(int64_t) * sub);
  if (st) return st;
  std::vector<double> w(sub), V((size_t)sub * sub);
  if (!host_syev((int)sub, hsub.data(), (int)sub, w.data(), V.data()))
    return set_err(c, ADCGPU_EIGEN_FAILED, "The diagonalisation of the subspace Hamiltonian failed");
  q0.assign((size_t)N * b, 0.0);
  for (int col = 0; col < b && col < sub; ++col)
    for (int64_t i = 0; i < sub; ++i) q0[(size_t)col * N + rows[i]] = V[(size_t)col * sub + i];
  return ADCGPU_OK;
}

}  // namespace adcgpu

extern "C" int adcgpu_chebyshev_auto(adcgpu_ctx* h, int nvec, const double* q0, const double* bounds, int chebyord,
                                     int df, double* auto_out, double* q1h1p, int* order_out) {
  using namespace adcgpu;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  ST(cheb_check(c, nvec, q0, bounds, chebyord));
  if (!auto_out) return set_err(c, ADCGPU_BAD_INPUT, "auto_out required");
  const int ord = chebyord - chebyord % 2;   // chebyshev_initialise (:136)
  const int64_t N = mat_dim(c), n1 = mat_n1(c);
  ChebGPU G;
  G.c = c; G.N = N; G.P = nvec; G.ord = ord;
  ST(G.alloc(false, n1, q1h1p != nullptr));
  ADC_CUDA(c, cudaMemcpyAsync(G.Q0, q0, G.blk_bytes, cudaMemcpyHostToDevice, c->stream));
  k_cheb_norm0<<<CHEB_BLK, CHEB_THR, 0, c->stream>>>(N, nvec, G.Q0, G.part); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  ST(G.reduce_into(0));
  ST(G.save_h1(0, G.Q0, n1));
  double a, b;
  cheb_scaling(bounds, a, b);
  ST(G.expand(a, b, nullptr, n1, df));
  std::vector<double> sums((size_t)3 * nvec * (ord + 1));
  ADC_CUDA(c, cudaMemcpyAsync(sums.data(), G.sums, G.sums_bytes, cudaMemcpyDeviceToHost, c->stream));
  if (q1h1p) ADC_CUDA(c, cudaMemcpyAsync(q1h1p, G.h1, G.h1_bytes, cudaMemcpyDeviceToHost, c->stream));
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  const int nk = 2 * ord + 1;
  auto S = [&](int k, int p, int j) { return sums[((size_t)k * nvec + p) * 3 + j]; };
  for (int p = 0; p < nvec; ++p) {
    double* A = auto_out + (size_t)p * nk;
    for (int k = 0; k < nk; ++k) A[k] = 0.0;
    A[0] = S(0, p, 0);
    for (int k = 1; k <= ord; ++k) {
      A[k] = S(k, p, 0);
      if (k > ord / 2) {
        A[2 * k] = 2.0 * S(k, p, 1) - A[0];
        A[2 * k - 1] = 2.0 * S(k, p, 2) - A[1];
      }
    }
  }
  if (order_out) *order_out = ord;
  return ADCGPU_OK;
}

extern "C" int adcgpu_chebyshev_project(adcgpu_ctx* h, int nvec, double* q0, const double* bounds, int chebyord,
                                        double projen, int df) {
  using namespace adcgpu;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  ST(cheb_check(c, nvec, q0, bounds, chebyord));
  const int ord = chebyord - chebyord % 2;
  const int64_t N = mat_dim(c);
  // project_psi0 (:420-446): escale, the Jackson damping g_k and the
  // step-function coefficients f_k, with the reference's expression order
  const double pi = 3.1415926535897932;   // constants.f90:8
  double escale = projen - (0.5 * (bounds[1] - bounds[0]) + bounds[0]);
  escale = escale / (bounds[1] - bounds[0]);
  escale = 2.0 * escale;
  if (!(std::fabs(escale) <= 1.0)) return set_err(c, ADCGPU_BAD_INPUT, "projen lies outside the spectral bounds");
  std::vector<double> gk(ord + 1), fk(ord + 1), coef(ord + 1);
  const double alpha = pi / (double)(ord + 2), cosa = std::cos(alpha), sina = std::sin(alpha);
  for (int k = 0; k <= ord; ++k)
    gk[k] = (1.0 - (double)k / ((double)(ord + 2))) * sina * std::cos(k * alpha) +
            (1.0 / (double)(ord + 2)) * cosa * std::sin(k * alpha);
  for (int k = 0; k <= ord; ++k) gk[k] = gk[k] / sina;
  fk[0] = 1.0 - std::acos(escale) / pi;
  for (int k = 1; k <= ord; ++k) fk[k] = -2.0 * std::sin(k * std::acos(escale)) / (k * pi);
  for (int k = 0; k <= ord; ++k) coef[k] = fk[k] * gk[k];
  ChebGPU G;
  G.c = c; G.N = N; G.P = nvec; G.ord = ord;
  ST(G.alloc(true, 0, false));
  ADC_CUDA(c, cudaMemcpyAsync(G.Q0, q0, G.blk_bytes, cudaMemcpyHostToDevice, c->stream));
  k_cheb_scale<<<c->nsm * 4, 256, 0, c->stream>>>(N * nvec, coef[0], G.Q0, G.acc); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  double a, b;
  cheb_scaling(bounds, a, b);
  ST(G.expand(a, b, &coef, 0, df));
  ADC_CUDA(c, cudaMemcpyAsync(q0, G.acc, G.blk_bytes, cudaMemcpyDeviceToHost, c->stream));
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  return ADCGPU_OK;
}

extern "C" int adcgpu_spectral_bounds(adcgpu_ctx* h, const adcgpu_dav_params* fp, double* bounds) {
  using namespace adcgpu;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "build the matrix first");
  if (!bounds) return set_err(c, ADCGPU_BAD_INPUT, "bounds required");
  if (mat_dim(c) < 200) return set_err(c, ADCGPU_BAD_INPUT, "the Lanczos estimate needs ndim >= 200 (2 x 100 vectors)");
  // lower bound: one-root block Davidson (specbounds.f90:151-176).  The
  // reference sets davstates_f, dmain_f, maxsubdim_f, davtol_f and
  // lsubdiag_f; maxiter, precon, ldfl and guessdim stay the caller's
  // final-space values (defaults.f90:84-94 when fp is NULL or a field is 0).
  adcgpu_dav_params p;
  std::memset(&p, 0, sizeof p);
  if (fp) {
    p.maxiter = fp->maxiter;
    p.precon = fp->precon;
    p.ldfl = fp->ldfl;
    p.guessdim = fp->guessdim;
  } else {
    p.ldfl = 1;
  }
  if (p.maxiter <= 0) p.maxiter = 100;
  if (p.precon == 0) p.precon = ADCGPU_PRECON_OLSEN;
  if (p.guessdim <= 0) p.guessdim = 800;
  p.davstates = 1;
  p.dmain = 5;
  p.maxsubdim = 20;
  p.davtol = 1e-8;
  p.lsubdiag = 1;
  p.precision = ADCGPU_FP64;
  double lower = 0.0;
  adcgpu_dav_info info;
  ST(adcgpu_davidson(h, &p, &lower, nullptr, &info));
  // upper bound: block Lanczos, block 2, 100 cycles, PRO, from the single
  // subspace diagonalisation (:178-199); the last Lanczos state energy
  std::vector<double> q0;
  ST(singlesubspace_block(c, 2, q0));
  std::vector<double> ev(200);
  ST(adcgpu_block_lanczos(h, 2, 100, 1, q0.data(), nullptr, ev.data(), nullptr));
  bounds[0] = lower;
  bounds[1] = ev[199];
  return ADCGPU_OK;
}
