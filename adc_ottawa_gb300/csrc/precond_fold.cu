// Folded singles-block preconditioner (ADCGPU_PRECON_FOLD).
//
// The Davidson correction t for a residual r = (H - lambda) x solves
// (lambda - H) t = r approximately.  With H = [[Hss, B^T], [B, D]] (dense
// singles block Hss = diag1 + A, coupling B, diagonal doubles block D) block
// elimination of the doubles rows gives
//     t_d = (lambda - D)^-1 (r_d + B t_s)
//     (lambda - Hss - B^T (lambda - D)^-1 B) t_s = r_s + B^T (lambda - D)^-1 r_d.
// The preconditioner keeps the two terms that carry almost all of the gain
// on ADC(2)-s matrices and drops the self-energy B^T (lambda-D)^-1 B and the
// B t_s back-coupling:
//     t_d = r_d / (lambda - D)                              (the DPR rows)
//     t_s = (lambda - Hss)^-1 (r_s + B^T t_d)               (folded residual)
// B^T t_d is the singles part of one sigma product of [0; t_d]; the dense
// singles solve runs FOLD_MINRES_STEPS steps of MINRES (Paige-Saunders),
// batched over the block's columns, on the device.  The reference
// preconditioners (dpr, olsen: block_davidson.f90:1288-1419) use only the
// diagonal; this one is an addition without a reference counterpart, and the
// converged eigenpairs are those of the same matrix whichever is used.
#include <cmath>

#include "dense.h"
#include "internal.h"

namespace adcgpu {

int singles_block_product(Ctx* c, int m, const double* V, int64_t ldv, double* W, int64_t ldw);
int singles_block_product(Ctx* c, int m, const float* V, int64_t ldv, float* W, int64_t ldw);

namespace {

constexpr int FOLD_MINRES_STEPS = 8;
constexpr int MR_THREADS = 256;

// rows >= n1: t_d = r_d / (lambda - h) (0 where the denominator vanishes);
// rows < n1: 0, so that sigma([0; t_d]) has B^T t_d as its singles part.
template <typename T>
__global__ void k_fold_prep(int64_t N, int n1, const T* __restrict__ R, int64_t ldr, const double* __restrict__ lam,
                            const T* __restrict__ hii, T* __restrict__ Tout, int64_t ldt) {
  const int c = blockIdx.y;
  const T l = (T)lam[c];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    T t = T(0);
    if (i >= n1) {
      const T den = l - hii[i];
      t = den != T(0) ? R[(int64_t)c * ldr + i] / den : T(0);
    }
    Tout[(int64_t)c * ldt + i] = t;
  }
}

__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < MR_THREADS / 32; ++k) s += red[k];
  return s;
}

// Per-column MINRES state: sc[8c + {0..5}] = beta, c_old, s_old, c, s, eta.
// One block per column; the right-hand side is r_s + (B^T t_d)_s.
template <typename T, typename M>
__global__ void __launch_bounds__(MR_THREADS) k_mr_init(int n1, const T* __restrict__ R, int64_t ldr,
                                                        const T* __restrict__ Z, int64_t ldz, M* __restrict__ V,
                                                        M* __restrict__ Vold, M* __restrict__ W, M* __restrict__ Wold,
                                                        M* __restrict__ X, double* __restrict__ sc) {
  __shared__ double red[MR_THREADS / 32];
  const int c = blockIdx.x;
  const int64_t o = (int64_t)c * n1;
  double ss = 0.0;
  for (int i = threadIdx.x; i < n1; i += MR_THREADS) {
    const double f = (double)R[(int64_t)c * ldr + i] + (double)Z[(int64_t)c * ldz + i];
    V[o + i] = M(f);
    ss += f * f;
  }
  const double beta1 = sqrt(block_sum(ss, red));
  for (int i = threadIdx.x; i < n1; i += MR_THREADS) {
    V[o + i] = beta1 > 0.0 ? M((double)V[o + i] / beta1) : M(0);
    Vold[o + i] = M(0);
    W[o + i] = M(0);
    Wold[o + i] = M(0);
    X[o + i] = M(0);
  }
  if (threadIdx.x == 0) {
    double* s = sc + 8 * c;
    s[0] = 0.0; s[1] = 1.0; s[2] = 0.0; s[3] = 1.0; s[4] = 0.0; s[5] = beta1;
  }
}

// One MINRES step for (lambda - Hss) x = b; HV = Hss V from the previous
// launch.  Vold holds the new Lanczos vector between passes 2 and 3; each
// element is read and written by the same thread in every pass.
template <typename M>
__global__ void __launch_bounds__(MR_THREADS) k_mr_step(int n1, const double* __restrict__ lam,
                                                        const M* __restrict__ HV, M* __restrict__ V,
                                                        M* __restrict__ Vold, M* __restrict__ W,
                                                        M* __restrict__ Wold, M* __restrict__ X,
                                                        double* __restrict__ sc) {
  __shared__ double red[MR_THREADS / 32];
  const int c = blockIdx.x;
  const int64_t o = (int64_t)c * n1;
  const double l = lam[c];
  double a = 0.0;
  for (int i = threadIdx.x; i < n1; i += MR_THREADS) {
    const double v = (double)V[o + i];
    a += v * (l * v - (double)HV[o + i]);
  }
  const double alpha = block_sum(a, red);
  double* s = sc + 8 * c;
  const double beta = s[0], c_old = s[1], s_old = s[2], cc = s[3], sn0 = s[4], eta = s[5];
  double b2 = 0.0;
  for (int i = threadIdx.x; i < n1; i += MR_THREADS) {
    const double v = (double)V[o + i];
    const double vn = (l * v - (double)HV[o + i]) - alpha * v - beta * (double)Vold[o + i];
    Vold[o + i] = M(vn);
    b2 += vn * vn;
  }
  const double beta_n = sqrt(block_sum(b2, red));
  const double delta = cc * alpha - c_old * sn0 * beta;
  const double rho2 = sn0 * alpha + c_old * cc * beta;
  const double rho3 = s_old * beta;
  double rho1 = sqrt(delta * delta + beta_n * beta_n);
  if (rho1 == 0.0) rho1 = 1.0;
  const double cn = delta / rho1, sn = beta_n / rho1;
  for (int i = threadIdx.x; i < n1; i += MR_THREADS) {
    const double v = (double)V[o + i], vn = (double)Vold[o + i];
    const double w = (double)W[o + i], wo = (double)Wold[o + i];
    const double wn = (v - rho3 * wo - rho2 * w) / rho1;
    X[o + i] = M((double)X[o + i] + cn * eta * wn);
    Wold[o + i] = M(w);
    W[o + i] = M(wn);
    Vold[o + i] = M(v);
    V[o + i] = beta_n > 0.0 ? M(vn / beta_n) : M(0);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    s[0] = beta_n; s[1] = cc; s[2] = sn0; s[3] = cn; s[4] = sn; s[5] = -sn * eta;
  }
}

template <typename T, typename M>
__global__ void k_mr_out(int n1, int nb, const M* __restrict__ X, T* __restrict__ Tout, int64_t ldt) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)n1 * nb;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(t / n1), i = (int)(t - (int64_t)c * n1);
    Tout[(int64_t)c * ldt + i] = T(X[t]);
  }
}

int sigma_any(Ctx* c, int m, const double* V, int64_t ldv, double* W, int64_t ldw) {
  return sigma_fp64(c, m, V, ldv, W, ldw);
}
int sigma_any(Ctx* c, int m, const float* V, int64_t ldv, float* W, int64_t ldw) {
  return sigma_fp32(c, m, V, ldv, W, ldw);
}

}  // namespace

namespace {

template <typename T>
int fold_impl(Ctx* c, Workspace& ws, int64_t N, int nb, const T* R, int64_t ldr, const double* d_lam,
              const T* hii, T* Tout, int64_t ldt, T* Z, int64_t ldz) {
  typedef T M;
  const int n1 = (int)c->geom.n1;
  if (nb <= 0) return ADCGPU_OK;
  const size_t vec = (size_t)n1 * nb;
  ST(ws.reserve(c, sizeof(M) * vec * 6 + sizeof(double) * 8 * nb));
  M* V = reinterpret_cast<M*>(ws.p);
  M* Vold = V + vec;
  M* W = Vold + vec;
  M* Wold = W + vec;
  M* X = Wold + vec;
  M* HV = X + vec;
  double* sc = reinterpret_cast<double*>(HV + vec);
  cudaStream_t s = c->stream;
  k_fold_prep<T><<<dim3(c->nsm * 2, nb), 256, 0, s>>>(N, n1, R, ldr, d_lam, hii, Tout, ldt); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  ST(sigma_any(c, nb, Tout, ldt, Z, ldz));
  k_mr_init<T, M><<<nb, MR_THREADS, 0, s>>>(n1, R, ldr, Z, ldz, V, Vold, W, Wold, X, sc); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  for (int it = 0; it < FOLD_MINRES_STEPS; ++it) {
    ST(singles_block_product(c, nb, V, n1, HV, n1));
    k_mr_step<M><<<nb, MR_THREADS, 0, s>>>(n1, d_lam, HV, V, Vold, W, Wold, X, sc); ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
  }
  k_mr_out<T, M><<<c->nsm * 2, 256, 0, s>>>(n1, nb, X, Tout, ldt); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

}  // namespace

// Tout (N x nb) = folded-singles-block correction of the residual block R.
// Z is scratch of at least 2 nb columns of N values; ws holds the MINRES
// vectors.  On a matrix built for ADCGPU_MIXED the fold always runs with FP32
// vectors and the BF16 matrix values, also inside the FP64 refinement: the
// preconditioner only shapes the search direction, and the FP64 residual
// still decides convergence.
template <>
int precond_fold<float>(Ctx* c, Workspace& ws, int64_t N, int nb, const float* R, int64_t ldr, const double* d_lam,
                        const float* hii, float* Tout, int64_t ldt, float* Z, int64_t ldz) {
  const int save = c->mixed_bf16;
  c->mixed_bf16 = c->d_Bt16 ? 1 : 0;
  const int st = fold_impl<float>(c, ws, N, nb, R, ldr, d_lam, hii, Tout, ldt, Z, ldz);
  c->mixed_bf16 = save;
  return st;
}

template <>
int precond_fold<double>(Ctx* c, Workspace& ws, int64_t N, int nb, const double* R, int64_t ldr,
                         const double* d_lam, const double* hii, double* Tout, int64_t ldt, double* Z, int64_t ldz) {
  // the FP32 route carves three float blocks (R, T, Z) = 1.5 nb doubles per
  // row out of Z
  if (c->precision == ADCGPU_MIXED && c->d_Bt16 && c->d_A32 && c->d_diag32 && ldr == N && ldt == N && ldz == N) {
    float* Rf = reinterpret_cast<float*>(Z);
    float* Tf = Rf + (size_t)N * nb;
    float* Zf = Tf + (size_t)N * nb;
    ST((convert<double, float>(c, R, Rf, N * nb)));
    ST(precond_fold<float>(c, ws, N, nb, Rf, N, d_lam, c->d_diag32, Tf, N, Zf, N));
    return convert<float, double>(c, Tf, Tout, N * nb);
  }
  return fold_impl<double>(c, ws, N, nb, R, ldr, d_lam, hii, Tout, ldt, Z, ldz);
}

}  // namespace adcgpu
