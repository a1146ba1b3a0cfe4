// Tall-skinny dense kernels of the solvers (N rows, <= a few hundred columns):
//
//   gemm_tn : C(p x q) = A(N x p)^T B(N x q)      calcrmat dgemm :961, the
//             Gram matrices of the orthogonalisation, Lanczos A_j = Q^T U
//   gemm_nn : C(N x q) = beta C + alpha A(N x p) B(p x q)    calcritzvec :1018,
//             calcres :1056, projections, Lanczos updates, Ritz vectors
//   precond : dpr (block_davidson.f90:1288-1342) and olsen (:1346-1419)
//   resid   : r_i = lambda_i x_i - (W y)_i and ||r_i|| (calcres :1029-1085)
//
// Reductions over N are two-pass (per-block partials, then a fixed-order
// sum), so results do not depend on scheduling.
#include <algorithm>
#include <type_traits>

#include "internal.h"
#include "dense.h"
#include "df.h"

namespace adcgpu {

namespace {

constexpr int TN_ROWS = 32;     // rows staged per step
constexpr int TN_P = 64, TN_Q = 32;   // output tile

// Accumulator helpers: plain types add; df accumulates with two-sums.
template <typename A> __device__ __forceinline__ A acc_zero() { return A(0); }
template <> __device__ __forceinline__ df acc_zero<df>() { return df{0.f, 0.f}; }
template <typename A, typename X> __device__ __forceinline__ void acc_add(A& a, X x) { a += (A)x; }
__device__ __forceinline__ void acc_add(df& a, float x) { a = df_add(a, df{x, 0.f}); }
template <typename R, typename A> __device__ __forceinline__ R acc_value(A a) { return (R)a; }
template <> __device__ __forceinline__ double acc_value<double, df>(df a) { return df_value(a); }

// double -> float without the FP64 pipe (truncating: relative error < 2^-23)
template <typename T, typename TB> __device__ __forceinline__ T to_t(TB x) { return (T)x; }
template <> __device__ __forceinline__ float to_t<float, double>(double x) { return df_split(x).hi; }

__device__ __forceinline__ void sq_add(double& a, double v) { a += v * v; }
__device__ __forceinline__ void sq_add(df& a, float v) { df_fma(a, df{v, 0.f}, df{v, 0.f}); }

// Partial C tiles: part[(blk * ntile + tile) * TN_P * TN_Q + ...]
// Block: a range of rows; output tile TN_P x TN_Q (64 x 32); thread -> 8
// outputs (p = ti + 16 u, q = tj + 16 v), conflict-free shared-memory reads.
// Products over one 32-row step are summed in T and added to TA accumulators
// (FP64 for FP32 inputs: one FP64 add per 32 FP32 FMAs keeps the Rayleigh and
// Gram matrices accurate to ~1e-7 over millions of rows).
template <typename T, typename TA>
__global__ void __launch_bounds__(256) k_gemm_tn_part(int64_t N, int p, int q, const T* __restrict__ A,
                                                      int64_t lda, const T* __restrict__ B, int64_t ldb,
                                                      TA* __restrict__ part, int64_t rows_per_blk) {
  __shared__ T sA[TN_ROWS][TN_P + 1];
  __shared__ T sB[TN_ROWS][TN_Q + 1];
  const int ntq = (q + TN_Q - 1) / TN_Q;
  const int tile = blockIdx.y;
  const int tp = tile / ntq, tq = tile % ntq;
  const int p0 = tp * TN_P, q0 = tq * TN_Q;
  const int tid = threadIdx.x;
  const int ti = tid & 15, tj = tid >> 4;
  // FP32 inputs: the step sums go into double-float accumulators (FP32-pipe
  // two-sums) instead of FP64 adds; FP64 inputs accumulate in FP64
  typedef typename std::conditional<std::is_same<T, float>::value && std::is_same<TA, double>::value, df, TA>::type
      TAcc;
  TAcc acc[4][2];
#pragma unroll
  for (int u = 0; u < 4; ++u) { acc[u][0] = acc_zero<TAcc>(); acc[u][1] = acc_zero<TAcc>(); }
  const int64_t r_begin = blockIdx.x * rows_per_blk;
  const int64_t r_end = min(N, r_begin + rows_per_blk);
  for (int64_t r0 = r_begin; r0 < r_end; r0 += TN_ROWS) {
    __syncthreads();
    for (int l = tid; l < TN_ROWS * TN_P; l += 256) {
      int c = l / TN_ROWS, rr = l % TN_ROWS;
      int64_t r = r0 + rr;
      sA[rr][c] = (r < r_end && p0 + c < p) ? A[(int64_t)(p0 + c) * lda + r] : T(0);
    }
    for (int l = tid; l < TN_ROWS * TN_Q; l += 256) {
      int c = l / TN_ROWS, rr = l % TN_ROWS;
      int64_t r = r0 + rr;
      sB[rr][c] = (r < r_end && q0 + c < q) ? B[(int64_t)(q0 + c) * ldb + r] : T(0);
    }
    __syncthreads();
    T st[4][2];
#pragma unroll
    for (int u = 0; u < 4; ++u) { st[u][0] = T(0); st[u][1] = T(0); }
#pragma unroll 8
    for (int rr = 0; rr < TN_ROWS; ++rr) {
      T b0 = sB[rr][tj], b1 = sB[rr][tj + 16];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        T a = sA[rr][ti + 16 * u];
        st[u][0] += a * b0;
        st[u][1] += a * b1;
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) { acc_add(acc[u][0], st[u][0]); acc_add(acc[u][1], st[u][1]); }
  }
  TA* out = part + ((int64_t)blockIdx.x * gridDim.y + tile) * (TN_P * TN_Q);
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    out[(ti + 16 * u) * TN_Q + tj] = acc_value<TA>(acc[u][0]);
    out[(ti + 16 * u) * TN_Q + tj + 16] = acc_value<TA>(acc[u][1]);
  }
}

// Threads walk the partial tiles in their stored order (jj fastest), so the
// nblk reads of consecutive threads are contiguous.
template <typename TA, typename TC>
__global__ void k_gemm_tn_reduce(int p, int q, int nblk, int ntile, const TA* __restrict__ part,
                                 TC* __restrict__ C, int ldc, TC alpha, TC beta) {
  const int ntq = (q + TN_Q - 1) / TN_Q;
  const int per_tile = TN_P * TN_Q;
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < ntile * per_tile; o += gridDim.x * blockDim.x) {
    const int tile = o / per_tile, w = o - tile * per_tile;
    const int ii = w / TN_Q, jj = w - ii * TN_Q;
    const int i = (tile / ntq) * TN_P + ii, j = (tile % ntq) * TN_Q + jj;
    if (i >= p || j >= q) continue;
    TA s = TA(0);
    for (int b = 0; b < nblk; ++b) s += part[((int64_t)b * ntile + tile) * per_tile + w];
    TC prev = beta == TC(0) ? TC(0) : beta * C[(int64_t)j * ldc + i];
    C[(int64_t)j * ldc + i] = prev + alpha * (TC)s;
  }
}


// k_gemm_tn_part for FP64 inputs: DF step sums added to DF accumulators.
__global__ void __launch_bounds__(256) k_gemm_tn_part_df(int64_t N, int p, int q, const double* __restrict__ A,
                                                         int64_t lda, const double* __restrict__ B, int64_t ldb,
                                                         double* __restrict__ part, int64_t rows_per_blk) {
  __shared__ df sA[TN_ROWS][TN_P + 1];
  __shared__ df sB[TN_ROWS][TN_Q + 1];
  const int ntq = (q + TN_Q - 1) / TN_Q;
  const int tile = blockIdx.y;
  const int tp = tile / ntq, tq = tile % ntq;
  const int p0 = tp * TN_P, q0 = tq * TN_Q;
  const int tid = threadIdx.x;
  const int ti = tid & 15, tj = tid >> 4;
  df acc[4][2];
#pragma unroll
  for (int u = 0; u < 4; ++u) { acc[u][0] = df{0.f, 0.f}; acc[u][1] = df{0.f, 0.f}; }
  const int64_t r_begin = blockIdx.x * rows_per_blk;
  const int64_t r_end = min(N, r_begin + rows_per_blk);
  for (int64_t r0 = r_begin; r0 < r_end; r0 += TN_ROWS) {
    __syncthreads();
    for (int l = tid; l < TN_ROWS * TN_P; l += 256) {
      int c = l / TN_ROWS, rr = l % TN_ROWS;
      int64_t r = r0 + rr;
      sA[rr][c] = df_split((r < r_end && p0 + c < p) ? A[(int64_t)(p0 + c) * lda + r] : 0.0);
    }
    for (int l = tid; l < TN_ROWS * TN_Q; l += 256) {
      int c = l / TN_ROWS, rr = l % TN_ROWS;
      int64_t r = r0 + rr;
      sB[rr][c] = df_split((r < r_end && q0 + c < q) ? B[(int64_t)(q0 + c) * ldb + r] : 0.0);
    }
    __syncthreads();
    df st[4][2];
#pragma unroll
    for (int u = 0; u < 4; ++u) { st[u][0] = df{0.f, 0.f}; st[u][1] = df{0.f, 0.f}; }
#pragma unroll 4
    for (int rr = 0; rr < TN_ROWS; ++rr) {
      const df b0 = sB[rr][tj], b1 = sB[rr][tj + 16];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const df a = sA[rr][ti + 16 * u];
        df_fma(st[u][0], a, b0);
        df_fma(st[u][1], a, b1);
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) { acc[u][0] = df_add(acc[u][0], st[u][0]); acc[u][1] = df_add(acc[u][1], st[u][1]); }
  }
  double* out = part + ((int64_t)blockIdx.x * gridDim.y + tile) * (TN_P * TN_Q);
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    out[(ti + 16 * u) * TN_Q + tj] = df_value(acc[u][0]);
    out[(ti + 16 * u) * TN_Q + tj + 16] = df_value(acc[u][1]);
  }
}

// C(N x q) = beta C + alpha A(N x p) B(p x q).  Block tile 128 rows x 64
// columns, K staged 16 at a time; thread micro tile 8 rows x 4 columns.
constexpr int NN_M = 128, NN_N = 64, NN_K = 16;
template <typename T, typename TB>
__global__ void __launch_bounds__(256) k_gemm_nn(int64_t N, int p, int q, T alpha, const T* __restrict__ A,
                                                 int64_t lda, const TB* __restrict__ B, int ldb, T beta,
                                                 T* __restrict__ C, int64_t ldc) {
  __shared__ __align__(16) T sA[NN_K][NN_M];
  __shared__ __align__(16) T sB[NN_K][NN_N];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;          // columns 4 tx.., rows 8 ty..
  const int64_t m0 = (int64_t)blockIdx.x * NN_M;
  const int n0 = blockIdx.y * NN_N;
  T acc[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
  for (int k0 = 0; k0 < p; k0 += NN_K) {
    __syncthreads();
    for (int l = tid; l < NN_K * NN_M; l += 256) {
      const int kk = l / NN_M, rr = l % NN_M;
      const int64_t r = m0 + rr;
      sA[kk][rr] = (r < N && k0 + kk < p) ? A[(int64_t)(k0 + kk) * lda + r] : T(0);
    }
    for (int l = tid; l < NN_K * NN_N; l += 256) {
      const int kk = l / NN_N, cc = l % NN_N;
      sB[kk][cc] = (k0 + kk < p && n0 + cc < q) ? to_t<T, TB>(B[(int64_t)(n0 + cc) * ldb + k0 + kk]) : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < NN_K; ++kk) {
      T a[8], b[4];
#pragma unroll
      for (int i = 0; i < 8; ++i) a[i] = sA[kk][8 * ty + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sB[kk][4 * tx + j];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int col = n0 + 4 * tx + j;
    if (col >= q) continue;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int64_t r = m0 + 8 * ty + i;
      if (r < N) {
        T prev = beta == T(0) ? T(0) : beta * C[(int64_t)col * ldc + r];
        C[(int64_t)col * ldc + r] = prev + alpha * acc[i][j];
      }
    }
  }
}

// k_gemm_nn for FP64 operands with DF products and DF sums over all of K.
__global__ void __launch_bounds__(256) k_gemm_nn_df(int64_t N, int p, int q, double alpha,
                                                    const double* __restrict__ A, int64_t lda,
                                                    const double* __restrict__ B, int ldb, double beta,
                                                    double* __restrict__ C, int64_t ldc) {
  __shared__ df sA[NN_K][NN_M];
  __shared__ df sB[NN_K][NN_N];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int64_t m0 = (int64_t)blockIdx.x * NN_M;
  const int n0 = blockIdx.y * NN_N;
  df acc[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = df{0.f, 0.f};
  for (int k0 = 0; k0 < p; k0 += NN_K) {
    __syncthreads();
    for (int l = tid; l < NN_K * NN_M; l += 256) {
      const int kk = l / NN_M, rr = l % NN_M;
      const int64_t r = m0 + rr;
      sA[kk][rr] = df_split((r < N && k0 + kk < p) ? A[(int64_t)(k0 + kk) * lda + r] : 0.0);
    }
    for (int l = tid; l < NN_K * NN_N; l += 256) {
      const int kk = l / NN_N, cc = l % NN_N;
      sB[kk][cc] = df_split((k0 + kk < p && n0 + cc < q) ? B[(int64_t)(n0 + cc) * ldb + k0 + kk] : 0.0);
    }
    __syncthreads();
#pragma unroll 2
    for (int kk = 0; kk < NN_K; ++kk) {
      df a[8], b[4];
#pragma unroll
      for (int i = 0; i < 8; ++i) a[i] = sA[kk][8 * ty + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sB[kk][4 * tx + j];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) df_fma(acc[i][j], a[i], b[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int col = n0 + 4 * tx + j;
    if (col >= q) continue;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int64_t r = m0 + 8 * ty + i;
      if (r < N) {
        double prev = beta == 0.0 ? 0.0 : beta * C[(int64_t)col * ldc + r];
        C[(int64_t)col * ldc + r] = prev + alpha * df_value(acc[i][j]);
      }
    }
  }
}

// FP32 tall-skinny C(N x q) = beta C + alpha A(N x p) B(p x q) (B FP64 or
// FP32, held as FP32 in shared memory for all row blocks of a persistent
// block).  A thread owns one row and the QT columns of a column tile: per k
// it loads one value of A (coalesced across the warp) and reads B's row k as
// QT/4 float4 broadcasts for QT FMAs.  The k loop runs in groups of NN_KG
// with the next group's A values loaded before the current group's FMAs, so
// each thread keeps NN_KG loads in flight (the kernel is otherwise bound by
// the latency of the column-strided loads of A).
constexpr int NN_KG = 16;
template <int QT>
__device__ __forceinline__ void nn_f32_step(float (&acc)[QT], float a, const float* __restrict__ brow) {
  const float4* b4 = reinterpret_cast<const float4*>(brow);
#pragma unroll
  for (int j4 = 0; j4 < QT / 4; ++j4) {
    const float4 b = b4[j4];
    acc[4 * j4 + 0] = fmaf(a, b.x, acc[4 * j4 + 0]);
    acc[4 * j4 + 1] = fmaf(a, b.y, acc[4 * j4 + 1]);
    acc[4 * j4 + 2] = fmaf(a, b.z, acc[4 * j4 + 2]);
    acc[4 * j4 + 3] = fmaf(a, b.w, acc[4 * j4 + 3]);
  }
}

template <typename TB, int QT>
__global__ void __launch_bounds__(256, 2) k_gemm_nn_f32(int64_t N, int p, int q, float alpha,
                                                        const float* __restrict__ A, int64_t lda,
                                                        const TB* __restrict__ B, int ldb, float beta,
                                                        float* __restrict__ C, int64_t ldc) {
  extern __shared__ __align__(16) float sBf[];   // [p][QT]
  const int q0 = blockIdx.y * QT;
  for (int l = threadIdx.x; l < p * QT; l += blockDim.x) {
    const int k = l / QT, j = l % QT;
    sBf[l] = q0 + j < q ? to_t<float, TB>(B[(int64_t)(q0 + j) * ldb + k]) : 0.f;
  }
  __syncthreads();
  const int qn = min(QT, q - q0);
  const int pg = p - p % NN_KG;
  for (int64_t r0 = blockIdx.x * 256ll; r0 < N; r0 += (int64_t)gridDim.x * 256) {
    const int64_t row = r0 + threadIdx.x;
    const bool ok = row < N;
    float acc[QT];
#pragma unroll
    for (int j = 0; j < QT; ++j) acc[j] = 0.f;
    float cur[NN_KG], nxt[NN_KG];
    if (pg > 0) {
#pragma unroll
      for (int u = 0; u < NN_KG; ++u) cur[u] = ok ? A[(int64_t)u * lda + row] : 0.f;
    }
    for (int k = 0; k < pg; k += NN_KG) {
      const bool more = ok && k + NN_KG < pg;
#pragma unroll
      for (int u = 0; u < NN_KG; ++u) nxt[u] = more ? A[(int64_t)(k + NN_KG + u) * lda + row] : 0.f;
#pragma unroll
      for (int u = 0; u < NN_KG; ++u) nn_f32_step<QT>(acc, cur[u], sBf + (k + u) * QT);
#pragma unroll
      for (int u = 0; u < NN_KG; ++u) cur[u] = nxt[u];
    }
    for (int k = pg; k < p; ++k) nn_f32_step<QT>(acc, ok ? A[(int64_t)k * lda + row] : 0.f, sBf + k * QT);
    if (ok) {
#pragma unroll
      for (int j = 0; j < QT; ++j) {
        if (j >= qn) break;
        float* cp = C + (int64_t)(q0 + j) * ldc + row;
        const float prev = beta == 0.f ? 0.f : beta * *cp;
        *cp = prev + alpha * acc[j];
      }
    }
  }
}

// FP32 tall-skinny partial Gram tiles C(p x q) = A(N x p)^T B(N x q): a block
// sums a range of rows for one 64 x 64 output tile; a thread owns a 4 x 4
// sub-tile read as float4 from row-major staged rows (32 rows per step).
// The products of one step are summed in FP32 and added to double-float
// accumulators, as in k_gemm_tn_part.  part: [blk][tile][64 x 64] doubles.
constexpr int TF_T = 64, TF_ROWS = 32, TF_LD = TF_T + 4;
__global__ void __launch_bounds__(256) k_gemm_tn_f32(int64_t N, int p, int q, const float* __restrict__ A,
                                                     int64_t lda, const float* __restrict__ B, int64_t ldb,
                                                     double* __restrict__ part, int64_t rows_per_blk) {
  __shared__ __align__(16) float sA[TF_ROWS][TF_LD];
  __shared__ __align__(16) float sB[TF_ROWS][TF_LD];
  const int ntq = (q + TF_T - 1) / TF_T;
  const int tile = blockIdx.y;
  const int p0 = (tile / ntq) * TF_T, q0 = (tile % ntq) * TF_T;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ti = tid & 15, tj = tid >> 4;        // outputs 4 ti.. (p) and 4 tj.. (q)
  df acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = df{0.f, 0.f};
  const int64_t r_begin = blockIdx.x * rows_per_blk;
  const int64_t r_end = min(N, r_begin + rows_per_blk);
  // a warp stages 32 consecutive rows of 8 columns (coalesced); the next
  // step's values are loaded into registers while the current step computes
  float pa[8], pb[8];
  auto fetch = [&](int64_t r0) {
    const int64_t r = r0 + lane;
    const bool rok = r < r_end;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int cidx = warp + 8 * u;
      pa[u] = (rok && p0 + cidx < p) ? A[(int64_t)(p0 + cidx) * lda + r] : 0.f;
      pb[u] = (rok && q0 + cidx < q) ? B[(int64_t)(q0 + cidx) * ldb + r] : 0.f;
    }
  };
  if (r_begin < r_end) fetch(r_begin);
  for (int64_t r0 = r_begin; r0 < r_end; r0 += TF_ROWS) {
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      sA[lane][warp + 8 * u] = pa[u];
      sB[lane][warp + 8 * u] = pb[u];
    }
    __syncthreads();
    if (r0 + TF_ROWS < r_end) fetch(r0 + TF_ROWS);
    float st[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) st[u][v] = 0.f;
#pragma unroll 8
    for (int rr = 0; rr < TF_ROWS; ++rr) {
      const float4 a = *reinterpret_cast<const float4*>(&sA[rr][4 * ti]);
      const float4 b = *reinterpret_cast<const float4*>(&sB[rr][4 * tj]);
      const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) st[u][v] = fmaf(av[u], bv[v], st[u][v]);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] = df_add(acc[u][v], df{st[u][v], 0.f});
  }
  double* out = part + ((int64_t)blockIdx.x * gridDim.y + tile) * (TF_T * TF_T);
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) out[(4 * ti + u) * TF_T + 4 * tj + v] = df_value(acc[u][v]);
}

// C(p x q) (col-major, ldc) = alpha * sum over blocks of the k_gemm_tn_f32
// partials + beta C, in a fixed block order
template <typename TC>
__global__ void k_gemm_tn_f32_reduce(int p, int q, int nblk, int ntile, const double* __restrict__ part,
                                     TC* __restrict__ C, int ldc, TC alpha, TC beta) {
  const int ntq = (q + TF_T - 1) / TF_T;
  const int per_tile = TF_T * TF_T;
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < ntile * per_tile; o += gridDim.x * blockDim.x) {
    const int tile = o / per_tile, w = o - tile * per_tile;
    const int ii = w / TF_T, jj = w - ii * TF_T;
    const int i = (tile / ntq) * TF_T + ii, j = (tile % ntq) * TF_T + jj;
    if (i >= p || j >= q) continue;
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += part[((int64_t)b * ntile + tile) * per_tile + w];
    TC prev = beta == TC(0) ? TC(0) : beta * C[(int64_t)j * ldc + i];
    C[(int64_t)j * ldc + i] = prev + alpha * (TC)s;
  }
}

// dpr: t_i(j) = r_i(j) / (lambda_i - hii(j)); exact zero denominators give 0.
template <typename T, typename TD>
__global__ void k_dpr(int64_t N, int nb, const T* __restrict__ R, int64_t ldr, const double* __restrict__ lam,
                      const TD* __restrict__ hii, T* __restrict__ Tout, int64_t ldt) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
    T h = (T)hii[r];
    for (int i = 0; i < nb; ++i) {
      T den = (T)lam[i] - h;
      Tout[(int64_t)i * ldt + r] = den == T(0) ? T(0) : R[(int64_t)i * ldr + r] * (T(1) / den);
    }
  }
}

// olsen, pass 1: per-block partial sums of x.(r*cd) and x.(x*cd)
template <typename T, typename TD>
__global__ void k_olsen_dots(int64_t N, int nb, const T* __restrict__ X, const T* __restrict__ R, int64_t ld,
                             const double* __restrict__ lam, const TD* __restrict__ hii, double* __restrict__ part) {
  __shared__ double red[2][8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = 0; i < nb; ++i) {
    double xz = 0.0, xy = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
      double den = (double)hii[r] - lam[i];
      double cd = den == 0.0 ? 0.0 : 1.0 / den;
      double x = X[(int64_t)i * ld + r], rr = R[(int64_t)i * ld + r];
      xz += x * (rr * cd);
      xy += x * (x * cd);
    }
    for (int o = 16; o; o >>= 1) { xz += __shfl_xor_sync(0xffffffffu, xz, o); xy += __shfl_xor_sync(0xffffffffu, xy, o); }
    if (lane == 0) { red[0][w][0] = xz; red[1][w][0] = xy; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0.0, b = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { a += red[0][q][0]; b += red[1][q][0]; }
      part[((int64_t)blockIdx.x * nb + i) * 2 + 0] = a;
      part[((int64_t)blockIdx.x * nb + i) * 2 + 1] = b;
    }
    __syncthreads();
  }
}

template <typename T, typename TD>
__global__ void k_olsen_apply(int64_t N, int nb, const T* __restrict__ X, const T* __restrict__ R, int64_t ld,
                              const double* __restrict__ lam, const double* __restrict__ alpha,
                              const TD* __restrict__ hii, T* __restrict__ Tout, int64_t ldt) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
    for (int i = 0; i < nb; ++i) {
      T den = (T)hii[r] - (T)lam[i];
      T cd = den == T(0) ? T(0) : T(1) / den;
      Tout[(int64_t)i * ldt + r] = (T)alpha[i] * cd * X[(int64_t)i * ld + r] - cd * R[(int64_t)i * ld + r];
    }
  }
}

// res_i = -(WY)_i + lambda_i X_i, and per-block partial ||res_i||^2 (FP64).
template <typename T>
__global__ void k_resid(int64_t N, int nb, const T* __restrict__ X, const T* __restrict__ WY, int64_t ld,
                        const double* __restrict__ lam, T* __restrict__ Rout, double* __restrict__ part) {
  __shared__ double red[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = 0; i < nb; ++i) {
    // FP32 vectors: squares summed in double-float on the FP32 pipe
    typedef typename std::conditional<std::is_same<T, float>::value, df, double>::type TS;
    TS s2a = acc_zero<TS>();
    const T li = (T)lam[i];
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
      T v = -WY[(int64_t)i * ld + r] + li * X[(int64_t)i * ld + r];
      Rout[(int64_t)i * ld + r] = v;
      sq_add(s2a, v);
    }
    double s2 = acc_value<double>(s2a);
    for (int o = 16; o; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    if (lane == 0) red[w] = s2;
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) a += red[q];
      part[(int64_t)blockIdx.x * nb + i] = a;
    }
    __syncthreads();
  }
}

__global__ void k_sum_parts(int nblk, int n, int stride, const double* __restrict__ part, double* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += part[(int64_t)b * stride + i];
  out[i] = s;
}

template <typename TS, typename TD>
__global__ void k_convert(const TS* __restrict__ x, TD* __restrict__ y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (TD)x[i];
}

}  // namespace

// ---------------------------------------------------------------------------
// Host wrappers
// ---------------------------------------------------------------------------
Workspace::~Workspace() { release(); }
void Workspace::release() {
  if (p && ctx) dfree(ctx, p, bytes);
  p = nullptr; bytes = 0;
}
int Workspace::reserve(Ctx* c, size_t need) {
  ctx = c;
  if (bytes >= need) return ADCGPU_OK;
  release();
  ctx = c;
  int st = dmalloc(c, &p, need);
  if (st) return st;
  bytes = need;
  return ADCGPU_OK;
}

// Row blocks of the TN reduction: at least 4 blocks per SM on large N.
static int tn_blocks(const Ctx* c, int64_t N) {
  int64_t b = (N + 1023) / 1024;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, c->nsm * 4));
}

template <typename T, typename TA, typename TC>
int gemm_tn(Ctx* c, Workspace& ws, int64_t N, int p, int q, const T* A, int64_t lda, const T* B, int64_t ldb,
            TC* C, int ldc, TC alpha, TC beta) {
  if (p <= 0 || q <= 0) return ADCGPU_OK;
  const int ntile = ((p + TN_P - 1) / TN_P) * ((q + TN_Q - 1) / TN_Q);
  const int nblk = tn_blocks(c, N);
  const int64_t rows = ((N + nblk - 1) / nblk + TN_ROWS - 1) / TN_ROWS * TN_ROWS;
  size_t need = sizeof(TA) * (size_t)nblk * ntile * TN_P * TN_Q;
  int st = ws.reserve(c, need);
  if (st) return st;
  if constexpr (std::is_same<T, double>::value && std::is_same<TA, double>::value) {
    if (c->dense_df) {
      k_gemm_tn_part_df<<<dim3(nblk, ntile), 256, 0, c->stream>>>(N, p, q, A, lda, B, ldb, (TA*)ws.p, rows); ADC_COUNT_LAUNCH();
    } else {
      k_gemm_tn_part<T, TA><<<dim3(nblk, ntile), 256, 0, c->stream>>>(N, p, q, A, lda, B, ldb, (TA*)ws.p, rows); ADC_COUNT_LAUNCH();
    }
  } else if constexpr (std::is_same<T, float>::value && std::is_same<TA, double>::value) {
    if constexpr (std::is_same<TC, double>::value) {
      // the tensor cores (three BF16 slices per value), q <= 48
      if (gram_umma_usable(c, N, p, q)) return gram_umma(c, ws, N, p, q, A, lda, B, ldb, C, ldc, alpha, beta);
    }
    // FP32 inputs: 64 x 64 tiles with 4 x 4 float4 sub-tiles per thread
    const int ntile2 = ((p + TF_T - 1) / TF_T) * ((q + TF_T - 1) / TF_T);
    const size_t need2 = sizeof(double) * (size_t)nblk * ntile2 * TF_T * TF_T;
    st = ws.reserve(c, need2);
    if (st) return st;
    k_gemm_tn_f32<<<dim3(nblk, ntile2), 256, 0, c->stream>>>(N, p, q, A, lda, B, ldb, (double*)ws.p, rows);
    ADC_COUNT_LAUNCH();
    const int nout2 = ntile2 * TF_T * TF_T;
    k_gemm_tn_f32_reduce<TC><<<std::min((nout2 + 255) / 256, c->nsm * 8), 256, 0, c->stream>>>(
        p, q, nblk, ntile2, (const double*)ws.p, C, ldc, alpha, beta);
    ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    return ADCGPU_OK;
  } else {
    k_gemm_tn_part<T, TA><<<dim3(nblk, ntile), 256, 0, c->stream>>>(N, p, q, A, lda, B, ldb, (TA*)ws.p, rows); ADC_COUNT_LAUNCH();
  }
  const int nout = ntile * TN_P * TN_Q;
  k_gemm_tn_reduce<TA, TC><<<std::min((nout + 255) / 256, c->nsm * 8), 256, 0, c->stream>>>(p, q, nblk, ntile,
                                                                                         (TA*)ws.p, C, ldc, alpha,
                                                                                         beta); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

template <typename T, typename TB>
int gemm_nn(Ctx* c, int64_t N, int p, int q, T alpha, const T* A, int64_t lda, const TB* B, int ldb, T beta, T* C,
            int64_t ldc) {
  if (q <= 0) return ADCGPU_OK;
  if (p <= 0) {
    // C = beta C
    if (beta == T(0)) {
      for (int j = 0; j < q; ++j) ADC_CUDA(c, cudaMemsetAsync(C + (int64_t)j * ldc, 0, sizeof(T) * N, c->stream));
    }
    return ADCGPU_OK;
  }
  dim3 grid((unsigned)((N + NN_M - 1) / NN_M), (unsigned)((q + NN_N - 1) / NN_N));
  if constexpr (std::is_same<T, double>::value && std::is_same<TB, double>::value) {
    if (c->dense_df) {
      k_gemm_nn_df<<<grid, 256, 0, c->stream>>>(N, p, q, alpha, A, lda, B, ldb, beta, C, ldc); ADC_COUNT_LAUNCH();
      ADC_CUDA(c, cudaGetLastError());
      return ADCGPU_OK;
    }
  }
  if constexpr (std::is_same<T, float>::value) {
    // FP32: B's column tile in shared memory, 2 rows x QT columns per thread
    const int QT = q <= 16 ? 16 : (q <= 32 ? 32 : (q <= 40 ? 40 : 48));
    const size_t smem = sizeof(float) * (size_t)p * QT;
    if (smem <= 200 * 1024) {
      const int nq = (q + QT - 1) / QT;
      const int64_t nrb = (N + 255) / 256;
      const int gx = (int)std::max<int64_t>(1, std::min<int64_t>(nrb, (int64_t)c->nsm * 2 / std::max(1, nq)));
      dim3 g2(gx, nq);
      switch (QT) {
        case 16:
          if (smem > 48 * 1024)
            ADC_CUDA(c, cudaFuncSetAttribute(k_gemm_nn_f32<TB, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
          k_gemm_nn_f32<TB, 16><<<g2, 256, smem, c->stream>>>(N, p, q, alpha, A, lda, B, ldb, beta, C, ldc);
          break;
        case 32:
          if (smem > 48 * 1024)
            ADC_CUDA(c, cudaFuncSetAttribute(k_gemm_nn_f32<TB, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
          k_gemm_nn_f32<TB, 32><<<g2, 256, smem, c->stream>>>(N, p, q, alpha, A, lda, B, ldb, beta, C, ldc);
          break;
        case 40:
          if (smem > 48 * 1024)
            ADC_CUDA(c, cudaFuncSetAttribute(k_gemm_nn_f32<TB, 40>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
          k_gemm_nn_f32<TB, 40><<<g2, 256, smem, c->stream>>>(N, p, q, alpha, A, lda, B, ldb, beta, C, ldc);
          break;
        default:
          if (smem > 48 * 1024)
            ADC_CUDA(c, cudaFuncSetAttribute(k_gemm_nn_f32<TB, 48>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
          k_gemm_nn_f32<TB, 48><<<g2, 256, smem, c->stream>>>(N, p, q, alpha, A, lda, B, ldb, beta, C, ldc);
          break;
      }
      ADC_COUNT_LAUNCH();
      ADC_CUDA(c, cudaGetLastError());
      return ADCGPU_OK;
    }
  }
  k_gemm_nn<T, TB><<<grid, 256, 0, c->stream>>>(N, p, q, alpha, A, lda, B, ldb, beta, C, ldc); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

template <typename T, typename TD>
int precond_dpr(Ctx* c, int64_t N, int nb, const T* R, int64_t ldr, const double* d_lam, const TD* hii, T* Tout,
                int64_t ldt) {
  k_dpr<T, TD><<<c->nsm * 8, 256, 0, c->stream>>>(N, nb, R, ldr, d_lam, hii, Tout, ldt); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

template <typename T, typename TD>
int precond_olsen(Ctx* c, Workspace& ws, int64_t N, int nb, const T* X, const T* R, int64_t ld, const double* d_lam,
                  const TD* hii, T* Tout, int64_t ldt, double* h_alpha_out) {
  const int nblk = c->nsm * 2;
  int st = ws.reserve(c, sizeof(double) * (size_t)nblk * nb * 2 + sizeof(double) * 4 * nb);
  if (st) return st;
  double* part = (double*)ws.p;
  double* sums = part + (size_t)nblk * nb * 2;
  k_olsen_dots<T, TD><<<nblk, 256, 0, c->stream>>>(N, nb, X, R, ld, d_lam, hii, part); ADC_COUNT_LAUNCH();
  k_sum_parts<<<(2 * nb + 127) / 128, 128, 0, c->stream>>>(nblk, 2 * nb, 2 * nb, part, sums); ADC_COUNT_LAUNCH();
  std::vector<double> h(2 * nb), alpha(nb);
  ADC_CUDA(c, cudaMemcpyAsync(h.data(), sums, sizeof(double) * 2 * nb, cudaMemcpyDeviceToHost, c->stream));
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  for (int i = 0; i < nb; ++i) alpha[i] = h[2 * i + 1] == 0.0 ? 0.0 : h[2 * i] / h[2 * i + 1];
  double* d_alpha = sums + 2 * nb;
  ADC_CUDA(c, cudaMemcpyAsync(d_alpha, alpha.data(), sizeof(double) * nb, cudaMemcpyHostToDevice, c->stream));
  k_olsen_apply<T, TD><<<c->nsm * 8, 256, 0, c->stream>>>(N, nb, X, R, ld, d_lam, d_alpha, hii, Tout, ldt); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  if (h_alpha_out) std::copy(alpha.begin(), alpha.end(), h_alpha_out);
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  return ADCGPU_OK;
}

template <typename T>
int residuals(Ctx* c, Workspace& ws, int64_t N, int nb, const T* X, const T* WY, int64_t ld, const double* d_lam,
              T* Rout, double* h_norm2) {
  const int nblk = c->nsm * 2;
  int st = ws.reserve(c, sizeof(double) * ((size_t)nblk * nb + nb));
  if (st) return st;
  double* part = (double*)ws.p;
  double* sums = part + (size_t)nblk * nb;
  k_resid<T><<<nblk, 256, 0, c->stream>>>(N, nb, X, WY, ld, d_lam, Rout, part); ADC_COUNT_LAUNCH();
  k_sum_parts<<<(nb + 127) / 128, 128, 0, c->stream>>>(nblk, nb, nb, part, sums); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  ADC_CUDA(c, cudaMemcpyAsync(h_norm2, sums, sizeof(double) * nb, cudaMemcpyDeviceToHost, c->stream));
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  return ADCGPU_OK;
}

template <typename TS, typename TD>
int convert(Ctx* c, const TS* x, TD* y, int64_t n) {
  k_convert<TS, TD><<<c->nsm * 8, 256, 0, c->stream>>>(x, y, n); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

// explicit instantiations
template int gemm_tn<double, double, double>(Ctx*, Workspace&, int64_t, int, int, const double*, int64_t,
                                             const double*, int64_t, double*, int, double, double);
template int gemm_tn<float, float, double>(Ctx*, Workspace&, int64_t, int, int, const float*, int64_t, const float*,
                                           int64_t, double*, int, double, double);
template int gemm_tn<float, double, double>(Ctx*, Workspace&, int64_t, int, int, const float*, int64_t, const float*,
                                            int64_t, double*, int, double, double);
template int gemm_nn<double, double>(Ctx*, int64_t, int, int, double, const double*, int64_t, const double*, int,
                                     double, double*, int64_t);
template int gemm_nn<float, double>(Ctx*, int64_t, int, int, float, const float*, int64_t, const double*, int, float,
                                    float*, int64_t);
template int gemm_nn<float, float>(Ctx*, int64_t, int, int, float, const float*, int64_t, const float*, int, float,
                                   float*, int64_t);
template int precond_dpr<double, double>(Ctx*, int64_t, int, const double*, int64_t, const double*, const double*,
                                         double*, int64_t);
template int precond_dpr<float, float>(Ctx*, int64_t, int, const float*, int64_t, const double*, const float*,
                                       float*, int64_t);
template int precond_olsen<double, double>(Ctx*, Workspace&, int64_t, int, const double*, const double*, int64_t,
                                           const double*, const double*, double*, int64_t, double*);
template int precond_olsen<float, float>(Ctx*, Workspace&, int64_t, int, const float*, const float*, int64_t,
                                         const double*, const float*, float*, int64_t, double*);
template int residuals<double>(Ctx*, Workspace&, int64_t, int, const double*, const double*, int64_t, const double*,
                               double*, double*);
template int residuals<float>(Ctx*, Workspace&, int64_t, int, const float*, const float*, int64_t, const double*,
                              float*, double*);
template int convert<double, float>(Ctx*, const double*, float*, int64_t);
template int convert<float, double>(Ctx*, const float*, double*, int64_t);

}  // namespace adcgpu
