// Learned preconditioner: a per-component MLP that rescales the diagonal
// (DPR) correction of block_davidson.f90:1288-1342,
//
//     t_ij = m_ij * r_ij / (lambda_i - h_jj),   m = MLP(features_ij),
//
// so that m = 1 is exactly the reference's preconditioner (the fallback).
// Features of configuration j for root i (MLP_NIN = 16, see mlp_feature):
//   g = lambda_i - h_jj, sign(g) exp(-|g|), 1/(1+|g|), single flag, one-hot of
//   the double class (1, 2, 3, 4I/4II), zeroth-order energy / 10 (e_a - e_k
//   or e_a + e_b - e_k - e_l), (h_jj - zeroth-order) / 10, lambda_i / 10.
// Network: 16 -> 256 -> 256 -> 1, SiLU, BF16 weights, FP32 accumulation.
//
// Tensor-core work uses mma.sync m16n8k16 (BF16 in, FP32 accumulate).
// Inference is one fused kernel: layer-1 outputs become layer-2 A fragments
// in registers and layer 2 is reduced against w3 on the fly, so activations
// never leave the SM.  Training (forward, backward, Adam) uses a generic BF16
// GEMM plus elementwise kernels; weights live in the context.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "davidson.h"
#include "dense.h"
#include "internal.h"

namespace adcgpu {

constexpr int MLP_NIN = 16, MLP_H = 256;

struct MlpState {
  // FP32 masters and Adam moments: W1[H][NIN], b1[H], W2[H][H], b2[H], w3[H], b3
  float* p = nullptr;        // all parameters, packed
  float* m1 = nullptr;       // Adam first moment
  float* m2 = nullptr;       // Adam second moment
  float* grad = nullptr;
  __nv_bfloat16* W1b = nullptr;
  __nv_bfloat16* W2b = nullptr;
  int64_t nparam = 0;
  int step = 0;
  // training scratch
  float* scratch = nullptr;
  size_t scratch_bytes = 0;
};

namespace {

constexpr int64_t OFF_W1 = 0;
constexpr int64_t OFF_B1 = OFF_W1 + MLP_H * MLP_NIN;
constexpr int64_t OFF_W2 = OFF_B1 + MLP_H;
constexpr int64_t OFF_B2 = OFF_W2 + MLP_H * MLP_H;
constexpr int64_t OFF_W3 = OFF_B2 + MLP_H;
constexpr int64_t OFF_B3 = OFF_W3 + MLP_H;
constexpr int64_t NPARAM = OFF_B3 + 1;

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  float s = 1.f / (1.f + __expf(-z));
  return s * (1.f + z * (1.f - s));
}

// Features of storage-independent configuration j (0-based, singles first).
__device__ __forceinline__ void mlp_feature(const GeomDev& g, const double* __restrict__ e, int64_t j, double lam,
                                            double h, float* f) {
  const int no = g.no;
  double d0;
  int cls;
  if (j < g.n1) {
    const int a = (int)(j / no), k = (int)(j % no);
    d0 = e[no + a] - e[k];
    cls = -1;
  } else {
    Double r = decode_double(g, j - g.n1);
    d0 = e[no + r.ap] + e[no + r.bp] - e[r.kp] - e[r.lp];
    cls = r.cls < 4 ? r.cls : 3;
  }
  const double gg = lam - h;
  f[0] = (float)gg;
  f[1] = (float)(gg >= 0 ? 1.0 : -1.0) * expf(-(float)fabs(gg));
  f[2] = 1.f / (1.f + (float)fabs(gg));
  f[3] = cls < 0 ? 1.f : 0.f;
  f[4] = cls == 0 ? 1.f : 0.f;
  f[5] = cls == 1 ? 1.f : 0.f;
  f[6] = cls == 2 ? 1.f : 0.f;
  f[7] = cls == 3 ? 1.f : 0.f;
  f[8] = (float)(d0 / 10.0);
  f[9] = (float)((h - d0) / 10.0);
  f[10] = (float)(lam / 10.0);
  f[11] = f[12] = f[13] = f[14] = f[15] = 0.f;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int W1S = 24;    // padded smem row strides (bf16 elements): conflict-free fragment loads
constexpr int W2S = 264;

// Fused inference: rows q = i*N + j (root i, configuration j).  Each warp
// handles 16 rows per step.  Writes t = m r / g (0 where g == 0).
template <typename T>
__global__ void __launch_bounds__(256) k_mlp_apply(GeomDev geo, const double* __restrict__ e, int64_t N, int nb,
                                                   const T* __restrict__ R, const double* __restrict__ lam,
                                                   const T* __restrict__ hii, const __nv_bfloat16* __restrict__ W1g,
                                                   const __nv_bfloat16* __restrict__ W2g,
                                                   const float* __restrict__ P, T* __restrict__ Tout,
                                                   float* __restrict__ m_out) {
  extern __shared__ unsigned char smem_raw[];
  __nv_bfloat16* sW2 = reinterpret_cast<__nv_bfloat16*>(smem_raw);      // [H][W2S]
  __nv_bfloat16* sW1 = sW2 + MLP_H * W2S;                                // [H][W1S]
  float* sb1 = reinterpret_cast<float*>(sW1 + MLP_H * W1S);
  float* sb2 = sb1 + MLP_H;
  float* sw3 = sb2 + MLP_H;
  for (int i = threadIdx.x; i < MLP_H * MLP_H; i += blockDim.x) sW2[(i / MLP_H) * W2S + (i % MLP_H)] = W2g[i];
  for (int i = threadIdx.x; i < MLP_H * MLP_NIN; i += blockDim.x) sW1[(i / MLP_NIN) * W1S + (i % MLP_NIN)] = W1g[i];
  for (int i = threadIdx.x; i < MLP_H; i += blockDim.x) {
    sb1[i] = P[OFF_B1 + i]; sb2[i] = P[OFF_B2 + i]; sw3[i] = P[OFF_W3 + i];
  }
  __syncthreads();
  const float b3 = P[OFF_B3];
  const int lane = threadIdx.x & 31, gid = lane >> 2, tig = lane & 3;
  const int64_t M = N * nb;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t q0 = warp * 16; q0 < M; q0 += nwarps * 16) {
    // rows of this thread: q0 + gid and q0 + gid + 8
    float f[2][MLP_NIN];
    float rv[2], gv[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t q = q0 + gid + 8 * h;
      if (q < M) {
        const int i = (int)(q / N);
        const int64_t j = q - (int64_t)i * N;
        const double hj = (double)hii[j];
        mlp_feature(geo, e, j, lam[i], hj, f[h]);
        rv[h] = (float)R[(int64_t)i * N + j];
        gv[h] = (float)(lam[i] - hj);
      } else {
#pragma unroll
        for (int k = 0; k < MLP_NIN; ++k) f[h][k] = 0.f;
        rv[h] = 0.f; gv[h] = 0.f;
      }
    }
    uint32_t a1[4];
    a1[0] = pack_bf16(f[0][tig * 2], f[0][tig * 2 + 1]);
    a1[1] = pack_bf16(f[1][tig * 2], f[1][tig * 2 + 1]);
    a1[2] = pack_bf16(f[0][tig * 2 + 8], f[0][tig * 2 + 9]);
    a1[3] = pack_bf16(f[1][tig * 2 + 8], f[1][tig * 2 + 9]);
    // layer 1 -> A fragments of layer 2 (16 K-chunks)
    uint32_t a2[16][4];
#pragma unroll
    for (int kc = 0; kc < 16; ++kc) {
      float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
      const int n0 = kc * 16 + gid, n1 = n0 + 8;
      const uint32_t* w0 = reinterpret_cast<const uint32_t*>(sW1 + n0 * W1S);
      const uint32_t* w1 = reinterpret_cast<const uint32_t*>(sW1 + n1 * W1S);
      mma_bf16(c0, a1, w0[tig], w0[tig + 4]);
      mma_bf16(c1, a1, w1[tig], w1[tig + 4]);
      const int col0 = kc * 16 + tig * 2, col1 = col0 + 8;
      a2[kc][0] = pack_bf16(silu(c0[0] + sb1[col0]), silu(c0[1] + sb1[col0 + 1]));
      a2[kc][1] = pack_bf16(silu(c0[2] + sb1[col0]), silu(c0[3] + sb1[col0 + 1]));
      a2[kc][2] = pack_bf16(silu(c1[0] + sb1[col1]), silu(c1[1] + sb1[col1 + 1]));
      a2[kc][3] = pack_bf16(silu(c1[2] + sb1[col1]), silu(c1[3] + sb1[col1 + 1]));
    }
    // layer 2 in blocks of 64 outputs, reduced against w3 on the fly
    float rs0 = 0.f, rs1 = 0.f;
#pragma unroll 1
    for (int nb64 = 0; nb64 < MLP_H; nb64 += 64) {
      float acc[8][4];
#pragma unroll
      for (int t = 0; t < 8; ++t) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
#pragma unroll
      for (int kc = 0; kc < 16; ++kc) {
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          const uint32_t* w = reinterpret_cast<const uint32_t*>(sW2 + (nb64 + t * 8 + gid) * W2S + kc * 16);
          mma_bf16(acc[t], a2[kc], w[tig], w[tig + 4]);
        }
      }
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int col = nb64 + t * 8 + tig * 2;
        rs0 += silu(acc[t][0] + sb2[col]) * sw3[col] + silu(acc[t][1] + sb2[col + 1]) * sw3[col + 1];
        rs1 += silu(acc[t][2] + sb2[col]) * sw3[col] + silu(acc[t][3] + sb2[col + 1]) * sw3[col + 1];
      }
    }
    rs0 += __shfl_xor_sync(0xffffffffu, rs0, 1);
    rs0 += __shfl_xor_sync(0xffffffffu, rs0, 2);
    rs1 += __shfl_xor_sync(0xffffffffu, rs1, 1);
    rs1 += __shfl_xor_sync(0xffffffffu, rs1, 2);
    if (tig == 0) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int64_t q = q0 + gid + 8 * h;
        if (q < M) {
          const float mm = (h ? rs1 : rs0) + b3;
          if (m_out) m_out[q] = mm;
          if (Tout) {
            const float gq = gv[h];
            Tout[q] = gq == 0.f ? T(0) : (T)(mm * rv[h] / gq);
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Training kernels.
// ---------------------------------------------------------------------------
// Generic C[M x N] (fp32) = alpha * op(A)[M x K] * op(B)[K x N] + beta C, BF16
// inputs.  op(A): transA ? A^T stored [K][lda] : A stored [M][lda].
// op(B): transB ? B^T stored [N][ldb] : B stored [K][ldb].  Tiles 64x64x16.
__global__ void __launch_bounds__(128) k_gemm_bf16(int M, int Nn, int K, const __nv_bfloat16* __restrict__ A,
                                                   int lda, int transA, const __nv_bfloat16* __restrict__ B, int ldb,
                                                   int transB, float* __restrict__ C, int ldc, float alpha,
                                                   float beta, int ksplit) {
  __shared__ __nv_bfloat16 sA[64][16 + 8];   // [m][k]
  __shared__ __nv_bfloat16 sB[64][16 + 8];   // [n][k]
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const int kz = blockIdx.z;
  const int kper = ((K + ksplit - 1) / ksplit + 15) / 16 * 16;
  const int kbeg = kz * kper, kend = min(K, kbeg + kper);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int gid = lane >> 2, tig = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;
  for (int k0 = kbeg; k0 < kend; k0 += 16) {
    __syncthreads();
    for (int l = threadIdx.x; l < 64 * 16; l += 128) {
      const int r = l / 16, kk = l % 16;
      const int gm = m0 + r, gk = k0 + kk, gn = n0 + r;
      __nv_bfloat16 va = __float2bfloat16(0.f), vb = __float2bfloat16(0.f);
      if (gm < M && gk < kend) va = transA ? A[(int64_t)gk * lda + gm] : A[(int64_t)gm * lda + gk];
      if (gn < Nn && gk < kend) vb = transB ? B[(int64_t)gn * ldb + gk] : B[(int64_t)gk * ldb + gn];
      sA[r][kk] = va;
      sB[r][kk] = vb;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int r = wm + i * 16;
      uint32_t a[4];
      a[0] = *reinterpret_cast<const uint32_t*>(&sA[r + gid][tig * 2]);
      a[1] = *reinterpret_cast<const uint32_t*>(&sA[r + gid + 8][tig * 2]);
      a[2] = *reinterpret_cast<const uint32_t*>(&sA[r + gid][tig * 2 + 8]);
      a[3] = *reinterpret_cast<const uint32_t*>(&sA[r + gid + 8][tig * 2 + 8]);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int cidx = wn + j * 8 + gid;
        uint32_t b0 = *reinterpret_cast<const uint32_t*>(&sB[cidx][tig * 2]);
        uint32_t b1 = *reinterpret_cast<const uint32_t*>(&sB[cidx][tig * 2 + 8]);
        mma_bf16(acc[i][j], a, b0, b1);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = m0 + wm + i * 16 + gid + 8 * h;
        const int cc = n0 + wn + j * 8 + tig * 2;
        for (int u = 0; u < 2; ++u) {
          if (r < M && cc + u < Nn) {
            float v = alpha * acc[i][j][2 * h + u];
            float* dst = &C[(int64_t)r * ldc + cc + u];
            if (ksplit > 1) atomicAdd(dst, v);
            else *dst = (beta == 0.f ? 0.f : beta * *dst) + v;
          }
        }
      }
}

// Z (fp32, M x H) += bias; H = SiLU(Z) as BF16
__global__ void k_bias_silu(int64_t M, const float* __restrict__ Z, const float* __restrict__ b,
                            __nv_bfloat16* __restrict__ Hb, float* __restrict__ Zout) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M * MLP_H; i += (int64_t)gridDim.x * blockDim.x) {
    float z = Z[i] + b[i % MLP_H];
    Zout[i] = z;
    Hb[i] = __float2bfloat16(silu(z));
  }
}

// m = H2 w3 + b3 (one warp per row)
__global__ void k_head(int64_t M, const __nv_bfloat16* __restrict__ H2, const float* __restrict__ P,
                       float* __restrict__ m) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < M;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    float s = 0.f;
    for (int k = lane; k < MLP_H; k += 32) s += __bfloat162float(H2[r * MLP_H + k]) * P[OFF_W3 + k];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) m[r] = s + P[OFF_B3];
  }
}

// Cosine loss per group of S rows: L = 1 - <t,e>^2 / (|t|^2 |e|^2), t = m t0.
// One block per group; writes dL/dm and the group loss.
__global__ void k_cos_loss(int S, const float* __restrict__ m, const float* __restrict__ t0,
                           const float* __restrict__ e, float* __restrict__ dm, float* __restrict__ loss) {
  const int gI = blockIdx.x;
  const float* mg = m + (int64_t)gI * S;
  const float* tg = t0 + (int64_t)gI * S;
  const float* eg = e + (int64_t)gI * S;
  float a = 0.f, b = 0.f, c = 0.f;
  for (int i = threadIdx.x; i < S; i += blockDim.x) {
    float t = mg[i] * tg[i];
    a += t * eg[i]; b += t * t; c += eg[i] * eg[i];
  }
  __shared__ float red[3][32];
  for (int o = 16; o; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) { red[0][w] = a; red[1][w] = b; red[2][w] = c; }
  __syncthreads();
  if (threadIdx.x == 0) {
    float A = 0, B = 0, Cc = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { A += red[0][q]; B += red[1][q]; Cc += red[2][q]; }
    red[0][0] = A; red[1][0] = fmaxf(B, 1e-30f); red[2][0] = fmaxf(Cc, 1e-30f);
  }
  __syncthreads();
  a = red[0][0]; b = red[1][0]; c = red[2][0];
  if (threadIdx.x == 0) loss[gI] = 1.f - a * a / (b * c);
  for (int i = threadIdx.x; i < S; i += blockDim.x) {
    float t = mg[i] * tg[i];
    float dLdt = -2.f * a / (b * c) * eg[i] + 2.f * a * a / (b * b * c) * t;
    dm[(int64_t)gI * S + i] = dLdt * tg[i];
  }
}

// dZ2 = (dm w3) * SiLU'(Z2) (bf16), dw3 partial sums
__global__ void k_back_head(int64_t M, const float* __restrict__ dm, const float* __restrict__ Z2,
                            const float* __restrict__ P, __nv_bfloat16* __restrict__ dZ2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M * MLP_H; i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % MLP_H);
    dZ2[i] = __float2bfloat16(dm[i / MLP_H] * P[OFF_W3 + k] * dsilu(Z2[i]));
  }
}

// column sums of X (M x H, bf16 or fp32 via float reader) into out[H] (atomic)
__global__ void k_colsum_bf16(int64_t M, const __nv_bfloat16* __restrict__ X, float* __restrict__ out) {
  const int k = threadIdx.x;   // blockDim = H
  float s = 0.f;
  for (int64_t r = blockIdx.x; r < M; r += gridDim.x) s += __bfloat162float(X[r * MLP_H + k]);
  atomicAdd(&out[k], s);
}

// dw3[k] = sum_r dm[r] H2[r][k]; db3 = sum dm
__global__ void k_grad_w3(int64_t M, const float* __restrict__ dm, const __nv_bfloat16* __restrict__ H2,
                          float* __restrict__ gw3, float* __restrict__ gb3) {
  const int k = threadIdx.x;
  float s = 0.f, sb = 0.f;
  for (int64_t r = blockIdx.x; r < M; r += gridDim.x) {
    s += dm[r] * __bfloat162float(H2[r * MLP_H + k]);
    if (k == 0) sb += dm[r];
  }
  atomicAdd(&gw3[k], s);
  if (k == 0) atomicAdd(gb3, sb);
}

// dZ1 = dH1 * SiLU'(Z1) (bf16)
__global__ void k_back_act(int64_t M, const float* __restrict__ dH, const float* __restrict__ Z,
                           __nv_bfloat16* __restrict__ dZ) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M * MLP_H; i += (int64_t)gridDim.x * blockDim.x)
    dZ[i] = __float2bfloat16(dH[i] * dsilu(Z[i]));
}

__global__ void k_adam(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, float lr, float b1, float b2, float c1, float c2, float eps,
                       float scale) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float gi = g[i] * scale;
    m1[i] = b1 * m1[i] + (1.f - b1) * gi;
    m2[i] = b2 * m2[i] + (1.f - b2) * gi * gi;
    p[i] -= lr * (m1[i] / c1) / (sqrtf(m2[i] / c2) + eps);
  }
}

__global__ void k_to_bf16_f(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = __float2bfloat16(x[i]);
}

__global__ void k_features(GeomDev g, const double* __restrict__ e, int64_t N, int nb, const double* __restrict__ lam,
                           const double* __restrict__ hii, float* __restrict__ F) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < N * nb; q += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(q / N);
    const int64_t j = q - (int64_t)i * N;
    mlp_feature(g, e, j, lam[i], hii[j], F + q * MLP_NIN);
  }
}

inline MlpState* state(Ctx* c) { return reinterpret_cast<MlpState*>(c->mlp); }

int ensure_state(Ctx* c) {
  if (c->mlp) return ADCGPU_OK;
  MlpState* s = new MlpState;
  c->mlp = s;
  s->nparam = NPARAM;
  int st;
  if ((st = dmalloc(c, (void**)&s->p, sizeof(float) * NPARAM))) return st;
  if ((st = dmalloc(c, (void**)&s->m1, sizeof(float) * NPARAM))) return st;
  if ((st = dmalloc(c, (void**)&s->m2, sizeof(float) * NPARAM))) return st;
  if ((st = dmalloc(c, (void**)&s->grad, sizeof(float) * NPARAM))) return st;
  if ((st = dmalloc(c, (void**)&s->W1b, sizeof(__nv_bfloat16) * MLP_H * MLP_NIN))) return st;
  if ((st = dmalloc(c, (void**)&s->W2b, sizeof(__nv_bfloat16) * MLP_H * MLP_H))) return st;
  ADC_CUDA(c, cudaMemsetAsync(s->m1, 0, sizeof(float) * NPARAM, c->stream));
  ADC_CUDA(c, cudaMemsetAsync(s->m2, 0, sizeof(float) * NPARAM, c->stream));
  return ADCGPU_OK;
}

int refresh_bf16(Ctx* c) {
  MlpState* s = state(c);
  k_to_bf16_f<<<64, 256, 0, c->stream>>>(s->p + OFF_W1, s->W1b, MLP_H * MLP_NIN); ADC_COUNT_LAUNCH();
  k_to_bf16_f<<<256, 256, 0, c->stream>>>(s->p + OFF_W2, s->W2b, MLP_H * MLP_H); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

size_t apply_smem() {
  return sizeof(__nv_bfloat16) * (MLP_H * W2S + MLP_H * W1S) + sizeof(float) * 3 * MLP_H;
}

// Forward + backward on G groups of S rows.  feats (G*S x 16, fp32 host or
// device), t0 = r/g, e = target.  Gradients into s->grad; returns mean loss.
int mlp_fwd_bwd(Ctx* c, int G, int S, const float* d_feat, const float* d_t0, const float* d_e, float* mean_loss,
                float* d_m_out) {
  MlpState* s = state(c);
  const int64_t M = (int64_t)G * S;
  // scratch: X(bf16 M x16) Z1 Z2 (f32 M x H) H1 H2 dZ (bf16 M x H) dH (f32 M x H) m dm (M) loss (G)
  size_t need = M * MLP_NIN * 2 + 3 * M * MLP_H * 4 + 3 * M * MLP_H * 2 + 2 * M * 4 + G * 4 + 1024;
  if (s->scratch_bytes < need) {
    if (s->scratch) dfree(c, s->scratch, s->scratch_bytes);
    s->scratch = nullptr;
    int st = dmalloc(c, (void**)&s->scratch, need);
    if (st) return st;
    s->scratch_bytes = need;
  }
  char* base = reinterpret_cast<char*>(s->scratch);
  __nv_bfloat16* X = reinterpret_cast<__nv_bfloat16*>(base); base += M * MLP_NIN * 2;
  float* Z1 = reinterpret_cast<float*>(base); base += M * MLP_H * 4;
  float* Z2 = reinterpret_cast<float*>(base); base += M * MLP_H * 4;
  float* dH = reinterpret_cast<float*>(base); base += M * MLP_H * 4;
  __nv_bfloat16* H1 = reinterpret_cast<__nv_bfloat16*>(base); base += M * MLP_H * 2;
  __nv_bfloat16* H2 = reinterpret_cast<__nv_bfloat16*>(base); base += M * MLP_H * 2;
  __nv_bfloat16* dZ = reinterpret_cast<__nv_bfloat16*>(base); base += M * MLP_H * 2;
  float* m = reinterpret_cast<float*>(base); base += M * 4;
  float* dm = reinterpret_cast<float*>(base); base += M * 4;
  float* loss = reinterpret_cast<float*>(base);
  cudaStream_t st = c->stream;
  const float* P = s->p;
  float* gr = s->grad;
  k_to_bf16_f<<<c->nsm * 4, 256, 0, st>>>(d_feat, X, M * MLP_NIN); ADC_COUNT_LAUNCH();
  // Z1 = X W1^T
  dim3 g1((MLP_H + 63) / 64, (unsigned)((M + 63) / 64), 1);
  k_gemm_bf16<<<g1, 128, 0, st>>>((int)M, MLP_H, MLP_NIN, X, MLP_NIN, 0, s->W1b, MLP_NIN, 1, Z1, MLP_H, 1.f, 0.f, 1); ADC_COUNT_LAUNCH();
  k_bias_silu<<<c->nsm * 4, 256, 0, st>>>(M, Z1, P + OFF_B1, H1, Z1); ADC_COUNT_LAUNCH();
  k_gemm_bf16<<<g1, 128, 0, st>>>((int)M, MLP_H, MLP_H, H1, MLP_H, 0, s->W2b, MLP_H, 1, Z2, MLP_H, 1.f, 0.f, 1); ADC_COUNT_LAUNCH();
  k_bias_silu<<<c->nsm * 4, 256, 0, st>>>(M, Z2, P + OFF_B2, H2, Z2); ADC_COUNT_LAUNCH();
  k_head<<<c->nsm * 4, 256, 0, st>>>(M, H2, P, m); ADC_COUNT_LAUNCH();
  if (d_m_out) ADC_CUDA(c, cudaMemcpyAsync(d_m_out, m, sizeof(float) * M, cudaMemcpyDeviceToDevice, st));
  k_cos_loss<<<G, 256, 0, st>>>(S, m, d_t0, d_e, dm, loss); ADC_COUNT_LAUNCH();
  // backward
  ADC_CUDA(c, cudaMemsetAsync(gr, 0, sizeof(float) * NPARAM, st));
  k_grad_w3<<<c->nsm, MLP_H, 0, st>>>(M, dm, H2, gr + OFF_W3, gr + OFF_B3); ADC_COUNT_LAUNCH();
  k_back_head<<<c->nsm * 4, 256, 0, st>>>(M, dm, Z2, P, dZ); ADC_COUNT_LAUNCH();          // dZ = dZ2
  k_colsum_bf16<<<c->nsm, MLP_H, 0, st>>>(M, dZ, gr + OFF_B2); ADC_COUNT_LAUNCH();
  const int ks = (int)std::min<int64_t>(64, std::max<int64_t>(1, M / 4096));
  // dW2 = dZ2^T H1  (H x H, K = M)
  dim3 g2((MLP_H + 63) / 64, (MLP_H + 63) / 64, ks);
  k_gemm_bf16<<<g2, 128, 0, st>>>(MLP_H, MLP_H, (int)M, dZ, MLP_H, 1, H1, MLP_H, 0, gr + OFF_W2, MLP_H, 1.f, 0.f, ks); ADC_COUNT_LAUNCH();
  // dH1 = dZ2 W2  (M x H)
  k_gemm_bf16<<<g1, 128, 0, st>>>((int)M, MLP_H, MLP_H, dZ, MLP_H, 0, s->W2b, MLP_H, 0, dH, MLP_H, 1.f, 0.f, 1); ADC_COUNT_LAUNCH();
  k_back_act<<<c->nsm * 4, 256, 0, st>>>(M, dH, Z1, dZ); ADC_COUNT_LAUNCH();               // dZ = dZ1
  k_colsum_bf16<<<c->nsm, MLP_H, 0, st>>>(M, dZ, gr + OFF_B1); ADC_COUNT_LAUNCH();
  // dW1 = dZ1^T X  (H x 16, K = M)
  dim3 g3(1, (MLP_H + 63) / 64, ks);
  k_gemm_bf16<<<g3, 128, 0, st>>>(MLP_H, MLP_NIN, (int)M, dZ, MLP_H, 1, X, MLP_NIN, 0, gr + OFF_W1, MLP_NIN, 1.f, 0.f, ks); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  std::vector<float> hl(G);
  ADC_CUDA(c, cudaMemcpyAsync(hl.data(), loss, sizeof(float) * G, cudaMemcpyDeviceToHost, st));
  ADC_CUDA(c, cudaStreamSynchronize(st));
  double sum = 0.0;
  for (float v : hl) sum += v;
  if (mean_loss) *mean_loss = (float)(sum / G);
  return ADCGPU_OK;
}

}  // namespace

template <typename T>
int mlp_apply(Ctx* c, const MlpPrecond&, int64_t N, int nb, const T* R, const T*, const double* d_lam, const T* hii,
              T* Tout) {
  MlpState* s = state(c);
  if (!s) return precond_dpr<T, T>(c, N, nb, R, N, d_lam, hii, Tout, N);
  const size_t smem = apply_smem();
  auto kern = k_mlp_apply<T>;
  ADC_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<c->nsm, 256, smem, c->stream>>>(to_dev(c->geom), c->d_e, N, nb, R, d_lam, hii, s->W1b, s->W2b, s->p, Tout,
                                      nullptr); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  return ADCGPU_OK;
}

template int mlp_apply<double>(Ctx*, const MlpPrecond&, int64_t, int, const double*, const double*, const double*,
                               const double*, double*);
template int mlp_apply<float>(Ctx*, const MlpPrecond&, int64_t, int, const float*, const float*, const double*,
                              const float*, float*);

void free_mlp(Ctx* c) {
  MlpState* s = state(c);
  if (!s) return;
  float* ps[] = {s->p, s->m1, s->m2, s->grad, s->scratch};
  for (float* p : ps) dfree(c, p);
  dfree(c, s->W1b);
  dfree(c, s->W2b);
  delete s;
  c->mlp = nullptr;
}

}  // namespace adcgpu

using namespace adcgpu;

extern "C" int adcgpu_mlp_set_params(adcgpu_ctx* h, const float* params, int64_t n) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || !params || n != NPARAM) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  int st = ensure_state(c);
  if (st) return st;
  MlpState* s = state(c);
  ADC_CUDA(c, h2d(c, s->p, params, sizeof(float) * NPARAM));
  ADC_CUDA(c, cudaMemsetAsync(s->m1, 0, sizeof(float) * NPARAM, c->stream));
  ADC_CUDA(c, cudaMemsetAsync(s->m2, 0, sizeof(float) * NPARAM, c->stream));
  s->step = 0;
  st = refresh_bf16(c);
  if (st) return st;
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  return ADCGPU_OK;
}

extern "C" int adcgpu_mlp_get_params(adcgpu_ctx* h, float* params, int64_t n) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || !params || n != NPARAM || !c->mlp) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  ADC_CUDA(c, d2h(c, params, state(c)->p, sizeof(float) * NPARAM));
  return ADCGPU_OK;
}

extern "C" int64_t adcgpu_mlp_num_params(void) { return NPARAM; }

// One optimisation step (or, with lr == 0, only the gradient) on G groups of
// S rows from host arrays; grad_out (may be NULL) receives the gradient.
extern "C" int adcgpu_mlp_train_step(adcgpu_ctx* h, int G, int S, const float* feats, const float* t0,
                                     const float* target, float lr, float* loss_out, float* grad_out) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || G <= 0 || S <= 0 || !feats || !t0 || !target || !c->mlp) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  const int64_t M = (int64_t)G * S;
  float *df = nullptr, *dt = nullptr, *de = nullptr;
  int st;
  if ((st = dmalloc(c, (void**)&df, sizeof(float) * M * MLP_NIN))) return st;
  if ((st = dmalloc(c, (void**)&dt, sizeof(float) * M))) return st;
  if ((st = dmalloc(c, (void**)&de, sizeof(float) * M))) return st;
  ADC_CUDA(c, cudaMemcpyAsync(df, feats, sizeof(float) * M * MLP_NIN, cudaMemcpyHostToDevice, c->stream));
  ADC_CUDA(c, cudaMemcpyAsync(dt, t0, sizeof(float) * M, cudaMemcpyHostToDevice, c->stream));
  ADC_CUDA(c, cudaMemcpyAsync(de, target, sizeof(float) * M, cudaMemcpyHostToDevice, c->stream));
  float loss = 0.f;
  st = mlp_fwd_bwd(c, G, S, df, dt, de, &loss, nullptr);
  MlpState* s = state(c);
  if (!st && grad_out) {
    ADC_CUDA(c, cudaMemcpyAsync(grad_out, s->grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, c->stream));
  }
  if (!st && lr > 0.f && std::isfinite(loss)) {
    s->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)s->step), c2 = 1.f - powf(b2, (float)s->step);
    k_adam<<<256, 256, 0, c->stream>>>(NPARAM, s->p, s->grad, s->m1, s->m2, lr, b1, b2, c1, c2, 1e-8f, 1.f / G); ADC_COUNT_LAUNCH();
    st = refresh_bf16(c);
  }
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  dfree(c, df, 0); dfree(c, dt, 0); dfree(c, de, 0);
  if (loss_out) *loss_out = loss;
  return st;
}

// Fused inference on host data: m_out[q] for q = i*N + j (N x nb rows of
// the built matrix), t_out = m r / g.  Also returns the features.
extern "C" int adcgpu_mlp_infer(adcgpu_ctx* h, int nb, const double* lam, const double* R, float* m_out,
                                double* t_out, float* feats_out) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || nb <= 0 || !lam || !c->mlp) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "build the matrix first");
  const int64_t N = c->geom.N, M = N * nb;
  double *dl = nullptr, *dR = nullptr, *dT = nullptr;
  float *dm = nullptr, *dF = nullptr;
  int st;
  if ((st = dmalloc(c, (void**)&dl, sizeof(double) * nb))) return st;
  if ((st = dmalloc(c, (void**)&dR, sizeof(double) * M))) return st;
  if ((st = dmalloc(c, (void**)&dT, sizeof(double) * M))) return st;
  if ((st = dmalloc(c, (void**)&dm, sizeof(float) * M))) return st;
  if ((st = dmalloc(c, (void**)&dF, sizeof(float) * M * MLP_NIN))) return st;
  ADC_CUDA(c, cudaMemcpyAsync(dl, lam, sizeof(double) * nb, cudaMemcpyHostToDevice, c->stream));
  if (R) ADC_CUDA(c, cudaMemcpyAsync(dR, R, sizeof(double) * M, cudaMemcpyHostToDevice, c->stream));
  else ADC_CUDA(c, cudaMemsetAsync(dR, 0, sizeof(double) * M, c->stream));
  const size_t smem = apply_smem();
  ADC_CUDA(c, cudaFuncSetAttribute(k_mlp_apply<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  MlpState* s = state(c);
  k_mlp_apply<double><<<c->nsm, 256, smem, c->stream>>>(to_dev(c->geom), c->d_e, N, nb, dR, dl, c->d_diag, s->W1b,
                                                     s->W2b, s->p, dT, dm); ADC_COUNT_LAUNCH();
  k_features<<<c->nsm * 4, 256, 0, c->stream>>>(to_dev(c->geom), c->d_e, N, nb, dl, c->d_diag, dF); ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  if (m_out) ADC_CUDA(c, cudaMemcpyAsync(m_out, dm, sizeof(float) * M, cudaMemcpyDeviceToHost, c->stream));
  if (t_out) ADC_CUDA(c, cudaMemcpyAsync(t_out, dT, sizeof(double) * M, cudaMemcpyDeviceToHost, c->stream));
  if (feats_out) ADC_CUDA(c, cudaMemcpyAsync(feats_out, dF, sizeof(float) * M * MLP_NIN, cudaMemcpyDeviceToHost, c->stream));
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  dfree(c, dl, 0); dfree(c, dR, 0); dfree(c, dT, 0); dfree(c, dm, 0); dfree(c, dF, 0);
  return ADCGPU_OK;
}
