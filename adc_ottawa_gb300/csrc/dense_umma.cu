// Tall-skinny Gram products C(p x q) = A(N x p)^T B(N x q) of FP32 vectors on
// the 5th-generation tensor cores: the Rayleigh matrix V^T (HV) (calcrmat,
// block_davidson.f90:954-967), the projections of the block
// orthogonalisation (subspace_projection / qrortho, :1226-1284, 1423-1465)
// and their Gram matrices, on the FP32 phases of the mixed-precision ladder.
//
// Precision.  Every FP32 value x is split into three BF16 slices
// x = x0 + x1 + x2 (x0 = bf16(x), x1 = bf16(x - x0), x2 = bf16(x - x0 - x1);
// the differences are exact in FP32), and the six slice products whose
// weight is at least 2^-18 (x0y0, x0y1, x1y0, x0y2, x1y1, x2y0) are
// accumulated by tcgen05.mma (kind::f16, FP32 accumulate in TMEM).  The
// dropped products are below 2^-26 of |x||y|, so each product carries about
// FP32 rounding.  A TMEM accumulator sums 128 rows; the epilogue adds it into
// double-float registers (df.h), and the per-block partials are summed in
// FP64 in a fixed order, as the CUDA-core kernel of dense.cu does.
//
// One CTA per (row block, 128-column tile of A), 256 threads: all threads
// load the next 64 rows of their columns into registers while the tensor
// cores work on the current ones, split them and store the slices into a
// 3-stage ring of 128-byte-swizzled K-major operand tiles; thread 0 issues
// the MMAs (24 per 64 rows) and commits them to mbarriers; threads 0-127
// (the 128 TMEM lanes) drain the accumulator every 128 rows.  TMEM holds two
// accumulators, so the MMAs of the next 128 rows run while one is drained.
// Every wait is bounded; a wait that gives up sets the error word and the
// call returns ADCGPU_DEVICE_TIMEOUT.
#include <cuda_bf16.h>

#include <algorithm>

#include "dense.h"
#include "df.h"
#include "internal.h"
#include "umma.h"

namespace adcgpu {

using namespace umma;

namespace {

constexpr int GU_THREADS = 256;
constexpr int GU_M = 128;      // A columns per CTA (MMA M)
constexpr int GU_K = 64;       // rows per stage: one 128-byte swizzled row of 64 BF16 values
constexpr int GU_NS = 3;       // ring stages
constexpr int GU_F = 2;        // stages summed per TMEM accumulator before it is drained
constexpr int GU_A_SLICE = GU_M * 128;   // bytes of one slice of the A tile

template <int NQ>
__host__ __device__ constexpr int gu_stage_bytes() { return 3 * GU_A_SLICE + 3 * NQ * 128; }

template <int NQ>
__host__ __device__ constexpr uint32_t gu_tmem_cols() { return 2 * NQ <= 32 ? 32 : (2 * NQ <= 64 ? 64 : 128); }

template <int NQ>
__host__ __device__ constexpr size_t gu_smem_bytes() {
  return 1024 + (size_t)GU_NS * gu_stage_bytes<NQ>() + 8 * (GU_NS + 2) + 16;
}

__device__ __forceinline__ bool gu_failed(const int* err) { return *(const volatile int*)err != 0; }

// three BF16 slices of a pair of FP32 values (stored as bf16x2 words)
__device__ __forceinline__ void split3(float x, float y, __nv_bfloat162& s0, __nv_bfloat162& s1,
                                       __nv_bfloat162& s2) {
  s0 = __floats2bfloat162_rn(x, y);
  const float2 f0 = __bfloat1622float2(s0);
  const float rx = x - f0.x, ry = y - f0.y;
  s1 = __floats2bfloat162_rn(rx, ry);
  const float2 f1 = __bfloat1622float2(s1);
  s2 = __floats2bfloat162_rn(rx - f1.x, ry - f1.y);
}

// part[blk][tile][GU_M][NQ]: the block's FP64 sums of its rows
template <int NQ>
__global__ void __launch_bounds__(GU_THREADS, 1)
    k_gram_umma(int64_t N, int p, int q, const float* __restrict__ A, int64_t lda, const float* __restrict__ B,
                int64_t ldb, int64_t rows_per_blk, double* __restrict__ part, int* __restrict__ err) {
  constexpr int SB = gu_stage_bytes<NQ>();
  constexpr int B_SLICE = NQ * 128;
  constexpr int NB = NQ / 8;          // B columns per warp
  constexpr uint32_t TCOLS = gu_tmem_cols<NQ>();
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + (size_t)GU_NS * SB);
  uint64_t* mma_done = bars;                 // [GU_NS]
  uint64_t* acc_full = bars + GU_NS;         // [2]
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + GU_NS + 2);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * GU_M;
  const int64_t r_begin = blockIdx.x * rows_per_blk;
  const int64_t r_end = min(N, r_begin + rows_per_blk);
  const int nch = r_begin < r_end ? (int)((r_end - r_begin + GU_K - 1) / GU_K) : 0;

  if (tid == 0) {
    for (int i = 0; i < GU_NS + 2; ++i) mbar_init(&bars[i], 1u);
  }
  if (warp == 0) tmem_alloc(tmem_holder, TCOLS);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tacc = *tmem_holder;

  // this thread's columns: A columns m0 + warp + 8u (u < 16), B columns
  // warp + 8u (u < NB); rows r0 + 2 lane, r0 + 2 lane + 1 of each stage
  float2 pa[GU_M / 8], pb[NB];
  auto fetch = [&](int i) {
    const int64_t r = r_begin + (int64_t)i * GU_K + 2 * lane;
    const bool ok0 = r < r_end, ok1 = r + 1 < r_end;
#pragma unroll
    for (int u = 0; u < GU_M / 8; ++u) {
      const int m = m0 + warp + 8 * u;
      const float* col = A + (int64_t)m * lda;
      pa[u].x = (m < p && ok0) ? __ldg(col + r) : 0.f;
      pa[u].y = (m < p && ok1) ? __ldg(col + r + 1) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      const int n = warp + 8 * u;
      const float* col = B + (int64_t)n * ldb;
      pb[u].x = (n < q && ok0) ? __ldg(col + r) : 0.f;
      pb[u].y = (n < q && ok1) ? __ldg(col + r + 1) : 0.f;
    }
  };
  auto store = [&](int s) {
    unsigned char* sa = base + (size_t)s * SB;
    unsigned char* sb = sa + 3 * GU_A_SLICE;
#pragma unroll
    for (int u = 0; u < GU_M / 8; ++u) {
      const uint32_t off = sw128_off(warp + 8 * u, 2 * lane);
      __nv_bfloat162 s0, s1, s2;
      split3(pa[u].x, pa[u].y, s0, s1, s2);
      *reinterpret_cast<__nv_bfloat162*>(sa + off) = s0;
      *reinterpret_cast<__nv_bfloat162*>(sa + GU_A_SLICE + off) = s1;
      *reinterpret_cast<__nv_bfloat162*>(sa + 2 * GU_A_SLICE + off) = s2;
    }
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      const uint32_t off = sw128_off(warp + 8 * u, 2 * lane);
      __nv_bfloat162 s0, s1, s2;
      split3(pb[u].x, pb[u].y, s0, s1, s2);
      *reinterpret_cast<__nv_bfloat162*>(sb + off) = s0;
      *reinterpret_cast<__nv_bfloat162*>(sb + B_SLICE + off) = s1;
      *reinterpret_cast<__nv_bfloat162*>(sb + 2 * B_SLICE + off) = s2;
    }
  };
  // double-float sums of this thread's row (TMEM lane = tid < 128) of C
  df acc[NQ];
#pragma unroll
  for (int j = 0; j < NQ; ++j) acc[j] = df{0.f, 0.f};
  const uint32_t lane_off = (uint32_t)(32 * (warp & 3)) << 16;
  auto drain = [&](int grp) -> bool {
    // threads 0-127 read accumulator grp & 1 once its MMAs are complete
    if (tid < GU_M) {
      // tcgen05.ld is warp-aligned: the warp leaves together if any lane's
      // wait gave up
      const bool w = mbar_wait(&acc_full[grp & 1], (uint32_t)(grp >> 1) & 1u, err, 3);
      if (!__all_sync(0xffffffffu, w)) return false;
      fence_after_sync();
#pragma unroll
      for (int j0 = 0; j0 < NQ; j0 += 8) {
        float v[8];
        tmem_ld8(tacc + (uint32_t)((grp & 1) * NQ + j0) + lane_off, v);
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[j0 + j] = df_add(acc[j0 + j], df{v[j], 0.f});
      }
    }
    return true;
  };

  const int ngrp = (nch + GU_F - 1) / GU_F;
  int drained = 0, issued = 0;
  bool ok = true;
  if (nch > 0) fetch(0);
  for (int i = 0; i < nch; ++i) {
    const int s = i % GU_NS;
    // the stage's previous MMAs (chunk i - GU_NS) have read it
    if (ok && i >= GU_NS) ok = mbar_wait(&mma_done[s], (uint32_t)((i - GU_NS) / GU_NS) & 1u, err, 1);
    if (ok) {
      store(s);
      fence_proxy_async();
    }
    if (i + 1 < nch) fetch(i + 1);
    // every thread takes the same branch: a failed wait anywhere ends the loop
    // for the whole CTA, so no thread is left at a barrier
    if (!__syncthreads_and(ok && !gu_failed(err))) {
      ok = false;
      break;
    }
    if (tid == 0) {
      fence_after_sync();
      const int grp = i / GU_F;
      const uint32_t idesc = idesc_bf16(GU_M, NQ, 0, 0);
      const uint32_t sa = smem_u32(base + (size_t)s * SB), sb = sa + 3 * GU_A_SLICE;
      const uint32_t d = tacc + (uint32_t)((grp & 1) * NQ);
      constexpr int PA[6] = {0, 0, 1, 0, 1, 2}, PB[6] = {0, 1, 0, 2, 1, 0};
      uint32_t accum = (i % GU_F) ? 1u : 0u;
#pragma unroll
      for (int pr = 0; pr < 6; ++pr)
#pragma unroll
        for (int ks = 0; ks < GU_K / 16; ++ks) {
          const uint64_t ad = sdesc(sa + PA[pr] * GU_A_SLICE + ks * 32, 16, 1024, LAYOUT_SW128);
          const uint64_t bd = sdesc(sb + PB[pr] * B_SLICE + ks * 32, 16, 1024, LAYOUT_SW128);
          mma_bf16(d, ad, bd, idesc, accum);
          accum = 1u;
        }
      mma_commit(&mma_done[s]);
      if (i % GU_F == GU_F - 1 || i == nch - 1) mma_commit(&acc_full[grp & 1]);
      issued = i + 1;
    }
    // the previous accumulator is complete once the first stage of the next
    // one is issued: drain it while the tensor cores work (its result joins
    // the next iteration's vote)
    if (i % GU_F == 0 && i > 0) {
      if (!drain(drained)) ok = false;
      ++drained;
      fence_before_sync();
    }
  }
  while (ok && drained < ngrp) {
    if (!drain(drained)) ok = false;
    ++drained;
  }
  // no MMA may still be running when TMEM is released: wait (bounded) for the
  // last commit of every stage
  if (tid == 0) {
    for (int k = 0; k < GU_NS && k < issued; ++k) {
      const int i = issued - 1 - k;
      mbar_wait(&mma_done[i % GU_NS], (uint32_t)(i / GU_NS) & 1u, err, 4);
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0) {
    tmem_dealloc(tacc, TCOLS);
    tmem_relinquish();
  }
  if (tid < GU_M) {
    double* out = part + ((int64_t)blockIdx.x * gridDim.y + blockIdx.y) * (GU_M * NQ) + (int64_t)tid * NQ;
#pragma unroll
    for (int j = 0; j < NQ; ++j) out[j] = df_value(acc[j]);
  }
}

// C(p x q) (col-major, ldc) = alpha * sum over blocks (fixed order) + beta C
__global__ void k_gram_umma_reduce(int p, int q, int nq, int nblk, int ntile, const double* __restrict__ part,
                                   double* __restrict__ C, int ldc, double alpha, double beta) {
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < p * q; o += gridDim.x * blockDim.x) {
    const int i = o % p, j = o / p;
    const int tile = i / GU_M, ii = i - tile * GU_M;
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += part[((int64_t)b * ntile + tile) * (GU_M * nq) + (int64_t)ii * nq + j];
    const double prev = beta == 0.0 ? 0.0 : beta * C[(int64_t)j * ldc + i];
    C[(int64_t)j * ldc + i] = prev + alpha * s;
  }
}

}  // namespace

struct GramPlan {
  int* d_err = nullptr;
  int* h_err = nullptr;
  int off = 0;                  // 1: the CUDA-core kernel is used instead
};

void gram_free(Ctx* c) {
  GramPlan* g = reinterpret_cast<GramPlan*>(c->gram);
  if (!g) return;
  dfree(c, g->d_err);
  if (g->h_err) cudaFreeHost(g->h_err);
  delete g;
  c->gram = nullptr;
}

int gram_set_off(Ctx* c, int off) {
  if (!c->gram) c->gram = new GramPlan;
  reinterpret_cast<GramPlan*>(c->gram)->off = off;
  return ADCGPU_OK;
}

bool gram_umma_usable(Ctx* c, int64_t N, int p, int q) {
  if (q < 1 || q > 48 || p < 1 || N < 1) return false;
  if (c->gram && reinterpret_cast<GramPlan*>(c->gram)->off) return false;
  int major = 0;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, c->device) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return major >= 10 && gu_smem_bytes<48>() <= (size_t)smem_optin_max(c);
}

int gram_umma(Ctx* c, Workspace& ws, int64_t N, int p, int q, const float* A, int64_t lda, const float* B,
              int64_t ldb, double* C, int ldc, double alpha, double beta) {
  if (!c->gram) c->gram = new GramPlan;
  GramPlan* gp = reinterpret_cast<GramPlan*>(c->gram);
  if (!gp->d_err) {
    ST(dmalloc(c, (void**)&gp->d_err, sizeof(int)));
    ADC_CUDA(c, cudaMallocHost((void**)&gp->h_err, sizeof(int)));
    ADC_CUDA(c, cudaMemsetAsync(gp->d_err, 0, sizeof(int), c->stream));
  }
  const int nq = q <= 16 ? 16 : (q <= 32 ? 32 : 48);
  const int ntile = (p + GU_M - 1) / GU_M;
  // at most two blocks per SM over all column tiles (one CTA fits an SM, so
  // that is two full waves), each row block a multiple of the stage height
  const int64_t want = std::max<int64_t>(1, ((int64_t)c->nsm * 2) / ntile);
  const int64_t rows = std::max<int64_t>(GU_K, ((N + want - 1) / want + GU_K - 1) / GU_K * GU_K);
  const int nblk = (int)((N + rows - 1) / rows);
  ST(ws.reserve(c, sizeof(double) * (size_t)nblk * ntile * GU_M * nq));
  double* part = reinterpret_cast<double*>(ws.p);
  const int smax = smem_optin_max(c);
  auto go = [&](auto kern, size_t smem) -> int {
    ADC_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
    kern<<<dim3(nblk, ntile), GU_THREADS, smem, c->stream>>>(N, p, q, A, lda, B, ldb, rows, part, gp->d_err);
    ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    return ADCGPU_OK;
  };
  if (nq == 16) ST(go(k_gram_umma<16>, gu_smem_bytes<16>()));
  else if (nq == 32) ST(go(k_gram_umma<32>, gu_smem_bytes<32>()));
  else ST(go(k_gram_umma<48>, gu_smem_bytes<48>()));
  k_gram_umma_reduce<<<std::min((p * q + 255) / 256, c->nsm * 8), 256, 0, c->stream>>>(p, q, nq, nblk, ntile, part,
                                                                                      C, ldc, alpha, beta);
  ADC_COUNT_LAUNCH();
  ADC_CUDA(c, cudaGetLastError());
  // the error word of the bounded waits (one small copy; the callers read C
  // on the host right after)
  ADC_CUDA(c, cudaMemcpyAsync(gp->h_err, gp->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  if (*gp->h_err) {
    const int code = *gp->h_err;
    ADC_CUDA(c, cudaMemsetAsync(gp->d_err, 0, sizeof(int), c->stream));
    return set_err(c, ADCGPU_DEVICE_TIMEOUT, "tensor-core Gram product: a pipeline wait timed out (stage " +
                                                  std::to_string(code) + ")");
  }
  return ADCGPU_OK;
}

}  // namespace adcgpu

using namespace adcgpu;

extern "C" int adcgpu_gram_f32(adcgpu_ctx* h, int64_t N, int p, int q, const void* dA, int64_t lda, const void* dB,
                               int64_t ldb, double* dC, int ldc) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || N < 1 || p < 1 || q < 1 || !dA || !dB || !dC || lda < N || ldb < N || ldc < p) return ADCGPU_BAD_INPUT;
  cudaSetDevice(c->device);
  Workspace ws;
  int st = gemm_tn<float, double, double>(c, ws, N, p, q, (const float*)dA, lda, (const float*)dB, ldb, dC, ldc, 1.0,
                                          0.0);
  if (st) return st;
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  return ADCGPU_OK;
}
