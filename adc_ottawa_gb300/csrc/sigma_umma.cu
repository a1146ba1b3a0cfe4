// Tensor-core (tcgen05) pass of the sigma product for BF16 matrix values
// and FP32 vectors: the C and D segments of every row of B^T (the singles
// (a, k') and (a, l') of a double (a', b', k', l'); the layout is described
// in internal.h).  Replaces the per-slab products of hxvec_incore
// (block_davidson.f90:844-883), hxq_incore (block_lanczos.f90:1325-1361)
// and matxvec_treal_incore (tdselib.f90:352-437) on the mixed-precision path.
//
// For one slab (fixed k', l', class) the C|D values of its rows form a dense
// rows x K matrix CD (K = nvP or 2 nvP) and the products are two GEMMs:
//   W2[rows, c] += CD . X          X[k, c] = V[(a, k'|l'), c]
//   W1[(a, k'|l'), c] += CD^T . V2  V2[r, c] = V[n1 + d(r), c]
// Both read the same tile of CD in shared memory: the first as a K-major A
// operand, the second as an MN-major A operand (rows of the tile are its K
// index).  The vectors enter as BF16 hi + lo pairs stacked along N (columns
// [0, NP) hi, [NP, 2 NP) lo), so one MMA gives both products and the
// epilogue adds them (x = hi + lo to ~2^-17 relative).
//
// One CTA per SM, persistent over work items (up to UMMA_ITEM_ROWS rows of
// one slab), warp-specialised:
//   warp 0, one thread : TMA producer.  Each tile of 128 rows is loaded as
//                        slots of two 64-column boxes (128-byte swizzle) into
//                        a ring of NSLOT slots.
//   warp 1, one thread : MMA issuer.  Per slot: W2 tile (M = 128 rows,
//                        N = 2 NP, K = 128) into a double-buffered TMEM
//                        accumulator D1; W1 part (M = 128 values of a,
//                        N = 2 NP, K = 128 rows) into D2[slot], summed over
//                        the item.
//   warps 2-9          : X and V2 operands (hi/lo split into swizzled
//                        shared memory), the diagonal term (and, with
//                        seg_a, the W2 part of segment A) on the CUDA cores,
//                        the D1 epilogue (W2 rows) and, at the end of an
//                        item, D2 into the FP64 W1 accumulator.  Thread =
//                        tile row = TMEM lane; two warps per lane quarter
//                        split the columns.
// Segments A and B run after this pass in the compact A/B kernels
// (sigma_ab.cu); without them (seg_a set), segment B runs in pass 2
// (k_sigma_p2 in sigma.cu) and the W1 part of segment A in k_sigma_p3.  The
// dense singles block is k_singles_gemm.  Every wait is bounded: a lost
// arrival sets the error word and the kernel ends (the host reports
// ADCGPU_DEVICE_TIMEOUT).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"
#include "umma.h"

namespace adcgpu {

using namespace umma;

constexpr int UMMA_ROWS = 128;              // rows per tile (MMA M)
constexpr int UMMA_BOX = 64;                // values per box row (128 bytes)
constexpr int UMMA_SLOT_BYTES = 2 * UMMA_ROWS * UMMA_BOX * 2;   // two boxes
constexpr int UMMA_MAX_BOXES = 6;           // K <= 384
constexpr int UMMA_THREADS = 320;             // producer, MMA issuer, 8 epilogue warps
constexpr int UMMA_NOP = 16;                  // segment A lengths (noP) up to 16 (nocc <= 16)
constexpr int UMMA_ITEM_ROWS_DEFAULT = 4096;  // rows per work item (a piece of one slab)
// rows per work item of the FP32-value main pass: the W1 sums of an item run
// in one TMEM chain (8 MMA steps per 128-row tile), and shorter chains keep
// the tensor cores' truncating FP32 accumulation near FP32 rounding
constexpr int UMMA_ITEM_ROWS_SHORT = 512;

// tensor maps of the five classes' B^T values (rows x L BF16, boxes of 64 x
// 128, 128-byte swizzle), passed by value to the kernel
struct UmmaMaps {
  CUtensorMap m[3][5];   // [value slice][class]; slices 1, 2 only for the FP32-value pass
};

namespace {

enum Bar {
  B_XFULL = 0, B_XEMPTY, B_V2FULL, B_V2EMPTY, B_D2FULL, B_D2EMPTY, B_D1FULL0, B_D1FULL1, B_D1EMPTY0, B_D1EMPTY1,
  B_SLOT0   // then NSLOT full barriers and NSLOT empty barriers
};

__device__ __forceinline__ bool failed(const int* err) { return *(const volatile int*)err != 0; }

// one X / V2 box: XS vector slices of NP columns, 64 values each
__host__ __device__ constexpr int umma_box_bytes(int NP, int XS) { return XS * NP * 128; }

template <int NP, int XS>
__host__ __device__ constexpr int umma_nslot(int smax) {
  // X (6 boxes) + V2 (2 boxes) + barriers and bookkeeping + alignment slack
  return (smax - 1024 - 1024 - 8 * umma_box_bytes(NP, XS)) / UMMA_SLOT_BYTES;
}

template <int NP, int XS>
__host__ __device__ constexpr int umma_tmem_cols() {
  // D1 x 2, D2 x 3 groups, XS NP columns each
  return 5 * XS * NP <= 256 ? 256 : 512;
}

// VS value slices (1: the BF16 store; 3: BF16 slices of the FP32 values,
// hi + mid + lo) and XS vector slices (2: hi | lo; 3: hi | mid | lo).  The
// slices of a product are accumulated by the same MMA chain.
template <int NP, int NSLOT, int VS, int XS>
// 320 threads: some SM sub-partitions hold three of the ten warps, so a
// thread may use at most 16384 / 96 -> 168 registers
__global__ void __launch_bounds__(UMMA_THREADS, 1)
    k_sigma_umma(GeomDev g, const int2* __restrict__ items, int nitems, const __grid_constant__ UmmaMaps maps,
                 const __nv_bfloat16* __restrict__ Bt, const float* __restrict__ diag, const float* __restrict__ V,
                 int64_t ldv, int mcols, float* __restrict__ W, int64_t ldw, double* __restrict__ W1, int64_t ld1,
                 int seg_a, int vbase, int w2_add, int* __restrict__ err) {
  constexpr int N2 = XS * NP;                      // MMA N (the vector slices side by side)
  constexpr int BOXB = umma_box_bytes(NP, XS);
  constexpr uint32_t TCOLS = umma_tmem_cols<NP, XS>();
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sX = base;                                   // 6 boxes [N2 rows x 64 k]
  unsigned char* sV2 = sX + UMMA_MAX_BOXES * BOXB;            // 2 boxes [N2 rows x 64 tile rows]
  unsigned char* sRing = sV2 + 2 * BOXB;                      // NSLOT x 32 KB
  uint64_t* bars = reinterpret_cast<uint64_t*>(sRing + (size_t)NSLOT * UMMA_SLOT_BYTES);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + B_SLOT0 + 2 * NSLOT);
  uint64_t* slot_full = bars + B_SLOT0;
  uint64_t* slot_empty = bars + B_SLOT0 + NSLOT;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int no = g.no, nv = g.nv, noP = g.noP, nvP = g.nvP;
  const int64_t n1 = g.n1;

  if (tid == 0) {
    for (int i = 0; i < B_SLOT0 + 2 * NSLOT; ++i) {
      const bool epi = i == B_XFULL || i == B_V2FULL || i == B_D2EMPTY || i == B_D1EMPTY0 || i == B_D1EMPTY1;
      mbar_init(&bars[i], epi ? 256u : 1u);
    }
  }
  if (warp == 0) tmem_alloc(tmem_holder, TCOLS);
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tbase = *tmem_holder;
  const uint32_t tD1[2] = {tbase, tbase + (uint32_t)N2};
  const uint32_t tD2 = tbase + 2u * N2;                       // + g * N2, g = 0..2

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      uint32_t use = 0;   // slots issued so far (ring position and phase)
      bool ok = true;
      for (int it = blockIdx.x; ok && it < nitems; it += gridDim.x) {
        const int2 item = items[it];
        const Double r0 = decode_row(g, item.x);
        const int cls = r0.cls;
        const bool twoa = (cls == 1 || cls >= 3);
        const int K = (cls >= 2 ? 2 : 1) * nvP;
        const int nslot = (K + 2 * UMMA_BOX - 1) / (2 * UMMA_BOX);
        const int offC = twoa ? 2 * noP : noP;
        for (int row0 = item.x; ok && row0 < item.y; row0 += UMMA_ROWS) {
          const int y = (int)(row0 - g.start[cls]);
          for (int vs = 0; vs < VS && ok; ++vs)
          for (int s = 0; s < nslot; ++s, ++use) {
            const CUtensorMap* tm = &maps.m[vbase + vs][cls];
            const int ri = (int)(use % NSLOT);
            const uint32_t ph = (use / NSLOT) & 1u;
            ok = !failed(err) && mbar_wait(&slot_empty[ri], ph ^ 1u, err, 1);
            if (!ok) break;
            unsigned char* dst = sRing + (size_t)ri * UMMA_SLOT_BYTES;
            mbar_expect_tx(&slot_full[ri], UMMA_SLOT_BYTES);
            // columns past the row's end (and whole boxes past K) read as zero
            tma_load_2d(dst, tm, offC + 2 * UMMA_BOX * s, y, &slot_full[ri]);
            tma_load_2d(dst + UMMA_SLOT_BYTES / 2, tm, offC + 2 * UMMA_BOX * s + UMMA_BOX, y, &slot_full[ri]);
          }
        }
      }
      // no copy may still be writing shared memory when the CTA exits: wait
      // for the last load into every slot (bounded)
      for (uint32_t k = 0; k < NSLOT && k < use; ++k) {
        const uint32_t u = use - 1 - k;
        mbar_wait(&slot_full[u % NSLOT], (u / NSLOT) & 1u, err, 11);
      }
    }
  } else if (warp == 1) {
    // ---------------------------------------------------------- MMA issuer
    if (lane == 0) {
      const uint32_t idK = idesc_bf16(UMMA_ROWS, N2, 0, 0);     // W2: A K-major
      const uint32_t idM = idesc_bf16(UMMA_ROWS, N2, 1, 0);     // W1: A MN-major
      const uint32_t sXa = smem_u32(sX), sVa = smem_u32(sV2), sRa = smem_u32(sRing);
      uint32_t use = 0, tile = 0, nitem = 0;
      bool ok = true;
      for (int it = blockIdx.x; it < nitems && ok && !failed(err); it += gridDim.x, ++nitem) {
        const int2 item = items[it];
        const Double r0 = decode_row(g, item.x);
        const int cls = r0.cls;
        const int K = (cls >= 2 ? 2 : 1) * nvP;
        const int nbox = (K + UMMA_BOX - 1) / UMMA_BOX;
        const int nslot = (nbox + 1) / 2;
        ok = mbar_wait(&bars[B_XFULL], nitem & 1u, err, 2);          // X of this item built
        ok = ok && mbar_wait(&bars[B_D2EMPTY], (nitem & 1u) ^ 1u, err, 3);   // D2 of the last item read
        fence_after_sync();
        bool first_tile = true;
        for (int row0 = item.x; ok && row0 < item.y; row0 += UMMA_ROWS, ++tile) {
          const int db = tile & 1;
          ok = mbar_wait(&bars[B_D1EMPTY0 + db], ((tile >> 1) & 1u) ^ 1u, err, 4);
          ok = ok && mbar_wait(&bars[B_V2FULL], tile & 1u, err, 5);
          fence_after_sync();
          for (int vs = 0; vs < VS && ok; ++vs)
          for (int s = 0; ok && s < nslot; ++s, ++use) {
            const int ri = (int)(use % NSLOT);
            const uint32_t ph = (use / NSLOT) & 1u;
            ok = mbar_wait(&slot_full[ri], ph, err, 6);
            if (!ok) break;
            fence_after_sync();
            const uint32_t slot = sRa + (uint32_t)ri * UMMA_SLOT_BYTES;
            // W2 tile: the slot's boxes as K-major A, X boxes 2s, 2s+1 as B
            for (int b = 0; b < 2; ++b) {
              const int box = 2 * s + b;
              if (box >= nbox) break;
              for (int ks = 0; ks < 4; ++ks) {
                const uint64_t ad = sdesc(slot + b * (UMMA_SLOT_BYTES / 2) + ks * 32, 16, 1024, LAYOUT_SW128);
                const uint64_t bd = sdesc(sXa + box * BOXB + ks * 32, 16, 1024, LAYOUT_SW128);
                mma_bf16(tD1[db], ad, bd, idK, (vs | box | ks) ? 1u : 0u);
              }
            }
            // W1 part: the slot's 128 values of a as MN-major A (two 64-wide
            // groups 16 KB apart), the tile's 128 rows as K; V2 as B
            for (int ks = 0; ks < 8; ++ks) {
              const uint64_t ad = sdesc(slot + ks * 2048, UMMA_SLOT_BYTES / 2, 1024, LAYOUT_SW128);
              const uint64_t bd = sdesc(sVa + (ks >> 2) * BOXB + (ks & 3) * 32, 16, 1024, LAYOUT_SW128);
              mma_bf16(tD2 + (uint32_t)s * N2, ad, bd, idM, (first_tile && vs == 0 && ks == 0) ? 0u : 1u);
            }
            mma_commit(&slot_empty[ri]);
          }
          mma_commit(&bars[B_D1FULL0 + db]);
          mma_commit(&bars[B_V2EMPTY]);
          first_tile = false;
        }
        mma_commit(&bars[B_D2FULL]);
        mma_commit(&bars[B_XEMPTY]);
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue
    // warps 2-9: two warps per TMEM lane quarter, each with half the columns
    const int et = tid - 64;                     // 0..255
    const int q = warp & 3;                      // TMEM lane quarter of this warp
    const int half = (warp - 2) >> 2;            // column half
    constexpr int NH = NP / 2;
    const int cbeg = half * NH;
    const int r = 32 * q + lane;                 // tile row = TMEM lane
    const uint32_t lane_off = (uint32_t)(32 * q) << 16;
    uint32_t tile = 0, nitem = 0;
    bool ok = true;
    // V2 of one tile: this thread's row, this warp's columns.  load_v2 reads
    // them into registers (issued a tile ahead, so the loads overlap the
    // current tile's work); store_v2 splits them into hi/lo in the swizzled
    // operand buffer once the previous tile's W1 products have read it.
    auto load_v2 = [&](int row, int item_end, float (&v2)[NP / 2], int& ap, int64_t& d, bool& valid) {
      valid = row < item_end;
      ap = 0;
      d = 0;
      if (valid) {
        const Double rr = decode_row(g, row);
        ap = rr.ap;
        d = row_to_d(g, rr, row);
      }
#pragma unroll
      for (int j = 0; j < NP / 2; ++j) {
        const int c = cbeg + j;
        v2[j] = (valid && c < mcols) ? __ldg(V + (int64_t)c * ldv + n1 + d) : 0.f;
      }
    };
    auto store_v2 = [&](const float (&v2)[NP / 2]) {
#pragma unroll
      for (int j = 0; j < NP / 2; ++j) {
        const int c = cbeg + j;
        unsigned char* bx = sV2 + (r >> 6) * BOXB;
        float rem = v2[j];
#pragma unroll
        for (int t = 0; t < XS; ++t) {
          const __nv_bfloat16 h = __float2bfloat16(rem);
          *reinterpret_cast<__nv_bfloat16*>(bx + sw128_off(t * NP + c, r & 63)) = h;
          rem -= __bfloat162float(h);
        }
      }
      fence_proxy_async();
      mbar_arrive(&bars[B_V2FULL]);
    };
    for (int it = blockIdx.x; it < nitems && ok && !failed(err); it += gridDim.x, ++nitem) {
      const int2 item = items[it];
      const Double r0 = decode_row(g, item.x);
      const int cls = r0.cls;
      const int K = (cls >= 2 ? 2 : 1) * nvP;
      const int nslot = (K + 2 * UMMA_BOX - 1) / (2 * UMMA_BOX);
      const int64_t L = g.len[cls];
      const int kp = r0.kp, lp = r0.lp;
      // X of this item: slice t of column c at row t NP + c of each box
      ok = mbar_wait(&bars[B_XEMPTY], (nitem & 1u) ^ 1u, err, 7);
      if (!ok) break;
      // eight independent loads in flight per thread, then the stores
      constexpr int XTOT = UMMA_MAX_BOXES * UMMA_BOX * NP;
      for (int o0 = et; o0 < XTOT; o0 += 256 * 8) {
        float xv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int o = o0 + 256 * u;
          const int c = o / (UMMA_MAX_BOXES * UMMA_BOX), k = o - c * (UMMA_MAX_BOXES * UMMA_BOX);
          const int seg = k / nvP, a = k - seg * nvP;
          xv[u] = (o < XTOT && c < mcols && k < K && a < nv)
                      ? __ldg(V + (int64_t)c * ldv + (int64_t)a * no + (seg ? lp : kp)) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int o = o0 + 256 * u;
          if (o >= XTOT) break;
          const int c = o / (UMMA_MAX_BOXES * UMMA_BOX), k = o - c * (UMMA_MAX_BOXES * UMMA_BOX);
          unsigned char* bx = sX + (k >> 6) * BOXB;
          float rem = xv[u];
#pragma unroll
          for (int t = 0; t < XS; ++t) {
            const __nv_bfloat16 h = __float2bfloat16(rem);
            *reinterpret_cast<__nv_bfloat16*>(bx + sw128_off(t * NP + c, k & 63)) = h;
            rem -= __bfloat162float(h);
          }
        }
      }
      fence_proxy_async();
      mbar_arrive(&bars[B_XFULL]);
      // V2 of the item's first tile
      float v2[NH];
      int ap;
      int64_t d;
      bool valid;
      load_v2(item.x + r, item.y, v2, ap, d, valid);
      ok = mbar_wait(&bars[B_V2EMPTY], (tile & 1u) ^ 1u, err, 8);
      if (!ok) break;
      store_v2(v2);
      for (int row0 = item.x; ok && row0 < item.y; row0 += UMMA_ROWS, ++tile) {
        const int db = tile & 1;
        const int row = row0 + r;
        // the next tile's V2, a tile ahead
        const bool has_next = row0 + UMMA_ROWS < item.y;
        float v2n[NH];
        int apn = 0;
        int64_t dn = 0;
        bool validn = false;
        if (has_next) load_v2(row0 + UMMA_ROWS + r, item.y, v2n, apn, dn, validn);
        // diagonal term and segment A (singles (a', k)) of the row's W2; the
        // lanes of a warp mostly share a', so the V loads are broadcasts
        float w2[NH];
        float sa[UMMA_NOP];
#pragma unroll
        for (int k = 0; k < UMMA_NOP; ++k) sa[k] = 0.f;
        if (valid && seg_a) {
          const __nv_bfloat16* rp = Bt + g.off[cls] + (int64_t)(row - g.start[cls]) * L;
#pragma unroll
          for (int k8 = 0; k8 < UMMA_NOP; k8 += 8) {
            if (k8 >= noP) break;
            const uint4 u = __ldg(reinterpret_cast<const uint4*>(rp + k8));
            const __nv_bfloat162* h2 = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const float2 f = __bfloat1622float2(h2[i]);
              sa[k8 + 2 * i] = f.x;
              sa[k8 + 2 * i + 1] = f.y;
            }
          }
        }
        // w2_add: a second pass over other value slices adds to the W2 rows
        // the first pass stored (which hold the diagonal term already)
        const float dg = (valid && !w2_add) ? diag[n1 + d] : 0.f;
#pragma unroll
        for (int j = 0; j < NH; ++j) {
          const int c = cbeg + j;
          w2[j] = w2_add ? ((valid && c < mcols) ? W[(int64_t)c * ldw + n1 + d] : 0.f) : dg * v2[j];
        }
        // segment A: sum_k A[row, k] V[(a', k), c].  The lanes of a warp with
        // the same a' (most of them: a' changes once per run of nv - 1 - a'
        // rows) share one cooperative load of those V values, spread over
        // the lanes (k fastest: coalesced) and broadcast by shuffles.
        if (seg_a) {
          constexpr unsigned FULL = 0xffffffffu;
          constexpr int NVL = (NH * UMMA_NOP + 31) / 32;
          unsigned pending = __ballot_sync(FULL, valid);
          while (pending) {
            const int apg = __shfl_sync(FULL, ap, __ffs(pending) - 1);
            const bool mine = valid && ap == apg;
            pending &= ~__ballot_sync(FULL, mine);
            float vc[NVL];
#pragma unroll
            for (int i = 0; i < NVL; ++i) {
              const int idx = lane + 32 * i;            // idx = j * UMMA_NOP + k
              const int j = idx / UMMA_NOP, k = idx - j * UMMA_NOP;
              const int c = cbeg + j;
              vc[i] = (j < NH && k < no && c < mcols) ? __ldg(V + (int64_t)c * ldv + (int64_t)apg * no + k) : 0.f;
            }
#pragma unroll
            for (int k = 0; k < UMMA_NOP; ++k) {
              if (k >= no) break;
              const float a = mine ? sa[k] : 0.f;
#pragma unroll
              for (int j = 0; j < NH; ++j) {
                const int idx = j * UMMA_NOP + k;
                w2[j] = fmaf(a, __shfl_sync(FULL, vc[idx / 32], idx % 32), w2[j]);
              }
            }
          }
        }
        const bool valid_t = valid;
        const int64_t d_t = d;
        // this tile's products are done: the V2 buffer takes the next tile
        // (so its products overlap this tile's epilogue), then D1 is read
        ok = mbar_wait(&bars[B_D1FULL0 + db], (tile >> 1) & 1u, err, 9);
        ok = ok && mbar_wait(&bars[B_V2EMPTY], ((tile + 1) & 1u) ^ 1u, err, 8);
        if (!ok) break;
        fence_after_sync();
        if (has_next) store_v2(v2n);
#pragma unroll
        for (int j0 = 0; j0 < NH; j0 += 8) {
          float hi[8], lo[8];
          tmem_ld8(tD1[db] + lane_off + (uint32_t)(cbeg + j0), hi);
          tmem_ld8(tD1[db] + lane_off + (uint32_t)(NP + cbeg + j0), lo);
          if (XS == 3) {
            float lo2[8];
            tmem_ld8(tD1[db] + lane_off + (uint32_t)(2 * NP + cbeg + j0), lo2);
#pragma unroll
            for (int j = 0; j < 8; ++j) lo[j] += lo2[j];
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int c = cbeg + j0 + j;
            if (valid_t && c < mcols) W[(int64_t)c * ldw + n1 + d_t] = w2[j0 + j] + (hi[j] + lo[j]);
          }
        }
        fence_before_sync();
        mbar_arrive(&bars[B_D1EMPTY0 + db]);
#pragma unroll
        for (int j = 0; j < NH; ++j) v2[j] = v2n[j];
        ap = apn;
        d = dn;
        valid = validn;
      }
      if (!ok) break;
      // the item's W1 (C|D) sums: TMEM lane = position k in group s
      ok = mbar_wait(&bars[B_D2FULL], nitem & 1u, err, 10);
      if (!ok) break;
      fence_after_sync();
      for (int s = 0; s < nslot; ++s) {
        const int k = 128 * s + r;
        const int seg = k / nvP, a = k - seg * nvP;
        const bool kv = k < K && a < nv;
        const int64_t single = (int64_t)a * no + (seg ? lp : kp);
#pragma unroll
        for (int j0 = 0; j0 < NH; j0 += 8) {
          float hi[8], lo[8];
          tmem_ld8(tD2 + (uint32_t)s * N2 + lane_off + (uint32_t)(cbeg + j0), hi);
          tmem_ld8(tD2 + (uint32_t)s * N2 + lane_off + (uint32_t)(NP + cbeg + j0), lo);
          if (XS == 3) {
            float lo2[8];
            tmem_ld8(tD2 + (uint32_t)s * N2 + lane_off + (uint32_t)(2 * NP + cbeg + j0), lo2);
#pragma unroll
            for (int j = 0; j < 8; ++j) lo[j] += lo2[j];
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int c = cbeg + j0 + j;
            const float v = hi[j] + lo[j];
            if (kv && c < mcols && v != 0.f) atomicAdd(&W1[(int64_t)c * ld1 + single], (double)v);
          }
        }
      }
      fence_before_sync();
      mbar_arrive(&bars[B_D2EMPTY]);
    }
  }
  // every role is done (or gave up): release TMEM
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0) {
    tmem_dealloc(tbase, TCOLS);
    tmem_relinquish();
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct UmmaPlan {
  UmmaMaps maps;
  const void* maps_for = nullptr;   // the B^T array the maps describe
  const void* slices_for = nullptr; // the mid slice array the slice maps describe (FP32-value pass)
  int2* d_items = nullptr;          // tensor-core work items (row ranges inside one slab)
  int nitems = 0;
  int2* d_items_s = nullptr;        // short items (UMMA_ITEM_ROWS_SHORT rows): the FP32-value main pass
  int nitems_s = 0;
  int2* d_runs = nullptr;           // pass-3 runs: (first row, rows) of equal a' in one slab
  int nruns = 0;
  int* d_err = nullptr;             // device error word of the kernel's bounded waits
  int* h_err = nullptr;             // pinned host copy
  int item_rows = UMMA_ITEM_ROWS_DEFAULT;
};

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  }
  return fn;
}

template <int NP, int XS>
size_t umma_smem_bytes(int nslot) {
  return 1024 + (size_t)(UMMA_MAX_BOXES + 2) * umma_box_bytes(NP, XS) + (size_t)nslot * UMMA_SLOT_BYTES +
         (size_t)(B_SLOT0 + 2 * nslot) * 8 + 16;
}

template <int NP, int VS, int XS>
int launch_umma_np(Ctx* c, UmmaPlan* u, const float* V, int64_t ldv, int m, float* W, int64_t ldw, double* W1,
                   int64_t ld1, int seg_a, int vbase = 0, int w2_add = 0, bool short_items = false) {
  const int2* items = short_items ? u->d_items_s : u->d_items;
  const int nitems = short_items ? u->nitems_s : u->nitems;
  const int smax = smem_optin_max(c);
  int nslot = umma_nslot<NP, XS>(smax);
  nslot = std::min(nslot, (VS == 1 && XS == 2) ? 6 : 4);
  if (nslot < 2) return set_err(c, ADCGPU_UNSUPPORTED, "tensor-core sigma pass: shared memory too small");
  const size_t smem = umma_smem_bytes<NP, XS>(nslot);
  if (smem > (size_t)smax) return set_err(c, ADCGPU_UNSUPPORTED, "tensor-core sigma pass: shared memory too small");
  const GeomDev g = to_dev(c->geom);
  const int grid = std::max(1, std::min(nitems, c->nsm));
  auto go = [&](auto kern) -> int {
    ADC_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smax));
    kern<<<grid, UMMA_THREADS, smem, c->stream>>>(g, items, nitems, u->maps,
                                                  (const __nv_bfloat16*)c->d_Bt16, c->d_diag32, V, ldv, m, W, ldw, W1,
                                                  ld1, seg_a, vbase, w2_add, u->d_err);
    ADC_COUNT_LAUNCH();
    ADC_CUDA(c, cudaGetLastError());
    return ADCGPU_OK;
  };
  if constexpr (VS == 1 && XS == 2) {
    switch (nslot) {
      case 2: return go(k_sigma_umma<NP, 2, VS, XS>);
      case 3: return go(k_sigma_umma<NP, 3, VS, XS>);
      case 4: return go(k_sigma_umma<NP, 4, VS, XS>);
      case 5: return go(k_sigma_umma<NP, 5, VS, XS>);
      default: return go(k_sigma_umma<NP, 6, VS, XS>);
    }
  } else {
    switch (nslot) {
      case 2: return go(k_sigma_umma<NP, 2, VS, XS>);
      case 3: return go(k_sigma_umma<NP, 3, VS, XS>);
      default: return go(k_sigma_umma<NP, 4, VS, XS>);
    }
  }
}

}  // namespace

bool umma_supported(const Ctx* c) {
  const Geometry& G = c->geom;
  int major = 0;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, c->device) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  // segment A in registers (noP <= 24), C|D of at most six 64-value boxes
  return major >= 10 && umma_geometry_ok(G) && c->d_Bt16 != nullptr && encode_fn() != nullptr;
}

bool umma_geometry_ok(const Geometry& G) {
  return G.noP <= UMMA_NOP && 2 * G.nvP <= UMMA_MAX_BOXES * UMMA_BOX && G.no >= 2 && G.nv >= 2;
}

bool umma3_supported(const Ctx* c) {
  return umma_supported(c) && c->d_Bt16s[0] != nullptr && c->d_Bt16s[1] != nullptr;
}

void umma_free(Ctx* c, void*& handle) {
  UmmaPlan* u = reinterpret_cast<UmmaPlan*>(handle);
  if (!u) return;
  dfree(c, u->d_items);
  dfree(c, u->d_items_s);
  dfree(c, u->d_runs);
  dfree(c, u->d_err);
  if (u->h_err) cudaFreeHost(u->h_err);
  delete u;
  handle = nullptr;
}

// Work items, pass-3 runs and the tensor maps of the BF16 B^T values.
int umma_prepare(Ctx* c, void*& handle, int item_rows) {
  if (handle && reinterpret_cast<UmmaPlan*>(handle)->maps_for == c->d_Bt16 &&
      reinterpret_cast<UmmaPlan*>(handle)->slices_for == c->d_Bt16s[0] &&
      reinterpret_cast<UmmaPlan*>(handle)->item_rows == item_rows)
    return ADCGPU_OK;
  umma_free(c, handle);
  const Geometry& G = c->geom;
  UmmaPlan* u = new UmmaPlan;
  handle = u;
  u->item_rows = item_rows;
  std::vector<int2> items, items_s, runs;
  for (int cls = 0; cls < 5; ++cls) {
    const int64_t r0 = G.start[cls], r1 = G.start[cls + 1], sl = G.slab_len(cls);
    const bool twoa = (cls == 1 || cls >= 3);
    for (int64_t s0 = r0; s0 < r1; s0 += sl) {
      const int64_t npc = (sl + item_rows - 1) / item_rows, per = (sl + npc - 1) / npc;
      for (int64_t a = s0; a < s0 + sl; a += per)
        items.push_back(make_int2((int)a, (int)std::min<int64_t>(a + per, s0 + sl)));
      const int64_t npcs = (sl + UMMA_ITEM_ROWS_SHORT - 1) / UMMA_ITEM_ROWS_SHORT, pers = (sl + npcs - 1) / npcs;
      for (int64_t a = s0; a < s0 + sl; a += pers)
        items_s.push_back(make_int2((int)a, (int)std::min<int64_t>(a + pers, s0 + sl)));
      if (twoa) {
        for (int ap = 0; ap + 1 < G.nv; ++ap)
          runs.push_back(make_int2((int)(s0 + pair_index(ap, ap + 1, G.nv)), G.nv - 1 - ap));
      } else {
        for (int a = 0; a < G.nv; ++a) runs.push_back(make_int2((int)(s0 + a), 1));
      }
    }
  }
  int st;
  if ((st = dmalloc(c, (void**)&u->d_items, sizeof(int2) * items.size()))) return st;
  if ((st = dmalloc(c, (void**)&u->d_items_s, sizeof(int2) * items_s.size()))) return st;
  ADC_CUDA(c, h2d(c, u->d_items_s, items_s.data(), sizeof(int2) * items_s.size()));
  u->nitems_s = (int)items_s.size();
  if ((st = dmalloc(c, (void**)&u->d_runs, sizeof(int2) * runs.size()))) return st;
  if ((st = dmalloc(c, (void**)&u->d_err, sizeof(int)))) return st;
  ADC_CUDA(c, cudaMallocHost((void**)&u->h_err, sizeof(int)));
  ADC_CUDA(c, h2d(c, u->d_items, items.data(), sizeof(int2) * items.size()));
  ADC_CUDA(c, h2d(c, u->d_runs, runs.data(), sizeof(int2) * runs.size()));
  ADC_CUDA(c, cudaMemsetAsync(u->d_err, 0, sizeof(int), c->stream));
  u->nitems = (int)items.size();
  u->nruns = (int)runs.size();
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return set_err(c, ADCGPU_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  // slice 0: the BF16 store; slices 1, 2: the mid and lo BF16 slices of the
  // FP32 values (when the matrix has them)
  const uint16_t* arrays[3] = {c->d_Bt16, c->d_Bt16s[0], c->d_Bt16s[1]};
  std::memset(&u->maps, 0, sizeof(UmmaMaps));
  for (int v = 0; v < 3; ++v) {
    if (!arrays[v]) continue;
    for (int cls = 0; cls < 5; ++cls) {
      const int64_t rows = G.start[cls + 1] - G.start[cls];
      if (rows <= 0) continue;
      void* basep = (void*)((const __nv_bfloat16*)arrays[v] + G.off[cls]);
      cuuint64_t gdim[2] = {(cuuint64_t)G.len[cls], (cuuint64_t)rows};
      cuuint64_t gstr[1] = {(cuuint64_t)G.len[cls] * 2};
      cuuint32_t box[2] = {UMMA_BOX, UMMA_ROWS};
      cuuint32_t es[2] = {1, 1};
      CUresult r = enc(&u->maps.m[v][cls], CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, basep, gdim, gstr, box, es,
                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (r != CUDA_SUCCESS)
        return set_err(c, ADCGPU_CUDA_ERROR, "cuTensorMapEncodeTiled failed for class " + std::to_string(cls));
    }
  }
  u->maps_for = c->d_Bt16;
  u->slices_for = c->d_Bt16s[0];
  return ADCGPU_OK;
}

int umma_runs(void* handle, const int2** runs, int* nruns) {
  UmmaPlan* u = reinterpret_cast<UmmaPlan*>(handle);
  if (!u) return ADCGPU_NO_MATRIX;
  *runs = u->d_runs;
  *nruns = u->nruns;
  return ADCGPU_OK;
}

// The C|D products and, when seg_a is set, the W2 part of segment A for
// m <= 48 columns (otherwise segment A is left to the compact A/B kernels of
// sigma_ab.cu).
int umma_launch(Ctx* c, void* handle, const float* V, int64_t ldv, int m, float* W, int64_t ldw, double* W1,
                int64_t ld1, int seg_a) {
  UmmaPlan* u = reinterpret_cast<UmmaPlan*>(handle);
  if (!u || m <= 0 || m > 48) return set_err(c, ADCGPU_BAD_INPUT, "tensor-core sigma pass: columns");
  if (m <= 16) return launch_umma_np<16, 1, 2>(c, u, V, ldv, m, W, ldw, W1, ld1, seg_a);
  if (m <= 32) return launch_umma_np<32, 1, 2>(c, u, V, ldv, m, W, ldw, W1, ld1, seg_a);
  return launch_umma_np<48, 1, 2>(c, u, V, ldv, m, W, ldw, W1, ld1, seg_a);
}

// The C|D products of the FP32-value matrix for m <= 32 columns, in two
// passes whose TMEM sums stay short: (1) the BF16 store (the leading 8 bits
// of each value) against the vectors as three BF16 slices, over short work
// items, storing W2 with the diagonal term; (2) the mid and lo value slices
// (2^-9 of the value and below) against the vectors as hi | lo, adding to
// W2.  The second pass's accumulation error is relative to its small
// products.  Segments A and B are left to the compact kernels.
int umma3_launch(Ctx* c, void* handle, const float* V, int64_t ldv, int m, float* W, int64_t ldw, double* W1,
                 int64_t ld1) {
  UmmaPlan* u = reinterpret_cast<UmmaPlan*>(handle);
  if (!u || m <= 0 || m > 32) return set_err(c, ADCGPU_BAD_INPUT, "tensor-core FP32-value sigma pass: columns");
  if (!u->slices_for) return set_err(c, ADCGPU_UNSUPPORTED, "tensor-core FP32-value sigma pass: no value slices");
  if (m <= 16) {
    ST((launch_umma_np<16, 1, 3>(c, u, V, ldv, m, W, ldw, W1, ld1, 0, 0, 0, true)));
    return launch_umma_np<16, 2, 2>(c, u, V, ldv, m, W, ldw, W1, ld1, 0, 1, 1, false);
  }
  ST((launch_umma_np<32, 1, 3>(c, u, V, ldv, m, W, ldw, W1, ld1, 0, 0, 0, true)));
  return launch_umma_np<32, 2, 2>(c, u, V, ldv, m, W, ldw, W1, ld1, 0, 1, 1, false);
}

// Reads the kernel's error word (waits for the stream) and clears it.
int umma_check(Ctx* c, void* handle) {
  UmmaPlan* u = reinterpret_cast<UmmaPlan*>(handle);
  if (!u) return ADCGPU_OK;
  ADC_CUDA(c, cudaMemcpyAsync(u->h_err, u->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  if (*u->h_err) {
    const int code = *u->h_err;
    ADC_CUDA(c, cudaMemsetAsync(u->d_err, 0, sizeof(int), c->stream));
    return set_err(c, ADCGPU_DEVICE_TIMEOUT, "tensor-core sigma pass: a pipeline wait timed out (stage " +
                                          std::to_string(code) + ")");
  }
  return ADCGPU_OK;
}

}  // namespace adcgpu
