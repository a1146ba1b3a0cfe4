// Internal declarations of libadcgpu: the device-resident problem, the
// configuration index maps and the layout of the stored matrix.
//
// Stored matrix (ADC(2)-s, C1 symmetry):
//
//     H = | A    B |   A  : n1 x n1 dense ph-ph block (symmetric, FP64)
//         | B^T  D |   B  : n1 x n2 ph-2p2h coupling
//                      D  : diagonal 2p2h block (get_matrix.f90:303-306)
//
// B is stored index-free.  A double d = (a',b',k',l') couples only to singles
// (a,k) with a in {a',b'} or k in {k',l'} (the coincidence tests of
// C1..C5_ph_2p2h, adc_ph.f90:974-1073), so the column pattern of each row of
// B^T is a closed-form function of d.  Each row holds its structural entries
// in a fixed segment order and values with |h| <= minc are stored as 0.0, so
// the matrix equals the reference's thresholded COO exactly while the sigma
// product streams only values (8, 4 or 2 bytes per entry), no indices.
//
//   segment A : singles (a',k), k = 0..no-1           (always)
//   segment B : singles (b',k), k = 0..no-1           (a' != b')
//   segment C : singles (a,k'),  a = 0..nv-1          (0 at a in {a',b'})
//   segment D : singles (a,l'),  a = 0..nv-1          (k' != l'; 0 likewise)
//
// Segments A/B are padded to noP = 8*ceil(no/8) and C/D to nvP = 8*ceil(nv/8)
// entries (zeros), so every segment starts on a 16-byte boundary for BF16
// (and on 32/64 bytes for FP32/FP64) and a lane can fetch 8 consecutive
// values with one vector load.  Row lengths: class 1 (a'=b',k'=l') noP+nvP;
// class 2 (a'<b',k'=l') 2noP+nvP; class 3 (a'=b',k'<l') noP+2nvP; classes
// 4I/4II 2noP+2nvP.  Because C and D cover the full virtual range, the lane
// that owns virtual a always owns single (a,k'): the sigma product
// accumulates B V2 in registers.
//
// Storage order of rows ("slabs" of fixed (k',l')): classes 1, 3, 4I, 4II in
// the kpq order (hole indices outer); class 2 hole-outer (k' outer, pair
// (a'<b') inner), the transpose of its kpq order (pair outer, hole inner).
//
// All indices below are 0-based: occupied i in [0,no), virtual a in [0,nv)
// (orbital no+a), single s = a*no + k (select_atom_is order), doubles in the
// select_atom_d order of select_fano.f90:539-718.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>
#include <atomic>
#include <thread>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/adcgpu.h"

namespace adcgpu {

constexpr double MINC = 1e-12;   // parameters.f90:139
constexpr int BUF_SIZE = 655360; // parameters.f90:425

// ---------------------------------------------------------------------------
// Configuration space geometry.
// ---------------------------------------------------------------------------
struct Geometry {
  int no = 0, nv = 0;
  int noP = 0, nvP = 0;   // segment lengths padded to multiples of 8
  int64_t n1 = 0;         // singles
  int64_t c1 = 0, c2 = 0, c3 = 0, c4 = 0;   // class sizes (4 = each of 4I, 4II)
  int64_t n2 = 0, N = 0;
  int64_t start[6];       // first doubles-local index of class 1,2,3,4I,4II and n2
  int64_t len[5];         // row length of B^T per class (4I and 4II equal)
  int64_t off[6];         // value offset of class c in the B^T store; off[5] = total
  int64_t npair_v = 0, npair_o = 0;   // nv(nv-1)/2, no(no-1)/2

  void init(int no_, int nv_) {
    no = no_; nv = nv_;
    noP = (no + 7) / 8 * 8;
    nvP = (nv + 7) / 8 * 8;
    n1 = (int64_t)no * nv;
    npair_v = (int64_t)nv * (nv - 1) / 2;
    npair_o = (int64_t)no * (no - 1) / 2;
    c1 = (int64_t)no * nv;
    c2 = npair_v * no;
    c3 = npair_o * nv;
    c4 = npair_o * npair_v;
    n2 = c1 + c2 + c3 + 2 * c4;
    N = n1 + n2;
    start[0] = 0; start[1] = c1; start[2] = c1 + c2; start[3] = c1 + c2 + c3;
    start[4] = start[3] + c4; start[5] = n2;
    len[0] = noP + nvP;
    len[1] = 2 * noP + nvP;
    len[2] = noP + 2 * nvP;
    len[3] = 2 * noP + 2 * nvP;
    len[4] = len[3];
    off[0] = 0;
    for (int c = 0; c < 5; ++c) off[c + 1] = off[c] + (start[c + 1] - start[c]) * len[c];
  }
  // rows of one slab (fixed k',l') per class
  int64_t slab_len(int c) const { return (c == 0 || c == 2) ? nv : npair_v; }
};

// Decoded double: virtuals a' <= b', occupied k' <= l', class 0..4.
struct Double {
  int ap, bp, kp, lp, cls;
};

// Index of pair (x<y) among pairs of n items in lexicographic order.
__host__ __device__ inline int64_t pair_index(int x, int y, int n) {
  return (int64_t)x * n - (int64_t)x * (x + 1) / 2 + (y - x - 1);
}

__host__ __device__ inline void pair_decode(int64_t p, int n, int& x, int& y) {
  // invert pair_index: estimate the row from the quadratic (FP32 is enough
  // for an estimate; GB300's FP64 square root is slow), then correct exactly
  const float b = 2.0f * (float)n - 1.0f;
  float disc = b * b - 8.0f * (float)p;
  int xx = (int)((b - sqrtf(disc > 0.0f ? disc : 0.0f)) * 0.5f);
  if (xx < 0) xx = 0;
  if (xx > n - 2) xx = n - 2;
  while (xx > 0 && pair_index(xx, xx + 1, n) > p) --xx;
  while (xx < n - 2 && pair_index(xx + 1, xx + 2, n) <= p) ++xx;
  x = xx;
  y = (int)(p - pair_index(xx, xx + 1, n)) + xx + 1;
}

struct GeomDev {
  int no, nv, noP, nvP;
  int64_t n1, n2, N;
  int64_t start[6];
  int64_t len[5];
  int64_t off[6];
  int64_t npair_v, npair_o;
};

inline GeomDev to_dev(const Geometry& g) {
  GeomDev d;
  d.no = g.no; d.nv = g.nv; d.noP = g.noP; d.nvP = g.nvP; d.n1 = g.n1; d.n2 = g.n2; d.N = g.N;
  for (int i = 0; i < 6; ++i) { d.start[i] = g.start[i]; d.off[i] = g.off[i]; }
  for (int i = 0; i < 5; ++i) d.len[i] = g.len[i];
  d.npair_v = g.npair_v; d.npair_o = g.npair_o;
  return d;
}

// Doubles-local index d in [0,n2) -> configuration, following select_atom_d.
__host__ __device__ inline Double decode_double(const GeomDev& g, int64_t d) {
  Double r;
  if (d < g.start[1]) {                       // class 1: hole outer, particle inner
    r.cls = 0; r.kp = r.lp = (int)(d / g.nv); r.ap = r.bp = (int)(d % g.nv);
  } else if (d < g.start[2]) {                // class 2: pair (a<b) outer, hole inner
    int64_t t = d - g.start[1];
    r.cls = 1; r.kp = r.lp = (int)(t % g.no);
    pair_decode(t / g.no, g.nv, r.ap, r.bp);
  } else if (d < g.start[3]) {                // class 3: hole pair outer, particle inner
    int64_t t = d - g.start[2];
    r.cls = 2; r.ap = r.bp = (int)(t % g.nv);
    pair_decode(t / g.nv, g.no, r.kp, r.lp);
  } else {                                     // classes 4I / 4II
    int64_t t = d - g.start[3];
    r.cls = 3;
    if (t >= g.start[4] - g.start[3]) { t -= g.start[4] - g.start[3]; r.cls = 4; }
    pair_decode(t / g.npair_v, g.no, r.kp, r.lp);
    pair_decode(t % g.npair_v, g.nv, r.ap, r.bp);
  }
  return r;
}

// Storage row -> configuration (storage order described above).
__host__ __device__ inline Double decode_row(const GeomDev& g, int64_t row) {
  if (row >= g.start[1] && row < g.start[2]) {
    int64_t t = row - g.start[1];
    Double r;
    r.cls = 1;
    r.kp = r.lp = (int)(t / g.npair_v);
    pair_decode(t % g.npair_v, g.nv, r.ap, r.bp);
    return r;
  }
  return decode_double(g, row);
}

// Storage row of a configuration -> its doubles-local (kpq) index.
__host__ __device__ inline int64_t row_to_d(const GeomDev& g, const Double& r, int64_t row) {
  if (r.cls == 1) return g.start[1] + pair_index(r.ap, r.bp, g.nv) * g.no + r.kp;
  return row;
}

// Single index of entry e of the B^T row of double r, or -1 for a padding
// position of segments C/D.
__host__ __device__ inline int64_t entry_single(const GeomDev& g, const Double& r, int e) {
  const int no = g.no;
  if (e < g.noP) return e < no ? (int64_t)r.ap * no + e : -1;  // segment A
  e -= g.noP;
  const bool twoa = r.ap != r.bp;
  if (twoa) {
    if (e < g.noP) return e < no ? (int64_t)r.bp * no + e : -1;  // segment B
    e -= g.noP;
  }
  const int seg = e / g.nvP;                                    // 0: C (k'), 1: D (l')
  const int a = e - seg * g.nvP;
  if (a >= g.nv || a == r.ap || a == r.bp) return -1;
  return (int64_t)a * no + (seg == 0 ? r.kp : r.lp);
}

// Chunk of whole slabs of the B^T store (the direct path recomputes the
// coupling values of one chunk at a time): storage rows [row0, row1), values
// [vbase, vbase + vlen), and the ranges of the sigma work lists that cover
// those rows (tiled items, pass-1 chunks, pass-2 items).
struct DirectChunk {
  int64_t row0 = 0, row1 = 0, vbase = 0, vlen = 0;
  int ti0 = 0, ti1 = 0, ch0 = 0, ch1 = 0, it0 = 0, it1 = 0;
};

// Whole slabs grouped in store order into chunks of at most 'budget' values
// (a slab larger than the budget forms a chunk of its own).
inline std::vector<DirectChunk> direct_chunk_rows(const Geometry& G, int64_t budget) {
  std::vector<DirectChunk> out;
  DirectChunk cur;
  bool open = false;
  for (int cls = 0; cls < 5; ++cls) {
    const int64_t sl = G.slab_len(cls), L = G.len[cls];
    for (int64_t s0 = G.start[cls]; s0 < G.start[cls + 1]; s0 += sl) {
      const int64_t v0 = G.off[cls] + (s0 - G.start[cls]) * L, nvals = sl * L;
      if (open && cur.vlen + nvals > budget) { out.push_back(cur); open = false; }
      if (!open) { cur = DirectChunk(); cur.row0 = s0; cur.vbase = v0; open = true; }
      cur.row1 = s0 + sl;
      cur.vlen += nvals;
    }
  }
  if (open) out.push_back(cur);
  return out;
}

// Value budget of a direct-path chunk: at most 2^27 values (1 GiB in FP64)
// and a quarter of the store, never less than the largest slab.
inline int64_t direct_budget(const Geometry& G) {
  int64_t slab = 0;
  for (int cls = 0; cls < 5; ++cls)
    if (G.start[cls + 1] > G.start[cls]) slab = std::max(slab, G.slab_len(cls) * G.len[cls]);
  return std::max(slab, std::min<int64_t>((G.off[5] + 3) / 4, (int64_t)1 << 27));
}

// ---------------------------------------------------------------------------
// Context.
// ---------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

struct Ctx {
  int device = 0;
  int nsm = 152;                  // streaming multiprocessors of the device (queried at creation)
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  Geometry geom;
  bool have_orb = false, have_eri = false, have_matrix = false;
  int precision = ADCGPU_FP64;
  int direct = 0;                 // 1: matrix-free coupling block (d_Bt is one chunk's buffer)
  std::vector<DirectChunk> dchunks;   // its chunks (row and value ranges)
  char flag = 'i';
  std::vector<double> e;          // orbital energies (host copy)
  double* d_e = nullptr;          // device orbital energies [nbas]
  // ERI blocks (0-based, see eri accessors in build_kernels.cu)
  double* d_vovo = nullptr;       // (a i|b j) [nv][no][nv][no]
  double* d_vvoo = nullptr;       // (a b|i j) [nv][nv][no][no]
  double* d_ooov = nullptr;       // (i j|k a) [no][no][no][nv]
  double* d_vvov = nullptr;       // (a b|i c) [nv][nv][no][nv]
  double* d_oooo = nullptr;       // (i j|k l) [no][no][no][no]
  double* d_vvvv = nullptr;       // (a c|b d) over virtual pairs: [tri(pair(a,c), pair(b,d))]
  double* d_dpl = nullptr;        // dipole matrix dpl(p,q) [nbas][nbas] (q-major), adcgpu_set_dipole
  // matrix
  double* d_diag = nullptr;       // hii [N]
  double* d_A = nullptr;          // ph-ph block, n1 x n1 dense symmetric (0 where |h|<=minc)
  double* d_Bt = nullptr;         // structured B^T values (geom.off[5] entries)
  float* d_A32 = nullptr;         // mixed-precision copies
  uint16_t* d_Bt16 = nullptr;     // bf16 bits of B^T values
  float* d_Bt32 = nullptr;        // fp32 B^T values (when bf16 is not safe)
  uint16_t* d_Bt16s[2] = {nullptr, nullptr};   // mid and lo BF16 slices of the fp32 values
                                               // (hi = d_Bt16), for the tcgen05 FP32-value pass
  float* d_diag32 = nullptr;
  int mixed_bf16 = 1;             // 1: B^T stored as bf16, 0: fp32
  int dense_df = 0;               // FP64 GEMMs in double-float on the FP32 pipe
  // heapsort order (1-based, the reference's dsortindxa1 tie order) of |hii|,
  // the initvec_ondiag guess selection: computed on a host thread from the
  // end of the matrix build, joined by the first solve that needs it
  std::vector<int64_t> diag_order;
  std::thread diag_order_thread;
  int64_t nnz_kept = 0;           // reference noffd
  int64_t nnz_ph = 0;             // kept ph-ph entries
  int64_t* d_rowcount = nullptr;  // kept entries per double row (for COO export)
  // sigma work lists (SigmaPlan, sigma.cu)
  void* sigma_plan = nullptr;
  void* d_ws = nullptr;
  size_t ws_bytes = 0;
  double last_sigma_ms = 0.0;
  // sigma statistics (adcgpu_sigma_stats)
  int64_t st_calls = 0, st_cols = 0;
  double st_ms = 0.0, st_bytes = 0.0;
  cudaEvent_t st_ev0 = nullptr, st_ev1 = nullptr;
  bool st_pending = false;
  double st_pending_bytes = 0.0;
  int st_pending_cols = 0;
  int st_pending_kind = 0;        // value store of the pending call: 0 BF16, 1 FP32, 2 FP64
  double st_by[3][4] = {};        // per value store: calls, ms, algorithmic bytes, columns
  int64_t dev_bytes = 0;          // sum of the live dmalloc sizes
  std::unordered_map<void*, size_t> dev_allocs;   // dmalloc pointer -> size
  // learned preconditioner (MlpState, mlp.cu); DPR is used when absent
  void* mlp = nullptr;
  // tensor-core Gram products (GramPlan, dense_umma.cu): error word, switch
  void* gram = nullptr;
  // CVS matrix (write_fspace_adc2_1_cvs): singles on core holes only; the
  // ph-ph block dense (diagonal included), the coupling block as CSR over the
  // doubles rows (kept entries, column = CVS single index)
  int cvs = 0;
  int64_t cvs_n1 = 0, cvs_N = 0, cvs_nnz = 0;
  std::vector<int32_t> cvs_kpq;   // 7 x (cvs_N + 1)
  double* d_Ac = nullptr;         // cvs_n1 x cvs_n1
  int64_t* d_crow = nullptr;      // row offsets, n2 + 1
  int32_t* d_ccol = nullptr;
  double* d_cval = nullptr;
  // SIL persistent state for adcgpu_silstep (device Krylov vectors)
  double* d_sil = nullptr;
  int64_t sil_cap = 0;
};

// Process-wide count of kernels this library has launched (every launch
// site is followed by ADC_COUNT_LAUNCH); read with adcgpu_kernel_launches.
extern std::atomic<unsigned long long> g_kernel_launches;
#define ADC_COUNT_LAUNCH() ::adcgpu::g_kernel_launches.fetch_add(1, std::memory_order_relaxed)

// error helpers
int set_err(Ctx* c, int code, const std::string& msg);
// the device's opt-in maximum of dynamic shared memory per block (cached)
int smem_optin_max(Ctx* c);
// |hii| heapsort order of the built matrix (waits for the build's host thread)
const std::vector<int64_t>& diag_order(Ctx* c);
// propagate a non-zero status
#define ST(x)                 \
  do {                        \
    int _s = (x);             \
    if (_s) return _s;        \
  } while (0)
#define ADC_CUDA(ctx, call)                                                     \
  do {                                                                         \
    cudaError_t _e = (call);                                                   \
    if (_e != cudaSuccess)                                                     \
      return ::adcgpu::set_err((ctx), _e == cudaErrorMemoryAllocation          \
                                         ? ADCGPU_OUT_OF_MEMORY                \
                                         : ADCGPU_CUDA_ERROR,                  \
                               std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// Device allocations of a context: dmalloc records each size, dfree (null is
// a no-op) releases the pointer and subtracts the recorded size, so
// adcgpu_device_bytes reports what the context holds.  dfree's third
// argument is not needed and is ignored.
// Host<->device copies on the context's stream.  The stream is created
// non-blocking, so it is not ordered with the legacy default stream that a
// plain cudaMemcpy uses: a copy there could overtake kernels still queued on
// the context's stream, or be overtaken by them.  Both return when the copy
// has completed (so a caller's buffer, pinned or not, may be reused at once)
// and are ordered after earlier and before later work on the stream.
inline cudaError_t h2d(Ctx* c, void* dst, const void* src, size_t bytes) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
  return e != cudaSuccess ? e : cudaStreamSynchronize(c->stream);
}
inline cudaError_t d2h(Ctx* c, void* dst, const void* src, size_t bytes) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
  return e != cudaSuccess ? e : cudaStreamSynchronize(c->stream);
}

int dmalloc(Ctx* c, void** p, size_t bytes);
void dfree(Ctx* c, void* p, size_t bytes = 0);

// ---------------------------------------------------------------------------
// Kernels launched from other translation units.
// ---------------------------------------------------------------------------
// build_kernels.cu
int build_eri_blocks_from_packed(Ctx* c, const double* d_packed);
int build_matrix(Ctx* c);
// the ADC(1) (TDA) singles matrix, n1 x n1 (d_M: n1 * n1 doubles)
int build_adc1_matrix(Ctx* c, double* d_M);
// coupling values of store rows [row0, row1) into buf, which holds the values
// from offset vbase on; kept-entry counts per row into rowcount (may be null)
int coupling_values(Ctx* c, double* buf, int64_t vbase, int64_t row0, int64_t row1, int64_t* rowcount);
int export_coo_device(Ctx* c, double* d_h, int32_t* d_oi, int32_t* d_oj);

// Dimension and singles count of the matrix the context holds (the CVS
// matrix when one was built, else the ADC(2)-s space of the orbitals).
inline int64_t mat_dim(const Ctx* c) { return c->cvs ? c->cvs_N : c->geom.N; }
inline int64_t mat_n1(const Ctx* c) { return c->cvs ? c->cvs_n1 : c->geom.n1; }

// CVS (build_kernels.cu, cvs.cu): build from a validated CVS kpq (host,
// 7 x (ndim+1)), the FP64 sigma product, the COO export and the release
int build_matrix_cvs(Ctx* c, const int32_t* kpq, int64_t ndim, int ncore, const int32_t* core);
int sigma_cvs(Ctx* c, int m, const double* dV, int64_t ldv, double* dW, int64_t ldw);
int export_coo_cvs(Ctx* c, double* d_h, int32_t* d_oi, int32_t* d_oj);
void free_cvs(Ctx* c);

// fvec.cu : the ADC(2) f-vector (get_modifiedtm_adc2) of the dipole matrix
// d_dpl over kpq columns 1..ndim (an ADC(2)-s or CVS list validated by the
// caller); mtm on the host
int modified_tm_adc2(Ctx* c, int64_t ndim, const int32_t* kpq, double* mtm);

// sigma.cu : W = H V for m columns (column-major, leading dim ld), FP64 or FP32.
struct SigmaPlan {
  int2* d_chunks = nullptr;   // pass 1: [row_begin, row_end) inside one slab
  int2* d_items = nullptr;    // pass 2: (first row of slab, b')
  int nchunks = 0, nitems = 0;
  int chunk = 64;             // rows per pass-1 work item (autotuned)
  int mc_cap[2] = {2, 4};     // columns per pass for FP64 / FP32 vectors (autotuned)
  int staged = 1;             // pass 1 through a cp.async shared-memory ring (autotuned)
  int tiled = 1;              // pass 1 tiled when its shared memory fits (1: tensor cores for
                              // BF16 values, 2: CUDA cores only, 0: per-warp pass 1)
  int2* d_titems = nullptr;   // tiled pass 1: [row_begin, row_end) inside one slab
  int ntitems = 0;
  void* d_acc = nullptr;      // FP64 accumulator of the singles rows (FP32 path)
  size_t acc_bytes = 0;
  void* d_sk = nullptr;       // split-K partials of the FP32 singles block
  size_t sk_bytes = 0;
  void* umma = nullptr;       // tensor-core pass plan (sigma_umma.cu), built on first use
  int umma_item_rows = 4096;  // rows per tensor-core work item (autotuned)
  int umma_off = 0;           // 1: the tensor-core pass is not used
  void* ab = nullptr;         // compact segment-A/B tables (sigma_ab.cu), built on first use
  int ab_off = 0;             // 1: segments A/B through pass 2 / pass 3 instead
  int umma3_on = 0;           // 1: FP32 values on the two tcgen05 passes (BF16 slices)
  std::vector<DirectChunk> dchunks;   // direct path: chunks with their work-list ranges
};
int prepare_desc(Ctx* c);
int build_chunks(Ctx* c, int chunk);
void free_sigma_plan(Ctx* c);
int sigma_fp64(Ctx* c, int m, const double* dV, int64_t ldv, double* dW, int64_t ldw);
int sigma_fp32(Ctx* c, int m, const float* dV, int64_t ldv, float* dW, int64_t ldw);
int prepare_mixed(Ctx* c);
void free_mlp(Ctx* c);
// dense_umma.cu: release the tensor-core Gram state; switch it off (1) or on
void gram_free(Ctx* c);
int gram_set_off(Ctx* c, int off);

// sigma_umma.cu : the tensor-core (tcgen05) pass of the BF16 sigma product
bool umma_supported(const Ctx* c);
int umma_prepare(Ctx* c, void*& handle, int item_rows);
void umma_free(Ctx* c, void*& handle);
int umma_launch(Ctx* c, void* handle, const float* V, int64_t ldv, int m, float* W, int64_t ldw, double* W1,
                int64_t ld1, int seg_a);
int umma_runs(void* handle, const int2** runs, int* nruns);
int umma_check(Ctx* c, void* handle);
bool umma_geometry_ok(const Geometry& G);
bool umma3_supported(const Ctx* c);
int umma3_launch(Ctx* c, void* handle, const float* V, int64_t ldv, int m, float* W, int64_t ldw, double* W1,
                 int64_t ld1);

// sigma_ab.cu : segments A and B of the mixed-precision sigma product in
// compact form (tables copied from the BF16 or FP32 value store on first use)
bool ab_supported(const Ctx* c);
void ab_free(Ctx* c, void*& handle);
void ab_invalidate(void* handle);
template <typename TV>
int ab_launch(Ctx* c, void*& handle, const TV* Bt, bool do_a, const float* V, int64_t ldv, int m, float* W,
              int64_t ldw, double* W1, int64_t ld1);

// hostla.cpp : dense host linear algebra (FP64)
// Symmetric eigen-decomposition (Householder tridiagonalisation + implicit QL).
// A: n x n column-major (upper triangle used); w ascending; V eigenvectors.
bool host_syev(int n, const double* A, int lda, double* w, double* V);
bool host_sbev_values(int n, int kd, const double* A, int lda, double* w);
// Cholesky of SPD G (n x n col-major) -> upper R with G = R^T R; returns the
// first column whose pivot fell below rel_tol * max diag (or -1 on success).
int host_cholesky_upper(int n, const double* G, double* R, double rel_tol);
// Inverse of an upper-triangular n x n matrix.
void host_triu_inverse(int n, const double* R, double* Rinv);
// NR heapsort index (dsortindxa1 'A', misc.f90:492+); indx 1-based.
void host_heapsort_index(int64_t n, const double* arr, std::vector<int64_t>& indx);

}  // namespace adcgpu
