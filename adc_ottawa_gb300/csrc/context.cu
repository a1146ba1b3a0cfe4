// Context management, integral upload and the builder / sigma entry points
// of the C ABI (include/adcgpu.h).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cmath>

#include "internal.h"

namespace adcgpu {

std::atomic<unsigned long long> g_kernel_launches{0};

int smem_optin_max(Ctx* c) {
  static std::atomic<int> cached[64];
  const int dev = (c && c->device >= 0 && c->device < 64) ? c->device : 0;
  int v = cached[dev].load();
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0) {
      cudaGetLastError();
      v = 48 * 1024;
    }
    cached[dev].store(v);
  }
  return v;
}

int set_err(Ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int dmalloc(Ctx* c, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    char buf[160];
    snprintf(buf, sizeof buf, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    return set_err(c, e == cudaErrorMemoryAllocation ? ADCGPU_OUT_OF_MEMORY : ADCGPU_CUDA_ERROR, buf);
  }
  c->dev_bytes += (int64_t)bytes;
  c->dev_allocs[*p] = bytes;
  return ADCGPU_OK;
}

void dfree(Ctx* c, void* p, size_t) {
  if (!p) return;
  cudaFree(p);
  if (!c) return;
  auto it = c->dev_allocs.find(p);
  if (it != c->dev_allocs.end()) {
    c->dev_bytes -= (int64_t)it->second;
    c->dev_allocs.erase(it);
  }
}

static void join_diag_order(Ctx* c) {
  if (c->diag_order_thread.joinable()) c->diag_order_thread.join();
}

const std::vector<int64_t>& diag_order(Ctx* c) {
  join_diag_order(c);
  return c->diag_order;
}

static void free_matrix(Ctx* c) {
  join_diag_order(c);
  c->diag_order.clear();
  void** ps[] = {(void**)&c->d_diag, (void**)&c->d_A, (void**)&c->d_Bt, (void**)&c->d_A32, (void**)&c->d_Bt16,
                 (void**)&c->d_Bt32, (void**)&c->d_diag32, (void**)&c->d_rowcount, &c->d_ws,
                 (void**)&c->d_Bt16s[0], (void**)&c->d_Bt16s[1]};
  for (void** p : ps) {
    dfree(c, *p);
    *p = nullptr;
  }
  c->ws_bytes = 0;
  free_sigma_plan(c);
  free_cvs(c);
  c->have_matrix = false;
  c->direct = 0;
  c->dchunks.clear();
}

static void free_eri(Ctx* c) {
  double** ps[] = {&c->d_vovo, &c->d_vvoo, &c->d_ooov, &c->d_vvov, &c->d_oooo, &c->d_vvvv};
  for (double** p : ps) {
    dfree(c, *p);
    *p = nullptr;
  }
  c->have_eri = false;
}

}  // namespace adcgpu

using namespace adcgpu;

#define CTX_CHECK(ctx)                     \
  do {                                     \
    if (!(ctx)) return ADCGPU_BAD_INPUT;   \
    cudaSetDevice((ctx)->device);          \
  } while (0)

extern "C" {

int adcgpu_ctx_create(int device, adcgpu_ctx** out) {
  if (!out) return ADCGPU_BAD_INPUT;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return ADCGPU_CUDA_ERROR;
  }
  if (device < 0 || device >= ndev) return ADCGPU_BAD_INPUT;
  if (cudaSetDevice(device) != cudaSuccess) return ADCGPU_CUDA_ERROR;
  Ctx* c = new Ctx;
  c->device = device;
  // grids are sized in multiples of the streaming-multiprocessor count
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && nsm > 0) c->nsm = nsm;
  else cudaGetLastError();
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
    delete c;
    return ADCGPU_CUDA_ERROR;
  }
  *out = reinterpret_cast<adcgpu_ctx*>(c);
  return ADCGPU_OK;
}

int adcgpu_ctx_destroy(adcgpu_ctx* h) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return ADCGPU_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_matrix(c);
  free_eri(c);
  free_mlp(c);
  gram_free(c);
  dfree(c, c->d_e);
  dfree(c, c->d_sil);
  dfree(c, c->d_dpl);
  cudaEventDestroy(c->ev0);
  cudaEventDestroy(c->ev1);
  if (c->st_ev0) cudaEventDestroy(c->st_ev0);
  if (c->st_ev1) cudaEventDestroy(c->st_ev1);
  cudaStreamDestroy(c->stream);
  delete c;
  return ADCGPU_OK;
}

const char* adcgpu_last_error(const adcgpu_ctx* h) {
  const Ctx* c = reinterpret_cast<const Ctx*>(h);
  return c ? c->err.c_str() : "null context";
}

int adcgpu_set_orbitals(adcgpu_ctx* h, int nocc, int nvirt, const double* e) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  CTX_CHECK(c);
  if (nocc <= 0 || nvirt <= 1 || nocc > 32 || nvirt > 256 || !e)
    return set_err(c, ADCGPU_BAD_INPUT, "nocc in [1,32], nvirt in [2,256] and e required");
  Geometry g;
  g.init(nocc, nvirt);
  if (g.N > INT32_MAX) return set_err(c, ADCGPU_UNSUPPORTED, "ADC(2) dimension exceeds int32 kpq indexing");
  free_matrix(c);
  free_eri(c);
  dfree(c, c->d_dpl);
  c->d_dpl = nullptr;
  c->geom = g;
  c->e.assign(e, e + nocc + nvirt);
  dfree(c, c->d_e);
  c->d_e = nullptr;
  int st = dmalloc(c, (void**)&c->d_e, sizeof(double) * (nocc + nvirt));
  if (st) return st;
  ADC_CUDA(c, h2d(c, c->d_e, e, sizeof(double) * (nocc + nvirt)));
  c->have_orb = true;
  return ADCGPU_OK;
}

int adcgpu_set_eri_packed(adcgpu_ctx* h, const double* eri) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  CTX_CHECK(c);
  if (!c->have_orb) return set_err(c, ADCGPU_BAD_INPUT, "set orbitals first");
  if (!eri) return set_err(c, ADCGPU_BAD_INPUT, "null eri");
  free_eri(c);
  const int nbas = c->geom.no + c->geom.nv;
  const int64_t n = adcgpu_eri_packed_size(nbas);
  double* d_packed = nullptr;
  int st = dmalloc(c, (void**)&d_packed, sizeof(double) * n);
  if (st) return st;
  ADC_CUDA(c, cudaMemcpyAsync(d_packed, eri, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  st = build_eri_blocks_from_packed(c, d_packed);
  dfree(c, d_packed, sizeof(double) * n);
  if (st) return st;
  c->have_eri = true;
  return ADCGPU_OK;
}

int adcgpu_set_eri_mo_complex(adcgpu_ctx* h, const double* buf) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  CTX_CHECK(c);
  if (!c->have_orb) return set_err(c, ADCGPU_BAD_INPUT, "set orbitals first");
  if (!buf) return set_err(c, ADCGPU_BAD_INPUT, "null buffer");
  free_eri(c);
  const int no = c->geom.no, nv = c->geom.nv;
  const int64_t n = no + nv;
  // Real part of buffer_real(r,s,u,v), column-major complex (vpqrsmod.f90:24)
  auto V = [&](int64_t r, int64_t s, int64_t u, int64_t v) {
    return buf[2 * (((v * n + u) * n + s) * n + r)];
  };
  const int64_t npv = (int64_t)nv * (nv + 1) / 2;
  const int64_t sz[6] = {(int64_t)nv * no * nv * no, (int64_t)nv * nv * no * no, (int64_t)no * no * no * nv,
                         (int64_t)nv * nv * no * nv, (int64_t)no * no * no * no, npv * (npv + 1) / 2};
  double** dst[6] = {&c->d_vovo, &c->d_vvoo, &c->d_ooov, &c->d_vvov, &c->d_oooo, &c->d_vvvv};
  // (P, Q), P >= Q, of the triangular index t = P(P+1)/2 + Q
  auto untri = [](int64_t t, int64_t& P, int64_t& Q) {
    P = (int64_t)((std::sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (P * (P + 1) / 2 > t) --P;
    while ((P + 1) * (P + 2) / 2 <= t) ++P;
    Q = t - P * (P + 1) / 2;
  };
  for (int k = 0; k < 6; ++k) {
    std::vector<double> hb(sz[k]);
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < sz[k]; ++t) {
      int64_t x = t;
      int64_t p, q, r, s;
      switch (k) {
        case 4: { int64_t l = x % no; x /= no; int64_t kk = x % no; x /= no; int64_t j = x % no; int64_t i = x / no;
                  p = i; q = j; r = kk; s = l; } break;
        case 5: { int64_t P, Q, a, cc, b, d;
                  untri(x, P, Q); untri(P, a, cc); untri(Q, b, d);
                  p = no + a; q = no + cc; r = no + b; s = no + d; } break;
        case 0: { int64_t j = x % no; x /= no; int64_t b = x % nv; x /= nv; int64_t i = x % no; int64_t a = x / no;
                  p = no + a; q = i; r = no + b; s = j; } break;
        case 1: { int64_t j = x % no; x /= no; int64_t i = x % no; x /= no; int64_t b = x % nv; int64_t a = x / nv;
                  p = no + a; q = no + b; r = i; s = j; } break;
        case 2: { int64_t a = x % nv; x /= nv; int64_t kk = x % no; x /= no; int64_t j = x % no; int64_t i = x / no;
                  p = i; q = j; r = kk; s = no + a; } break;
        default: { int64_t cc = x % nv; x /= nv; int64_t i = x % no; x /= no; int64_t b = x % nv; int64_t a = x / nv;
                   p = no + a; q = no + b; r = i; s = no + cc; } break;
      }
      hb[t] = V(p, q, r, s);
    }
    int st = dmalloc(c, (void**)dst[k], sizeof(double) * sz[k]);
    if (st) return st;
    ADC_CUDA(c, h2d(c, *dst[k], hb.data(), sizeof(double) * sz[k]));
  }
  c->have_eri = true;
  return ADCGPU_OK;
}

int adcgpu_build_adc2s(adcgpu_ctx* h, int ndim, const int32_t* kpq, int64_t* noffd_out, char flag, int precision) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  CTX_CHECK(c);
  if (!c->have_orb || !c->have_eri) return set_err(c, ADCGPU_BAD_INPUT, "orbitals and ERIs must be set");
  if (ndim != c->geom.N) return set_err(c, ADCGPU_BAD_INPUT, "ndim does not match nocc/nvirt");
  if (precision != ADCGPU_FP64 && precision != ADCGPU_MIXED && precision != ADCGPU_DIRECT)
    return set_err(c, ADCGPU_BAD_INPUT, "precision");
  if (kpq) {
    std::vector<int32_t> ref((size_t)7 * (ndim + 1));
    adcgpu_select_adc2s(c->geom.no, c->geom.nv, ref.data());
    for (size_t i = 0; i < ref.size(); ++i)
      if (ref[i] != kpq[i] && !(i >= 5 && i < 7))
        return set_err(c, ADCGPU_UNSUPPORTED,
                       "kpq is not the C1 ADC(2)-s list of select_atom_is/select_atom_d (flag -1)");
  }
  free_matrix(c);
  c->direct = precision == ADCGPU_DIRECT ? 1 : 0;
  int st = build_matrix(c);
  if (st) return st;
  st = prepare_desc(c);
  if (st) return st;
  // the direct path multiplies in FP64 like the stored FP64 path
  c->precision = precision == ADCGPU_DIRECT ? ADCGPU_FP64 : precision;
  if (precision == ADCGPU_MIXED) {
    st = prepare_mixed(c);
    if (st) return st;
  }
  ADC_CUDA(c, cudaStreamSynchronize(c->stream));
  {
    // the guess selection order of |hii| (initvec_ondiag), sorted on a host
    // thread while the caller goes on (it depends only on the diagonal)
    std::vector<double> ah((size_t)c->geom.N);
    ADC_CUDA(c, d2h(c, ah.data(), c->d_diag, sizeof(double) * ah.size()));
    c->diag_order_thread = std::thread([c, ah = std::move(ah)]() mutable {
      for (double& x : ah) x = std::fabs(x);
      host_heapsort_index((int64_t)ah.size(), ah.data(), c->diag_order);
    });
  }
  c->flag = flag;
  c->have_matrix = true;
  if (noffd_out) *noffd_out = c->nnz_kept;
  return ADCGPU_OK;
}

int adcgpu_set_dipole(adcgpu_ctx* h, const double* dpl) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  CTX_CHECK(c);
  if (!c->have_orb) return set_err(c, ADCGPU_BAD_INPUT, "set orbitals first");
  if (!dpl) return set_err(c, ADCGPU_BAD_INPUT, "null dipole matrix");
  const int64_t nb = c->geom.no + c->geom.nv;
  if (!c->d_dpl) ST(dmalloc(c, (void**)&c->d_dpl, sizeof(double) * nb * nb));
  ADC_CUDA(c, h2d(c, c->d_dpl, dpl, sizeof(double) * nb * nb));
  return ADCGPU_OK;
}

int adcgpu_modified_tm_adc2(adcgpu_ctx* h, int ndim, const int32_t* kpq, double* mtm) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  CTX_CHECK(c);
  if (!c->have_orb || !c->have_eri) return set_err(c, ADCGPU_BAD_INPUT, "orbitals and ERIs must be set");
  if (!c->d_dpl) return set_err(c, ADCGPU_BAD_INPUT, "set the dipole matrix first (adcgpu_set_dipole)");
  if (!mtm) return set_err(c, ADCGPU_BAD_INPUT, "null mtm");
  if (ndim == c->geom.N) {
    std::vector<int32_t> ref((size_t)7 * (ndim + 1));
    adcgpu_select_adc2s(c->geom.no, c->geom.nv, ref.data());
    if (kpq) {
      for (size_t i = 0; i < ref.size(); ++i)
        if (ref[i] != kpq[i] && !(i >= 5 && i < 7))
          return set_err(c, ADCGPU_UNSUPPORTED,
                         "kpq is not the C1 ADC(2)-s list of select_atom_is/select_atom_d (flag -1)");
    }
    return modified_tm_adc2(c, ndim, ref.data(), mtm);
  }
  // a CVS list: its core orbitals are the holes of its singles
  if (!kpq || kpq[1] != 0 || kpq[2] != 0 || kpq[0] <= 0 || kpq[0] % c->geom.nv != 0)
    return set_err(c, ADCGPU_BAD_INPUT, "ndim matches neither the ADC(2)-s nor a CVS list (kpq required)");
  std::vector<int32_t> core;
  for (int i = 1; i <= kpq[0] / c->geom.nv; ++i) core.push_back(kpq[7 * i + 2]);
  int32_t cnt[5];
  if (adcgpu_cvs_dim(c->geom.no, c->geom.nv, (int)core.size(), core.data(), cnt) != ndim)
    return set_err(c, ADCGPU_BAD_INPUT, "ndim does not match the CVS list");
  std::vector<int32_t> ref((size_t)7 * (ndim + 1));
  adcgpu_select_adc2s_cvs(c->geom.no, c->geom.nv, (int)core.size(), core.data(), ref.data());
  for (size_t i = 0; i < ref.size(); ++i)
    if (ref[i] != kpq[i] && !(i >= 5 && i < 7))
      return set_err(c, ADCGPU_UNSUPPORTED, "kpq is not a C1 CVS list of select_atom_is_cvs/select_atom_d_cvs");
  return modified_tm_adc2(c, ndim, ref.data(), mtm);
}

int adcgpu_build_adc2s_cvs(adcgpu_ctx* h, int ndim, const int32_t* kpq, int ncore, const int32_t* core,
                           int64_t* noffd_out, char flag) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  CTX_CHECK(c);
  if (!c->have_orb || !c->have_eri) return set_err(c, ADCGPU_BAD_INPUT, "orbitals and ERIs must be set");
  int32_t cnt[5];
  const int64_t nd = adcgpu_cvs_dim(c->geom.no, c->geom.nv, ncore, core, cnt);
  if (nd <= 0) return set_err(c, ADCGPU_BAD_INPUT, "core: 0 < ncore < nocc distinct occupied orbitals (1-based)");
  if (ndim != nd) return set_err(c, ADCGPU_BAD_INPUT, "ndim does not match the CVS space of the core orbitals");
  std::vector<int32_t> ref((size_t)7 * (ndim + 1));
  if (adcgpu_select_adc2s_cvs(c->geom.no, c->geom.nv, ncore, core, ref.data()) != ADCGPU_OK)
    return set_err(c, ADCGPU_BAD_INPUT, "CVS configuration list");
  if (kpq) {
    for (size_t i = 0; i < ref.size(); ++i)
      if (ref[i] != kpq[i] && !(i >= 5 && i < 7))
        return set_err(c, ADCGPU_UNSUPPORTED,
                       "kpq is not the C1 CVS list of select_atom_is_cvs/select_atom_d_cvs for these core orbitals");
  }
  free_matrix(c);
  int st = build_matrix_cvs(c, ref.data(), ndim, ncore, core);
  if (st) { free_matrix(c); return st; }
  c->cvs = 1;
  c->cvs_kpq = std::move(ref);
  c->precision = ADCGPU_FP64;
  {
    std::vector<double> ah((size_t)ndim);
    ADC_CUDA(c, d2h(c, ah.data(), c->d_diag, sizeof(double) * ah.size()));
    c->diag_order_thread = std::thread([c, ah = std::move(ah)]() mutable {
      for (double& x : ah) x = std::fabs(x);
      host_heapsort_index((int64_t)ah.size(), ah.data(), c->diag_order);
    });
  }
  c->flag = flag;
  c->have_matrix = true;
  if (noffd_out) *noffd_out = c->nnz_kept;
  return ADCGPU_OK;
}

int adcgpu_get_diag(adcgpu_ctx* h, double* hii) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  CTX_CHECK(c);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "no matrix");
  ADC_CUDA(c, d2h(c, hii, c->d_diag, sizeof(double) * mat_dim(c)));
  return ADCGPU_OK;
}

int adcgpu_export_coo(adcgpu_ctx* h, int64_t cap, double* hv, int32_t* oi, int32_t* oj) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  CTX_CHECK(c);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "no matrix");
  if (c->direct) return set_err(c, ADCGPU_UNSUPPORTED, "the direct path stores no coupling block");
  if (cap < c->nnz_kept || !hv || !oi || !oj) return set_err(c, ADCGPU_BAD_INPUT, "cap < noffd");
  const int64_t n = c->nnz_kept;
  double* d_h = nullptr;
  int32_t *d_i = nullptr, *d_j = nullptr;
  int st;
  if ((st = dmalloc(c, (void**)&d_h, sizeof(double) * n))) return st;
  if ((st = dmalloc(c, (void**)&d_i, sizeof(int32_t) * n))) { dfree(c, d_h, sizeof(double) * n); return st; }
  if ((st = dmalloc(c, (void**)&d_j, sizeof(int32_t) * n))) {
    dfree(c, d_h, sizeof(double) * n); dfree(c, d_i, sizeof(int32_t) * n); return st;
  }
  st = c->cvs ? export_coo_cvs(c, d_h, d_i, d_j) : export_coo_device(c, d_h, d_i, d_j);
  if (!st) {
    d2h(c, hv, d_h, sizeof(double) * n);
    d2h(c, oi, d_i, sizeof(int32_t) * n);
    cudaError_t e = d2h(c, oj, d_j, sizeof(int32_t) * n);
    if (e != cudaSuccess) st = set_err(c, ADCGPU_CUDA_ERROR, cudaGetErrorString(e));
  }
  dfree(c, d_h, sizeof(double) * n);
  dfree(c, d_i, sizeof(int32_t) * n);
  dfree(c, d_j, sizeof(int32_t) * n);
  return st;
}

// Fortran unformatted sequential record: 4-byte length, payload, 4-byte length.
static bool write_record(FILE* f, const void* const* parts, const size_t* sizes, int nparts) {
  size_t total = 0;
  for (int i = 0; i < nparts; ++i) total += sizes[i];
  if (total > 0x7FFFFFFFu) return false;
  int32_t len = (int32_t)total;
  if (fwrite(&len, 4, 1, f) != 1) return false;
  for (int i = 0; i < nparts; ++i)
    if (sizes[i] && fwrite(parts[i], 1, sizes[i], f) != sizes[i]) return false;
  return fwrite(&len, 4, 1, f) == 1;
}

int adcgpu_write_hmlt_files(adcgpu_ctx* h, const char* dir, char flag) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  CTX_CHECK(c);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "no matrix");
  if (c->direct) return set_err(c, ADCGPU_UNSUPPORTED, "the direct path stores no coupling block");
  const int64_t n = c->nnz_kept, N = mat_dim(c);
  std::vector<double> hv(n), diag(N);
  std::vector<int32_t> oi(n), oj(n);
  int st = adcgpu_export_coo(h, n, hv.data(), oi.data(), oj.data());
  if (st) return st;
  if ((st = adcgpu_get_diag(h, diag.data()))) return st;
  std::string base = std::string(dir ? dir : ".") + "/hmlt.";
  // hmlt.off<flag>: records of buf_size triples + nlim (filetools.f90:36-44);
  // the last record may be incomplete (get_matrix.f90:1124-1126).
  std::string offname = base + "off" + flag;
  FILE* f = fopen(offname.c_str(), "wb");
  if (!f) return set_err(c, ADCGPU_BAD_INPUT, "cannot open " + offname);
  std::vector<double> bh(BUF_SIZE);
  std::vector<int32_t> bi(BUF_SIZE), bj(BUF_SIZE);
  int32_t nrec = 0;
  for (int64_t k0 = 0;; k0 += BUF_SIZE) {
    int64_t nlim64 = std::min<int64_t>(BUF_SIZE, n - k0);
    if (nlim64 < 0) nlim64 = 0;
    std::fill(bh.begin(), bh.end(), 0.0);
    std::fill(bi.begin(), bi.end(), 0);
    std::fill(bj.begin(), bj.end(), 0);
    std::copy(hv.begin() + k0, hv.begin() + k0 + nlim64, bh.begin());
    std::copy(oi.begin() + k0, oi.begin() + k0 + nlim64, bi.begin());
    std::copy(oj.begin() + k0, oj.begin() + k0 + nlim64, bj.begin());
    int32_t nlim = (int32_t)nlim64;
    const void* parts[4] = {bh.data(), bi.data(), bj.data(), &nlim};
    size_t sizes[4] = {sizeof(double) * BUF_SIZE, sizeof(int32_t) * BUF_SIZE, sizeof(int32_t) * BUF_SIZE, 4};
    if (!write_record(f, parts, sizes, 4)) { fclose(f); return set_err(c, ADCGPU_BAD_INPUT, "write failed"); }
    ++nrec;
    if (nlim64 < BUF_SIZE) break;
  }
  fclose(f);
  // hmlt.dia<flag>: (buf_size, nbuf) then hii(ndim) (filetools.f90:24-34)
  std::string dianame = base + "dia" + flag;
  f = fopen(dianame.c_str(), "wb");
  if (!f) return set_err(c, ADCGPU_BAD_INPUT, "cannot open " + dianame);
  int32_t hdr[2] = {BUF_SIZE, nrec};
  const void* p1[1] = {hdr};
  size_t s1[1] = {8};
  const void* p2[1] = {diag.data()};
  size_t s2[1] = {sizeof(double) * (size_t)N};
  bool ok = write_record(f, p1, s1, 1) && write_record(f, p2, s2, 1);
  fclose(f);
  if (!ok) return set_err(c, ADCGPU_BAD_INPUT, "write failed");
  return ADCGPU_OK;
}

int adcgpu_sigma_device(adcgpu_ctx* h, int m, const void* dv, void* dw, int64_t ld) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  CTX_CHECK(c);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "no matrix");
  if (m <= 0 || ld < mat_dim(c) || !dv || !dw) return set_err(c, ADCGPU_BAD_INPUT, "sigma arguments");
  ADC_CUDA(c, cudaEventRecord(c->ev0, c->stream));
  int st = c->precision == ADCGPU_MIXED
               ? sigma_fp32(c, m, (const float*)dv, ld, (float*)dw, ld)
               : sigma_fp64(c, m, (const double*)dv, ld, (double*)dw, ld);
  if (st) return st;
  ADC_CUDA(c, cudaEventRecord(c->ev1, c->stream));
  ADC_CUDA(c, cudaEventSynchronize(c->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->last_sigma_ms = ms;
  return ADCGPU_OK;
}

int adcgpu_sigma(adcgpu_ctx* h, int m, const double* v, double* w) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  CTX_CHECK(c);
  if (!c->have_matrix) return set_err(c, ADCGPU_NO_MATRIX, "no matrix");
  if (m <= 0 || !v || !w) return set_err(c, ADCGPU_BAD_INPUT, "sigma arguments");
  const int64_t N = mat_dim(c);
  const size_t n = (size_t)N * m;
  int st;
  if (c->precision == ADCGPU_FP64) {
    double *dv = nullptr, *dw = nullptr;
    if ((st = dmalloc(c, (void**)&dv, sizeof(double) * n))) return st;
    if ((st = dmalloc(c, (void**)&dw, sizeof(double) * n))) { dfree(c, dv, sizeof(double) * n); return st; }
    ADC_CUDA(c, cudaMemcpyAsync(dv, v, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    st = adcgpu_sigma_device(h, m, dv, dw, N);
    if (!st) ADC_CUDA(c, d2h(c, w, dw, sizeof(double) * n));
    dfree(c, dv, sizeof(double) * n);
    dfree(c, dw, sizeof(double) * n);
    return st;
  }
  // mixed: host FP64 in/out, FP32 on the device
  std::vector<float> hv(n);
  for (size_t i = 0; i < n; ++i) hv[i] = (float)v[i];
  float *dv = nullptr, *dw = nullptr;
  if ((st = dmalloc(c, (void**)&dv, sizeof(float) * n))) return st;
  if ((st = dmalloc(c, (void**)&dw, sizeof(float) * n))) { dfree(c, dv, sizeof(float) * n); return st; }
  ADC_CUDA(c, h2d(c, dv, hv.data(), sizeof(float) * n));
  st = adcgpu_sigma_device(h, m, dv, dw, N);
  if (!st) {
    ADC_CUDA(c, d2h(c, hv.data(), dw, sizeof(float) * n));
    for (size_t i = 0; i < n; ++i) w[i] = hv[i];
  }
  dfree(c, dv, sizeof(float) * n);
  dfree(c, dw, sizeof(float) * n);
  return st;
}

double adcgpu_last_sigma_ms(const adcgpu_ctx* h) {
  const Ctx* c = reinterpret_cast<const Ctx*>(h);
  return c ? c->last_sigma_ms : 0.0;
}

int64_t adcgpu_device_bytes(const adcgpu_ctx* h) {
  const Ctx* c = reinterpret_cast<const Ctx*>(h);
  return c ? c->dev_bytes : 0;
}

int adcgpu_set_fp64_arith(adcgpu_ctx* h, int mode) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c) return ADCGPU_BAD_INPUT;
  if (mode != 0 && mode != 1) return set_err(c, ADCGPU_BAD_INPUT, "fp64 arithmetic mode is 0 or 1");
  c->dense_df = mode;
  return ADCGPU_OK;
}

uint64_t adcgpu_kernel_launches(void) { return adcgpu::g_kernel_launches.load(); }

}  // extern "C"
