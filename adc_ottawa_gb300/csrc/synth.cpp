// Seeded synthetic ADC(2) system and the ADC(2)-s configuration list.
//
// The synthetic system replaces the GAMESS import and AO->MO transform of the
// reference (source/qclib/load_electronic_structure.f90:153-342): orbital
// energies e(1:nbas), occupied first, and real MO ERIs (pq|rs) with 8-fold
// symmetry.  Every random number comes from a counter-based hash, and every
// floating-point operation is an IEEE basic operation (+ - * / sqrt, no FMA
// contraction), so the arrays are bit-identical on any host that compiles
// this file with -ffp-contract=off.  exp and log are evaluated by the series
// below (own code, from the Taylor / atanh expansions) rather than libm, whose
// last-bit behaviour differs between x86-64 and aarch64.
//
// The configuration list follows select_atom_is (source/adclib/select_fano.f90
// :16-60) and select_atom_d with flag -1 (:539-718) for C1 symmetry and no
// frozen core: the order of configurations and the kpq column layout
// (cnf, spin, j, k, a, b, type) of fill_indices (source/utilities/misc.f90
// :458-471) are kept because the solvers' guess vectors depend on them.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/adcgpu.h"
#include "synth_math.h"

namespace {

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Stream key: one independent stream per (seed, purpose).
inline uint64_t stream_key(uint64_t seed, uint64_t purpose) {
  return splitmix64(splitmix64(seed) ^ (purpose * 0xD1B54A32D192ED03ull));
}

// Uniform double in (0,1): 53 random bits, centred in their cell.
inline double uniform01(uint64_t key, uint64_t counter) {
  uint64_t h = splitmix64(key ^ splitmix64(counter));
  return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

// Standard normal deviate for one counter, Marsaglia's polar method with
// sub-counters for the rejected pairs.
inline double normal01(uint64_t key, uint64_t counter) {
  for (uint64_t t = 0;; ++t) {
    uint64_t c = counter * 64 + 2 * t;
    double u = 2.0 * uniform01(key, c) - 1.0;
    double v = 2.0 * uniform01(key, c + 1) - 1.0;
    double s = u * u + v * v;
    if (s > 0.0 && s < 1.0) {
      double f = adcsynth::sqrt_rn(-2.0 * adcsynth::log_series(s) / s);
      return u * f;
    }
    if (t == 31) return 0.0;  // probability < 1e-20; keeps the loop finite
  }
}

enum : uint64_t { PURPOSE_OCC = 1, PURPOSE_VIRT = 2, PURPOSE_ERI = 3, PURPOSE_BLOCK = 4, PURPOSE_DIPOLE = 5 };

}  // namespace

extern "C" int adcgpu_synth_orbitals(int nocc, int nvirt, uint64_t seed, double* e) {
  if (nocc <= 0 || nvirt <= 0 || !e) return ADCGPU_BAD_INPUT;
  uint64_t ko = stream_key(seed, PURPOSE_OCC), kv = stream_key(seed, PURPOSE_VIRT);
  for (int i = 0; i < nocc; ++i) e[i] = -1.4 + 1.0 * uniform01(ko, (uint64_t)i);
  for (int a = 0; a < nvirt; ++a) e[nocc + a] = 0.1 + 2.9 * uniform01(kv, (uint64_t)a);
  std::sort(e, e + nocc);
  std::sort(e + nocc, e + nocc + nvirt);
  return ADCGPU_OK;
}

extern "C" int64_t adcgpu_eri_packed_size(int nbas) {
  int64_t m = (int64_t)nbas * (nbas + 1) / 2;
  return m * (m + 1) / 2;
}

extern "C" int adcgpu_synth_eri_packed(int nbas, uint64_t seed, double* eri, int nthreads) {
  if (nbas <= 0 || !eri) return ADCGPU_BAD_INPUT;
  const uint64_t key = stream_key(seed, PURPOSE_ERI);
  // exp(-0.15 d1 - 0.15 d2) for d1,d2 in [0,nbas): exponent formed as
  // (-0.15*d1) - (0.15*d2) exactly as written in the generator spec.
  std::vector<double> decay((size_t)nbas * nbas);
  for (int d1 = 0; d1 < nbas; ++d1)
    for (int d2 = 0; d2 < nbas; ++d2)
      decay[(size_t)d1 * nbas + d2] = adcsynth::exp_series(-0.15 * d1 - 0.15 * d2);
  const int64_t M = (int64_t)nbas * (nbas + 1) / 2;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
  for (int64_t PQ = 0; PQ < M; ++PQ) {
    // PQ = p(p+1)/2 + q with p >= q (0-based)
    int p = (int)((std::sqrt(8.0 * (double)PQ + 1.0) - 1.0) / 2.0);
    while ((int64_t)p * (p + 1) / 2 > PQ) --p;
    while ((int64_t)(p + 1) * (p + 2) / 2 <= PQ) ++p;
    int q = (int)(PQ - (int64_t)p * (p + 1) / 2);
    int64_t base = PQ * (PQ + 1) / 2;
    int r = 0, s = 0;
    for (int64_t RS = 0; RS <= PQ; ++RS) {
      // RS walks (r,s) = (0,0),(1,0),(1,1),(2,0),...
      int dr = p > r ? p - r : r - p;
      int ds = q > s ? q - s : s - q;
      int64_t idx = base + RS;
      double z = normal01(key, (uint64_t)idx);
      eri[idx] = z * 0.3 * decay[(size_t)dr * nbas + ds];
      if (s == r) { ++r; s = 0; } else { ++s; }
    }
  }
  return ADCGPU_OK;
}

extern "C" int adcgpu_synth_uniform_block(int64_t nrow, int ncol, uint64_t seed, double* out) {
  if (nrow <= 0 || ncol <= 0 || !out) return ADCGPU_BAD_INPUT;
  const uint64_t key = stream_key(seed, PURPOSE_BLOCK);
  for (int64_t k = 0; k < nrow * (int64_t)ncol; ++k) out[k] = uniform01(key, (uint64_t)k);
  return ADCGPU_OK;
}

extern "C" int adcgpu_synth_dipole(int nbas, uint64_t seed, double* dpl) {
  if (nbas <= 0 || !dpl) return ADCGPU_BAD_INPUT;
  const uint64_t key = stream_key(seed, PURPOSE_DIPOLE);
  for (int p = 0; p < nbas; ++p)
    for (int q = 0; q <= p; ++q) {
      const uint64_t idx = (uint64_t)p * (p + 1) / 2 + q;
      const double x = normal01(key, idx) * 0.5 * adcsynth::exp_series(-0.1 * (p - q));
      dpl[(size_t)q * nbas + p] = x;
      dpl[(size_t)p * nbas + q] = x;
    }
  return ADCGPU_OK;
}

// ---------------------------------------------------------------------------
// kpq
// ---------------------------------------------------------------------------
extern "C" int64_t adcgpu_adc2s_dim(int nocc, int nvirt, int32_t* counts5) {
  if (nocc <= 0 || nvirt <= 0) return -1;
  int64_t no = nocc, nv = nvirt;
  int64_t c1 = no * nv;                     // singles
  int64_t c2 = no * nv;                     // a=b, i=j
  int64_t c3 = nv * (nv - 1) / 2 * no;      // a<b, i=j
  int64_t c4 = no * (no - 1) / 2 * nv;      // a=b, i<j
  int64_t c5 = no * (no - 1) / 2 * (nv * (nv - 1) / 2);  // a<b, i<j (each spin)
  if (counts5) {
    counts5[0] = (int32_t)c1; counts5[1] = (int32_t)c2; counts5[2] = (int32_t)c3;
    counts5[3] = (int32_t)c4; counts5[4] = (int32_t)c5;
  }
  return c1 + c2 + c3 + c4 + 2 * c5;   // adc2_ener.f90:78
}

extern "C" int adcgpu_select_adc2s(int nocc, int nvirt, int32_t* kpq) {
  if (!kpq) return ADCGPU_BAD_INPUT;
  int32_t cnt[5];
  int64_t ndim = adcgpu_adc2s_dim(nocc, nvirt, cnt);
  if (ndim <= 0 || ndim > INT32_MAX) return ADCGPU_BAD_INPUT;
  const int nbas = nocc + nvirt;
  std::memset(kpq, 0, sizeof(int32_t) * 7 * (size_t)(ndim + 1));
  auto put = [&](int64_t col, int cnf, int spin, int a, int b, int j, int k, int type) {
    int32_t* c = kpq + 7 * col;   // fill_indices column layout
    c[0] = cnf; c[1] = spin; c[2] = j; c[3] = k; c[4] = a; c[5] = b; c[6] = type;
  };
  int64_t n = 0;
  // singles: ap outer over virtuals, hole inner (hcentre = 1..nocc)
  for (int a = nocc + 1; a <= nbas; ++a)
    for (int i = 1; i <= nocc; ++i) put(++n, 1, 1, a, -1, i, -1, 0);
  // class 1: a=b, i=j; hole outer
  for (int i = 1; i <= nocc; ++i)
    for (int a = nocc + 1; a <= nbas; ++a) put(++n, 2, 1, a, a, i, i, 1);
  // class 2: a<b, i=j; pair outer, hole inner
  for (int a = nocc + 1; a <= nbas; ++a)
    for (int b = a + 1; b <= nbas; ++b)
      for (int i = 1; i <= nocc; ++i) put(++n, 2, 1, a, b, i, i, 2);
  // class 3: a=b, i<j; hole pair outer, particle inner
  for (int i = 1; i <= nocc; ++i)
    for (int j = i + 1; j <= nocc; ++j)
      for (int a = nocc + 1; a <= nbas; ++a) put(++n, 2, 1, a, a, i, j, 3);
  // class 4I: a<b, i<j, spin 11
  int64_t start4 = n;
  for (int i = 1; i <= nocc; ++i)
    for (int j = i + 1; j <= nocc; ++j)
      for (int a = nocc + 1; a <= nbas; ++a)
        for (int b = a + 1; b <= nbas; ++b) put(++n, 2, 11, a, b, i, j, 4);
  // class 4II: copy of 4I with spin 12 and type 5
  for (int64_t t = 1; t <= cnt[4]; ++t) {
    int32_t* src = kpq + 7 * (start4 + t);
    int32_t* dst = kpq + 7 * (start4 + cnt[4] + t);
    std::memcpy(dst, src, 7 * sizeof(int32_t));
    dst[1] = 12; dst[6] = 5;
  }
  n += cnt[4];
  for (int k = 0; k < 5; ++k) kpq[k] = cnt[k];
  return n == ndim ? ADCGPU_OK : ADCGPU_BAD_INPUT;
}

// ---------------------------------------------------------------------------
// CVS kpq: select_atom_is_cvs (select_fano.f90:112-142) and select_atom_d_cvs
// (:903-1027) for C1 symmetry, no frozen orbitals, hcentre = 1..nocc.  core
// lists the core orbitals (icore, 1-based occupied indices).  Singles: ap
// outer, core hole inner (in hcentre order).  Doubles: classes 3 (a=b, i<j)
// and 4I/4II (a<b, i<j) whose hole pair holds exactly one core orbital; no
// i=j classes.
// ---------------------------------------------------------------------------
static bool cvs_mask(int nocc, int ncore, const int32_t* core, std::vector<char>& is_core) {
  if (ncore <= 0 || ncore >= nocc || !core) return false;
  is_core.assign(nocc + 1, 0);
  for (int i = 0; i < ncore; ++i) {
    if (core[i] < 1 || core[i] > nocc || is_core[core[i]]) return false;
    is_core[core[i]] = 1;
  }
  return true;
}

extern "C" int64_t adcgpu_cvs_dim(int nocc, int nvirt, int ncore, const int32_t* core, int32_t* counts5) {
  std::vector<char> ic;
  if (nocc <= 0 || nvirt <= 1 || !cvs_mask(nocc, ncore, core, ic)) return -1;
  int64_t pairs = (int64_t)ncore * (nocc - ncore);   // hole pairs with exactly one core orbital
  int64_t c1 = (int64_t)ncore * nvirt;
  int64_t c4 = pairs * nvirt;
  int64_t c5 = pairs * ((int64_t)nvirt * (nvirt - 1) / 2);
  if (counts5) {
    counts5[0] = (int32_t)c1; counts5[1] = 0; counts5[2] = 0;
    counts5[3] = (int32_t)c4; counts5[4] = (int32_t)c5;
  }
  return c1 + c4 + 2 * c5;
}

extern "C" int adcgpu_select_adc2s_cvs(int nocc, int nvirt, int ncore, const int32_t* core, int32_t* kpq) {
  std::vector<char> ic;
  if (!kpq || !cvs_mask(nocc, ncore, core, ic)) return ADCGPU_BAD_INPUT;
  int32_t cnt[5];
  const int64_t ndim = adcgpu_cvs_dim(nocc, nvirt, ncore, core, cnt);
  if (ndim <= 0 || ndim > INT32_MAX) return ADCGPU_BAD_INPUT;
  const int nbas = nocc + nvirt;
  std::memset(kpq, 0, sizeof(int32_t) * 7 * (size_t)(ndim + 1));
  auto put = [&](int64_t col, int cnf, int spin, int a, int b, int j, int k, int type) {
    int32_t* c = kpq + 7 * col;
    c[0] = cnf; c[1] = spin; c[2] = j; c[3] = k; c[4] = a; c[5] = b; c[6] = type;
  };
  int64_t n = 0;
  for (int a = nocc + 1; a <= nbas; ++a)                 // select_atom_is_cvs :124-138
    for (int i = 1; i <= nocc; ++i)
      if (ic[i]) put(++n, 1, 1, a, -1, i, -1, 0);
  for (int i = 1; i <= nocc; ++i)                        // a=b, i|=j, one core hole :937-962
    for (int j = i + 1; j <= nocc; ++j)
      if (ic[i] + ic[j] == 1)
        for (int a = nocc + 1; a <= nbas; ++a) put(++n, 2, 1, a, a, i, j, 3);
  const int64_t start4 = n;
  for (int i = 1; i <= nocc; ++i)                        // a|=b, i|=j spin I :967-1017
    for (int j = i + 1; j <= nocc; ++j)
      if (ic[i] + ic[j] == 1)
        for (int a = nocc + 1; a <= nbas; ++a)
          for (int b = a + 1; b <= nbas; ++b) put(++n, 2, 11, a, b, i, j, 4);
  for (int64_t t = 1; t <= cnt[4]; ++t) {                // spin II copy :1019-1021
    int32_t* src = kpq + 7 * (start4 + t);
    int32_t* dst = kpq + 7 * (start4 + cnt[4] + t);
    std::memcpy(dst, src, 7 * sizeof(int32_t));
    dst[1] = 12; dst[6] = 5;
  }
  n += cnt[4];
  for (int k = 0; k < 5; ++k) kpq[k] = cnt[k];
  return n == ndim ? ADCGPU_OK : ADCGPU_BAD_INPUT;
}
