// Small dense FP64 linear algebra on the host, standing in for the LAPACK
// calls of the reference's solvers on subspace-sized matrices (dsyev in
// diagrmat block_davidson.f90:991 and initvec_subdiag :400; dsbev in
// diagmat_banded block_lanczos.f90:2041; dsteqr in SILStep sillib.f90:355).
//
// Symmetric eigenproblem: Householder reduction to tridiagonal form followed
// by the implicit QL iteration with Wilkinson shifts (the classical
// tred2/tql2 pair of the EISPACK literature), written here for column-major
// storage.  These matrices are at most a few thousand wide; the O(N)
// tall-skinny work that forms them runs on the GPU.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

namespace adcgpu {

namespace {

// Reduce symmetric a (n x n, row-major view z[i][j] = a(i,j)) to tridiagonal
// form; on exit z holds the orthogonal transformation, d the diagonal and
// e the sub-diagonal (e[0] = 0).
void tred2(int n, std::vector<double>& z, std::vector<double>& d, std::vector<double>& e) {
  auto Z = [&](int i, int j) -> double& { return z[(size_t)i * n + j]; };
  for (int i = n - 1; i > 0; --i) {
    int l = i - 1;
    double h = 0.0, scale = 0.0;
    if (l > 0) {
      for (int k = 0; k <= l; ++k) scale += std::fabs(Z(i, k));
      if (scale == 0.0) {
        e[i] = Z(i, l);
      } else {
        for (int k = 0; k <= l; ++k) { Z(i, k) /= scale; h += Z(i, k) * Z(i, k); }
        double f = Z(i, l);
        double g = f >= 0.0 ? -std::sqrt(h) : std::sqrt(h);
        e[i] = scale * g;
        h -= f * g;
        Z(i, l) = f - g;
        f = 0.0;
        for (int j = 0; j <= l; ++j) {
          Z(j, i) = Z(i, j) / h;
          g = 0.0;
          for (int k = 0; k <= j; ++k) g += Z(j, k) * Z(i, k);
          for (int k = j + 1; k <= l; ++k) g += Z(k, j) * Z(i, k);
          e[j] = g / h;
          f += e[j] * Z(i, j);
        }
        double hh = f / (h + h);
        for (int j = 0; j <= l; ++j) {
          f = Z(i, j);
          e[j] = g = e[j] - hh * f;
          for (int k = 0; k <= j; ++k) Z(j, k) -= (f * e[k] + g * Z(i, k));
        }
      }
    } else {
      e[i] = Z(i, l);
    }
    d[i] = h;
  }
  d[0] = 0.0;
  e[0] = 0.0;
  for (int i = 0; i < n; ++i) {
    int l = i - 1;
    if (d[i] != 0.0) {
      for (int j = 0; j <= l; ++j) {
        double g = 0.0;
        for (int k = 0; k <= l; ++k) g += Z(i, k) * Z(k, j);
        for (int k = 0; k <= l; ++k) Z(k, j) -= g * Z(k, i);
      }
    }
    d[i] = Z(i, i);
    Z(i, i) = 1.0;
    for (int j = 0; j <= l; ++j) Z(j, i) = Z(i, j) = 0.0;
  }
}

// Implicit QL on the tridiagonal (d, e); accumulates into z (row-major).
bool tql2(int n, std::vector<double>& d, std::vector<double>& e, std::vector<double>* z) {
  for (int i = 1; i < n; ++i) e[i - 1] = e[i];
  if (n > 0) e[n - 1] = 0.0;
  for (int l = 0; l < n; ++l) {
    int iter = 0, m;
    do {
      for (m = l; m < n - 1; ++m) {
        double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= 1e-300 || std::fabs(e[m]) + dd == dd) break;
      }
      if (m != l) {
        if (iter++ == 60) return false;
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        double r = std::hypot(g, 1.0);
        g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? std::fabs(r) : -std::fabs(r)));
        double s = 1.0, c = 1.0, p = 0.0;
        int i;
        for (i = m - 1; i >= l; --i) {
          double f = s * e[i], b = c * e[i];
          e[i + 1] = (r = std::hypot(f, g));
          if (r == 0.0) { d[i + 1] -= p; e[m] = 0.0; break; }
          s = f / r; c = g / r;
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0 * c * b;
          d[i + 1] = g + (p = s * r);
          g = c * r - b;
          if (z) {
            for (int k = 0; k < n; ++k) {
              double& zk1 = (*z)[(size_t)k * n + i + 1];
              double& zk = (*z)[(size_t)k * n + i];
              f = zk1;
              zk1 = s * zk + c * f;
              zk = c * zk - s * f;
            }
          }
        }
        if (r == 0.0 && i >= l) continue;
        d[l] -= p; e[l] = g; e[m] = 0.0;
      }
    } while (m != l);
  }
  return true;
}

}  // namespace

bool host_syev(int n, const double* A, int lda, double* w, double* V) {
  if (n <= 0) return true;
  std::vector<double> z((size_t)n * n), d(n), e(n);
  // row-major z[i][j] = A(i,j) from the upper triangle of column-major A
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= j; ++i) {
      double x = A[(size_t)j * lda + i];
      z[(size_t)i * n + j] = x;
      z[(size_t)j * n + i] = x;
    }
  tred2(n, z, d, e);
  if (!tql2(n, d, e, V ? &z : nullptr)) return false;
  // sort ascending; eigenvector k is column k of z (row-major z[i][k])
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
  for (int c = 0; c < n; ++c) {
    w[c] = d[idx[c]];
    if (V)
      for (int r = 0; r < n; ++r) V[(size_t)c * n + r] = z[(size_t)r * n + idx[c]];
  }
  return true;
}

// Eigenvalues of a symmetric band matrix (bandwidth kd, the lower band of
// column-major A is read), as dsbev('N') in diagmat_banded
// (block_lanczos.f90:2006-2052): the band is reduced to tridiagonal form by
// Givens rotations, one bandwidth at a time, each fill-in element chased
// down the band (the band-reduction scheme of Rutishauser and Schwarz), in
// O(n^2 kd) operations; the implicit QL iteration then gives the
// eigenvalues in O(n^2).
bool host_sbev_values(int n, int kd, const double* A, int lda, double* w) {
  if (n <= 0) return true;
  kd = std::max(0, std::min(kd, n - 1));
  // row-major symmetric working copy of the band (+ one bulge diagonal)
  std::vector<double> z((size_t)n * n, 0.0);
  auto Z = [&](int i, int j) -> double& { return z[(size_t)i * n + j]; };
  for (int j = 0; j < n; ++j)
    for (int i = j; i < std::min(n, j + kd + 1); ++i) {
      const double x = A[(size_t)j * lda + i];
      Z(i, j) = x;
      Z(j, i) = x;
    }
  for (int b = kd; b >= 2; --b) {
    for (int j = 0; j + b < n; ++j) {
      int p = j + b, col = j;
      while (p < n) {
        const double x = Z(p - 1, col), y = Z(p, col);
        if (y != 0.0) {
          const double r = std::hypot(x, y), c = x / r, s = y / r;
          // rows/columns p-1 and p: A <- G A G^T, G = [[c, s], [-s, c]]
          const int lo = std::max(0, p - 1 - b - 1), hi = std::min(n - 1, p + b + 1);
          for (int k = lo; k <= hi; ++k) {
            if (k == p - 1 || k == p) continue;
            const double a1 = Z(p - 1, k), a2 = Z(p, k);
            const double n1v = c * a1 + s * a2, n2v = -s * a1 + c * a2;
            Z(p - 1, k) = n1v; Z(k, p - 1) = n1v;
            Z(p, k) = n2v; Z(k, p) = n2v;
          }
          const double a11 = Z(p - 1, p - 1), a12 = Z(p - 1, p), a22 = Z(p, p);
          Z(p - 1, p - 1) = c * c * a11 + 2.0 * c * s * a12 + s * s * a22;
          Z(p, p) = s * s * a11 - 2.0 * c * s * a12 + c * c * a22;
          const double o = c * s * (a22 - a11) + (c * c - s * s) * a12;
          Z(p - 1, p) = o; Z(p, p - 1) = o;
          Z(p, col) = 0.0; Z(col, p) = 0.0;
        }
        // the rotation fills (p + b, p - 1); chase it one band-width down
        col = p - 1;
        p += b;
      }
    }
  }
  std::vector<double> d(n), e(n, 0.0);
  for (int i = 0; i < n; ++i) d[i] = Z(i, i);
  for (int i = 1; i < n; ++i) e[i] = Z(i, i - 1);
  if (!tql2(n, d, e, nullptr)) return false;
  std::sort(d.begin(), d.end());
  std::memcpy(w, d.data(), sizeof(double) * n);
  return true;
}

int host_cholesky_upper(int n, const double* G, double* R, double rel_tol) {
  double dmax = 0.0;
  for (int i = 0; i < n; ++i) dmax = std::max(dmax, std::fabs(G[(size_t)i * n + i]));
  std::memset(R, 0, sizeof(double) * (size_t)n * n);
  for (int j = 0; j < n; ++j) {
    double s = G[(size_t)j * n + j];
    for (int k = 0; k < j; ++k) s -= R[(size_t)j * n + k] * R[(size_t)j * n + k];
    if (!(s > rel_tol * dmax) || s <= 0.0) return j;
    double rjj = std::sqrt(s);
    R[(size_t)j * n + j] = rjj;
    for (int i = j + 1; i < n; ++i) {
      double t = G[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) t -= R[(size_t)j * n + k] * R[(size_t)i * n + k];
      R[(size_t)i * n + j] = t / rjj;   // R(j,i), column-major
    }
  }
  return -1;
}

void host_triu_inverse(int n, const double* R, double* Ri) {
  std::memset(Ri, 0, sizeof(double) * (size_t)n * n);
  for (int j = 0; j < n; ++j) {
    Ri[(size_t)j * n + j] = 1.0 / R[(size_t)j * n + j];
    for (int i = j - 1; i >= 0; --i) {
      double s = 0.0;
      for (int k = i + 1; k <= j; ++k) s += R[(size_t)k * n + i] * Ri[(size_t)j * n + k];
      Ri[(size_t)j * n + i] = -s / R[(size_t)i * n + i];
    }
  }
}

// Numerical Recipes heapsort of an index array, ascending (dsortindxa1 'A').
// The order of equal keys is that of the heap construction, as in the
// reference, because the Davidson guess vectors are taken from it.
void host_heapsort_index(int64_t n, const double* arrin, std::vector<int64_t>& indx) {
  // The keys travel with their indices (one array of pairs), so a sift step
  // reads one location instead of an index and then its key; comparisons and
  // moves are those of the index-array formulation, so the permutation, and
  // the order of ties, is the same.
  struct KI { double key; int64_t idx; };
  indx.resize(n);
  if (n <= 0) return;
  if (n == 1) { indx[0] = 1; return; }
  std::vector<KI> h((size_t)n);
  for (int64_t i = 0; i < n; ++i) h[i] = KI{arrin[i], i + 1};
  int64_t l = n / 2 + 1, ir = n, i, j;
  KI t;
  for (;;) {
    if (l > 1) {
      l = l - 1;
      t = h[l - 1];
    } else {
      t = h[ir - 1];
      h[ir - 1] = h[0];
      ir = ir - 1;
      if (ir == 1) { h[0] = t; break; }
    }
    i = l; j = l + l;
    while (j <= ir) {
      if (j < ir && h[j - 1].key < h[j].key) j = j + 1;
      if (t.key < h[j - 1].key) { h[i - 1] = h[j - 1]; i = j; j = j + j; }
      else j = ir + 1;
    }
    h[i - 1] = t;
  }
  for (int64_t k = 0; k < n; ++k) indx[k] = h[k].idx;
}

}  // namespace adcgpu
