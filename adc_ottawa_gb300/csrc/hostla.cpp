// Small dense FP64 linear algebra on the host, standing in for the LAPACK
// calls of the reference's solvers on subspace-sized matrices (dsyev in
// diagrmat block_davidson.f90:991 and initvec_subdiag :400; dsbev in
// diagmat_banded block_lanczos.f90:2041; dsteqr in SILStep sillib.f90:355).
//
// Symmetric eigenproblem, in the formulation of Golub and Van Loan (Matrix
// Computations, 4th ed.): Householder reduction to tridiagonal form by
// symmetric rank-2 updates (Alg. 8.3.1, with the Householder vector of
// Alg. 5.1.1), then the implicit symmetric QR iteration with a Wilkinson
// shift, each step a chase of one Givens bulge down the unreduced block
// (Alg. 8.3.2/8.3.3), eigenvectors accumulated from the rotations.  These
// matrices are at most a few thousand wide; the O(N) tall-skinny work that
// forms them runs on the GPU.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

namespace adcgpu {

namespace {

// Householder vector of x[0..m): v[0] = 1 and beta with
// (I - beta v v^T) x = mu e_0, mu = ||x|| (beta = 0 and mu = x[0] when x is
// already a multiple of e_0).
double house(int m, const double* x, double* v, double* mu) {
  double sigma = 0.0;
  for (int i = 1; i < m; ++i) sigma += x[i] * x[i];
  v[0] = 1.0;
  for (int i = 1; i < m; ++i) v[i] = x[i];
  if (sigma == 0.0) { *mu = x[0]; return 0.0; }
  const double norm = std::sqrt(x[0] * x[0] + sigma);
  // v0 = x0 - ||x||, written without cancellation when x0 > 0
  const double v0 = x[0] <= 0.0 ? x[0] - norm : -sigma / (x[0] + norm);
  for (int i = 1; i < m; ++i) v[i] /= v0;
  *mu = norm;
  return 2.0 * v0 * v0 / (sigma + v0 * v0);
}

// A (n x n column-major, full symmetric, overwritten) = Q T Q^T with T
// tridiagonal: diagonal d[0..n), sub-diagonal e[0..n-1).  With Q != null
// the orthogonal Q (n x n column-major) is formed.
void tridiagonalise(int n, double* A, double* d, double* e, double* Q) {
  auto a = [&](int i, int j) -> double& { return A[(size_t)j * n + i]; };
  std::vector<double> V((size_t)n * n, 0.0), beta(n, 0.0), p(n), w(n);
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1;
    double* v = &V[(size_t)k * n];
    double mu;
    beta[k] = house(m, &a(k + 1, k), v, &mu);
    d[k] = a(k, k);
    e[k] = mu;
    const double bk = beta[k];
    if (bk == 0.0) continue;
    // p = beta A22 v; w = p - (beta p^T v / 2) v; A22 -= v w^T + w v^T
    for (int i = 0; i < m; ++i) p[i] = 0.0;
    for (int j = 0; j < m; ++j) {
      const double vj = v[j];
      const double* col = &a(k + 1, k + 1 + j);
      for (int i = 0; i < m; ++i) p[i] += col[i] * vj;
    }
    double pv = 0.0;
    for (int i = 0; i < m; ++i) { p[i] *= bk; pv += p[i] * v[i]; }
    const double K = 0.5 * bk * pv;
    for (int i = 0; i < m; ++i) w[i] = p[i] - K * v[i];
    for (int j = 0; j < m; ++j) {
      double* col = &a(k + 1, k + 1 + j);
      const double vj = v[j], wj = w[j];
      for (int i = 0; i < m; ++i) col[i] -= v[i] * wj + w[i] * vj;
    }
  }
  if (n >= 2) {
    d[n - 2] = a(n - 2, n - 2);
    e[n - 2] = a(n - 1, n - 2);
  }
  d[n - 1] = a(n - 1, n - 1);
  if (!Q) return;
  // Q = H_0 H_1 ... H_{n-3}, accumulated from the right end
  std::memset(Q, 0, sizeof(double) * (size_t)n * n);
  for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;
  for (int k = n - 3; k >= 0; --k) {
    const double bk = beta[k];
    if (bk == 0.0) continue;
    const int m = n - k - 1;
    const double* v = &V[(size_t)k * n];
    for (int j = k + 1; j < n; ++j) {
      double* col = &Q[(size_t)j * n + k + 1];
      double s = 0.0;
      for (int i = 0; i < m; ++i) s += v[i] * col[i];
      s *= bk;
      for (int i = 0; i < m; ++i) col[i] -= s * v[i];
    }
  }
}

// Eigenvalues of the symmetric tridiagonal (d, e) in place (d, unsorted);
// with Z != null (n x n column-major, holding the basis the tridiagonal is
// expressed in) the rotations are applied to its columns, so column i ends
// as the eigenvector of d[i].  False if the iteration did not converge.
bool tridiagonal_qr(int n, double* d, double* e, double* Z) {
  int sweeps = 0;
  int q = n - 1;
  while (q > 0) {
    for (int i = 0; i < q; ++i)
      if (std::fabs(e[i]) <= DBL_EPSILON * (std::fabs(d[i]) + std::fabs(d[i + 1])) || std::fabs(e[i]) < DBL_MIN)
        e[i] = 0.0;
    while (q > 0 && e[q - 1] == 0.0) --q;
    if (q == 0) break;
    int p = q - 1;
    while (p > 0 && e[p - 1] != 0.0) --p;
    if (++sweeps > 30 * n) return false;
    // Wilkinson shift from the trailing 2 x 2 of the block [p, q]
    const double half = 0.5 * (d[q - 1] - d[q]), bq = e[q - 1];
    const double mu = d[q] - bq * bq / (half + std::copysign(std::hypot(half, bq), half));
    double x = d[p] - mu, z = e[p];
    for (int k = p; k < q; ++k) {
      const double r = std::hypot(x, z);
      const double c = r == 0.0 ? 1.0 : x / r, s = r == 0.0 ? 0.0 : z / r;
      if (k > p) e[k - 1] = r;
      const double ak = d[k], ak1 = d[k + 1], bk = e[k];
      d[k] = c * c * ak + 2.0 * c * s * bk + s * s * ak1;
      d[k + 1] = s * s * ak - 2.0 * c * s * bk + c * c * ak1;
      e[k] = c * s * (ak1 - ak) + (c * c - s * s) * bk;
      if (k + 1 < q) {
        z = s * e[k + 1];          // the bulge at (k + 2, k)
        e[k + 1] *= c;
        x = e[k];
      }
      if (Z) {
        double* zk = Z + (size_t)k * n;
        double* zk1 = Z + (size_t)(k + 1) * n;
        for (int i = 0; i < n; ++i) {
          const double u = zk[i], t = zk1[i];
          zk[i] = c * u + s * t;
          zk1[i] = c * t - s * u;
        }
      }
    }
  }
  return true;
}

}  // namespace

bool host_syev(int n, const double* A, int lda, double* w, double* V) {
  if (n <= 0) return true;
  std::vector<double> a((size_t)n * n), d(n), e(std::max(n - 1, 1), 0.0), Z;
  // full symmetric copy from the upper triangle of column-major A
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= j; ++i) {
      const double x = A[(size_t)j * lda + i];
      a[(size_t)j * n + i] = x;
      a[(size_t)i * n + j] = x;
    }
  if (V) Z.resize((size_t)n * n);
  tridiagonalise(n, a.data(), d.data(), e.data(), V ? Z.data() : nullptr);
  if (!tridiagonal_qr(n, d.data(), e.data(), V ? Z.data() : nullptr)) return false;
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
  for (int c = 0; c < n; ++c) {
    w[c] = d[idx[c]];
    if (V) std::memcpy(V + (size_t)c * n, &Z[(size_t)idx[c] * n], sizeof(double) * n);
  }
  return true;
}

// Eigenvalues of a symmetric band matrix (bandwidth kd, the lower band of
// column-major A is read), as dsbev('N') in diagmat_banded
// (block_lanczos.f90:2006-2052): the band is reduced to tridiagonal form by
// Givens rotations, one bandwidth at a time, each fill-in element chased
// down the band (the band-reduction scheme of Rutishauser and Schwarz), in
// O(n^2 kd) operations; the implicit symmetric QR iteration then gives the
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
  std::vector<double> d(n), e(std::max(n - 1, 1), 0.0);
  for (int i = 0; i < n; ++i) d[i] = Z(i, i);
  for (int i = 0; i + 1 < n; ++i) e[i] = Z(i + 1, i);
  if (!tridiagonal_qr(n, d.data(), e.data(), nullptr)) return false;
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
