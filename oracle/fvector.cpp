// ORACLE -- test infrastructure only.  Never linked into, imported by or
// called from the product library.  Only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg use it, as the checker.
//
// A CPU FP64 restatement of get_modifiedtm_adc2 (source/adclib/get_moment.f90
// :153-442): the ADC(2) f-vector F_J = <Psi_J|D|Psi_0> of one dipole
// component over the intermediate states of kpq, with the formulas of
// source/adclib/dipole_ph.f90 (F0_ph :24-46, F21_ph..F210_ph :189-656,
// FI_2p2h..FIV1_2p2h :662-846, tauA..tauC :896-1209, FC_ph_new :1213-1242).
// Every loop runs in the reference's order and every expression is written
// in the reference's left-to-right order (-ffp-contract=off), so each entry
// is the reference's value under IEEE FP64.  C1 symmetry: every MT test of
// those loops passes (CHECK_dip = 1), so the tests are not written out.
// roccnum is the identity (occupied orbitals first).
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

struct FvecSystem {
  int no = 0, nv = 0, nbas = 0;
  std::vector<double> e;        // e(1:nbas) at e[1..nbas]
  const double* eri = nullptr;  // canonical 8-fold packed (pq|rs), 0-based
  const double* dpl = nullptr;  // nbas x nbas, column-major
  // vpqrs(r,s,u,v) = (rs|uv), vpqrsmod.f90:13-27; 1-based
  inline double v(int p, int q, int r, int s) const {
    int64_t a = p - 1, b = q - 1, c = r - 1, d = s - 1;
    int64_t pq = a >= b ? a * (a + 1) / 2 + b : b * (b + 1) / 2 + a;
    int64_t rs = c >= d ? c * (c + 1) / 2 + d : d * (d + 1) / 2 + c;
    int64_t idx = pq >= rs ? pq * (pq + 1) / 2 + rs : rs * (rs + 1) / 2 + pq;
    return eri[idx];
  }
  inline double d(int p, int q) const { return dpl[(int64_t)(q - 1) * nbas + (p - 1)]; }
};

// ---- 1h1p terms, dipole_ph.f90 ------------------------------------------

double F0_ph(const FvecSystem& S, int a, int k) {  // :24-46
  double f = 0.0;
  for (int b = S.no + 1; b <= S.nbas; ++b)
    for (int l = 1; l <= S.no; ++l) {
      double e_abkl = S.e[a] + S.e[b] - S.e[k] - S.e[l];
      f = f + S.d(b, l) / e_abkl * (2.0 * S.v(a, k, b, l) - S.v(a, l, b, k));
    }
  return -f;
}

double F25_ph(const FvecSystem& S, int a, int k) {  // :390-428
  double f = 0.0;
  for (int m = 1; m <= S.no; ++m)
    for (int c = S.no + 1; c <= S.nbas; ++c) {
      double e_kmac = S.e[k] + S.e[m] - S.e[a] - S.e[c];
      for (int l = 1; l <= S.no; ++l)
        for (int b = S.no + 1; b <= S.nbas; ++b) {
          double e_lmbc = S.e[l] + S.e[m] - S.e[b] - S.e[c];
          f = f + S.d(m, c) / e_kmac / e_lmbc * (2.0 * S.v(a, k, l, b) - S.v(a, b, l, k)) *
                      (2.0 * S.v(b, l, c, m) - S.v(b, m, c, l));
        }
    }
  return f;
}

double F26_ph(const FvecSystem& S, int a, int k) {  // :432-469
  double f = 0.0;
  for (int m = 1; m <= S.no; ++m)
    for (int c = S.no + 1; c <= S.nbas; ++c) {
      double e_kmac = S.e[k] + S.e[m] - S.e[a] - S.e[c];
      for (int l = 1; l <= S.no; ++l)
        for (int b = S.no + 1; b <= S.nbas; ++b) {
          double e_klab = S.e[k] + S.e[l] - S.e[a] - S.e[b];
          f = f + S.d(m, c) / e_klab / e_kmac * (2.0 * S.v(l, b, c, m) - S.v(l, m, c, b)) *
                      (2.0 * S.v(a, k, b, l) - S.v(a, l, b, k));
        }
    }
  return f;
}

double F27_ph(const FvecSystem& S, int a, int k) {  // :473-513
  double f = 0.0;
  for (int l = 1; l <= S.no; ++l)
    for (int b = S.no + 1; b <= S.nbas; ++b) {
      double e_klab = S.e[k] + S.e[l] - S.e[a] - S.e[b];
      for (int m = 1; m <= S.no; ++m)
        for (int c = S.no + 1; c <= S.nbas; ++c) {
          double e_kmbc = S.e[k] + S.e[m] - S.e[b] - S.e[c];
          f = f - S.d(l, b) / e_klab / e_kmbc *
                      (S.v(a, l, m, c) * (2.0 * S.v(c, m, b, k) - S.v(c, k, b, m)) +
                       S.v(a, c, m, l) * (2.0 * S.v(c, k, b, m) - S.v(c, m, b, k)));
        }
    }
  return f;
}

double F28_ph(const FvecSystem& S, int a, int k) {  // :517-557
  double f = 0.0;
  for (int m = 1; m <= S.no; ++m)
    for (int b = S.no + 1; b <= S.nbas; ++b) {
      double e_kmab = S.e[k] + S.e[m] - S.e[a] - S.e[b];
      for (int l = 1; l <= S.no; ++l)
        for (int c = S.no + 1; c <= S.nbas; ++c) {
          double e_lmac = S.e[l] + S.e[m] - S.e[a] - S.e[c];
          f = f - S.d(m, b) / e_kmab / e_lmac *
                      (S.v(a, m, c, l) * (2.0 * S.v(l, c, b, k) - S.v(l, k, b, c)) +
                       S.v(a, l, c, m) * (2.0 * S.v(l, k, b, c) - S.v(l, c, b, k)));
        }
    }
  return f;
}

double F29_ph(const FvecSystem& S, int a, int k) {  // :561-606
  double f = 0.0;
  for (int b = S.no + 1; b <= S.nbas; ++b)
    for (int l = 1; l <= S.no; ++l) {
      double e_klab = S.e[k] + S.e[l] - S.e[a] - S.e[b];
      for (int c = S.no + 1; c <= S.nbas; ++c) {
        double e_klcd = S.e[k] + S.e[l] - S.e[c] - S.e[c];
        f = f + S.d(l, b) / e_klab / e_klcd * S.v(a, c, b, c) * S.v(c, k, c, l);
        for (int dd = c + 1; dd <= S.nbas; ++dd) {
          e_klcd = S.e[k] + S.e[l] - S.e[c] - S.e[dd];
          f = f + S.d(l, b) / e_klab / e_klcd *
                      (S.v(a, c, b, dd) * (2.0 * S.v(c, k, dd, l) - S.v(c, l, dd, k)) +
                       S.v(a, dd, b, c) * (2.0 * S.v(dd, k, c, l) - S.v(dd, l, c, k)));
        }
      }
    }
  return f;
}

double F210_ph(const FvecSystem& S, int a, int k) {  // :610-656
  double f = 0.0;
  for (int b = S.no + 1; b <= S.nbas; ++b)
    for (int l = 1; l <= S.no; ++l) {
      double e_klab = S.e[k] + S.e[l] - S.e[a] - S.e[b];
      for (int m = 1; m <= S.no; ++m) {
        double e_mnab = S.e[m] + S.e[m] - S.e[a] - S.e[b];
        f = f + S.d(l, b) / e_klab / e_mnab * S.v(a, m, b, m) * S.v(m, k, m, l);
        for (int n = m + 1; n <= S.no; ++n) {
          e_mnab = S.e[m] + S.e[n] - S.e[a] - S.e[b];
          f = f + S.d(l, b) / e_klab / e_mnab *
                      (S.v(a, m, b, n) * (2.0 * S.v(m, k, n, l) - S.v(m, l, n, k)) +
                       S.v(a, n, b, m) * (2.0 * S.v(n, k, m, l) - S.v(n, l, m, k)));
        }
      }
    }
  return f;
}

// ---- intermediates, dipole_ph.f90:896-1242 --------------------------------

double tauA(const FvecSystem& S, int c, int a) {  // :896-935
  double t = 0.0;
  for (int b = S.no + 1; b <= S.nbas; ++b)
    for (int l = 1; l <= S.no; ++l) {
      double e_lmba = 2.0 * S.e[l] - S.e[b] - S.e[a];
      double e_lmbc = 2.0 * S.e[l] - S.e[b] - S.e[c];
      t = t - 0.5 / e_lmba / e_lmbc * S.v(a, l, b, l) * S.v(l, c, l, b);
      for (int m = l + 1; m <= S.no; ++m) {
        e_lmba = S.e[l] + S.e[m] - S.e[b] - S.e[a];
        e_lmbc = S.e[l] + S.e[m] - S.e[b] - S.e[c];
        t = t - 0.5 / e_lmba / e_lmbc *
                    (S.v(a, l, b, m) * (2.0 * S.v(l, c, m, b) - S.v(l, b, m, c)) +
                     S.v(a, m, b, l) * (2.0 * S.v(l, b, m, c) - S.v(l, c, m, b)));
      }
    }
  return t;
}

double tauB(const FvecSystem& S, int m, int k) {  // :939-981
  double t = 0.0;
  for (int l = 1; l <= S.no; ++l)
    for (int b = S.no + 1; b <= S.nbas; ++b) {
      double e_klbc = S.e[k] + S.e[l] - S.e[b] - S.e[b];
      double e_lmbc = S.e[l] + S.e[m] - S.e[b] - S.e[b];
      t = t - 0.5 / e_klbc / e_lmbc * S.v(b, k, b, l) * S.v(m, b, l, b);
      for (int c = b + 1; c <= S.nbas; ++c) {
        e_klbc = S.e[k] + S.e[l] - S.e[b] - S.e[c];
        e_lmbc = S.e[l] + S.e[m] - S.e[b] - S.e[c];
        t = t - 0.5 / e_klbc / e_lmbc *
                    (S.v(b, k, c, l) * (2.0 * S.v(m, b, l, c) - S.v(m, c, l, b)) +
                     S.v(b, l, c, k) * (2.0 * S.v(m, c, l, b) - S.v(m, b, l, c)));
      }
    }
  return t;
}

double tau21(const FvecSystem& S, int a, int m) {  // :985-1029
  double t = 0.0;
  double e_ma = S.e[m] - S.e[a];
  for (int l = 1; l <= S.no; ++l)
    for (int b = S.no + 1; b <= S.nbas; ++b) {
      double e_lmbc = S.e[l] + S.e[m] - S.e[b] - S.e[b];
      t = t - 1.0 / e_ma / e_lmbc * S.v(b, l, b, m) * S.v(l, b, a, b);
      for (int c = b + 1; c <= S.nbas; ++c) {
        e_lmbc = S.e[l] + S.e[m] - S.e[b] - S.e[c];
        t = t - 1.0 / e_ma / e_lmbc *
                    (S.v(b, l, c, m) * (2.0 * S.v(l, b, a, c) - S.v(l, c, a, b)) +
                     S.v(b, m, c, l) * (2.0 * S.v(l, c, a, b) - S.v(l, b, a, c)));
      }
    }
  return t;
}

double tau22(const FvecSystem& S, int a, int n) {  // :1033-1076
  double t = 0.0;
  double e_na = S.e[n] - S.e[a];
  for (int l = 1; l <= S.no; ++l)
    for (int b = S.no + 1; b <= S.nbas; ++b) {
      double e_lmba = S.e[l] + S.e[l] - S.e[b] - S.e[a];
      t = t + 1.0 / e_na / e_lmba * S.v(l, b, l, n) * S.v(b, l, a, l);
      for (int m = l + 1; m <= S.no; ++m) {
        e_lmba = S.e[l] + S.e[m] - S.e[b] - S.e[a];
        t = t + 1.0 / e_na / e_lmba *
                    (S.v(l, b, m, n) * (2.0 * S.v(b, l, a, m) - S.v(b, m, a, l)) +
                     S.v(l, n, m, b) * (2.0 * S.v(b, m, a, l) - S.v(b, l, a, m)));
      }
    }
  return t;
}

double tau23(const FvecSystem& S, int b, int k) {  // :1080-1125
  double t = 0.0;
  double e_kb = S.e[k] - S.e[b];
  for (int c = S.no + 1; c <= S.nbas; ++c)
    for (int l = 1; l <= S.no; ++l) {
      double e_lmbc = S.e[l] + S.e[l] - S.e[b] - S.e[c];
      t = t - 1.0 / e_kb / e_lmbc * S.v(b, l, c, l) * S.v(l, k, l, c);
      for (int m = l + 1; m <= S.no; ++m) {
        e_lmbc = S.e[l] + S.e[m] - S.e[b] - S.e[c];
        t = t - 1.0 / e_kb / e_lmbc *
                    (S.v(b, l, c, m) * (2.0 * S.v(l, k, m, c) - S.v(l, c, m, k)) +
                     S.v(b, m, c, l) * (2.0 * S.v(l, c, m, k) - S.v(l, k, m, c)));
      }
    }
  return t;
}

double tau24(const FvecSystem& S, int dd, int k) {  // :1129-1177
  double t = 0.0;
  double e_kd = S.e[k] - S.e[dd];
  for (int l = 1; l <= S.no; ++l)
    for (int b = S.no + 1; b <= S.nbas; ++b) {
      double e_klbc = S.e[k] + S.e[l] - S.e[b] - S.e[b];
      t = t + 1.0 / e_kd / e_klbc * S.v(b, k, b, l) * S.v(dd, b, l, b);
      for (int c = b + 1; c <= S.nbas; ++c) {
        e_klbc = S.e[k] + S.e[l] - S.e[b] - S.e[c];
        t = t + 1.0 / e_kd / e_klbc *
                    (S.v(b, k, c, l) * (2.0 * S.v(dd, b, l, c) - S.v(dd, c, l, b)) +
                     S.v(b, l, c, k) * (2.0 * S.v(dd, c, l, b) - S.v(dd, b, l, c)));
      }
    }
  return t;
}

double tauC(const FvecSystem& S, int b, int l) {  // :1181-1209
  double t = 0.0;
  for (int c = S.no + 1; c <= S.nbas; ++c)
    for (int m = 1; m <= S.no; ++m) {
      double e_mlcb = S.e[m] + S.e[l] - S.e[c] - S.e[b];
      t = t + 0.5 * S.d(c, m) / e_mlcb * (2.0 * S.v(m, c, l, b) - S.v(m, b, l, c));
    }
  return t;
}

// FC_ph_new, :1213-1242; tau(b - nocc, l) = tauC(b, l)
double FC_ph_new(const FvecSystem& S, int a, int k, const std::vector<double>& tau) {
  double f = 0.0;
  for (int b = S.no + 1; b <= S.nbas; ++b)
    for (int l = 1; l <= S.no; ++l) {
      double e_klab = S.e[k] + S.e[l] - S.e[a] - S.e[b];
      f = f + tau[(size_t)(b - S.no - 1) * S.no + (l - 1)] / e_klab * (2.0 * S.v(a, k, b, l) - S.v(a, l, b, k));
    }
  return f;
}

// ---- 2h2p terms, dipole_ph.f90:662-846 ------------------------------------

double FI_2p2h(const FvecSystem& S, int a, int k) {  // :662-690
  double f = 0.0;
  for (int m = 1; m <= S.no; ++m) {
    double e_mkaa = S.e[m] + S.e[k] - S.e[a] - S.e[a];
    f = f - S.d(m, k) / e_mkaa * S.v(a, k, a, m);
  }
  for (int c = S.no + 1; c <= S.nbas; ++c) {
    double e_kkac = S.e[k] + S.e[k] - S.e[a] - S.e[c];
    f = f + S.d(a, c) / e_kkac * S.v(c, k, a, k);
  }
  return 2.0 * f;
}

double FII_2p2h(const FvecSystem& S, int a, int b, int k) {  // :694-727
  double f = 0.0;
  for (int m = 1; m <= S.no; ++m) {
    double e_mkab = S.e[m] + S.e[k] - S.e[a] - S.e[b];
    f = f - S.d(m, k) / e_mkab * (S.v(a, m, b, k) + S.v(a, k, b, m));
  }
  for (int c = S.no + 1; c <= S.nbas; ++c) {
    double e_kkbc = S.e[k] + S.e[k] - S.e[b] - S.e[c];
    f = f + S.d(a, c) / e_kkbc * S.v(c, k, b, k);
    double e_kkac = S.e[k] + S.e[k] - S.e[a] - S.e[c];
    f = f + S.d(b, c) / e_kkac * S.v(c, k, a, k);
  }
  return std::sqrt(2.0) * f;
}

double FIII_2p2h(const FvecSystem& S, int a, int k, int l) {  // :731-764
  double f = 0.0;
  for (int m = 1; m <= S.no; ++m) {
    double e_mlaa = S.e[m] + S.e[l] - S.e[a] - S.e[a];
    f = f + S.d(m, k) / e_mlaa * S.v(a, m, a, l);
    double e_kmaa = S.e[k] + S.e[m] - S.e[a] - S.e[a];
    f = f + S.d(m, l) / e_kmaa * S.v(a, k, a, m);
  }
  for (int c = S.no + 1; c <= S.nbas; ++c) {
    double e_klac = S.e[k] + S.e[l] - S.e[a] - S.e[c];
    f = f - S.d(a, c) / e_klac * (S.v(c, k, a, l) + S.v(c, l, a, k));
  }
  return std::sqrt(2.0) * f;
}

double FIV2_2p2h(const FvecSystem& S, int a, int b, int k, int l) {  // :768-806
  double f = 0.0;
  for (int m = 1; m <= S.no; ++m) {
    double e_mlab = S.e[m] + S.e[l] - S.e[a] - S.e[b];
    f = f + S.d(m, k) / e_mlab * (S.v(a, m, b, l) - S.v(a, l, m, b));
    double e_kmab = S.e[k] + S.e[m] - S.e[a] - S.e[b];
    f = f + S.d(m, l) / e_kmab * (S.v(a, k, m, b) - S.v(a, m, b, k));
  }
  for (int c = S.no + 1; c <= S.nbas; ++c) {
    double e_klbc = S.e[k] + S.e[l] - S.e[b] - S.e[c];
    f = f - S.d(a, c) / e_klbc * (S.v(c, k, b, l) - S.v(c, l, b, k));
    double e_klac = S.e[k] + S.e[l] - S.e[a] - S.e[c];
    f = f - S.d(b, c) / e_klac * (S.v(c, l, a, k) - S.v(c, k, a, l));
  }
  return std::sqrt(3.0) * f;
}

double FIV1_2p2h(const FvecSystem& S, int a, int b, int k, int l) {  // :810-846
  double f = 0.0;
  for (int m = 1; m <= S.no; ++m) {
    double e_mlab = S.e[m] + S.e[l] - S.e[a] - S.e[b];
    f = f + S.d(m, k) / e_mlab * (S.v(a, m, b, l) + S.v(a, l, m, b));
    double e_kmab = S.e[k] + S.e[m] - S.e[a] - S.e[b];
    f = f + S.d(m, l) / e_kmab * (S.v(a, k, m, b) + S.v(a, m, b, k));
  }
  for (int c = S.no + 1; c <= S.nbas; ++c) {
    double e_klbc = S.e[k] + S.e[l] - S.e[b] - S.e[c];
    f = f - S.d(a, c) / e_klbc * (S.v(c, k, b, l) + S.v(c, l, b, k));
    double e_klac = S.e[k] + S.e[l] - S.e[a] - S.e[c];
    f = f - S.d(b, c) / e_klac * (S.v(c, l, a, k) + S.v(c, k, a, l));
  }
  return f;
}

}  // namespace

extern "C" {

// get_modifiedtm_adc2(ndim,kpq,mtm,ista), get_moment.f90:153-442, for a kpq of
// the ADC(2)-s form (singles, then the 2h2p classes I, II, III, IV1, IV2 with
// counts kpq(1..5,0)).  kpq: 7 x (ndim+1) int32, column-major, 1-based.
// sections: bit 0 the 1h1p block, bit 1 the 2h2p block (a subset lets a test
// time one part on a bounded sample); the other entries are left at zero.
int orc_modified_tm_adc2(int no, int nv, const double* e, const double* eri, const double* dpl,
                         int64_t ndim, const int32_t* kpq, double* mtm, int sections) {
  FvecSystem S;
  S.no = no; S.nv = nv; S.nbas = no + nv;
  S.e.assign(S.nbas + 1, 0.0);
  for (int p = 1; p <= S.nbas; ++p) S.e[p] = e[p - 1];
  S.eri = eri; S.dpl = dpl;
  auto K = [&](int row, int64_t col) { return kpq[7 * col + (row - 1)]; };
  for (int64_t i = 0; i < ndim; ++i) mtm[i] = 0.0;
  const int64_t n1 = K(1, 0);
  int64_t nlim1 = 1, nlim2 = n1;
  if (sections & 1) {
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t cnt = nlim1; cnt <= nlim2; ++cnt) {
      int k = K(3, cnt), a = K(5, cnt);
      double x = S.d(a, k);
      x = x + F0_ph(S, a, k);
      x = x + F25_ph(S, a, k);
      x = x + F26_ph(S, a, k);
      x = x + F27_ph(S, a, k);
      x = x + F28_ph(S, a, k);
      x = x + F29_ph(S, a, k);
      x = x + F210_ph(S, a, k);
      mtm[cnt - 1] = x;
    }
    const int nb = S.nbas;
    // FA_ph: tau(a,c) = tauA(c,a); mtm += sum_c tau(a,c) dpl(c,k)
    std::vector<double> tau((size_t)nv * nv);
#pragma omp parallel for schedule(dynamic, 1)
    for (int a = no + 1; a <= nb; ++a)
      for (int c = no + 1; c <= nb; ++c) tau[(size_t)(a - no - 1) * nv + (c - no - 1)] = tauA(S, c, a);
    for (int64_t cnt = nlim1; cnt <= nlim2; ++cnt) {
      int k = K(3, cnt), a = K(5, cnt);
      double f = 0.0;
      for (int c = no + 1; c <= nb; ++c) f = f + tau[(size_t)(a - no - 1) * nv + (c - no - 1)] * S.d(c, k);
      mtm[cnt - 1] = mtm[cnt - 1] + f;
    }
    // FB_ph: tau(l,k) = tauB(l,k); mtm += sum_l dpl(a,l) tau(l,k)
    std::vector<double> tb((size_t)no * no);
    for (int l = 1; l <= no; ++l)
      for (int k = 1; k <= no; ++k) tb[(size_t)(l - 1) * no + (k - 1)] = tauB(S, l, k);
    for (int64_t cnt = nlim1; cnt <= nlim2; ++cnt) {
      int k = K(3, cnt), a = K(5, cnt);
      double f = 0.0;
      for (int l = 1; l <= no; ++l) f = f + S.d(a, l) * tb[(size_t)(l - 1) * no + (k - 1)];
      mtm[cnt - 1] = mtm[cnt - 1] + f;
    }
    // FC_ph: tau(b,l) = tauC(b,l); mtm += FC_ph_new(a,k,tau)
    std::vector<double> tc((size_t)nv * no);
    for (int b = no + 1; b <= nb; ++b)
      for (int l = 1; l <= no; ++l) tc[(size_t)(b - no - 1) * no + (l - 1)] = tauC(S, b, l);
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t cnt = nlim1; cnt <= nlim2; ++cnt) {
      int k = K(3, cnt), a = K(5, cnt);
      mtm[cnt - 1] = mtm[cnt - 1] + FC_ph_new(S, a, k, tc);
    }
    // F21_ph, F22_ph: tau(a,l); mtm += sum_l tau(a,l) dpl(l,k)
    for (int which = 0; which < 2; ++which) {
      std::vector<double> t2((size_t)nv * no);
#pragma omp parallel for schedule(dynamic, 1)
      for (int a = no + 1; a <= nb; ++a)
        for (int l = 1; l <= no; ++l)
          t2[(size_t)(a - no - 1) * no + (l - 1)] = which == 0 ? tau21(S, a, l) : tau22(S, a, l);
      for (int64_t cnt = nlim1; cnt <= nlim2; ++cnt) {
        int k = K(3, cnt), a = K(5, cnt);
        double f = 0.0;
        for (int l = 1; l <= no; ++l) f = f + t2[(size_t)(a - no - 1) * no + (l - 1)] * S.d(l, k);
        mtm[cnt - 1] = mtm[cnt - 1] + f;
      }
    }
    // F23_ph, F24_ph: tau(c,k); mtm += sum_c dpl(a,c) tau(c,k)
    for (int which = 0; which < 2; ++which) {
      std::vector<double> t2((size_t)nv * no);
#pragma omp parallel for schedule(dynamic, 1)
      for (int c = no + 1; c <= nb; ++c)
        for (int k = 1; k <= no; ++k)
          t2[(size_t)(c - no - 1) * no + (k - 1)] = which == 0 ? tau23(S, c, k) : tau24(S, c, k);
      for (int64_t cnt = nlim1; cnt <= nlim2; ++cnt) {
        int k = K(3, cnt), a = K(5, cnt);
        double f = 0.0;
        for (int c = no + 1; c <= nb; ++c) f = f + S.d(a, c) * t2[(size_t)(c - no - 1) * no + (k - 1)];
        mtm[cnt - 1] = mtm[cnt - 1] + f;
      }
    }
    const double s2 = -std::sqrt(2.0);
    for (int64_t cnt = nlim1; cnt <= nlim2; ++cnt) mtm[cnt - 1] = s2 * mtm[cnt - 1];
  }
  if (sections & 2) {
    // I: a=b, i=j
    nlim1 = nlim2 + 1; nlim2 = nlim2 + K(2, 0);
#pragma omp parallel for schedule(static)
    for (int64_t cnt = nlim1; cnt <= nlim2; ++cnt) mtm[cnt - 1] = FI_2p2h(S, K(5, cnt), K(3, cnt));
    // II: a|=b, i=j
    nlim1 = nlim2 + 1; nlim2 = nlim2 + K(3, 0);
#pragma omp parallel for schedule(static)
    for (int64_t cnt = nlim1; cnt <= nlim2; ++cnt) mtm[cnt - 1] = FII_2p2h(S, K(5, cnt), K(6, cnt), K(3, cnt));
    // III: a=b, i|=j
    nlim1 = nlim2 + 1; nlim2 = nlim2 + K(4, 0);
#pragma omp parallel for schedule(static)
    for (int64_t cnt = nlim1; cnt <= nlim2; ++cnt) mtm[cnt - 1] = FIII_2p2h(S, K(5, cnt), K(3, cnt), K(4, cnt));
    // IV1 and IV2 (the second copy of the a|=b, i|=j block)
    nlim1 = nlim2 + 1; nlim2 = nlim2 + K(5, 0);
    const int64_t n5 = K(5, 0);
#pragma omp parallel for schedule(static)
    for (int64_t cnt = nlim1; cnt <= nlim2; ++cnt) {
      int k = K(3, cnt), j = K(4, cnt), a = K(5, cnt), b = K(6, cnt);
      mtm[cnt - 1] = FIV1_2p2h(S, a, b, k, j);
      mtm[cnt + n5 - 1] = FIV2_2p2h(S, a, b, k, j);
    }
  }
  return 0;
}

}  // extern "C"
