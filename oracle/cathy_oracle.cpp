// CPU FP64 oracle for CATHY's FLOW3D hot path -- TEST INFRASTRUCTURE ONLY.
//
// A serial double-precision restatement of the reference Fortran, keeping the
// reference's loop order and 1-based indexing so that it can serve as the
// parity truth and as the timed CPU baseline.  Every routine cites the
// reference source it follows; paths are relative to the vendored CATHY tree
// pyCATHY/tests/weil_exemple/my_cathy_prj/src/ (all 36 vendored copies of the
// *.f files are byte-identical).
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// this library.  It is never linked into, or called by, the product.
#include "cathy_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using std::vector;
typedef vector<double> dvec;
typedef vector<int> ivec;

namespace {

const double RMAX = 1.7e100;  // cathy_main.f:2488
const double RMIN = 1.7e-100; // cathy_main.f:2489

// ---------------------------------------------------------------------------
// Sparse solver pieces (solscal-extended.f)
// ---------------------------------------------------------------------------

// INCLDP: IC(0) of a symmetric upper CSR matrix (diagonal first in each row),
// with the reference's breakdown patch.  solscal-extended.f:2142-2192
void incldp(const int* ja, const int* topol, const double* coefr, double* lriga,
            int n, int nterm) {
  for (int k = 1; k <= nterm; ++k) lriga[k] = 0.0;
  for (int kk = 1; kk <= n; ++kk) {
    int k = topol[kk];
    double a = coefr[k] - lriga[k];
    if (a <= 0.0) a = lriga[topol[kk - 1]] * lriga[topol[kk - 1]];
    lriga[k] = std::sqrt(a);
    if (kk == n) continue;
    int i = topol[kk] + 1, j = topol[kk + 1] - 1;
    if (j < i) continue;
    for (int k1 = i; k1 <= j; ++k1) lriga[k1] = (coefr[k1] - lriga[k1]) / lriga[k];
    for (int k2 = i; k2 <= j; ++k2) {
      int i1 = k2 + 1;
      int j1 = topol[ja[k2]];
      lriga[j1] += lriga[k2] * lriga[k2];
      if (k2 == j) continue;
      j1 = j1 + 1;
      if (j1 >= topol[ja[k2] + 1]) continue;
      // merge walk of row ja[k2] (from j1) against row kk (from i1)
      for (;;) {
        if (ja[j1] < ja[i1]) {
          j1++;
          if (j1 >= topol[ja[k2] + 1]) break;
        } else if (ja[j1] == ja[i1]) {
          lriga[j1] += lriga[k2] * lriga[i1];
          i1++;
          if (i1 > j) break;
        } else {
          i1++;
          if (i1 > j) break;
        }
      }
    }
  }
}

// PRODDP: x = (U^T U)^-1 b with U in upper CSR.  solscal-extended.f:4169-4204
void proddp(double* x, const double* b, int n, const int* topol, const int* ja,
            const double* coef2) {
  for (int k = 1; k <= n; ++k) x[k] = 0.0;
  for (int k = 1; k <= n; ++k) {
    int i = topol[k], j = topol[k + 1] - 1;
    for (int m = i; m <= j; ++m) {
      if (m == i) x[k] = (b[k] - x[k]) / coef2[m];
      else x[ja[m]] += coef2[m] * x[k];
    }
  }
  double a = 0.0;
  for (int kk = 1; kk <= n; ++kk) {
    int row = n - kk + 1;
    int i = topol[row], j = topol[row + 1] - 1;
    for (int m = i; m <= j; ++m) {
      int mm = j - m + i;
      if (mm == i) {
        x[row] = (x[row] - a) / coef2[mm];
        a = 0.0;
      } else {
        a += coef2[mm] * x[ja[mm]];
      }
    }
  }
}

// Jacobi variant of PRODDP (documented Picard+Jacobi option, not in the
// reference's Picard path): x = D^-1 b.
void prodjac(double* x, const double* b, int n, const int* topol,
             const double* coef1) {
  for (int k = 1; k <= n; ++k) x[k] = b[k] / coef1[topol[k]];
}

// symmetric SpMV from upper storage, y -= A x (accumulating form of GRADDP)
void symmv_acc(double* y, const double* x, int n, const int* topol,
               const int* ja, const double* a, double sign) {
  for (int k = 1; k <= n; ++k) {
    int i = topol[k], j = topol[k + 1] - 1;
    for (int m = i; m <= j; ++m) {
      y[k] += sign * a[m] * x[ja[m]];
      if (m != i) y[ja[m]] += sign * a[m] * x[k];
    }
  }
}

// GRADDP: preconditioned CG with the reference's recurrences and stopping
// rule (masked residual norm over masked RHS norm).
// solscal-extended.f:1260-1386
void graddp(int n, double* poten, double* scr, double* res, double* b,
            double* r, double* p, const int* topol, const int* ja,
            const double* coef1, const double* coef2, const double* tnoti,
            double tol, int imax, int np, const int* contp, int* niter,
            double* err, bool jacobi) {
  *niter = 1;
  for (int k = 1; k <= n; ++k) { scr[k] = tnoti[k]; r[k] = tnoti[k]; }
  for (int i = 1; i <= np; ++i) scr[contp[i]] = 0.0;
  double xlung = 0.0;
  for (int i = 1; i <= n; ++i) xlung += scr[i] * scr[i];
  for (int i = 1; i <= np; ++i) scr[contp[i]] = tnoti[contp[i]];
  for (int k = 1; k <= n; ++k) {
    int i = topol[k], j = topol[k + 1] - 1;
    for (int m = i; m <= j; ++m) {
      r[k] -= coef1[m] * poten[ja[m]];
      res[k] = r[k];
      if (m != i) {
        r[ja[m]] -= coef1[m] * poten[k];
        res[ja[m]] = r[ja[m]];
      }
    }
  }
  if (jacobi) prodjac(p, r, n, topol, coef1);
  else proddp(p, r, n, topol, ja, coef2);
  for (;;) {
    for (int k = 1; k <= n; ++k) b[k] = 0.0;
    for (int k = 1; k <= n; ++k) {
      int i = topol[k], j = topol[k + 1] - 1;
      for (int m = i; m <= j; ++m) {
        b[k] += coef1[m] * p[ja[m]];
        if (m != i) b[ja[m]] += coef1[m] * p[k];
      }
    }
    double a = 0.0, bb = 0.0;
    for (int k = 1; k <= n; ++k) { a += p[k] * r[k]; bb += p[k] * b[k]; }
    double alfa = a / bb;
    for (int k = 1; k <= n; ++k) { r[k] -= alfa * b[k]; poten[k] += alfa * p[k]; }
    if (jacobi) prodjac(scr, r, n, topol, coef1);
    else proddp(scr, r, n, topol, ja, coef2);
    double c = 0.0;
    for (int k = 1; k <= n; ++k) c += b[k] * scr[k];
    double beta = -c / bb;
    for (int k = 1; k <= n; ++k) p[k] = scr[k] + beta * p[k];
    for (int k = 1; k <= n; ++k) res[k] = r[k];
    for (int k = 1; k <= np; ++k) res[contp[k]] = 0.0;
    a = 0.0;
    for (int k = 1; k <= n; ++k) a += res[k] * res[k];
    *err = (xlung > 0.0) ? std::sqrt(a / xlung) : std::sqrt(a / n);
    if (*err > tol && *niter < imax) { (*niter)++; continue; }
    break;
  }
}

// RESSYM: true residual of the symmetric solve.  solscal-extended.f:4389-4438
double ressym(const int* topol, const int* ja, const double* coef1,
              const double* tnoti, const double* pnew, double* resv, int n,
              int numdir, const int* noddir) {
  for (int k = 1; k <= n; ++k) resv[k] = tnoti[k];
  for (int k = 1; k <= numdir; ++k) resv[noddir[k]] = 0.0;
  double xlung = 0.0;
  for (int k = 1; k <= n; ++k) xlung += resv[k] * resv[k];
  for (int k = 1; k <= n; ++k) {
    int m = topol[k], mm = topol[k + 1] - 1;
    for (int i = m; i <= mm; ++i) {
      if (i > m) resv[ja[i]] -= coef1[i] * pnew[k];
      resv[k] -= coef1[i] * pnew[ja[i]];
    }
  }
  for (int k = 1; k <= numdir; ++k) resv[noddir[k]] = 0.0;
  double res = 0.0;
  for (int k = 1; k <= n; ++k) res += resv[k] * resv[k];
  return (xlung <= RMIN) ? std::sqrt(res / n) : std::sqrt(res / xlung);
}

// SYMSLV: IC(0) factor, x0 = M^-1 b, GRADDP, RESSYM.
// solscal-extended.f:4669-4699
int symslv(int n, int nterm, int numdir, int* niter, int itmxcg, double tolcg,
           const int* noddir, const int* ja, const int* topol, double* pnew,
           const double* tnoti, const double* coef1, double* coef2, double* scr,
           double* err, double* res, bool jacobi) {
  int in1 = 0, in2 = in1 + n, in3 = in2 + n, in4 = in3 + n, in5 = in4 + n;
  if (jacobi) {
    prodjac(pnew, tnoti, n, topol, coef1);
  } else {
    incldp(ja, topol, coef1, coef2, n, nterm);
    proddp(pnew, tnoti, n, topol, ja, coef2);
  }
  graddp(n, pnew, scr + in1, scr + in2, scr + in3, scr + in4, scr + in5, topol,
         ja, coef1, coef2, tnoti, tolcg, itmxcg, numdir, noddir, niter, err,
         jacobi);
  *res = ressym(topol, ja, coef1, tnoti, pnew, scr + in1, n, numdir, noddir);
  return *niter;
}

// ---- nonsymmetric (Newton) solvers -------------------------------------

// aperbn: r = A v on full CSR.  solscal-extended.f:97-107
void aperbn(int n, const int* topol, const int* ja, const double* coeff,
            const double* vet, double* r) {
  for (int k = 1; k <= n; ++k) {
    double s = 0.0;
    for (int i = topol[k]; i < topol[k + 1]; ++i) s += coeff[i] * vet[ja[i]];
    r[k] = s;
  }
}

// ILU(0) in the reference's split: L lower with diagonal, U unit upper, both
// stored in COEF2 on the pattern of A (INCLU, solscal-extended.f:2194-2277).
// INCLU is a Crout-type incomplete factorisation; ILU(0) factors are unique
// for a fixed pattern and diagonal normalisation, so this restatement uses a
// row-wise (IKJ) elimination producing the same L (with diagonal) and unit U,
// with the reference's zero-pivot patch (use the previous diagonal).
void inclu(const int* ia, const int* ja, const int* topol, const double* a,
           double* lu, int n) {
  int nterm = topol[n + 1] - 1;
  // Doolittle IKJ on a copy, then move the diagonal scaling into L.
  dvec w(nterm + 1);
  for (int k = 1; k <= nterm; ++k) w[k] = a[k];
  ivec diag(n + 1), pos(n + 1, 0);
  for (int i = 1; i <= n; ++i)
    for (int m = topol[i]; m < topol[i + 1]; ++m)
      if (ja[m] == i) diag[i] = m;
  double prevd = 1.0;
  for (int i = 1; i <= n; ++i) {
    for (int m = topol[i]; m < topol[i + 1]; ++m) pos[ja[m]] = m;
    for (int m = topol[i]; m < topol[i + 1]; ++m) {
      int k = ja[m];
      if (k >= i) break;
      // w[m] = l_ik (Doolittle: divided by u_kk)
      double ukk = w[diag[k]];
      w[m] /= ukk;
      for (int mm = diag[k] + 1; mm < topol[k + 1]; ++mm) {
        int j = ja[mm];
        if (pos[j]) w[pos[j]] -= w[m] * w[mm];
      }
    }
    if (w[diag[i]] == 0.0) w[diag[i]] = prevd;
    prevd = w[diag[i]];
    for (int m = topol[i]; m < topol[i + 1]; ++m) pos[ja[m]] = 0;
  }
  // convert Doolittle (unit L, U with diag) -> reference split (L with diag,
  // unit U):  L' = L D, U' = D^-1 U
  for (int i = 1; i <= n; ++i) {
    for (int m = topol[i]; m < topol[i + 1]; ++m) {
      int j = ja[m];
      if (j < i) lu[m] = w[m] * w[diag[j]];
      else if (j == i) lu[m] = w[m];
      else lu[m] = w[m] / w[diag[i]];
    }
  }
  (void)ia;
}

// PRODL: z = L^-1 y (L with diagonal).  solscal-extended.f:4205-4226
void prodl(double* z, const double* y, int n, const int* topol, const int* ja,
           const double* c2) {
  for (int i = 1; i <= n; ++i) {
    double a = 0.0, d = 1.0;
    for (int m = topol[i]; m < topol[i + 1]; ++m) {
      int j = ja[m];
      if (j < i) a += c2[m] * z[j];
      else if (j == i) d = c2[m];
    }
    z[i] = (y[i] - a) / d;
  }
}
// PRODU: x = U^-1 h (unit U).  solscal-extended.f:4228-4249
void produ(double* x, const double* h, int n, const int* topol, const int* ja,
           const double* c2) {
  for (int i = n; i >= 1; --i) {
    double a = 0.0;
    for (int m = topol[i]; m < topol[i + 1]; ++m) {
      int j = ja[m];
      if (j > i) a += c2[m] * x[j];
    }
    x[i] = h[i] - a;
  }
}
// PRU: y = U x.  solscal-extended.f:4251-4266
void pru(double* y, const double* x, int n, const int* topol, const int* ja,
         const double* c2) {
  for (int i = 1; i <= n; ++i) {
    double s = x[i];
    for (int m = topol[i]; m < topol[i + 1]; ++m)
      if (ja[m] > i) s += c2[m] * x[ja[m]];
    y[i] = s;
  }
}
// PROD1: x = (LU)^-1 b.  solscal-extended.f:4107-4140
void prod1(double* x, const double* b, int n, const int* topol, const int* ja,
           const double* c2, double* tmp) {
  prodl(tmp, b, n, topol, ja, c2);
  produ(x, tmp, n, topol, ja, c2);
}
// PRODBH: z = L^-1 A U^-1 h.  solscal-extended.f:4142-4160
void prodbh(double* z, const double* h, int n, const int* topol, const int* ja,
            const double* c1, const double* c2, double* x, double* y) {
  produ(x, h, n, topol, ja, c2);
  aperbn(n, topol, ja, c1, x, y);
  prodl(z, y, n, topol, ja, c2);
}

// RESNSY: true residual of the nonsymmetric solve (same form as RESSYM on
// full storage).  solscal-extended.f:4332-4388
double resnsy(const int* topol, const int* ja, const double* c1,
              const double* tnoti, const double* pnew, double* resv, int n,
              int numdir, const int* noddir) {
  for (int k = 1; k <= n; ++k) resv[k] = tnoti[k];
  for (int k = 1; k <= numdir; ++k) resv[noddir[k]] = 0.0;
  double xlung = 0.0;
  for (int k = 1; k <= n; ++k) xlung += resv[k] * resv[k];
  for (int k = 1; k <= n; ++k)
    for (int i = topol[k]; i < topol[k + 1]; ++i) resv[k] -= c1[i] * pnew[ja[i]];
  for (int k = 1; k <= numdir; ++k) resv[noddir[k]] = 0.0;
  double res = 0.0;
  for (int k = 1; k <= n; ++k) res += resv[k] * resv[k];
  return (xlung <= RMIN) ? std::sqrt(res / n) : std::sqrt(res / xlung);
}

// GCSTAS (ISOLV=0, split ILU(0)) and GCSTAD (ISOLV=-5, Jacobi) BiCGSTAB.
// solscal-extended.f:1010-1130 and :786-900.  `jac` != NULL selects GCSTAD.
void bicgstab(int n, double* poten, const double* tnoti, const int* topol,
              const int* ja, const double* c1, const double* c2,
              const double* jac, int imax, double tol, int np,
              const int* contp, int* niter, double* err) {
  dvec pjm(n + 1), vjm(n + 1), p(n + 1), v(n + 1), s(n + 1), t(n + 1),
      r(n + 1), rt(n + 1), scr1(n + 1), scr2(n + 1);
  *niter = 1;
  double xlung = 0.0;
  for (int i = 1; i <= n; ++i) pjm[i] = tnoti[i];
  for (int i = 1; i <= np; ++i) pjm[contp[i]] = 0.0;
  for (int i = 1; i <= n; ++i) xlung += pjm[i] * pjm[i];
  aperbn(n, topol, ja, c1, poten, scr1.data());
  for (int k = 1; k <= n; ++k) scr1[k] = tnoti[k] - scr1[k];
  if (jac) {
    for (int k = 1; k <= n; ++k) r[k] = scr1[k] * jac[k];
  } else {
    prodl(r.data(), scr1.data(), n, topol, ja, c2);
    pru(scr1.data(), poten, n, topol, ja, c2);
    for (int k = 1; k <= n; ++k) poten[k] = scr1[k];
  }
  for (int i = 1; i <= n; ++i) { rt[i] = r[i]; pjm[i] = 0.0; vjm[i] = 0.0; }
  double rojm1 = 1.0, alfjm1 = 1.0, etaj = 1.0;
  for (;;) {
    double roj = 0.0;
    for (int i = 1; i <= n; ++i) roj += rt[i] * r[i];
    double beta = (roj / rojm1) * (alfjm1 / etaj);
    for (int i = 1; i <= n; ++i) p[i] = r[i] + beta * (pjm[i] - etaj * vjm[i]);
    if (jac) {
      aperbn(n, topol, ja, c1, p.data(), v.data());
      for (int i = 1; i <= n; ++i) v[i] *= jac[i];
    } else {
      prodbh(v.data(), p.data(), n, topol, ja, c1, c2, scr1.data(), scr2.data());
    }
    double sigma = 0.0;
    for (int i = 1; i <= n; ++i) sigma += rt[i] * v[i];
    double alfj = roj / sigma;
    for (int i = 1; i <= n; ++i) s[i] = r[i] - alfj * v[i];
    if (jac) {
      aperbn(n, topol, ja, c1, s.data(), t.data());
      for (int i = 1; i <= n; ++i) t[i] *= jac[i];
    } else {
      prodbh(t.data(), s.data(), n, topol, ja, c1, c2, scr1.data(), scr2.data());
    }
    double aa = 0.0, bb = 0.0;
    for (int i = 1; i <= n; ++i) { aa += s[i] * t[i]; bb += t[i] * t[i]; }
    etaj = aa / bb;
    for (int i = 1; i <= n; ++i) {
      poten[i] += alfj * p[i] + etaj * s[i];
      r[i] = s[i] - etaj * t[i];
    }
    for (int i = 1; i <= np; ++i) r[contp[i]] = 0.0;
    aa = 0.0;
    for (int i = 1; i <= n; ++i) aa += r[i] * r[i];
    *err = (xlung > 0.0) ? std::sqrt(aa / xlung) : std::sqrt(aa / n);
    if (*niter <= imax && *err > tol) {
      (*niter)++;
      rojm1 = roj;
      alfjm1 = alfj;
      for (int i = 1; i <= n; ++i) { pjm[i] = p[i]; vjm[i] = v[i]; }
      continue;
    }
    break;
  }
  if (!jac) {
    for (int i = 1; i <= n; ++i) { r[i] = poten[i]; poten[i] = 0.0; }
    produ(poten, r.data(), n, topol, ja, c2);
  }
}

// NSYSLV for ISOLV 0 and -5.  solscal-extended.f:3063-3170
int nsyslv(int isolv, int n, int numdir, const int* noddir, int itmxcg,
           double tolcg, const int* ia, const int* ja, const int* topol,
           const double* c1, double* c2, double* pnew, const double* tnoti,
           double* err, double* res) {
  double rhsn = 0.0;
  for (int i = 1; i <= n; ++i) rhsn += tnoti[i] * tnoti[i];
  if (rhsn == 0.0) {
    for (int i = 1; i <= n; ++i) pnew[i] = 0.0;
    *err = 0.0; *res = 0.0;
    return 0;
  }
  int niter = 0;
  dvec tmp(n + 1);
  if (isolv == -5) {
    dvec d(n + 1);
    for (int i = 1; i <= n; ++i)
      for (int m = topol[i]; m < topol[i + 1]; ++m)
        if (ja[m] == i) d[i] = 1.0 / c1[m];  // diagn
    for (int i = 1; i <= n; ++i) pnew[i] = tnoti[i] * d[i];  // PRDY
    bicgstab(n, pnew, tnoti, topol, ja, c1, nullptr, d.data(), itmxcg, tolcg,
             numdir, noddir, &niter, err);
  } else {
    inclu(ia, ja, topol, c1, c2, n);
    prod1(pnew, tnoti, n, topol, ja, c2, tmp.data());
    bicgstab(n, pnew, tnoti, topol, ja, c1, c2, nullptr, itmxcg, tolcg, numdir,
             noddir, &niter, err);
  }
  *res = resnsy(topol, ja, c1, tnoti, pnew, tmp.data(), n, numdir, noddir);
  return niter;
}

// ---------------------------------------------------------------------------
// The oracle state
// ---------------------------------------------------------------------------
// ASSPIC (asspic.f:9-54) on the reference's own arrays: 1-based TETRA(5,NT)
// and TETJA(4,4,NT) contents, column-major LMASS(4,4), BI/CI/DI(4,NT) and
// PERMX/PERMY/PERMZ(MAXSTR,*); COEF1/COEF2/COEF4 (C pointers to the Fortran
// arrays, 1-based contents) are accumulated in the reference's element order
// with its left-to-right sums: COEF1(IND) + PVKB*BI(L) + PVKC*CI(L) + PVKD*DI(L).
void asspic(int nt, int ntri, const int* tetra, const int* tetja, const double* lmass,
            double* coef1, double* coef2, double* coef4, const double* et1e,
            const double* pel, const double* permx, const double* permy,
            const double* permz, const double* ckrwe, const double* volu,
            const double* volur, const double* bi, const double* ci, const double* di,
            int maxstr) {
  for (int iel = 1; iel <= nt; ++iel) {
    int istr = 1 + iel / (ntri * 3);
    const int ir = iel % (ntri * 3);
    if (ir == 0) istr -= 1;
    const int mtype = tetra[5 * (iel - 1) + 4];
    const int id = (istr - 1) + maxstr * (mtype - 1);
    const int e = iel - 1;
    const double vk = volur[e] * ckrwe[e];
    const double ve1 = volu[e] * et1e[e];
    const double ve = volu[e] * pel[e];
    const double pvk1 = permx[id] * vk, pvk2 = permy[id] * vk, pvk3 = permz[id] * vk;
    for (int k = 1; k <= 4; ++k) {
      const double pvkb = pvk1 * bi[4 * e + k - 1], pvkc = pvk2 * ci[4 * e + k - 1],
                   pvkd = pvk3 * di[4 * e + k - 1];
      for (int l = k; l <= 4; ++l) {
        const int ind = tetja[16 * e + 4 * (l - 1) + (k - 1)] - 1;
        const double lm = lmass[4 * (l - 1) + (k - 1)];
        coef1[ind] = coef1[ind] + pvkb * bi[4 * e + l - 1] + pvkc * ci[4 * e + l - 1] +
                     pvkd * di[4 * e + l - 1];
        coef2[ind] = coef2[ind] + ve1 * lm;
        coef4[ind] = coef4[ind] + ve * lm;
      }
    }
  }
}

struct Oracle {
  // sizes
  int nrow = 0, ncol = 0, nnod = 0, ntri = 0, nstr = 0, n = 0, nt = 0,
      nterm = 0, nzone = 0;
  orc_parm_t parm;
  // mesh
  dvec x, y, z, arenod, volnod, volu, volur;
  ivec triang, tetra, tetra_gen3d, ivol, topol, ja, ia, tetja, tp;
  dvec bi, ci, di;
  double lmass[5][5];
  // soil tables per (layer, zone)
  dvec permx, permy, permz, elstor, poros, vgncell, vgrmccell, vgpsatcell;
  double pmin = -5.0, scf = 0.0, tolksl = 0.01;
  int kslope = 0;
  // Feddes root-water uptake (SOILCHAR.H /FEDDES/): VEG_TYPE per surface
  // node and 6 parameters per type (PCANA, PCREF, PCWLT, ZROOT, PZ, OMGC)
  ivec veg_type;
  dvec feddes;
  // seepage faces (sfvone.f, sfinit.f, extall.f): one entry per face node,
  // the faces' lists one after another; SFEXIT equals SFEX at the start of
  // every iteration, so KSF counts the exit flags EXTALL changes
  int nsfn = 0;
  ivec sfnode, sfex, sfexp;
  dvec sfq, sfqp;
  double sfflw = 0.0, sfflwp = 0.0;
  double vnd = 0.0, vnn = 0.0;  // VNDIN+VNDOUT, VNNIN+VNNOUT of the last MASBAL
  int ksf = 0;
  bool sfchek = false, ksfzer = true;
  // nodal soil parameters (SOILCHAR.H) and element porosity
  dvec pnodi, snodi, vgn, vgm, vgrmc, vgpsat, vgn1, vgm52, vgnr, vgmm1, vgmr,
      vgpsn, vgpnot, pel;
  // state vectors
  dvec pnew, pold, ptnew, ptold, ptimep, pdiff, swnew, swtimep, sw, ckrw, etai,
      et1, et2, ckrwe, etae, et1e, dckrw, detai, swp;
  dvec coef1, coef2, coef3, coef4, coef5, tnoti, xt5, scr, lhsp, lhsatm, lhssf;
  // boundary conditions
  int np = 0, nq = 0, numdir = 0;
  ivec contp, contq, noddir, ifatm, ifatmp;
  dvec presc, q, qpnew, qpold, atmpot, atmact, atmold, qtranie;
  // atmospheric series
  int hspatm = 1, ieto = 0, natm = 0, atm_next = 0, htiatm = 0;
  dvec atm_t, atm_v;  // natm records
  double atmtim[4] = {0, 0, 0, 0};
  dvec atminp[4];
  // mass balance (MB_HGRAPH.H)
  double adin = 0, adout = 0, adinp = 0, adoutp = 0, ndin = 0, ndout = 0,
         ndinp = 0, ndoutp = 0, anin = 0, anout = 0, aninp = 0, anoutp = 0,
         nnin = 0, nnout = 0, nninp = 0, nnoutp = 0, vin = 0, vout = 0,
         cvin = 0, cvout = 0, dstore = 0, cdstor = 0, erras = 0, cerras = 0,
         caeras = 0, errel = 0, store1 = 0, store2 = 0, vtot = 0;
  // time stepping
  double time = 0, timep = 0, deltat = 0, pondh_min = 0;
  int nstep = 1, iter = 1, nitert = 0, itlin = 0, itrtot = 0, kbackt = 0,
      kback = 0, klsfai = 0;
  bool dtgmin = true, finished = false;
  // diagnostics
  double pinf = 0, pl2 = 0, finf = 0, fl2 = 0, pikmax = 0;
  int ikmax = 0;
  int niter_last = 0;
  double lin_err = 0, lin_res = 0;
  vector<orc_iter_rec_t> iter_recs;
  vector<orc_step_rec_t> step_recs;

  int idx(int istr, int mtype) const { return (mtype - 1) * nstr + (istr - 1); }
  int T(int j, int iel) const { return tetra[(iel - 1) * 5 + (j - 1)]; }
  int& Tr(int j, int iel) { return tetra[(iel - 1) * 5 + (j - 1)]; }
  double B(int k, int iel) const { return bi[(iel - 1) * 4 + (k - 1)]; }
  double C(int k, int iel) const { return ci[(iel - 1) * 4 + (k - 1)]; }
  double D(int k, int iel) const { return di[(iel - 1) * 4 + (k - 1)]; }
  int TJ(int k, int l, int iel) const { return tetja[(iel - 1) * 16 + (l - 1) * 4 + (k - 1)]; }
  // layer of element iel (asspic.f:27-29)
  int istr_of(int iel) const {
    int istr = 1 + iel / (ntri * 3);
    if (iel % (ntri * 3) == 0) istr -= 1;
    return istr;
  }

  // ---- van Genuchten (fvgse.f, fvgdse.f, fvgkr.f, fvgdkr.f, fvgdds.f) ----
  double fvgse(double psi, int i) const {
    if (psi < -1.0e-14) {
      double beta = std::pow(std::fabs(psi / vgpsat[i]), vgn[i]);
      return std::pow(std::fabs(1.0 / (beta + 1.0)), vgm[i]);
    }
    return 1.0;
  }
  double fvgdse(double psi, int i) const {
    if (psi < -1.0e-14) {
      double beta = std::pow(std::fabs(psi / vgpsat[i]), vgn[i]);
      double b1 = beta + 1.0, b1r = 1.0 / b1;
      return vgn1[i] * (std::pow(std::fabs(psi), vgn1[i]) / vgpsn[i]) *
             std::pow(std::fabs(b1), vgnr[i]) * b1r * b1r;
    }
    return 0.0;
  }
  double fvgkr(double psi, double se, int i) const {
    if (psi < -1.0e-14) {
      double omega = std::pow(std::fabs(se), vgmr[i]);
      double v1 = 1.0 - std::pow(std::fabs(1.0 - omega), vgm[i]);
      return std::sqrt(se) * v1 * v1;
    }
    return 1.0;
  }
  double fvgdkr(double psi, int i) const {
    if (psi < -1.0e-14) {
      double beta = std::pow(std::fabs(psi / vgpsat[i]), vgn[i]);
      double b1 = beta + 1.0;
      double v1 = std::pow(std::fabs(b1), vgm[i]) - std::pow(std::fabs(beta), vgm[i]);
      double v2 = vgpsat[i] / psi;
      double v3 = vgn1[i] * beta * v2 * std::pow(std::fabs(1.0 / b1), vgm52[i]) / vgpsat[i];
      double v4 = v2 * ((2.5 / b1) * beta - 2.0) - 0.5 * std::pow(std::fabs(b1), vgmm1[i]);
      return v3 * v1 * v4;
    }
    return 0.0;
  }
  double fvgdds(double psi, int i) const {
    if (psi < -1.0e-14) {
      double beta = std::pow(std::fabs(psi / vgpsat[i]), vgn[i]);
      double b1 = beta + 1.0, b1r = 1.0 / b1;
      return vgn1[i] * (beta / psi) * (1.0 / psi) *
             ((1.0 + vgn[i] * (beta - 1.0)) / std::pow(std::fabs(b1), vgm[i])) *
             b1r * b1r;
    }
    return 0.0;
  }

  // ASSPIC on the oracle's state (element arrays are 1-based vectors)
  void asspic_state() {
    double lm[16];
    for (int k = 1; k <= 4; ++k)
      for (int l = 1; l <= 4; ++l) lm[4 * (l - 1) + (k - 1)] = lmass[k][l];
    asspic(nt, ntri, tetra.data(), tetja.data(), lm, coef1.data() + 1, coef2.data() + 1,
           coef4.data() + 1, et1e.data() + 1, pel.data() + 1, permx.data(), permy.data(),
           permz.data(), ckrwe.data() + 1, volu.data() + 1, volur.data() + 1, bi.data(),
           ci.data(), di.data(), nstr);
  }

  // NODELT (nodelt.f:9-29)
  void nodelt(const dvec& vnod, dvec& velt) const {
    const double r4 = 1.0 / 4.0;
    for (int iel = 1; iel <= nt; ++iel) {
      double s = 0.0;
      for (int j = 1; j <= 4; ++j) s += vnod[T(j, iel)];
      velt[iel] = s * r4;
    }
  }

  // ---- mesh construction ----
  bool build_mesh(const orc_dem_t* d);
  void tpnodi(const orc_soil_t* s);
  void chparm();
  // ---- nonlinear step pieces ----
  void chpic(void);
  void picard(void);
  void newton(void);
  void masbal(void);
  void conver(void);
  void switch_old(void);
  void etran(void);
  void extall(void);
  bool flow3d(bool first_only);
  void atm_read_next(double& t, dvec& v, bool& ok);
  void atmone(void);
  void atmnxt(void);
  void atmbak(void);
  void timupd(void);
  void bkstep(void);
  int  step(void);
};

// ---------------------------------------------------------------------------
// Mesh: TRIANGOLI (triangoli.f:1-159) + TPNODI2D (tpnodi2d.f) + RIORD
// (riord.f) + AREA2D (area2d.f/areas.f) + GEN3D (gen3d.f:28-77) + RIORD on
// tets for IOPT=1 + VOLBAS/VOLUMS/BASIS6 (volbas.f, volums.f, basis6.f) +
// LOCMAS (locmas.f) + STRPIC/TETPIC or STRNEW/TETNEW/TOPIA.
// ---------------------------------------------------------------------------
static void riord(int nelt, int* eltcon, int nod) {
  for (int i = 0; i < nelt; ++i) {
    int* e = eltcon + i * (nod + 1);
    for (int k = 0; k < nod - 1; ++k)
      for (int j = k + 1; j < nod; ++j)
        if (e[k] > e[j]) std::swap(e[k], e[j]);
  }
}

static const int IP4[5][5] = {  // IP4(II,NN): cathy_main.f:2491 (column-major DATA)
    {0, 0, 0, 0, 0}, {0, 1, 2, 3, 4}, {0, 2, 3, 4, 1}, {0, 3, 4, 1, 2}, {0, 4, 1, 2, 3}};
// IP4 as declared: IP4(II,NN) with DATA column-major -> IP4(II,NN) = ((NN-1)+(II-1))%4+1
static int ip4(int ii, int nn) { return ((nn - 1) + (ii - 1)) % 4 + 1; }

// local IP3 built from IP4 as in VOLUMS/BASIS6
static void make_ip3(int nn, int ip3[4][4]) {
  for (int ii = 2; ii <= 4; ++ii) ip3[ii - 1][1] = ip4(ii, nn);
  for (int lc = 2; lc <= 3; ++lc)
    for (int lr = 1; lr <= 3; ++lr) {
      if (lr == 3) ip3[lr][lc] = ip3[1][lc - 1];
      else ip3[lr][lc] = ip3[lr + 1][lc - 1];
    }
}

static double volums(const int* tl, const double* X, const double* Y,
                     const double* Z) {
  const double amen[5] = {0, -1.0, 1.0, -1.0, 1.0};
  double vol = 0.0;
  for (int nn = 1; nn <= 4; ++nn) {
    int ip3[4][4];
    make_ip3(nn, ip3);
    double a2 = 0.0, a3 = 0.0;
    for (int ii = 1; ii <= 3; ++ii) {
      int i = tl[ip3[ii][1] - 1], j = tl[ip3[ii][2] - 1], m = tl[ip3[ii][3] - 1];
      a3 = Y[i] * Z[j] + a3;
      a2 = Y[i] * Z[m] + a2;
    }
    vol = vol + X[tl[nn - 1]] * amen[nn] * (a3 - a2) / 6.0;
  }
  return vol;
}

static void basis6(const int* tl, const double* X, const double* Y,
                   const double* Z, double* bil, double* cil, double* dil) {
  const double amen[6] = {0, -1.0, 1.0, -1.0, 1.0, -1.0};
  for (int nn = 1; nn <= 4; ++nn) {
    int ip3[4][4];
    make_ip3(nn, ip3);
    double a2 = 0.0, a3 = 0.0;
    for (int ii = 1; ii <= 3; ++ii) {
      int i = tl[ip3[ii][1] - 1], j = tl[ip3[ii][2] - 1], m = tl[ip3[ii][3] - 1];
      a3 = Y[i] * Z[j] + a3;
      a2 = Y[i] * Z[m] + a2;
    }
    bil[nn - 1] = amen[nn] * (a3 - a2) / 6.0;
    a2 = 0.0; a3 = 0.0;
    for (int ii = 1; ii <= 3; ++ii) {
      int i = tl[ip3[ii][1] - 1], j = tl[ip3[ii][2] - 1], m = tl[ip3[ii][3] - 1];
      a3 = X[i] * Z[j] + a3;
      a2 = X[i] * Z[m] + a2;
    }
    cil[nn - 1] = amen[nn + 1] * (a3 - a2) / 6.0;
    a2 = 0.0; a3 = 0.0;
    for (int ii = 1; ii <= 3; ++ii) {
      int i = tl[ip3[ii][1] - 1], j = tl[ip3[ii][2] - 1], m = tl[ip3[ii][3] - 1];
      a3 = X[i] * Y[j] + a3;
      a2 = X[i] * Y[m] + a2;
    }
    dil[nn - 1] = amen[nn] * (a3 - a2) / 6.0;
  }
}

static double areas(const int* tl, const double* X, const double* Y) {
  // IP3 DATA (cathy_main.f:2490): IP3(:,1)=1,2,3 IP3(:,2)=2,3,1 IP3(:,3)=3,1,2
  const int ip3[4][4] = {{0, 0, 0, 0}, {0, 1, 2, 3}, {0, 2, 3, 1}, {0, 3, 1, 2}};
  double a2 = 0.0, a3 = 0.0;
  for (int ii = 1; ii <= 3; ++ii) {
    int i = tl[ip3[ii][1] - 1], j = tl[ip3[ii][2] - 1], m = tl[ip3[ii][3] - 1];
    a3 = X[i] * Y[j] + a3;
    a2 = X[i] * Y[m] + a2;
  }
  return 0.5 * (a3 - a2);
}

// STRPIC / STRNEW: fixed-stride sorted insertion (strpic.f:8-104,
// strnew.f:8-...), then TOPOL and compaction.
static void str_build(int n, int nt, const ivec& tetra, int n1, bool sym,
                      ivec& topol, ivec& ja, int& nterm) {
  int nt0 = n1 * n;
  ivec jb(nt0 + 2, 0);
  if (sym) {
    jb[1] = 1;
    for (int k = 1; k <= nt0 - 1; ++k)
      if ((k / n1) * n1 == k) jb[k + 1] = k / n1 + 1;
  }
  for (int k = 1; k <= nt; ++k) {
    int i1[5];
    int i2[5];
    for (int i = 1; i <= 4; ++i) i2[i] = tetra[(k - 1) * 5 + i - 1];
    for (int j = 1; j <= 4; ++j) {
      int kkk = 1, kk = i2[1];
      for (int i = 2; i <= 4; ++i)
        if (i2[i] < kk) { kk = i2[i]; kkk = i; }
      i1[j] = kk;
      i2[kkk] = 2147483647;
    }
    int ilo = sym ? 1 : 1, ihi = sym ? 3 : 4;
    for (int i = ilo; i <= ihi; ++i) {
      int llo = sym ? i + 1 : 1;
      for (int l = llo; l <= 4; ++l) {
        int m = sym ? n1 * (i1[i] - 1) + l - (i + 1) + 2 : n1 * (i1[i] - 1) + l;
        int mcontr = n1 * i1[i];
        for (;;) {
          if (i1[l] < jb[m]) {
            // shift right and insert at m
            int mm = m;
            do {
              mm++;
              if (mm - mcontr >= 0) { fprintf(stderr, "oracle: increase N1\n"); abort(); }
            } while (jb[mm] != 0);
            while (mm > m) { jb[mm] = jb[mm - 1]; mm--; }
            jb[m] = i1[l];
            break;
          } else if (i1[l] == jb[m]) {
            break;
          } else {
            if (jb[m] == 0) { jb[m] = i1[l]; break; }
            m++;
            if (m - mcontr >= 0) { fprintf(stderr, "oracle: increase N1\n"); abort(); }
          }
        }
      }
    }
  }
  topol.assign(n + 2, 0);
  topol[1] = 1;
  int m = 1, j = 1;
  for (int k = 1; k <= nt0; k += n1) {
    for (int i = 1; i <= n1; ++i)
      if (jb[k + i - 1] != 0) m++;
    j++;
    topol[j] = m;
  }
  ja.assign(1, 0);
  for (int k = 1; k <= nt0; ++k)
    if (jb[k] != 0) ja.push_back(jb[k]);
  nterm = (int)ja.size() - 1;
}

bool Oracle::build_mesh(const orc_dem_t* d) {
  // IVERT 3 needs the per-node DEPTH map of gen3d.f:67-68: not an input here
  if (d->ivert != 0 && d->ivert != 1 && d->ivert != 2 && d->ivert != 4) return false;
  nrow = d->nrow; ncol = d->ncol; nstr = d->nstr;
  // TRIANGOLI with DOSTEP=1
  vector<int> nodi((nrow + 2) * (ncol + 2), 0);
  auto NODI = [&](int i, int j) -> int& { return nodi[i * (ncol + 2) + j]; };
  auto DEM = [&](int i, int j) { return d->dem[(i - 1) * ncol + (j - 1)]; };
  auto ZONE = [&](int i, int j) { return d->zone ? d->zone[(i - 1) * ncol + (j - 1)] : 1; };
  for (int i = 1; i <= nrow; ++i)
    for (int j = 1; j <= ncol; ++j)
      if (DEM(i, j) != 0.0) {
        NODI(i, j) = 1; NODI(i + 1, j) = 1; NODI(i + 1, j + 1) = 1; NODI(i, j + 1) = 1;
      }
  dvec x2(1), y2(1);
  int inod = 0;
  for (int i = 1; i <= nrow + 1; ++i)
    for (int j = 1; j <= ncol + 1; ++j)
      if (NODI(i, j) == 1) {
        inod++;
        x2.push_back(d->west + (j - 1) * d->delta_x);
        y2.push_back(d->south + (nrow - i + 1) * d->delta_y);
        NODI(i, j) = inod;
      }
  nnod = inod;
  triang.assign(1 * 4, 0);  // dummy element 0
  dvec eltria(1);
  int itria = 0;
  nzone = 1;
  for (int i = 1; i <= nrow; ++i)
    for (int j = 1; j <= ncol; ++j) {
      if (DEM(i, j) == 0.0) continue;
      double e = DEM(i, j) * d->factor / 1;
      int zn = ZONE(i, j);
      nzone = std::max(nzone, zn);
      itria++;
      eltria.push_back(e);
      triang.push_back(NODI(i, j)); triang.push_back(NODI(i + 1, j));
      triang.push_back(NODI(i + 1, j + 1)); triang.push_back(zn);
      itria++;
      eltria.push_back(e);
      triang.push_back(NODI(i, j)); triang.push_back(NODI(i + 1, j + 1));
      triang.push_back(NODI(i, j + 1)); triang.push_back(zn);
    }
  ntri = itria;
  // TPNODI2D
  dvec z2(nnod + 1, 0.0);
  ivec tp2(nnod + 1, 0);
  for (int k = 1; k <= ntri; ++k)
    for (int ii = 1; ii <= 3; ++ii) {
      int nd = triang[k * 4 + ii - 1];
      z2[nd] += eltria[k];
      tp2[nd] += 1;
    }
  for (int k = 1; k <= nnod; ++k) {
    if (tp2[k] == 0) return false;
    z2[k] = z2[k] / tp2[k];
  }
  // RIORD on triangles (grdsys.f)
  riord(ntri, triang.data() + 4, 3);
  n = nnod * (nstr + 1);
  nt = 3 * ntri * nstr;
  x.assign(n + 1, 0.0); y.assign(n + 1, 0.0); z.assign(n + 1, 0.0);
  for (int i = 1; i <= nnod; ++i) { x[i] = x2[i]; y[i] = y2[i]; z[i] = z2[i]; }
  // AREA2D
  arenod.assign(nnod + 1, 0.0);
  const double r3 = 1.0 / 3.0;
  for (int iel = 1; iel <= ntri; ++iel) {
    int tl[3] = {triang[iel * 4], triang[iel * 4 + 1], triang[iel * 4 + 2]};
    double are = areas(tl, x.data(), y.data());
    if (are == 0.0) return false;
    double are3 = std::fabs(are) * r3;
    for (int q = 0; q < 3; ++q) arenod[tl[q]] += are3;
  }
  // GEN3D
  tetra.assign(5 * nt, 0);
  for (int j = 1; j <= nstr; ++j)
    for (int i = 1; i <= ntri; ++i) {
      int ntet = 3 * ((j - 1) * ntri + i - 1);
      const int* tr = &triang[i * 4];
      int* t1 = &tetra[(ntet) * 5];
      int* t2 = &tetra[(ntet + 1) * 5];
      int* t3 = &tetra[(ntet + 2) * 5];
      t1[0] = (j - 1) * nnod + tr[0]; t1[1] = (j - 1) * nnod + tr[1];
      t1[2] = (j - 1) * nnod + tr[2]; t1[3] = j * nnod + tr[0]; t1[4] = tr[3];
      t2[0] = t1[3]; t2[1] = j * nnod + tr[1]; t2[2] = j * nnod + tr[2];
      t2[3] = t1[2]; t2[4] = tr[3];
      t3[0] = t1[1]; t3[1] = t1[2]; t3[2] = t2[1]; t3[3] = t1[3]; t3[4] = tr[3];
    }
  double zmin = RMAX;
  for (int i = 1; i <= nnod; ++i) if (z[i] < zmin) zmin = z[i];
  for (int i = 1; i <= nnod; ++i) {
    double zthick = (z[i] - zmin) + d->base;
    double zrsum = 0.0;
    for (int j = 1; j <= nstr; ++j) {
      int kk = j * nnod + i;
      x[kk] = x[i]; y[kk] = y[i];
      zrsum = zrsum + d->zratio[j - 1];
      if (d->ivert == 0) z[kk] = z[i] - zrsum * d->base;
      else if (d->ivert == 1) z[kk] = z[i] - zrsum * zthick;
      else if (d->ivert == 2) z[kk] = zmin - zrsum * d->base;
      else if (d->ivert == 4) {
        z[kk] = z[i] - zrsum * d->base;
        if (j == nstr) z[kk] = zmin - d->base;
      } else z[kk] = z[i] - zrsum * d->base;
    }
  }
  tetra_gen3d = tetra;
  if (parm.iopt == 1) riord(nt, tetra.data(), 4);
  // VOLBAS
  volnod.assign(n + 1, 0.0); volu.assign(nt + 1, 0.0); volur.assign(nt + 1, 0.0);
  ivol.assign(nt + 1, 0);
  bi.assign(4 * nt + 4, 0.0); ci.assign(4 * nt + 4, 0.0); di.assign(4 * nt + 4, 0.0);
  const double r4 = 0.25;
  for (int iel = 1; iel <= nt; ++iel) {
    const int* tl = &tetra[(iel - 1) * 5];
    double vol = volums(tl, x.data(), y.data(), z.data());
    basis6(tl, x.data(), y.data(), z.data(), &bi[(iel - 1) * 4],
           &ci[(iel - 1) * 4], &di[(iel - 1) * 4]);
    if (vol == 0.0) return false;
    double vol4 = std::fabs(vol) * r4;
    for (int q = 0; q < 4; ++q) volnod[tl[q]] += vol4;
    ivol[iel] = 1;
    if (vol < 0.0) { ivol[iel] = -1; vol = -vol; }
    volu[iel] = vol;
    volur[iel] = 1.0 / vol;
  }
  // LOCMAS
  for (int k = 1; k <= 4; ++k)
    for (int i = k; i <= 4; ++i) {
      if (parm.lump == 0) lmass[k][i] = (k == i) ? 1.0 / 10.0 : 1.0 / 20.0;
      else lmass[k][i] = (k == i) ? 1.0 / 4.0 : 0.0;
    }
  for (int k = 2; k <= 4; ++k)
    for (int i = 1; i <= k - 1; ++i) lmass[k][i] = lmass[i][k];
  // STRPIC/TETPIC or STRNEW/TETNEW/TOPIA (cathy_main.f:2598-2606)
  int n1 = 40;
  str_build(n, nt, tetra, n1, parm.iopt == 1, topol, ja, nterm);
  tetja.assign(16 * nt, 0);
  for (int iel = 1; iel <= nt; ++iel)
    for (int i = 1; i <= 4; ++i) {
      int ii = T(i, iel);
      for (int j = (parm.iopt == 1 ? i : 1); j <= 4; ++j) {
        int jj = T(j, iel);
        int ind = topol[ii] - 1;
        do { ind++; } while (ja[ind] != jj);
        tetja[(iel - 1) * 16 + (j - 1) * 4 + (i - 1)] = ind;
      }
    }
  ia.assign(nterm + 1, 0);
  for (int k = 1; k <= n; ++k)
    for (int m = topol[k]; m < topol[k + 1]; ++m) ia[m] = k;
  (void)IP4;
  return true;
}

// TPNODI (tpnodi.f:9-99) for POROS, ELSTOR and the VG cell parameters
void Oracle::tpnodi(const orc_soil_t* s) {
  pnodi.assign(n + 1, 0.0); snodi.assign(n + 1, 0.0); vgn.assign(n + 1, 0.0);
  vgrmc.assign(n + 1, 0.0); vgpsat.assign(n + 1, 0.0); tp.assign(n + 1, 0);
  for (int k = 1; k <= nt; ++k) {
    int mtype = T(5, k);
    int istr = istr_of(k);
    int id = idx(istr, mtype);
    for (int ii = 1; ii <= 4; ++ii) {
      int nd = T(ii, k);
      pnodi[nd] += poros[id];
      snodi[nd] += elstor[id];
      vgn[nd] += vgncell[id];
      vgrmc[nd] += vgrmccell[id];
      vgpsat[nd] += vgpsatcell[id];
      tp[nd] += 1;
    }
  }
  for (int k = 1; k <= n; ++k) {
    pnodi[k] /= tp[k]; snodi[k] /= tp[k]; vgn[k] /= tp[k];
    vgpsat[k] /= tp[k]; vgrmc[k] /= tp[k];
  }
  (void)s;
}

// CHPARM for IVGHU=0 (chparm.f:24-45)
void Oracle::chparm() {
  vgm.assign(n + 1, 0); vgn1.assign(n + 1, 0); vgnr.assign(n + 1, 0);
  vgmm1.assign(n + 1, 0); vgpsn.assign(n + 1, 0); vgmr.assign(n + 1, 0);
  vgm52.assign(n + 1, 0); vgpnot.assign(n + 1, 0);
  for (int i = 1; i <= n; ++i) {
    vgm[i] = (vgn[i] - 1.0) / vgn[i];
    vgn1[i] = vgn[i] - 1.0;
    vgnr[i] = 1.0 / vgn[i];
    vgmm1[i] = vgm[i] - 1.0;
    vgpsn[i] = std::pow(std::fabs(vgpsat[i]), vgn[i]);
    vgmr[i] = 1.0 / vgm[i];
    vgm52[i] = 2.5 * vgm[i];
    vgpnot[i] = (pnodi[i] - vgrmc[i]) / pnodi[i];
  }
}

// ---- atmospheric BCs (atmone.f, atmnxt.f, atmbak.f) ----
void Oracle::atm_read_next(double& t, dvec& v, bool& ok) {
  if (atm_next >= natm) { ok = false; return; }
  t = atm_t[atm_next];
  v.assign(nnod + 1, 0.0);
  if (hspatm != 0) {
    for (int i = 1; i <= nnod; ++i) v[i] = atm_v[(size_t)atm_next];
  } else {
    for (int i = 1; i <= nnod; ++i) v[i] = atm_v[(size_t)atm_next * nnod + i - 1];
  }
  atm_next++;
  ok = true;
}

void Oracle::atmone() {
  htiatm = 0;
  atmtim[1] = 0.0; atmtim[2] = 0.0;
  for (int k = 1; k <= 3; ++k) atminp[k].assign(nnod + 1, 0.0);
  ifatm.assign(nnod + 1, 0); ifatmp.assign(nnod + 1, 0);
  atmpot.assign(nnod + 1, 0.0); atmact.assign(nnod + 1, 0.0);
  atmold.assign(nnod + 1, 0.0);
  bool ok;
  double t;
  dvec v;
  atm_read_next(t, v, ok);
  if (!ok) {
    htiatm = 1;
  } else {
    atmtim[3] = t;
    atminp[3] = v;
    if (atmtim[3] <= 0.0)
      for (int i = 1; i <= nnod; ++i) atmold[i] = atminp[3][i] * arenod[i];
    while (time > atmtim[3]) {
      atmtim[1] = atmtim[2]; atmtim[2] = atmtim[3];
      atminp[1] = atminp[2]; atminp[2] = atminp[3];
      atm_read_next(t, v, ok);
      if (!ok) { htiatm = 1; break; }
      atmtim[3] = t;
      atminp[3] = v;
    }
    if (atmtim[3] > atmtim[2]) {
      for (int i = 1; i <= nnod; ++i) {
        double slope = (atminp[3][i] - atminp[2][i]) / (atmtim[3] - atmtim[2]);
        if (ieto != 0) slope = 0.0;
        atmpot[i] = (atminp[2][i] + slope * (time - atmtim[2])) * arenod[i];
      }
    } else {
      for (int i = 1; i <= nnod; ++i) atmpot[i] = atminp[3][i] * arenod[i];
    }
  }
  for (int i = 1; i <= np; ++i)
    if (contp[i] <= nnod) { ifatm[contp[i]] = -1; ifatmp[contp[i]] = -1; }
  for (int i = 1; i <= nq; ++i)
    if (contq[i] <= nnod) { ifatm[contq[i]] = -1; ifatmp[contq[i]] = -1; }
  for (int e = 0; e < nsfn; ++e)  // atmone.f:112-119
    if (sfnode[e] <= nnod) { ifatm[sfnode[e]] = -1; ifatmp[sfnode[e]] = -1; }
  for (int i = 1; i <= nnod; ++i) {
    if (ifatm[i] == -1) continue;
    if (pnew[i] >= pondh_min) { ifatm[i] = 2; ifatmp[i] = 2; continue; }
    if (pnew[i] >= 0.0 && atmpot[i] > 0.0) ifatm[i] = 1;
    if (ptimep[i] >= 0.0 && atmold[i] > 0.0) ifatmp[i] = 1;
    if (pnew[i] <= pmin && atmpot[i] < 0.0) { pnew[i] = pmin; ifatm[i] = 1; }
    if (ptimep[i] <= pmin && atmold[i] < 0.0) { ptimep[i] = pmin; ifatmp[i] = 1; }
  }
  for (int i = 1; i <= nnod; ++i) {
    if (ifatm[i] == 0) atmact[i] = (atmpot[i] >= 0.0) ? atmpot[i] : (1.0 - scf) * atmpot[i];
    else atmact[i] = 0.0;
    if (ifatmp[i] == 1 || ifatmp[i] == 2) atmold[i] = 0.0;
  }
}

void Oracle::atmnxt() {
  if (htiatm == 0) {
    bool ok = true;
    double t;
    dvec v;
    while (time > atmtim[3]) {
      atmtim[1] = atmtim[2]; atmtim[2] = atmtim[3];
      atminp[1] = atminp[2]; atminp[2] = atminp[3];
      atm_read_next(t, v, ok);
      if (!ok) { htiatm = 1; break; }
      atmtim[3] = t;
      atminp[3] = v;
    }
    for (int i = 1; i <= nnod; ++i) {
      if (atmtim[3] > atmtim[2]) {
        double slope = (atminp[3][i] - atminp[2][i]) / (atmtim[3] - atmtim[2]);
        if (ieto != 0) slope = 0.0;
        atmpot[i] = (atminp[2][i] + slope * (time - atmtim[2])) * arenod[i];
      } else {
        atmpot[i] = atminp[3][i] * arenod[i];
      }
      if (ifatm[i] == 0) atmact[i] = (atmpot[i] >= 0.0) ? atmpot[i] : (1.0 - scf) * atmpot[i];
    }
  }
  for (int i = 1; i <= np; ++i) if (contp[i] <= nnod) ifatm[contp[i]] = -1;
  for (int i = 1; i <= nq; ++i) if (contq[i] <= nnod) ifatm[contq[i]] = -1;
  for (int e = 0; e < nsfn; ++e)  // atmnxt.f:94-101
    if (sfnode[e] <= nnod) ifatm[sfnode[e]] = -1;
}

void Oracle::atmbak() {
  if (atmtim[1] >= atmtim[2]) return;
  for (int i = 1; i <= nnod; ++i) {
    double slope = (atminp[2][i] - atminp[1][i]) / (atmtim[2] - atmtim[1]);
    if (ieto != 0) slope = 0.0;
    atmpot[i] = (atminp[1][i] + slope * (time - atmtim[1])) * arenod[i];
    if (ifatm[i] == 0) atmact[i] = (atmpot[i] >= 0.0) ? atmpot[i] : (1.0 - scf) * atmpot[i];
  }
}

// SWITCH_OLD (switch_old.f:12-53)
void Oracle::switch_old() {
  for (int i = 1; i <= nnod; ++i) {
    if (ifatm[i] == -1) continue;
    if (ifatm[i] == 1 && pnew[i] >= 0.0) {
      if (atmpot[i] < 0.0 || atmact[i] > atmpot[i]) {
        ifatm[i] = 0; atmact[i] = atmpot[i]; continue;
      }
    }
    if (ifatm[i] == 1 && pnew[i] <= pmin) {
      if (atmpot[i] > 0.0 || atmact[i] < atmpot[i]) {
        ifatm[i] = 0; atmact[i] = atmpot[i]; continue;
      }
    }
    if (ifatm[i] == 0 && pnew[i] >= 0.0 && atmpot[i] >= 0.0) {
      ifatm[i] = 1; pnew[i] = 0.0; continue;
    }
    if (ifatm[i] == 0 && pnew[i] <= pmin && atmpot[i] < 0.0) {
      ifatm[i] = 1; pnew[i] = pmin; continue;
    }
  }
}

// PICUNS -> CHPIC0 / CHPIC1 + NODELT (picuns.f, chpic0.f:23-36, chpic1.f)
void Oracle::chpic() {
  for (int i = 1; i <= n; ++i) {
    swnew[i] = vgpnot[i] * fvgse(pnew[i], i) + vgrmc[i] / pnodi[i];
    swtimep[i] = vgpnot[i] * fvgse(ptimep[i], i) + vgrmc[i] / pnodi[i];
  }
  for (int i = 1; i <= n; ++i) {
    double psi = ptnew[i];
    double se = fvgse(psi, i);
    sw[i] = vgpnot[i] * se + vgrmc[i] / pnodi[i];
    if (kslope == 0) {
      double dse = fvgdse(psi, i);
      etai[i] = sw[i] * snodi[i] + pnodi[i] * vgpnot[i] * dse;
      et1[i] = sw[i] * snodi[i];
      et2[i] = vgpnot[i] * dse;
    } else {
      double dp = psi - ptold[i];
      if (std::fabs(dp) < tolksl) {
        double dse = fvgdse(psi, i);
        etai[i] = sw[i] * snodi[i] + pnodi[i] * vgpnot[i] * dse;
        et1[i] = sw[i] * snodi[i];
        et2[i] = vgpnot[i] * dse;
      } else {
        double seold = fvgse(ptold[i], i);
        etai[i] = sw[i] * snodi[i] + pnodi[i] * vgpnot[i] * ((se - seold) / dp);
        et1[i] = sw[i] * snodi[i];
        et2[i] = vgpnot[i] * ((se - seold) / dp);
      }
    }
    ckrw[i] = fvgkr(psi, se, i);
  }
  nodelt(ckrw, ckrwe);
  nodelt(etai, etae);
  nodelt(et1, et1e);
  nodelt(pnodi, pel);
}

// PICARD (picard.f:8-205) with ASSPIC, RHSPIC, CFMATP, RHSGRV, BCPIC, SYMSLV,
// SHLPIC.  Nudging is zero (NUDN=0).
void Oracle::picard() {
  chpic();
  std::fill(coef1.begin(), coef1.end(), 0.0);
  std::fill(coef2.begin(), coef2.end(), 0.0);
  std::fill(coef4.begin(), coef4.end(), 0.0);
  std::fill(coef5.begin(), coef5.end(), 0.0);
  // ASSPIC (asspic.f:26-51)
  asspic_state();
  // RHSPIC (rhspic.f:22-38)
  for (int k = 1; k <= n; ++k) tnoti[k] = 0.0;
  double rdt = 1.0 / deltat;
  for (int k = 1; k <= n; ++k) {
    int i = topol[k], j = topol[k + 1] - 1;
    for (int m = i; m <= j; ++m) {
      double coef = coef2[m] * rdt, coeff = coef4[m] * rdt;
      int jm = ja[m];
      tnoti[k] = tnoti[k] - coef1[m] * ptnew[jm] - coef * (pnew[jm] - ptimep[jm]) -
                 coeff * (swnew[jm] - swtimep[jm]);
      if (m != i)
        tnoti[jm] = tnoti[jm] - coef1[m] * ptnew[k] - coef * (pnew[k] - ptimep[k]) -
                    coeff * (swnew[k] - swtimep[k]);
    }
  }
  // CFMATP (cfmatp.f:20-26)
  for (int k = 1; k <= n; ++k) coef5[topol[k]] = coef4[topol[k]] * et2[k];
  for (int k = 1; k <= nterm; ++k)
    coef1[k] = parm.tetaf * coef1[k] + coef2[k] * rdt + coef5[k] * rdt;
  // RHSGRV (rhsgrv.f:20-30)
  for (int ke = 1; ke <= nt; ++ke) {
    int istr = istr_of(ke);
    double t3 = ckrwe[ke] * permz[idx(istr, T(5, ke))];
    for (int in = 1; in <= 4; ++in) {
      int nd = T(in, ke);
      double t1 = t3 * D(in, ke) * ivol[ke];
      tnoti[nd] = tnoti[nd] - t1;
    }
  }
  xt5 = tnoti;  // VCOPYR(N,XT5,TNOTI)
  // BCPIC (bcpic.f:33-86)
  for (int k = 1; k <= np; ++k) {
    int j = contp[k];
    int ind = topol[j];
    tnoti[j] = 0.0;
    lhsp[k] = coef1[ind];
    coef1[ind] = 1.0e-9 * RMAX;
  }
  numdir = np;
  for (int k = 1; k <= np; ++k) noddir[k] = contp[k];
  for (int e = 0; e < nsfn; ++e)
    if (sfex[e] == 1) {
      const int inod = sfnode[e];
      numdir++;
      noddir[numdir] = inod;
      int ind = topol[inod];
      tnoti[inod] = 0.0;
      lhssf[e] = coef1[ind];
      coef1[ind] = 1.0e-9 * RMAX;
    }
  for (int k = 1; k <= nnod; ++k) {
    if (ifatm[k] == 1 || ifatm[k] == 2) {
      numdir++;
      noddir[numdir] = k;
      int ind = topol[k];
      tnoti[k] = 0.0;
      lhsatm[k] = coef1[ind];
      coef1[ind] = 1.0e-9 * RMAX;
    }
  }
  for (int k = 1; k <= nq; ++k) tnoti[contq[k]] += q[k];
  for (int k = 1; k <= nnod; ++k)
    if (ifatm[k] == 0)
      tnoti[k] = tnoti[k] + (parm.tetaf * atmact[k] + (1.0 - parm.tetaf) * atmold[k]);
  for (int k = 1; k <= n; ++k) tnoti[k] = tnoti[k] - qtranie[k];
  // SYMSLV
  int niter = 0;
  symslv(n, nterm, numdir, &niter, parm.itmxcg, parm.tolcg, noddir.data(),
         ja.data(), topol.data(), pdiff.data(), tnoti.data(), coef1.data(),
         coef2.data(), scr.data(), &lin_err, &lin_res, parm.precond == 1);
  itlin += niter;
  nitert += niter;
  niter_last = niter;
  // PNEW = PNEW + PDIFF, SHLPIC (shlpic.f:30-56)
  for (int k = 1; k <= n; ++k) pnew[k] = pnew[k] + pdiff[k];
  for (int i = 1; i <= np; ++i) {
    int j = contp[i];
    pnew[j] = presc[i];
    coef1[topol[j]] = lhsp[i];
  }
  for (int e = 0; e < nsfn; ++e)
    if (sfex[e] == 1) {
      pnew[sfnode[e]] = 0.0;
      coef1[topol[sfnode[e]]] = lhssf[e];
    }
  for (int i = 1; i <= nnod; ++i)
    if (ifatm[i] == 1 || ifatm[i] == 2) {
      pnew[i] = pold[i];
      coef1[topol[i]] = lhsatm[i];
    }
}

// NEWTON (newton.f) with NEWUNS/CHNEW0, ASSNEW, RHSNEW, CFMATN, RHSGRV, BCNEW,
// NSYSLV, SHLNEW.  KSLOPE=0 only.
void Oracle::newton() {
  // NEWUNS -> CHNEW0 (chnew0.f IVGHU=0) or, for KSLOPE=1, CHNEW1
  // (chnew1.f:27-53: chord slopes between PTOLD and PTNEW once they differ by
  // TOLKSL or more) + NODELT
  for (int i = 1; i <= n; ++i) {
    double psi = ptnew[i];
    double se = fvgse(psi, i);
    sw[i] = vgpnot[i] * se + vgrmc[i] / pnodi[i];
    ckrw[i] = fvgkr(psi, se, i);
    const double dp = psi - ptold[i];
    if (kslope == 0 || std::fabs(dp) < tolksl) {
      double dsedp = fvgdse(psi, i);
      double dswdp = vgpnot[i] * dsedp;
      etai[i] = sw[i] * snodi[i] + pnodi[i] * dswdp;
      detai[i] = dswdp * snodi[i] + pnodi[i] * vgpnot[i] * fvgdds(psi, i);
      dckrw[i] = fvgdkr(psi, i);
    } else {
      const double pold = ptold[i];
      const double seold = fvgse(pold, i);
      const double dsenew = fvgdse(psi, i), dseold = fvgdse(pold, i);
      const double dswdp = vgpnot[i] * ((se - seold) / dp);
      const double krold = fvgkr(pold, seold, i);
      etai[i] = sw[i] * snodi[i] + pnodi[i] * dswdp;
      detai[i] = dswdp * snodi[i] + pnodi[i] * vgpnot[i] * ((dsenew - dseold) / dp);
      dckrw[i] = (ckrw[i] - krold) / dp;
    }
  }
  nodelt(ckrw, ckrwe);
  nodelt(etai, etae);
  std::fill(coef1.begin(), coef1.end(), 0.0);
  std::fill(coef2.begin(), coef2.end(), 0.0);
  std::fill(coef3.begin(), coef3.end(), 0.0);
  // ASSNEW (assnew.f:30-87)
  double rdt = 1.0 / deltat;
  double tetaf = parm.tetaf;
  for (int iel = 1; iel <= nt; ++iel) {
    int istr = istr_of(iel);
    int id = idx(istr, T(5, iel));
    double ve = volu[iel] * etae[iel];
    double pv1 = permx[id] * volur[iel], pv2 = permy[id] * volur[iel],
           pv3 = permz[id] * volur[iel];
    double pvk1 = pv1 * ckrwe[iel], pvk2 = pv2 * ckrwe[iel], pvk3 = pv3 * ckrwe[iel];
    double tpi = tetaf * permz[id] * ivol[iel];
    double tvd = tetaf * volu[iel] * rdt;
    for (int k = 1; k <= 4; ++k) {
      int knod = T(k, iel);
      double pvb = pv1 * B(k, iel), pvc = pv2 * C(k, iel), pvd = pv3 * D(k, iel);
      double pvkb = pvk1 * B(k, iel), pvkc = pvk2 * C(k, iel), pvkd = pvk3 * D(k, iel);
      double sum = 0.0, sum1 = 0.0;
      for (int m = 1; m <= 4; ++m) {
        int mnod = T(m, iel);
        sum = sum + (pvb * B(m, iel) + pvc * C(m, iel) + pvd * D(m, iel)) * ptnew[mnod];
        sum1 = sum1 + lmass[k][m] * (pnew[mnod] - ptimep[mnod]);
      }
      double tsumtd = tetaf * sum + tpi * D(k, iel);
      double sum1tv = sum1 * tvd;
      for (int l = 1; l <= 4; ++l) {
        int lnod = T(l, iel);
        int ind = TJ(k, l, iel);
        if (lnod >= knod) {
          coef1[ind] = coef1[ind] + pvkb * B(l, iel) + pvkc * C(l, iel) + pvkd * D(l, iel);
          coef2[ind] = coef2[ind] + ve * lmass[k][l];
        }
        coef3[ind] = coef3[ind] + dckrw[lnod] * tsumtd + detai[lnod] * sum1tv;
      }
    }
    for (int k = 1; k <= 4; ++k) {
      int knod = T(k, iel);
      for (int l = 1; l <= 4; ++l) {
        int lnod = T(l, iel);
        if (lnod < knod) {
          int ind = TJ(k, l, iel), inds = TJ(l, k, iel);
          coef1[ind] = coef1[inds];
          coef2[ind] = coef2[inds];
        }
      }
    }
  }
  // RHSNEW (rhsnew.f)
  for (int k = 1; k <= n; ++k) {
    tnoti[k] = 0.0;
    for (int m = topol[k]; m < topol[k + 1]; ++m)
      tnoti[k] = tnoti[k] - coef1[m] * ptnew[ja[m]] -
                 coef2[m] * (pnew[ja[m]] - ptimep[ja[m]]) * rdt;
  }
  // CFMATN
  for (int k = 1; k <= nterm; ++k)
    coef1[k] = tetaf * coef1[k] + coef2[k] * rdt + coef3[k];
  // RHSGRV
  for (int ke = 1; ke <= nt; ++ke) {
    double t3 = ckrwe[ke] * permz[idx(istr_of(ke), T(5, ke))];
    for (int in = 1; in <= 4; ++in) {
      int nd = T(in, ke);
      tnoti[nd] = tnoti[nd] - t3 * D(in, ke) * ivol[ke];
    }
  }
  xt5 = tnoti;
  // BCNEW (bcnew.f)
  auto diagpos = [&](int j) {
    int ind = topol[j] - 1;
    do { ind++; } while (ja[ind] != j);
    return ind;
  };
  for (int k = 1; k <= np; ++k) {
    int j = contp[k];
    tnoti[j] = 0.0;
    int ind = diagpos(j);
    lhsp[k] = coef1[ind];
    coef1[ind] = 1.0e-9 * RMAX;
  }
  numdir = np;
  for (int k = 1; k <= np; ++k) noddir[k] = contp[k];
  for (int e = 0; e < nsfn; ++e)
    if (sfex[e] == 1) {
      const int inod = sfnode[e];
      numdir++;
      noddir[numdir] = inod;
      tnoti[inod] = 0.0;
      int ind = diagpos(inod);
      lhssf[e] = coef1[ind];
      coef1[ind] = 1.0e-9 * RMAX;
    }
  for (int k = 1; k <= nnod; ++k)
    if (ifatm[k] == 1 || ifatm[k] == 2) {
      numdir++;
      noddir[numdir] = k;
      tnoti[k] = 0.0;
      int ind = diagpos(k);
      lhsatm[k] = coef1[ind];
      coef1[ind] = 1.0e-9 * RMAX;
    }
  for (int k = 1; k <= nq; ++k) tnoti[contq[k]] += q[k];
  for (int k = 1; k <= nnod; ++k)
    if (ifatm[k] == 0)
      tnoti[k] = tnoti[k] + (tetaf * atmact[k] + (1.0 - tetaf) * atmold[k]);
  // NSYSLV
  int niter = nsyslv(parm.isolv, n, numdir, noddir.data(), parm.itmxcg,
                     parm.tolcg, ia.data(), ja.data(), topol.data(),
                     coef1.data(), coef2.data(), pdiff.data(), tnoti.data(),
                     &lin_err, &lin_res);
  itlin += niter;
  nitert += niter;
  niter_last = niter;
  for (int k = 1; k <= n; ++k) pnew[k] = pnew[k] + pdiff[k];
  // SHLNEW
  for (int i = 1; i <= np; ++i) {
    int j = contp[i];
    pnew[j] = presc[i];
    coef1[diagpos(j)] = lhsp[i];
  }
  for (int e = 0; e < nsfn; ++e)
    if (sfex[e] == 1) {
      pnew[sfnode[e]] = 0.0;
      coef1[diagpos(sfnode[e])] = lhssf[e];
    }
  for (int i = 1; i <= nnod; ++i)
    if (ifatm[i] == 1 || ifatm[i] == 2) {
      pnew[i] = pold[i];
      coef1[diagpos(i)] = lhsatm[i];
    }
}

// MASBAL (masbal.f:36-109) with BKPIC/BKNEW, STORMB and FLUXMB.
// Newton branch: the reference's STORMB reads a saturation array that the
// Newton branch never fills (flow3d.f declares SWNEW locally and only PICARD
// writes it), so its Newton storage change is not meaningful; the oracle
// evaluates SWNEW/SWTIMEP at the current and previous heads instead.
void Oracle::masbal() {
  double tetaf = parm.tetaf, tetafr = 1.0 / tetaf;
  // back-calculated fluxes: SCR = A * PDIFF - XT5 (bkpic.f:25-53)
  std::fill(scr.begin(), scr.begin() + n + 1, 0.0);
  if (parm.iopt == 1) {
    for (int k = 1; k <= n; ++k) {
      int i = topol[k], j = topol[k + 1] - 1;
      for (int m = i; m <= j; ++m) {
        int jm = ja[m];
        scr[k] += coef1[m] * pdiff[jm];
        if (m != i) scr[jm] += coef1[m] * pdiff[k];
      }
      scr[k] -= xt5[k];
    }
  } else {
    for (int k = 1; k <= n; ++k) {
      double s = 0.0;
      for (int m = topol[k]; m < topol[k + 1]; ++m) s += coef1[m] * pdiff[ja[m]];
      scr[k] = s - xt5[k];
    }
  }
  for (int i = 1; i <= np; ++i)
    qpnew[i] = (scr[contp[i]] - (1.0 - tetaf) * qpold[i]) * tetafr;
  for (int e = 0; e < nsfn; ++e)  // bkpic.f:44-51
    if (sfex[e] == 1) sfq[e] = (scr[sfnode[e]] - (1.0 - tetaf) * sfqp[e]) * tetafr;
  for (int k = 1; k <= nnod; ++k)
    if (ifatm[k] == 1 || ifatm[k] == 2)
      atmact[k] = (scr[k] - (1.0 - tetaf) * atmold[k]) * tetafr;
  if (parm.iopt != 1) {
    for (int i = 1; i <= n; ++i) {
      swnew[i] = vgpnot[i] * fvgse(pnew[i], i) + vgrmc[i] / pnodi[i];
      swtimep[i] = vgpnot[i] * fvgse(ptimep[i], i) + vgrmc[i] / pnodi[i];
    }
  }
  double deltam;
  if (deltat < 1.0e15) {
    deltam = 0.5 * deltat;
    dstore = 0.0;
    for (int k = 1; k <= n; ++k)
      dstore = dstore + volnod[k] * (snodi[k] * (swnew[k] + swtimep[k]) * 0.5 *
                                         (pnew[k] - ptimep[k]) +
                                     pnodi[k] * (swnew[k] - swtimep[k]));
  } else {
    deltam = 1.0;
    dstore = 0.0;
  }
  // FLUXMB (fluxmb.f)
  ndin = ndout = 0.0;
  for (int k = 1; k <= np; ++k) {
    if (qpnew[k] > 0.0) ndin += qpnew[k];
    else ndout += qpnew[k];
  }
  nnin = nnout = 0.0;
  for (int k = 1; k <= nq; ++k) {
    if (q[k] > 0.0) nnin += q[k];
    else nnout += q[k];
  }
  sfflw = 0.0;  // fluxmb.f:46-60 (SFFLAG(5) is a diagnostic only)
  for (int e = 0; e < nsfn; ++e)
    if (sfex[e] == 1) sfflw = sfflw + sfq[e];
  adin = adout = anin = anout = 0.0;
  for (int k = 1; k <= nnod; ++k) {
    if (ifatm[k] == -1) continue;
    if (ifatm[k] == 1 || ifatm[k] == 2) {
      if (atmact[k] > 0.0) adin += atmact[k];
      else adout += atmact[k];
    } else {
      if (atmact[k] > 0.0) anin += atmact[k];
      else anout += atmact[k];
    }
  }
  double vadin = (adin + adinp) * deltam, vadout = (adout + adoutp) * deltam;
  double vndin = (ndin + ndinp) * deltam, vndout = (ndout + ndoutp) * deltam;
  double vanin = (anin + aninp) * deltam, vanout = (anout + anoutp) * deltam;
  double vnnin = (nnin + nninp) * deltam, vnnout = (nnout + nnoutp) * deltam;
  const double vsfflw = (sfflw + sfflwp) * deltam;
  vnd = vndin + vndout;
  vnn = vnnin + vnnout;
  vin = vadin + vndin + vanin + vnnin;
  vout = vadout + vndout + vanout + vnnout + vsfflw;
  erras = vin + vout - dstore;
  if (deltat >= 1.0e15) errel = (vin != 0.0) ? 100.0 * erras / vin : 0.0;
  else errel = ((vin + vout) != 0.0) ? 100.0 * erras / (vin + vout) : 0.0;
}

// CONVER (conver.f) -> NORMS (norms.f:22-38) + SWITCH_OLD when allowed.
void Oracle::conver() {
  pl2 = fl2 = pinf = finf = 0.0;
  for (int k = 1; k <= n; ++k) {
    double diff = pnew[k] - pold[k];
    double difabs = std::fabs(diff);
    pl2 += diff * diff;
    fl2 += tnoti[k] * tnoti[k];
    if (difabs >= pinf) { pinf = difabs; pikmax = diff; ikmax = k; }
    double fabs_ = std::fabs(tnoti[k]);
    if (fabs_ >= finf) finf = fabs_;
  }
  pl2 = std::sqrt(pl2);
  fl2 = std::sqrt(fl2);
  orc_iter_rec_t rec;
  rec.nstep = nstep; rec.iter = iter; rec.niter = niter_last; rec.ikmax = ikmax;
  rec.deltat = deltat; rec.time = time; rec.pl2 = pl2; rec.pinf = pinf;
  rec.pnew_ik = pnew[ikmax]; rec.pold_ik = pold[ikmax]; rec.fl2 = fl2;
  rec.finf = finf; rec.lin_err = lin_err; rec.lin_res = lin_res;
  iter_recs.push_back(rec);
  if ((parm.l2norm == 0 && pinf <= parm.tolswi) ||
      (parm.l2norm != 0 && pl2 <= parm.tolswi))
    switch_old();
  if (nsfn > 0) {  // conver.f:82-104
    extall();
    ksfzer = (ksf == 0);
  }
}

// EXTALL (extall.f:27-55) + EXTCVG (extcvg.f): an exit node whose
// back-calculated flux is an inflow (SFQ >= 0) leaves the seepage face; a
// potential node with PNEW > 1e-8 becomes an exit node at PNEW = 0
// (DUPUIT = 0).  KSF counts the changed flags (SFEXIT = SFEX before).
void Oracle::extall() {
  ksf = 0;
  for (int e = 0; e < nsfn; ++e) {
    const int inod = sfnode[e];
    const int before = sfex[e];
    if (sfex[e] == 1) {
      if (sfq[e] >= 0.0) { sfex[e] = 0; sfq[e] = 0.0; }
    } else if (pnew[inod] > 1.0e-8) {
      pnew[inod] = 0.0;
      sfex[e] = 1;
    }
    if (sfex[e] != before) ksf++;
  }
}

// FLOW3D (flow3d.f:93-294); returns true when BCKSTP or NOBACK is set.
bool Oracle::flow3d(bool first_only) {
  bool lsfail;
  for (;;) {
    if (parm.iopt == 1) picard();
    else newton();
    lsfail = (niter_last >= parm.itmxcg);
    if (lsfail) klsfai++;
    masbal();
    if (parm.nlrelx == 1) {
      for (int k = 1; k <= n; ++k)
        pnew[k] = parm.omega * pnew[k] + (1.0 - parm.omega) * pold[k];
    }
    conver();
    if (first_only) return false;
    bool itagen = iter < parm.ituns;
    bool errgmx = (pl2 >= parm.ernlmx || pinf >= parm.ernlmx ||
                   fl2 >= parm.ernlmx || finf >= parm.ernlmx);
    bool normcv = (parm.l2norm == 0) ? (pinf <= parm.toluns) : (pl2 <= parm.toluns);
    if ((!lsfail && !errgmx && !normcv && itagen) ||
        (!lsfail && !errgmx && itagen && sfchek && !ksfzer)) {
      pold = pnew;
      ptold = ptnew;
      for (int k = 1; k <= n; ++k)
        ptnew[k] = parm.tetaf * pnew[k] + (1.0 - parm.tetaf) * ptimep[k];
      iter++;
      continue;
    }
    itrtot += iter;
    if ((!sfchek && !lsfail && !errgmx && normcv) ||
        (sfchek && !lsfail && !errgmx && normcv && ksfzer))
      return false;  // converged
    return true;  // back-step (DTGMIN) or abort (!DTGMIN)
  }
}

// TIMUPD (timupd.f:18-38)
void Oracle::timupd() {
  timep = time;
  if (iter < parm.ituns1) {
    deltat = deltat * parm.dtmagm + parm.dtmaga;
    if (deltat > parm.dtmax) deltat = parm.dtmax;
  }
  if (iter >= parm.ituns2) {
    deltat = deltat * parm.dtredm - parm.dtreds;
    if (deltat < parm.dtmin) deltat = parm.dtmin;
  }
  if ((time + deltat) >= parm.tmax) {
    deltat = parm.tmax - time;
    time = parm.tmax;
  } else {
    if ((time + 2 * deltat) > parm.tmax) deltat = (parm.tmax - time) / 2;
    time = time + deltat;
  }
  dtgmin = !(deltat <= parm.dtmin);
}

// BKSTEP (bkstep.f:54-166) for the subsurface-only case
void Oracle::bkstep() {
  pnew = ptimep;
  for (int e = 0; e < nsfn; ++e) { sfex[e] = sfexp[e]; sfq[e] = sfqp[e]; }  // bkstep.f:56-66
  for (int i = 1; i <= np; ++i) qpnew[i] = qpold[i];
  for (int i = 1; i <= nnod; ++i) { ifatm[i] = ifatmp[i]; atmact[i] = atmold[i]; }
  time = timep;
  deltat = deltat * parm.dtredm - parm.dtreds;
  if (deltat <= parm.dtmin) { deltat = parm.dtmin; dtgmin = false; }
  else dtgmin = true;
  time = time + deltat;
  kbackt++;
  kback++;
  iter = 1;
  nitert = 0;
  if (time > atmtim[2]) atmnxt();
  else atmbak();
  switch_old();
  pold = pnew;
  for (int k = 1; k <= n; ++k)
    ptnew[k] = parm.tetaf * pnew[k] + (1.0 - parm.tetaf) * ptimep[k];
  ptold = ptnew;
}

// ETRAN (etran.f:6-81): root water uptake QTRANIE of the new time step
// from PNEW before SWITCH_OLD and the new ATMPOT; with SCF = 0 the potential
// transpiration ETP is zero and so is QTRANIE.  The reference stops when a
// root zone reaches the bottom node (etran.f:60-65); orc_create rejects such
// a mesh instead.
void Oracle::etran() {
  for (int k = 1; k <= n; ++k) qtranie[k] = 0.0;
  if (scf <= 0.0) return;
  dvec btrani(n + 1, 0.0);
  dvec btran(nnod + 1, 0.0), omg(nnod + 1, 0.0), etp(nnod + 1, 0.0);
  for (int i = 1; i <= nnod; ++i) {
    const double* fp = &feddes[6 * (veg_type[i] - 1)];
    const double pcana = fp[0], pcref = fp[1], pcwlt = fp[2], zroot = fp[3], pz = fp[4];
    int j = 1;
    const double zsurf = z[i];
    double depth = 0.0;
    etp[i] = (atmpot[i] < 0.0) ? -1.0 * scf * atmpot[i] : 0.0;
    while (depth <= zroot) {
      const int k = (j - 1) * nnod + i;
      const double s1 = pcana, s2 = pcana + 1.0e-3;
      const double dz = (j == 1) ? (zsurf - z[k + nnod]) / 2.0 : (z[k - nnod] - z[k + nnod]) / 2.0;
      const double sh2o = pnew[k];
      double gx1 = (sh2o - pcwlt) / (pcref - pcwlt);
      gx1 = std::min(1.0, std::max(0.0, gx1));
      double gx2 = 1.0 - (sh2o - s1) / (s2 - s1);
      gx2 = std::min(1.0, std::max(0.0, gx2));
      const double gx = std::min(gx1, gx2);
      const double beta = (1 - depth / zroot) * std::exp(-1.0 * pz * depth / zroot);
      btrani[k] = std::max(0.0, beta * dz * gx);
      btran[i] = btran[i] + beta * dz;
      omg[i] = omg[i] + gx * beta * dz;
      j = j + 1;
      depth = zsurf - z[(j - 1) * nnod + i];  // in range: checked in orc_create
    }
    btran[i] = std::max(0.0, btran[i]);
    omg[i] = omg[i] / btran[i];
  }
  for (int i = 1; i <= nnod; ++i) {
    const double omgc = feddes[6 * (veg_type[i] - 1) + 5];
    for (int j = 1; j <= nstr + 1; ++j) {
      const int k = (j - 1) * nnod + i;
      qtranie[k] = etp[i] * btrani[k] / btran[i] / std::max(omg[i], omgc);
    }
  }
}

// One pass of the main time loop (cathy_main.f:2882-3843) for FL3D, no
// surface routing.  Returns 0 = step accepted, 1 = abort (no back-step
// possible), 2 = finished.
int Oracle::step() {
  if (finished) return 2;
  // input/interpolate BCs for the new time level, switching (cathy_main.f:2886-2945)
  atmnxt();
  etran();
  switch_old();
  pold = pnew;
  for (int k = 1; k <= n; ++k)
    ptnew[k] = parm.tetaf * pnew[k] + (1.0 - parm.tetaf) * ptimep[k];
  ptold = ptnew;
  for (;;) {
    for (int i = 1; i <= nnod; ++i) pold[i] = pnew[i];  // cathy_main.f:3100
    bool bad = flow3d(false);
    if (!bad) break;
    if (!dtgmin) {  // NOBACK
      finished = true;
      return 1;
    }
    bkstep();
  }
  // storage and mass-balance bookkeeping (cathy_main.f:3233-3290)
  for (int i = 1; i <= n; ++i) sw[i] = vgpnot[i] * fvgse(pnew[i], i) + vgrmc[i] / pnodi[i];
  store1 = 0.0;
  for (int i = 1; i <= n; ++i) store1 += sw[i] * volnod[i] * pnodi[i];
  store2 = store2 + dstore;
  vtot += vin + vout;
  cvin += vin; cvout += vout; cdstor += dstore; cerras += erras;
  caeras += std::fabs(erras);
  orc_step_rec_t rec;
  rec.nstep = nstep; rec.iter = iter; rec.nitert = nitert; rec.nback = kbackt;
  rec.deltat = deltat; rec.time = time; rec.store1 = store1; rec.store2 = store2;
  rec.dstore = dstore; rec.cdstor = cdstor; rec.vin = vin; rec.cvin = cvin;
  rec.vout = vout; rec.cvout = cvout; rec.erras = erras; rec.errel = errel;
  rec.cerras = cerras; rec.caeras = caeras;
  rec.sfflw = sfflw;
  rec.vnd = vnd;
  rec.vnn = vnn;
  step_recs.push_back(rec);
  adinp = adin; adoutp = adout; ndinp = ndin; ndoutp = ndout;
  aninp = anin; anoutp = anout; nninp = nnin; nnoutp = nnout;
  sfflwp = sfflw;  // cathy_main.f:3282, :3294-3300
  for (int e = 0; e < nsfn; ++e) { sfexp[e] = sfex[e]; sfqp[e] = sfq[e]; }
  for (int i = 1; i <= np; ++i) qpold[i] = qpnew[i];
  for (int i = 1; i <= nnod; ++i) { ifatmp[i] = ifatm[i]; atmold[i] = atmact[i]; }
  ptimep = pnew;
  if (deltat >= 1.0e15 || std::fabs(time - parm.tmax) <= 0.001 * deltat) {
    finished = true;
    return 0;
  }
  timupd();
  nstep++;
  iter = 1;
  nitert = 0;
  kbackt = 0;
  return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// C entry points
// ---------------------------------------------------------------------------
extern "C" {

void* orc_create(const orc_dem_t* dem, const orc_soil_t* soil,
                 const orc_parm_t* parm, const orc_bc_t* bc) {
  Oracle* o = new Oracle();
  o->parm = *parm;
  // NLRELX 2 (RELXOM's variable relaxation factor) is not restated
  if (parm->nlrelx != 0 && parm->nlrelx != 1) { delete o; return nullptr; }
  // NSYSLV restated for ISOLV 0 and -5 only (the Newton scheme's solvers)
  if (parm->iopt == 2 && parm->isolv != 0 && parm->isolv != -5) { delete o; return nullptr; }
  if (!o->build_mesh(dem)) { delete o; return nullptr; }
  int n = o->n, nt = o->nt, nnod = o->nnod, nstr = o->nstr;
  int nz = std::max(o->nzone, soil->nzone);
  o->nzone = nz;
  size_t tsz = (size_t)nz * nstr;
  auto cp = [&](const double* src, dvec& dst) { dst.assign(src, src + tsz); };
  cp(soil->permx, o->permx); cp(soil->permy, o->permy); cp(soil->permz, o->permz);
  cp(soil->elstor, o->elstor); cp(soil->poros, o->poros); cp(soil->vgn, o->vgncell);
  cp(soil->vgrmc, o->vgrmccell); cp(soil->vgpsat, o->vgpsatcell);
  o->pmin = soil->pmin; o->scf = soil->scf; o->kslope = soil->kslope;
  o->tolksl = soil->tolksl;
  o->pondh_min = (parm->isimgr <= 1) ? 1.0e10 : parm->pondh_min;  // datin.f:123
  // VEG_TYPE (datin.f:221-233): TRIANGOLI + TPNODI2D applied to the root
  // map, i.e. the mean of FACTOR * map over the triangles of each surface
  // node, truncated; the map must be active on the DEM's cells
  o->veg_type.assign(o->nnod + 1, 1);
  if (soil->scf > 0.0) {
    if (soil->nveg < 1 || !soil->feddes) { delete o; return nullptr; }
    o->feddes.assign(soil->feddes, soil->feddes + 6 * (size_t)soil->nveg);
    if (soil->root_map) {
      dvec sum(o->nnod + 1, 0.0);
      ivec cnt(o->nnod + 1, 0);
      int itria = 0;
      for (int i = 0; i < dem->nrow; ++i)
        for (int j = 0; j < dem->ncol; ++j) {
          const size_t c = (size_t)i * dem->ncol + j;
          if (dem->dem[c] == 0.0) continue;
          if (soil->root_map[c] == 0.0) { delete o; return nullptr; }
          const double e = soil->root_map[c] * dem->factor;
          for (int t = 0; t < 2; ++t) {
            ++itria;
            for (int v = 0; v < 3; ++v) {
              const int nd = o->triang[itria * 4 + v];
              sum[nd] += e;
              cnt[nd] += 1;
            }
          }
        }
      for (int i = 1; i <= o->nnod; ++i) o->veg_type[i] = (int)(sum[i] / cnt[i]);
    }
    for (int i = 1; i <= o->nnod; ++i) {
      const int vt = o->veg_type[i];
      if (vt < 1 || vt > soil->nveg) { delete o; return nullptr; }
      // the root zone must end above the bottom node (etran.f:60-65)
      const double zroot = o->feddes[6 * (vt - 1) + 3];
      if (o->z[i] - o->z[nstr * nnod + i] <= zroot) { delete o; return nullptr; }
    }
  }
  auto z0 = [&](dvec& v, size_t s) { v.assign(s, 0.0); };
  for (dvec* v : {&o->pnew, &o->pold, &o->ptnew, &o->ptold, &o->ptimep, &o->pdiff,
                  &o->swnew, &o->swtimep, &o->sw, &o->ckrw, &o->etai, &o->et1,
                  &o->et2, &o->dckrw, &o->detai, &o->swp, &o->tnoti, &o->xt5,
                  &o->qtranie})
    z0(*v, n + 1);
  for (dvec* v : {&o->ckrwe, &o->etae, &o->et1e, &o->pel}) z0(*v, nt + 1);
  for (dvec* v : {&o->coef1, &o->coef2, &o->coef3, &o->coef4, &o->coef5})
    z0(*v, o->nterm + 1);
  z0(o->scr, 6 * (size_t)n + 8);
  z0(o->lhsatm, nnod + 1);
  // BCs (constant non-atmospheric Dirichlet / Neumann lists)
  o->np = bc->np; o->nq = bc->nq;
  o->contp.assign(o->np + 1, 0); o->presc.assign(o->np + 1, 0.0);
  o->qpnew.assign(o->np + 1, 0.0); o->qpold.assign(o->np + 1, 0.0);
  o->lhsp.assign(o->np + 1, 0.0);
  for (int i = 1; i <= o->np; ++i) { o->contp[i] = bc->contp[i - 1]; o->presc[i] = bc->presc[i - 1]; }
  o->contq.assign(o->nq + 1, 0); o->q.assign(o->nq + 1, 0.0);
  for (int i = 1; i <= o->nq; ++i) { o->contq[i] = bc->contq[i - 1]; o->q[i] = bc->q[i - 1]; }
  o->noddir.assign(o->np + nnod + 2, 0);
  o->hspatm = bc->hspatm; o->ieto = bc->ieto; o->natm = bc->natm;
  o->atm_t.assign(bc->atmtim, bc->atmtim + bc->natm);
  size_t nv = (size_t)bc->natm * (bc->hspatm ? 1 : nnod);
  o->atm_v.assign(bc->atminp, bc->atminp + nv);
  // initial conditions (inital.f:97-103; icvhe.f, icvhwt.f, icvdwt.f;
  // INDP 0/1 direct)
  if (bc->indp < 0 || bc->indp > 4) { delete o; return nullptr; }
  if (bc->indp == 0) {
    for (int k = 1; k <= n; ++k) o->ptimep[k] = bc->pinit[0];
  } else if (bc->indp == 1) {
    for (int k = 1; k <= n; ++k) o->ptimep[k] = bc->pinit[k - 1];
  } else if (bc->indp == 2) {
    for (int i = 1; i <= nnod; ++i)
      for (int k = 0; k <= nstr; ++k) {
        int kk = k * nnod + i;
        o->ptimep[kk] = o->z[i] - o->z[kk];
      }
  } else if (bc->indp == 3) {
    // ICVHWT (icvhwt.f:31-37): water table WTPOSITION above the bottom node
    for (int i = 1; i <= nnod; ++i)
      for (int k = 0; k <= nstr; ++k) {
        int kk = k * nnod + i;
        o->ptimep[kk] = bc->wtposition - o->z[kk] + o->z[nstr * nnod + i];
      }
  } else {  // INDP = 4, ICVDWT: water table WTPOSITION below the surface
    for (int i = 1; i <= nnod; ++i)
      for (int k = 0; k <= nstr; ++k) {
        int kk = k * nnod + i;
        o->ptimep[kk] = o->z[i] - o->z[kk] - bc->wtposition;
      }
  }
  // INIT1 (init1.f)
  o->deltat = parm->deltat;
  if (o->deltat > parm->dtmax) o->deltat = parm->dtmax;
  if (o->deltat <= parm->dtmin) { o->deltat = parm->dtmin; o->dtgmin = false; }
  else o->dtgmin = true;
  o->timep = 0.0;
  o->time = o->deltat;
  // seepage faces (sfvone.f: elevations descending along each face) and
  // SFINIT (sfinit.f:22-50): nodes at PTIMEP >= 1e-8 start as exit points
  // at zero head
  if (bc->nsf > 0) {
    std::vector<char> seen(n + 1, 0);
    for (int i = 1; i <= o->np; ++i) seen[o->contp[i]] = 1;
    for (int i = 1; i <= o->nq; ++i) seen[o->contq[i]] = 1;
    int e = 0;
    for (int f = 0; f < bc->nsf; ++f) {
      for (int j = 0; j < bc->sfnum[f]; ++j, ++e) {
        const int nd = bc->sfnod[e];
        if (nd < 1 || nd > n || seen[nd]) { delete o; return nullptr; }
        seen[nd] = 1;
        if (j > 0 && o->z[bc->sfnod[e - 1]] < o->z[nd]) { delete o; return nullptr; }
        o->sfnode.push_back(nd);
      }
    }
    o->nsfn = e;
    o->sfex.assign(e, 0); o->sfq.assign(e, 0.0); o->sfqp.assign(e, 0.0);
    o->lhssf.assign(e, 0.0);
    o->noddir.assign(o->np + e + nnod + 2, 0);
    for (int k = 0; k < e; ++k)
      if (o->ptimep[o->sfnode[k]] >= 1.0e-8) { o->sfex[k] = 1; o->ptimep[o->sfnode[k]] = 0.0; }
    o->sfexp = o->sfex;
    o->sfchek = (parm->isfcvg == 1);
  }
  o->pnew = o->ptimep;
  o->atmone();
  // POLD, PTNEW, PTOLD (inital.f)
  o->pold = o->pnew;
  for (int k = 1; k <= n; ++k)
    o->ptnew[k] = parm->tetaf * o->pnew[k] + (1.0 - parm->tetaf) * o->ptimep[k];
  o->ptold = o->ptnew;
  // MBINIT: previous-level fluxes
  o->adinp = o->adoutp = o->ndinp = o->ndoutp = 0.0;
  o->aninp = o->anoutp = o->nninp = o->nnoutp = 0.0;
  for (int i = 1; i <= nnod; ++i) {
    if (o->ifatmp[i] == 0) {
      if (o->atmold[i] > 0.0) o->aninp += o->atmold[i];
      else o->anoutp += o->atmold[i];
    }
  }
  for (int k = 1; k <= o->nq; ++k) {
    if (o->q[k] > 0.0) o->nninp += o->q[k];
    else o->nnoutp += o->q[k];
  }
  o->tpnodi(soil);
  o->chparm();
  // initial storage (cathy_main.f:2660-2662)
  for (int i = 1; i <= n; ++i)
    o->sw[i] = o->vgpnot[i] * o->fvgse(o->ptimep[i], i) + o->vgrmc[i] / o->pnodi[i];
  o->store1 = 0.0;
  for (int i = 1; i <= n; ++i) o->store1 += o->sw[i] * o->volnod[i] * o->pnodi[i];
  o->store2 = o->store1;
  return o;
}

void orc_destroy(void* h) { delete (Oracle*)h; }

void orc_sizes(void* h, int32_t* out) {
  Oracle* o = (Oracle*)h;
  out[0] = o->n; out[1] = o->nt; out[2] = o->nnod; out[3] = o->ntri; out[4] = o->nterm;
}

void orc_get_mesh(void* h, double* x, double* y, double* z, int32_t* tetra,
                  int32_t* topol, int32_t* ja, double* arenod, double* volnod) {
  Oracle* o = (Oracle*)h;
  for (int i = 0; i < o->n; ++i) { x[i] = o->x[i + 1]; y[i] = o->y[i + 1]; z[i] = o->z[i + 1]; }
  std::memcpy(tetra, o->tetra.data(), sizeof(int) * 5 * o->nt);
  std::memcpy(topol, o->topol.data() + 1, sizeof(int) * (o->n + 1));
  std::memcpy(ja, o->ja.data() + 1, sizeof(int) * o->nterm);
  for (int i = 0; i < o->nnod; ++i) arenod[i] = o->arenod[i + 1];
  for (int i = 0; i < o->n; ++i) volnod[i] = o->volnod[i + 1];
}

void orc_get_tetra_gen3d(void* h, int32_t* tetra) {
  Oracle* o = (Oracle*)h;
  std::memcpy(tetra, o->tetra_gen3d.data(), sizeof(int) * 5 * o->nt);
}

int32_t orc_step(void* h) { return ((Oracle*)h)->step(); }

int32_t orc_run(void* h, int32_t max_steps) {
  Oracle* o = (Oracle*)h;
  int steps = 0;
  while (!o->finished && steps < max_steps) {
    int r = o->step();
    if (r == 1) return -1;
    steps++;
  }
  return steps;
}

void orc_first_iteration(void* h, orc_iter_rec_t* rec) {
  Oracle* o = (Oracle*)h;
  o->atmnxt();
  o->etran();
  o->switch_old();
  o->pold = o->pnew;
  for (int k = 1; k <= o->n; ++k)
    o->ptnew[k] = o->parm.tetaf * o->pnew[k] + (1.0 - o->parm.tetaf) * o->ptimep[k];
  o->ptold = o->ptnew;
  o->flow3d(true);
  *rec = o->iter_recs.back();
}

void orc_get_seepage(void* h, int32_t* sfex, double* sfq) {
  Oracle* o = (Oracle*)h;
  for (int e = 0; e < o->nsfn; ++e) { sfex[e] = o->sfex[e]; sfq[e] = o->sfq[e]; }
}

void orc_get_qtranie(void* h, double* qtranie, int32_t* veg_type) {
  Oracle* o = (Oracle*)h;
  for (int k = 1; k <= o->n; ++k) qtranie[k - 1] = o->qtranie[k];
  for (int i = 1; i <= o->nnod; ++i) veg_type[i - 1] = o->veg_type[i];
}

int32_t orc_num_iter_recs(void* h) { return (int32_t)((Oracle*)h)->iter_recs.size(); }
void orc_get_iter_recs(void* h, orc_iter_rec_t* out) {
  Oracle* o = (Oracle*)h;
  std::memcpy(out, o->iter_recs.data(), sizeof(orc_iter_rec_t) * o->iter_recs.size());
}
int32_t orc_num_step_recs(void* h) { return (int32_t)((Oracle*)h)->step_recs.size(); }
void orc_get_step_recs(void* h, orc_step_rec_t* out) {
  Oracle* o = (Oracle*)h;
  std::memcpy(out, o->step_recs.data(), sizeof(orc_step_rec_t) * o->step_recs.size());
}

void orc_get_state(void* h, double* pnew, double* td) {
  Oracle* o = (Oracle*)h;
  for (int i = 0; i < o->n; ++i) pnew[i] = o->pnew[i + 1];
  td[0] = o->time; td[1] = o->deltat;
}

void orc_set_state(void* h, const double* ptimep, double time, double deltat) {
  Oracle* o = (Oracle*)h;
  for (int i = 0; i < o->n; ++i) { o->ptimep[i + 1] = ptimep[i]; o->pnew[i + 1] = ptimep[i]; }
  for (int e = 0; e < o->nsfn; ++e) {  // SFINIT on the new heads
    const int nd = o->sfnode[e];
    o->sfex[e] = o->ptimep[nd] >= 1.0e-8 ? 1 : 0;
    if (o->sfex[e]) { o->ptimep[nd] = 0.0; o->pnew[nd] = 0.0; }
    o->sfq[e] = 0.0; o->sfqp[e] = 0.0;
  }
  o->sfexp = o->sfex;
  o->sfflwp = 0.0;
  o->time = time; o->deltat = deltat;
}

void orc_picard_system(void* h, double* coef1, double* tnoti, double* xt5,
                       int32_t* dirmask) {
  Oracle* o = (Oracle*)h;
  // replicate PICARD up to BCPIC, then restore diagonals (as SHLPIC does)
  o->pold = o->pnew;
  for (int k = 1; k <= o->n; ++k)
    o->ptnew[k] = o->parm.tetaf * o->pnew[k] + (1.0 - o->parm.tetaf) * o->ptimep[k];
  o->ptold = o->ptnew;
  o->chpic();
  Oracle& r = *o;
  std::fill(r.coef1.begin(), r.coef1.end(), 0.0);
  std::fill(r.coef2.begin(), r.coef2.end(), 0.0);
  std::fill(r.coef4.begin(), r.coef4.end(), 0.0);
  std::fill(r.coef5.begin(), r.coef5.end(), 0.0);
  r.asspic_state();
  double rdt = 1.0 / r.deltat;
  for (int k = 1; k <= r.n; ++k) r.tnoti[k] = 0.0;
  for (int k = 1; k <= r.n; ++k) {
    int i = r.topol[k], j = r.topol[k + 1] - 1;
    for (int m = i; m <= j; ++m) {
      double coef = r.coef2[m] * rdt, coeff = r.coef4[m] * rdt;
      int jm = r.ja[m];
      r.tnoti[k] = r.tnoti[k] - r.coef1[m] * r.ptnew[jm] - coef * (r.pnew[jm] - r.ptimep[jm]) -
                   coeff * (r.swnew[jm] - r.swtimep[jm]);
      if (m != i)
        r.tnoti[jm] = r.tnoti[jm] - r.coef1[m] * r.ptnew[k] - coef * (r.pnew[k] - r.ptimep[k]) -
                      coeff * (r.swnew[k] - r.swtimep[k]);
    }
  }
  for (int k = 1; k <= r.n; ++k) r.coef5[r.topol[k]] = r.coef4[r.topol[k]] * r.et2[k];
  for (int k = 1; k <= r.nterm; ++k)
    r.coef1[k] = r.parm.tetaf * r.coef1[k] + r.coef2[k] * rdt + r.coef5[k] * rdt;
  for (int ke = 1; ke <= r.nt; ++ke) {
    double t3 = r.ckrwe[ke] * r.permz[r.idx(r.istr_of(ke), r.T(5, ke))];
    for (int in = 1; in <= 4; ++in)
      r.tnoti[r.T(in, ke)] -= t3 * r.D(in, ke) * r.ivol[ke];
  }
  for (int k = 1; k <= r.n; ++k) xt5[k - 1] = r.tnoti[k];
  for (int k = 0; k < r.n; ++k) dirmask[k] = 0;
  for (int k = 1; k <= r.np; ++k) { r.tnoti[r.contp[k]] = 0.0; dirmask[r.contp[k] - 1] = 1; }
  for (int k = 1; k <= r.nnod; ++k)
    if (r.ifatm[k] == 1 || r.ifatm[k] == 2) { r.tnoti[k] = 0.0; dirmask[k - 1] = 1; }
  for (int k = 1; k <= r.nq; ++k) r.tnoti[r.contq[k]] += r.q[k];
  for (int k = 1; k <= r.nnod; ++k)
    if (r.ifatm[k] == 0)
      r.tnoti[k] += r.parm.tetaf * r.atmact[k] + (1.0 - r.parm.tetaf) * r.atmold[k];
  for (int k = 1; k <= r.n; ++k) tnoti[k - 1] = r.tnoti[k];
  for (int k = 1; k <= r.nterm; ++k) coef1[k - 1] = r.coef1[k];
}

void orc_asspic(int32_t nt, int32_t ntri, const int32_t* tetra, const int32_t* tetja,
                const double* lmass, double* coef1, double* coef2, double* coef4,
                const double* et1e, const double* pel, const double* permx,
                const double* permy, const double* permz, const double* ckrwe,
                const double* volu, const double* volur, const double* bi,
                const double* ci, const double* di, int32_t maxstr) {
  asspic(nt, ntri, tetra, tetja, lmass, coef1, coef2, coef4, et1e, pel, permx, permy, permz,
         ckrwe, volu, volur, bi, ci, di, maxstr);
}

void orc_asspic_inputs(void* h, int32_t* tetja, double* lmass, double* et1e, double* pel,
                       double* permx, double* permy, double* permz, double* ckrwe,
                       double* volu, double* volur, double* bi, double* ci, double* di) {
  Oracle* o = (Oracle*)h;
  std::copy(o->tetja.begin(), o->tetja.begin() + 16 * (size_t)o->nt, tetja);
  for (int k = 1; k <= 4; ++k)
    for (int l = 1; l <= 4; ++l) lmass[4 * (l - 1) + (k - 1)] = o->lmass[k][l];
  for (int e = 1; e <= o->nt; ++e) {
    et1e[e - 1] = o->et1e[e]; pel[e - 1] = o->pel[e]; ckrwe[e - 1] = o->ckrwe[e];
    volu[e - 1] = o->volu[e]; volur[e - 1] = o->volur[e];
  }
  std::copy(o->permx.begin(), o->permx.end(), permx);
  std::copy(o->permy.begin(), o->permy.end(), permy);
  std::copy(o->permz.begin(), o->permz.end(), permz);
  std::copy(o->bi.begin(), o->bi.begin() + 4 * (size_t)o->nt, bi);
  std::copy(o->ci.begin(), o->ci.begin() + 4 * (size_t)o->nt, ci);
  std::copy(o->di.begin(), o->di.begin() + 4 * (size_t)o->nt, di);
}

void orc_vg_nodal(void* h, const double* psi, double* sw, double* ckrw,
                  double* etai, double* et2) {
  Oracle* o = (Oracle*)h;
  for (int i = 1; i <= o->n; ++i) {
    double p = psi[i - 1];
    double se = o->fvgse(p, i);
    double dse = o->fvgdse(p, i);
    sw[i - 1] = o->vgpnot[i] * se + o->vgrmc[i] / o->pnodi[i];
    etai[i - 1] = sw[i - 1] * o->snodi[i] + o->pnodi[i] * o->vgpnot[i] * dse;
    et2[i - 1] = o->vgpnot[i] * dse;
    ckrw[i - 1] = o->fvgkr(p, se, i);
  }
}

// fine-grained solvers on caller-provided 1-based-content arrays (0-based
// C pointers to the Fortran arrays)
int32_t orc_symslv(int32_t n, int32_t nterm, int32_t numdir,
                   const int32_t* noddir, const int32_t* ja,
                   const int32_t* topol, double* x, const double* b,
                   const double* coef1, int32_t itmxcg, double tolcg,
                   int32_t jacobi, double* err_res) {
  ivec nd(numdir + 1), jv(nterm + 1), tp(n + 2);
  for (int i = 0; i < numdir; ++i) nd[i + 1] = noddir[i];
  for (int i = 0; i < nterm; ++i) jv[i + 1] = ja[i];
  for (int i = 0; i <= n; ++i) tp[i + 1] = topol[i];
  dvec xv(n + 1), bv(n + 1), c1(nterm + 1), c2(nterm + 1), scr(5 * (size_t)n + 8);
  for (int i = 0; i < n; ++i) bv[i + 1] = b[i];
  for (int i = 0; i < nterm; ++i) c1[i + 1] = coef1[i];
  int niter = 0;
  symslv(n, nterm, numdir, &niter, itmxcg, tolcg, nd.data(), jv.data(),
         tp.data(), xv.data(), bv.data(), c1.data(), c2.data(), scr.data(),
         &err_res[0], &err_res[1], jacobi != 0);
  for (int i = 0; i < n; ++i) x[i] = xv[i + 1];
  return niter;
}

int32_t orc_nsyslv(int32_t isolv, int32_t n, int32_t nterm, int32_t numdir,
                   const int32_t* noddir, const int32_t* ja,
                   const int32_t* topol, double* x, const double* b,
                   const double* coef1, int32_t itmxcg, double tolcg,
                   double* err_res) {
  ivec nd(numdir + 1), jv(nterm + 1), tp(n + 2), iav(nterm + 1);
  for (int i = 0; i < numdir; ++i) nd[i + 1] = noddir[i];
  for (int i = 0; i < nterm; ++i) jv[i + 1] = ja[i];
  for (int i = 0; i <= n; ++i) tp[i + 1] = topol[i];
  for (int k = 1; k <= n; ++k)
    for (int m = tp[k]; m < tp[k + 1]; ++m) iav[m] = k;
  dvec xv(n + 1), bv(n + 1), c1(nterm + 1), c2(nterm + 1);
  for (int i = 0; i < n; ++i) bv[i + 1] = b[i];
  for (int i = 0; i < nterm; ++i) c1[i + 1] = coef1[i];
  int niter = nsyslv(isolv, n, numdir, nd.data(), itmxcg, tolcg, iav.data(),
                     jv.data(), tp.data(), c1.data(), c2.data(), xv.data(),
                     bv.data(), &err_res[0], &err_res[1]);
  for (int i = 0; i < n; ++i) x[i] = xv[i + 1];
  return niter;
}

}  // extern "C"
