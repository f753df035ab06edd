// Host-side force-field tables of the GB300 force path.
//
// The device kernels consume three tables that cook builds at start-up:
//   * per type pair smoothed-LJ constants      (sim/setss.c:137-300,
//                                               sim/lj/sitesite.c:37-112)
//   * the hyperbolic erfc spline of the r-space (sim/erfc.c:119-191,
//                                               sim/splines.c:23-158)
//   * the half-space k-vector set and ekk       (sim/ewald.c:334-612)
// They are rebuilt here from the same inputs with the same arithmetic, so
// the device path evaluates the very functions cook evaluates.
#include "mg_internal.h"

#include <cmath>
#include <cstdlib>

namespace mg {

static inline double sq(double x) { return x * x; }
static const double kSqrtPi = 1.772453850905516;

// u(r) = -eps[(sig/r)^12 - 2 (sig/r)^6] and f(r) = -du/dr
static double lj_u(double eps, double sig, double r) {
  double x = sig / r;
  x = sq(x) * sq(x) * sq(x);
  return -eps * (x * x - 2 * x);
}
static double lj_f(double eps, double sig, double r) {
  double x = sig / r;
  x = sq(x) * sq(x) * sq(x);
  return -12 * eps * (x * x - x) / r;
}

void combining_rule(double E0, double R0, double a0, double E1, double R1, double a1,
                    int comb_rule, double* eps, double* sig) {
  int cr = (comb_rule | (a0 <= 0)) | (comb_rule | (a1 <= 0));
  if (E0 > 0) E0 = -E0;
  if (E1 > 0) E1 = -E1;
  double g0 = E0 != 0 ? sq(a0) / E0 / (sq(R0) * sq(R0) * sq(R0)) / -256 : 3e37;
  double g1 = E1 != 0 ? sq(a1) / E1 / (sq(R1) * sq(R1) * sq(R1)) / -256 : 3e37;
  double r;
  if (cr & 2) {
    double x = R0 * R1 * 4;
    r = x * x * x;
  } else {
    double x = sq(R0 + R1);
    r = x * x * x;
  }
  double B = (cr & 1) ? std::sqrt(-2 * E0) * std::sqrt(-2 * E1) * r : a0 * a1 / (g0 + g1);
  double A = B * r;
  *sig = B == 0 ? 0 : std::pow(A / B, 1. / 6);
  *eps = A == 0 ? 0 : B * B / (-2 * A);
}

int smooth_lj(double eps, double sig, double C2, PairLJ* p) {
  *p = PairLJ{};
  p->Sq = sq(sig) * 0.7937005259840998;  // sigma^2 of 4 eps[(s/r)^12-(s/r)^6]
  p->E4 = -4 * eps;
  if (p->Sq != 0) {
    p->E24 = -24 * eps / p->Sq;
    p->E48 = -48 * eps / p->Sq;
  }
  double C1;
  if (eps == 0 || C2 == 0) {
    C1 = C2 = 0;
  } else {
    // C1 from C2 by the fixed-point iteration that makes u, f continuous
    const double meps = 2.220446049250313e-16;
    int n = 0;
    double oldC1;
    C1 = 0.775 * C2;
    do {
      double den = lj_f(eps, sig, C1);
      if (std::fabs(den) < 1e-50) { C1 = -C1; break; }
      oldC1 = C1;
      C1 = 1 + 4 * lj_u(eps, sig, C1) / C1 / den;
      if (n++ > 2000 || C1 < 0) return -1;
      C1 = C2 / std::sqrt(C1);
    } while (std::fabs(1 - C1 / oldC1) > meps * n);
    if (C1 > 0 && (C1 > 0.999 * C2 || C1 < 0.5 * C2)) return -2;
    p->A = lj_u(eps, sig, C1) / sq(C2 * C2 - C1 * C1);
  }
  if (C1 < 0) {
    C1 = -C1;
    p->A = p->A4 = 0;
  } else if (C2 > 0) {
    p->A4 = -lj_f(eps, sig, C1) / (C2 * C2 - C1 * C1) / C1;
  }
  p->C1q = C1 * C1;
  p->C2q = C2 * C2;
  return 0;
}

// Cutoff correction of one type pair for a homogeneous fluid (the integral
// of the missing tail, sim/setss.c:454-500): the smoothing region C1..C2
// analytically, r > C1 by 4th-order Gauss on 64 intervals in 1/r
double lj_tail_correction(double eps, double sig, const PairLJ& p) {
  if (eps == 0 || p.C1q == 0) return 0;
  const double C1 = std::sqrt(p.C1q), C2 = std::sqrt(p.C2q);
  const double C14 = sq(C1) * sq(C1), C16 = C14 * sq(C1), C24 = sq(C2) * sq(C2);
  const double pi = 3.14159265358979323846;
  double c0 = 4 * pi * p.A *
              (C1 * (C16 / 7 - 0.4 * C14 * sq(C2) + sq(C1) * C24 / 3) - 8.0 / 105 * std::pow(C2, 7));
  const double h = 1.0 / 64 / C1, g = 0.2113248654051871;
  double c1 = 0;
  for (int n = 0; n < 64; n++) {
    double r = 1 / ((n + g) * h);
    c1 += sq(r) * sq(r) * lj_u(eps, sig, r);
    r = 1 / ((n + (1 - g)) * h);
    c1 += sq(r) * sq(r) * lj_u(eps, sig, r);
  }
  return c0 + c1 * 2 * pi * h;
}

int erfc_table_size(int grid, double maxr, double alpha) {
  return (int)(sq(maxr * alpha) * grid) + 1;
}

// Hyperbolic splines A+B/(C+x) in x=r^2 for eru = erfc(alpha r)/r and
// erd = -(d eru/dr)/r, built downwards from the end of the table with the
// slope carried from the previous interval; then the rshift shifts.
void erfc_table(int grid, double maxr, double cutoff, double alpha, int shift,
                std::vector<double>* tab, double* sgrid) {
  int n = erfc_table_size(grid, maxr, alpha);
  std::vector<double> fu(n + 3), fd(n + 3);
  double h = 1.0 / grid;
  for (int i = n + 2; i >= 0; i--) {
    if (i) {
      double rr = i * h, r = std::sqrt(rr), er = std::erfc(r);
      fu[i] = er / r;
      fd[i] = ((2 / kSqrtPi) * std::exp(-rr) + er / r) / rr;
    } else {
      fu[i] = fd[i] = 9e9;
    }
  }
  double Du = (-fu[n + 2] + 8 * fu[n + 1] - 8 * fu[n - 1] + fu[n - 2]) / (12 * h);
  double Dd = (-fd[n + 2] + 8 * fd[n + 1] - 8 * fd[n - 1] + fd[n - 2]) / (12 * h);
  double x = n * h, xh;
  tab->assign(6 * (size_t)n, 0.0);
  double a = alpha;
  for (int i = n - 1; i >= 0; i--) {
    xh = x;
    x = i * h;
    double Cu = (x * (fu[i + 1] - fu[i]) - xh * Du * h) / (Du * h - (fu[i + 1] - fu[i]));
    double Bu = -Du * sq(Cu + xh);
    double Au = fu[i + 1] + Du * (Cu + xh);
    Du = -Bu / sq(Cu + x);
    double Cd = (x * (fd[i + 1] - fd[i]) - xh * Dd * h) / (Dd * h - (fd[i + 1] - fd[i]));
    double Bd = -Dd * sq(Cd + xh);
    double Ad = fd[i + 1] + Dd * (Cd + xh);
    Dd = -Bd / sq(Cd + x);
    double* p = tab->data() + 6 * (size_t)i;
    p[0] = Au * a;
    p[1] = Bu / a;
    p[2] = Cu / sq(a);
    p[3] = Ad * (a * a * a);
    p[4] = Bd * a;
    p[5] = Cd / sq(a);
  }
  *sgrid = grid * sq(a);
  double z = sq(cutoff);
  auto eval = [&](int off, double rr) {
    const double* p = tab->data() + 6 * (size_t)(int)(rr * *sgrid) + off;
    return p[1] / (p[2] + rr) + p[0];
  };
  if (shift & 1) {
    double v = eval(0, z);
    for (int i = 0; i < n; i++) (*tab)[6 * (size_t)i] -= v;
  }
  if (shift & 2) {
    double v = eval(3, z);
    for (int i = 0; i < n; i++) (*tab)[6 * (size_t)i + 3] -= v;
  }
}

static bool almost_integer(double x) {
  x -= (int)x;
  return std::fabs(0.5 - std::fabs(x - 0.5)) < 1e-9;
}

// Half-space k-vector set of cook: kx>=0 octant entries expanded to the sign
// combinations (+,+,+) (+,+,-) (+,-,+) (+,-,-) that are distinct; kappa is
// nudged upwards when a bound lands within 1e-9 of an integer.
int kvector_set(const double L[3], double* kappa, std::vector<int>* kv) {
  double dK = 2e-9;
  for (int again = 0; again <= 25; again++) {
    bool retry = false;
    kv->clear();
    double Kk = sq(*kappa), KX = L[0] * *kappa;
    int kxmax = (int)KX;
    for (int kx = 0; kx <= kxmax && !retry; kx++) {
      double kxq = Kk - sq(kx / L[0]);
      double aux = L[1] * std::sqrt(kxq);
      if (almost_integer(aux)) { retry = true; break; }
      int kymax = (int)aux;
      for (int ky = 0; ky <= kymax; ky++) {
        double kyq = kxq - sq(ky / L[1]);
        aux = L[2] * std::sqrt(kyq);
        if (almost_integer(aux)) { retry = true; break; }
        int kzmax = (int)aux;
        for (int kz = !(kx + ky); kz <= kzmax; kz++) {
          auto push = [&](int a, int b, int c) {
            kv->push_back(a);
            kv->push_back(b);
            kv->push_back(c);
          };
          int nz = (kx > 0) + (ky > 0) + (kz > 0);
          push(kx, ky, kz);
          if (nz == 3) {
            push(kx, ky, -kz);
            push(kx, -ky, kz);
            push(kx, -ky, -kz);
          } else if (nz == 2) {
            if (kz == 0) push(kx, -ky, kz);
            else push(kx, ky, -kz);
          }
        }
      }
    }
    if (!retry) return (int)(kv->size() / 3);
    *kappa += *kappa * dK;
    dK *= 1.4;
  }
  return -1;
}

// ASPC predictor of Kolafa (J. Comput. Chem. 25, 335 (2004)) as set up in
// sim/pred2.c:70-97: B[0..k+1] for predictor length k (k=0: the linear
// predictor 2, -1) and the mixing omega = (k+2)/(2k+3) that keeps it stable
void aspc_coefficients(int k, double* B, double* omega) {
  if (k == 0) {
    B[0] = 2;
    B[1] = -1;
    *omega = 2.0 / 3.0;
    return;
  }
  double o = (double)(4 * k + 6) / (double)(k + 3);
  for (int i = 0; i < k + 2; i++) {
    B[i] = o * (i + 1);
    o *= (double)(i - k - 1) / (double)(k + i + 4);
  }
  *omega = (k + 2) / (double)(2 * k + 3);
}

}  // namespace mg
