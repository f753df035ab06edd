/*
 * cookoracle.c -- CPU restatement of cook's force path (TEST INFRASTRUCTURE).
 *
 * Used only by tests/, the smoke check and the benchmark's CPU-baseline leg,
 * as the checker.  Never part of the product path.  Each function cites the
 * reference file:line it restates.  Plain C99, double precision, pthreads.
 */
#include "cookoracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define SQ(x) ((x) * (x))
#define SQRTPI 1.772453850905516
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ LJ --- */

/* sim/lj/sitesite.c:37-93 (initcombrule + combrule) */
void orc_combrule(double E0, double R0, double a0, double E1, double R1, double a1,
                  int comb_rule, double *eps, double *sig)
{
  int cr0 = comb_rule | (a0 <= 0), cr1 = comb_rule | (a1 <= 0);
  int cr = cr0 | cr1;
  double g0, g1, r, A, B;
  if (E0 > 0) E0 = -E0;
  if (E1 > 0) E1 = -E1;
  g0 = E0 != 0 ? SQ(a0) / E0 / (SQ(R0) * SQ(R0) * SQ(R0)) / -256 : 3e37;
  g1 = E1 != 0 ? SQ(a1) / E1 / (SQ(R1) * SQ(R1) * SQ(R1)) / -256 : 3e37;
  if (cr & 2) { double x = R0 * R1 * 4; r = x * x * x; }
  else { double x = SQ(R0 + R1); r = x * x * x; }
  if (cr & 1) B = sqrt(-2 * E0) * sqrt(-2 * E1) * r;
  else B = a0 * a1 / (g0 + g1);
  A = B * r;
  *sig = B == 0 ? 0 : pow(A / B, 1. / 6);
  *eps = A == 0 ? 0 : B * B / (-2 * A);
}

/* potential and force of the LJ form u=-eps[(sig/r)^12-2(sig/r)^6]
   (SS_U / SS_F of sim/lj/sitesite.h:85-86) */
static double ss_u(double eps, double sig, double r)
{
  double x = sig / r;
  x = SQ(x) * SQ(x) * SQ(x);
  return -eps * (x * x - 2 * x);
}
static double ss_f(double eps, double sig, double r)
{
  double x = sig / r;
  x = SQ(x) * SQ(x) * SQ(x);
  return -12 * eps * (x * x - x) / r;
}

/* sim/setss.c:137-300 (smooth cutoff) + 460-510 (cutoff correction) and
   initssaux sim/lj/sitesite.c:96-112 */
int orc_setss(double eps, double sig, double C2, orc_ss_t *ss)
{
  double C1, oldC1;
  int n = 0;
  const double meps = 2.220446049250313e-16; /* machine precision (No.eps) */
  memset(ss, 0, sizeof(*ss));
  ss->eps = eps;
  ss->sig = sig;
  /* initssaux */
  ss->Sq = SQ(sig) * 0.7937005259840998;
  ss->E4 = -4 * eps;
  if (ss->Sq != 0) {
    ss->E24 = -24 * eps / ss->Sq;
    ss->E48 = -48 * eps / ss->Sq;
  }
  if (eps == 0 || C2 == 0) {
    C1 = C2 = ss->A = 0;
  } else {
    if (C2 < 0) C2 = -sig * C2;
    C1 = 0.775 * C2;
    do {
      double den = ss_f(eps, sig, C1);
      if (fabs(den) < 1e-50) { C1 = -C1; break; }
      oldC1 = C1;
      C1 = 1 + 4 * ss_u(eps, sig, C1) / C1 / den;
      if (n++ > 2000 || C1 < 0) { C1 = 0.775 * C2; return -1; }
      C1 = C2 / sqrt(C1);
    } while (fabs(1 - C1 / oldC1) > meps * n);
    if (C1 > 0 && (C1 > 0.999 * C2 || C1 < 0.5 * C2)) return -2;
    ss->A = ss_u(eps, sig, C1) / SQ(C2 * C2 - C1 * C1);
  }
  if (C1 < 0) { C1 = -C1; ss->A = ss->A4 = 0; }
  else if (C2 > 0) ss->A4 = -ss_f(eps, sig, C1) / (C2 * C2 - C1 * C1) / C1;
  ss->C2q = C2 * C2;
  ss->C1q = C1 * C1;
  /* normalized cutoff correction: analytic part + 4th order Gauss on 1/r */
  if (eps != 0) {
    double C14 = SQ(C1) * SQ(C1), C16 = C14 * SQ(C1), C24 = SQ(C2) * SQ(C2);
    double corr0 = 4 * M_PI * ss->A *
      (C1 * (C16 / 7 - 0.4 * C14 * SQ(C2) + SQ(C1) * C24 / 3) - 8.0 / 105 * pow(C2, 7));
    double h = 1.0 / 64 / C1, corr1 = 0, r;
    const double g4 = 0.2113248654051871;
    for (n = 0; n < 64; n++) {
      r = 1 / ((n + g4) * h); corr1 += SQ(r) * SQ(r) * ss_u(eps, sig, r);
      r = 1 / ((n + (1 - g4)) * h); corr1 += SQ(r) * SQ(r) * ss_u(eps, sig, r);
    }
    corr1 *= 2 * M_PI * h;
    ss->corr = corr0 + corr1;
  }
  return 0;
}

/* ---------------------------------------------------------------- erfc --- */

/* sim/erfc.c:119-150: number of spline intervals for [0,maxr) */
int orc_erfc_ntab(int grid, double maxr, double alpha)
{
  return (int)(SQ(maxr * alpha) * grid) + 1;
}

/* values at alpha=1: e=erfc(sqrt x)/sqrt x, z=(2/sqrt(pi) exp(-x)+e)/x
   (erfcs, sim/erfc.c:76-85) */
static void erfcs(long to, double h, double *e, double *z)
{
  if (to) {
    double rr = to * h, r = sqrt(rr), er = erfc(r);
    *e = er / r;
    *z = ((2 / SQRTPI) * exp(-rr) + er / r) / rr;
  } else
    *e = *z = 9e9;
}

/* makesplines SPLINE=-2, SUBGRID=1 (sim/splines.c:23-158) followed by the
   shifts of initerfc (sim/erfc.c:176-187).  tab: 6 doubles per interval */
void orc_erfc_build(int grid, double maxr, double cutoff, double alpha, int shift,
                    double *tab, double *sgrid_out)
{
  int ito = orc_erfc_ntab(grid, maxr, alpha), i, n = ito;
  double h = 1.0 / grid, Du, Dd, x, xh;
  double *fu = malloc(sizeof(double) * (n + 3)), *fd = malloc(sizeof(double) * (n + 3));
  double a = alpha, sgrid;
  for (i = n + 2; i >= 0; i--) erfcs(i, h, &fu[i], &fd[i]);
  Du = (-fu[n + 2] + 8 * fu[n + 1] - 8 * fu[n - 1] + fu[n - 2]) / (12 * h);
  Dd = (-fd[n + 2] + 8 * fd[n + 1] - 8 * fd[n - 1] + fd[n - 2]) / (12 * h);
  x = n * h;
  while (ito--) {
    double *p = tab + 6 * ito;
    double Au, Bu, Cu, Ad, Bd, Cd;
    xh = x;
    i = ito;
    x = i * h;
    Cu = (x * (fu[i + 1] - fu[i]) - xh * Du * h) / (Du * h - (fu[i + 1] - fu[i]));
    Bu = -Du * SQ(Cu + xh);
    Au = fu[i + 1] + Du * (Cu + xh);
    Du = -Bu / SQ(Cu + x);
    Cd = (x * (fd[i + 1] - fd[i]) - xh * Dd * h) / (Dd * h - (fd[i + 1] - fd[i]));
    Bd = -Dd * SQ(Cd + xh);
    Ad = fd[i + 1] + Dd * (Cd + xh);
    Dd = -Bd / SQ(Cd + x);
    p[0] = Au * a;
    p[1] = Bu / a;
    p[2] = Cu / SQ(a);
    p[3] = Ad * (a * a * a);
    p[4] = Bd * a;
    p[5] = Cd / SQ(a);
  }
  sgrid = grid * SQ(a);
  free(fu);
  free(fd);
  {
    int nt = orc_erfc_ntab(grid, maxr, alpha);
    double z = SQ(cutoff), v;
    if (shift & 1) {
      v = orc_eru(tab, sgrid, z);
      for (i = 0; i < nt; i++) tab[6 * i] -= v;
    }
    if (shift & 2) {
      v = orc_erd(tab, sgrid, z);
      for (i = 0; i < nt; i++) tab[6 * i + 3] -= v;
    }
  }
  *sgrid_out = sgrid;
}

/* eru/erd macros of sim/elst.h:122-130 */
double orc_eru(const double *tab, double sgrid, double rr)
{
  const double *p = tab + 6 * (int)(rr * sgrid);
  return p[1] / (p[2] + rr) + p[0];
}
double orc_erd(const double *tab, double sgrid, double rr)
{
  const double *p = tab + 6 * (int)(rr * sgrid);
  return p[4] / (p[5] + rr) + p[3];
}

/* sim/erexact.c:25-75 (SUBGRID==1): -erf(alpha r)/r and its derivative term */
static double exacterud_core(double rr, double alpha, double *erd, int minus1)
{
  double A = alpha * (-2 / SQRTPI), alphaq = SQ(alpha), B = A * alphaq * 2;
  double err = alphaq * rr;
  if (err < 0.01) {
    int n = 1;
    double su = 0, sd = 0, q = 1, r;
    for (;;) {
      r = q / (2 * n + 1);
      sd += r * n;
      su += r;
      if (fabs(q) < (minus1 ? 1e-17 : 1e-16)) break;
      q *= -err / ++n;
    }
    *erd = B * sd;
    return minus1 ? A * (-su * err) : A * (1 - su * err);
  } else {
    double r = sqrt(rr);
    double y = -erf(alpha * r) / r;
    *erd = (y - A * exp(-err)) / rr;
    return minus1 ? y - A : y;
  }
}
double orc_exacterud_sqrt(double rr, double alpha, double *erd)
{
  return exacterud_core(rr, alpha, erd, 0);
}
double orc_exacterud_sqrt_1(double rr, double alpha, double *erd)
{
  return exacterud_core(rr, alpha, erd, 1);
}

/* ---------------------------------------------------------- k-vectors --- */

static int almostint(double x)
{
  x -= (int)x;
  return fabs(0.5 - fabs(x - 0.5)) < 1e-9;
}

/* sim/ewald.c:410-510: k-vector count with the rounding-problem guard */
int orc_kvectors(const double L[3], double *kappa, int maxk, int *kv)
{
  double dK = 2e-9;
  int nagain = 0;
again:
  if (nagain++ > 25) return -1;
  {
    double Kk = SQ(*kappa), KX = L[0] * *kappa;
    int kx, ky, kz, kxmax = (int)KX, iQ = 0;
    for (kx = 0; kx <= kxmax; kx++) {
      double kxq = Kk - SQ(kx / L[0]), aux = L[1] * sqrt(kxq);
      int kymax;
      if (almostint(aux)) { *kappa += *kappa * dK; dK *= 1.4; goto again; }
      kymax = (int)aux;
      for (ky = 0; ky <= kymax; ky++) {
        double kyq = kxq - SQ(ky / L[1]);
        int kzmax;
        aux = L[2] * sqrt(kyq);
        if (almostint(aux)) { *kappa += *kappa * dK; dK *= 1.4; goto again; }
        kzmax = (int)aux;
        for (kz = !(kx + ky); kz <= kzmax; kz++) {
          int c = (kx > 0) + (ky > 0) + (kz > 0), m;
          /* sign combos in the order of sim/ewpass1.c: xyz xyZ xYz xYZ */
          int combos[4][3] = {{kx, ky, kz}, {kx, ky, -kz}, {kx, -ky, kz}, {kx, -ky, -kz}};
          int list[4], nl = 0;
          if (c == 3) { list[0] = 0; list[1] = 1; list[2] = 2; list[3] = 3; nl = 4; }
          else if (c == 2) {
            if (kz == 0) { list[0] = 0; list[1] = 2; nl = 2; }
            else { list[0] = 0; list[1] = 1; nl = 2; }
          } else { list[0] = 0; nl = 1; }
          for (m = 0; m < nl; m++) {
            if (kv && iQ < maxk) {
              kv[3 * iQ] = combos[list[m]][0];
              kv[3 * iQ + 1] = combos[list[m]][1];
              kv[3 * iQ + 2] = combos[list[m]][2];
            }
            iQ++;
          }
        }
      }
    }
    return iQ;
  }
}

/* ------------------------------------------------------------ threads --- */

static int is_polar(const orc_sys_t *s) { return s->qpol != NULL; }

typedef struct {
  const orc_sys_t *s;
  const double *r;
  int ith, nth;
  double *f;            /* thread-private force array (3*ns or 6*ns) */
  double el, lj, vir, Pvir[6];
  /* k-space */
  int nk;
  const int *kv;
  double *Sre, *Sim;    /* thread-partial structure factors */
  const double *ekk;
  const double *gre, *gim; /* full S for pass 2 */
  /* cells */
  const int *cellhead, *cellnext;
  int nc[3];
} orc_work_t;

static void run_threads(void *(*fn)(void *), orc_work_t *w, int nth)
{
  pthread_t th[64];
  int i;
  if (nth == 1) { fn(w); return; }
  for (i = 0; i < nth; i++) pthread_create(&th[i], NULL, fn, &w[i]);
  for (i = 0; i < nth; i++) pthread_join(th[i], NULL);
}


/* -------------------------------------------------------------- r-space --- */

/* one pair (cook/ljqqnp.c LJqqm, non-polar, COULOMB=-2): dr = ri - rj with
   nearest image, rr=|dr|^2 < cutoff^2 already checked.  Adds forces to fi
   (and -fdr to fj when fj!=NULL).  Returns f/r. */
static void pair_np(orc_work_t *w, int i, int j, const double dr[3], double rr,
                    double *fi, double *fj, int measure)
{
  const orc_sys_t *s = w->s;
  double f = 0, U = 0, qq = s->q[i] * s->q[j], x, y, z;
  if (s->mol[i] == s->mol[j]) {
    /* EXCL: no LJ; exact Ewald intramolecular correction (cook/ljqqnp.c:124-144) */
    if (qq != 0) {
      double fe;
      double e = orc_exacterud_sqrt(rr, s->alpha, &fe);
      if (measure) w->el += e * qq;
      f = fe * qq;
    }
  } else {
    const orc_ss_t *ss = s->ss + s->type[i] * s->ntypes + s->type[j];
    if (rr < ss->C2q) {
      if (rr < ss->C1q) {
        x = ss->Sq / rr;
        y = x * x * x;
        z = y * y;
        if (measure) {
          U += ss->E4 * (z - y);
          f = ss->E24 * (z + z - y) * x;
        } else
          f = ss->E48 * y * (y - 0.5) * x;
      } else {
        x = rr - ss->C2q;
        U = x * x * ss->A;
        f = ss->A4 * x;
      }
      if (measure) w->vir += rr * f;
    }
    if (qq != 0) {
      const double *p = s->ertab + 6 * (int)(rr * s->sgrid);
      f += (p[4] / (p[5] + rr) + p[3]) * qq;
      if (measure) w->el += (p[1] / (p[2] + rr) + p[0]) * qq;
    }
  }
  {
    double fx = f * dr[0], fy = f * dr[1], fz = f * dr[2];
    fi[0] += fx; fi[1] += fy; fi[2] += fz;
    if (fj) { fj[0] -= fx; fj[1] -= fy; fj[2] -= fz; }
    if (measure) {
      w->lj += U;
      w->Pvir[0] += dr[0] * fx;
      w->Pvir[1] += dr[1] * fy;
      w->Pvir[2] += dr[2] * fz;
      w->Pvir[3] += dr[2] * fy;
      w->Pvir[4] += dr[0] * fz;
      w->Pvir[5] += dr[1] * fx;
    }
  }
}

/* one pair of polarizable sites (cook/ljqqpol.c polarLJqqm, POLAR=0,
   COULOMB=-2): centre-centre LJ + charge, Drude(i)-centre(j),
   centre(i)-Drude(j), Drude-Drude terms, each at its own separation; an
   intramolecular pair takes the exact Ewald exclusion term for all four.
   dr = centre(i) - centre(j) (nearest image).  Centre forces go to
   f[3*ns..], Drude forces to the second half (cook's polar_off half). */
static void pair_pol(orc_work_t *w, int i, int j, const double dr0[3], double rr0,
                     double *fo, int measure)
{
  const orc_sys_t *s = w->s;
  const int ns = s->ns;
  const double *di = w->r + 3 * ns + 3 * i, *dj = w->r + 3 * ns + 3 * j;
  double *fci = fo + 3 * i, *fcj = fo + 3 * j, *fpi = fo + 3 * ns + 3 * i, *fpj = fo + 3 * ns + 3 * j;
  const double qi = s->q[i], qj = s->q[j], pi_ = s->qpol[i], pj_ = s->qpol[j];
  const int excl = s->mol[i] == s->mol[j];
  double U = 0, f = 0, x, y, z;
  int k, m;
  struct { double q; double sgn_i, sgn_j; double *fa, *fb; } t[4] = {
    {qi * qj, 0, 0, fci, fcj}, {pi_ * qj, 1, 0, fpi, fcj},
    {qi * pj_, 0, 1, fci, fpj}, {pi_ * pj_, 1, 1, fpi, fpj}};
  if (!excl) {
    const orc_ss_t *ss = s->ss + s->type[i] * s->ntypes + s->type[j];
    if (rr0 < ss->C2q) {
      if (rr0 < ss->C1q) {
        x = ss->Sq / rr0; y = x * x * x; z = y * y;
        U = ss->E4 * (z - y);
        f = ss->E24 * (z + z - y) * x;
      } else {
        x = rr0 - ss->C2q;
        U = x * x * ss->A;
        f = ss->A4 * x;
      }
      if (measure) { w->vir += rr0 * f; w->lj += U; }
    }
  }
  for (m = 0; m < 4; m++) {
    double d[3], rr, fe = 0, e = 0;
    if (t[m].q == 0 && !(m == 0 && f != 0)) continue;
    for (k = 0; k < 3; k++) d[k] = dr0[k] + (t[m].sgn_i ? di[k] : 0) - (t[m].sgn_j ? dj[k] : 0);
    rr = SQ(d[0]) + SQ(d[1]) + SQ(d[2]);
    if (t[m].q != 0) {
      if (excl) {
        e = orc_exacterud_sqrt(rr, s->alpha, &fe) * t[m].q;
        fe *= t[m].q;
      } else {
        const double *p = s->ertab + 6 * (int)(rr * s->sgrid);
        fe = (p[4] / (p[5] + rr) + p[3]) * t[m].q;
        e = (p[1] / (p[2] + rr) + p[0]) * t[m].q;
      }
    }
    if (m == 0) fe += f;
    if (measure) w->el += e;
    {
      double fx = fe * d[0], fy = fe * d[1], fz = fe * d[2];
      t[m].fa[0] += fx; t[m].fa[1] += fy; t[m].fa[2] += fz;
      t[m].fb[0] -= fx; t[m].fb[1] -= fy; t[m].fb[2] -= fz;
      if (measure) {
        w->Pvir[0] += d[0] * fx; w->Pvir[1] += d[1] * fy; w->Pvir[2] += d[2] * fz;
        w->Pvir[3] += d[2] * fy; w->Pvir[4] += d[0] * fz; w->Pvir[5] += d[1] * fx;
      }
    }
  }
}

static void nearest(const double L[3], const double *ri, const double *rj, double dr[3])
{
  int k;
  for (k = 0; k < 3; k++) {
    double d = ri[k] - rj[k], Lh = 0.5 * L[k];
    if (d < -Lh) d += L[k];
    else if (d > Lh) d -= L[k];
    dr[k] = d;
  }
}

static int cell_of(const double L[3], const int nc[3], const double *r, int k)
{
  double x = r[k] / L[k];
  int c;
  x -= floor(x);
  c = (int)(x * nc[k]);
  if (c >= nc[k]) c = nc[k] - 1;
  if (c < 0) c = 0;
  return c;
}

static int g_measure;

/* r-space worker: cells ≥ cutoff, half stencil over the 27 neighbours when
   every dimension has >=3 cells, otherwise all pairs with nearest image */
static void *rspace_worker(void *arg)
{
  orc_work_t *w = arg;
  const orc_sys_t *s = w->s;
  int ns = s->ns, measure = g_measure;
  const double *r = w->r;
  if (w->cellhead == NULL) {
    int i, j;
    for (i = w->ith; i < ns; i += w->nth)
      for (j = i + 1; j < ns; j++) {
        double dr[3], rr;
        nearest(s->L, r + 3 * i, r + 3 * j, dr);
        rr = SQ(dr[0]) + SQ(dr[1]) + SQ(dr[2]);
        if (rr >= SQ(s->cutoff)) continue;
        if (is_polar(s)) pair_pol(w, i, j, dr, rr, w->f, measure);
        else pair_np(w, i, j, dr, rr, w->f + 3 * i, w->f + 3 * j, measure);
      }
  } else {
    const int *nc = w->nc;
    int ncell = nc[0] * nc[1] * nc[2], c;
    for (c = w->ith; c < ncell; c += w->nth) {
      int cx = c / (nc[1] * nc[2]), cy = (c / nc[2]) % nc[1], cz = c % nc[2];
      int d;
      for (d = 0; d < 27; d++) {
        int dx = d / 9 - 1, dy = (d / 3) % 3 - 1, dz = d % 3 - 1;
        int c2 = ((cx + dx + nc[0]) % nc[0]) * nc[1] * nc[2] +
                 ((cy + dy + nc[1]) % nc[1]) * nc[2] + ((cz + dz + nc[2]) % nc[2]);
        int i, j;
        if (c2 < c) continue; /* half stencil: each unordered cell pair once */
        for (i = w->cellhead[c]; i >= 0; i = w->cellnext[i])
          for (j = w->cellhead[c2]; j >= 0; j = w->cellnext[j]) {
            double dr[3], rr;
            if (c2 == c && j <= i) continue;
            nearest(s->L, r + 3 * i, r + 3 * j, dr);
            rr = SQ(dr[0]) + SQ(dr[1]) + SQ(dr[2]);
            if (rr >= SQ(s->cutoff)) continue;
            if (is_polar(s)) pair_pol(w, i, j, dr, rr, w->f, measure);
            else pair_np(w, i, j, dr, rr, w->f + 3 * i, w->f + 3 * j, measure);
          }
      }
    }
  }
  return NULL;
}

/* -------------------------------------------------------------- k-space --- */

/* charge list: non-polar = sites with q != 0 (order of sim/ewald.c:632-690) */
typedef struct { int site; double q; int drude; } qitem_t;

static qitem_t *g_qlist;
static int g_nq;

static void charge_pos(const orc_sys_t *s, const double *r, const qitem_t *it, double p[3])
{
  int k;
  for (k = 0; k < 3; k++) {
    p[k] = r[3 * it->site + k];
    if (it->drude) p[k] += r[3 * s->ns + 3 * it->site + k];
  }
}

/* powers e^{2 pi i n x/L} for n = -nmax..nmax by incremental complex
   products, as the reference builds its per-charge factors (sim/ewald.c:632-690,
   sim/ewpass1.c: CxE/CxiE recurrences) */
static void phase_powers(double x, double L, int nmax, double *pre, double *pim)
{
  double er = cos(2 * M_PI / L * x), ei = sin(2 * M_PI / L * x);
  int n;
  pre[nmax] = 1; pim[nmax] = 0;
  for (n = 1; n <= nmax; n++) {
    double a = pre[nmax + n - 1], b = pim[nmax + n - 1];
    pre[nmax + n] = a * er - b * ei;
    pim[nmax + n] = a * ei + b * er;
    pre[nmax - n] = pre[nmax + n];
    pim[nmax - n] = -pim[nmax + n];
  }
}

static int g_kmax[3];

/* q e^{2 pi i k.r/L} of charge j for every k-vector */
static void charge_phases(const orc_sys_t *s, const double *r, const qitem_t *it,
                          int nk, const int *kv, double *xr, double *xi)
{
  double p[3];
  double *pw[3][2];
  int d, m;
  charge_pos(s, r, it, p);
  for (d = 0; d < 3; d++) {
    pw[d][0] = malloc(sizeof(double) * (2 * g_kmax[d] + 1));
    pw[d][1] = malloc(sizeof(double) * (2 * g_kmax[d] + 1));
    phase_powers(p[d], s->L[d], g_kmax[d], pw[d][0], pw[d][1]);
  }
  for (m = 0; m < nk; m++) {
    const int *k = kv + 3 * m;
    int a = k[0] + g_kmax[0], b = k[1] + g_kmax[1], c = k[2] + g_kmax[2];
    double ar = pw[0][0][a], ai = pw[0][1][a], br = pw[1][0][b], bi = pw[1][1][b];
    double xyr = ar * br - ai * bi, xyi = ar * bi + ai * br;
    double cr = pw[2][0][c], ci = pw[2][1][c];
    xr[m] = it->q * (xyr * cr - xyi * ci);
    xi[m] = it->q * (xyr * ci + xyi * cr);
  }
  for (d = 0; d < 3; d++) { free(pw[d][0]); free(pw[d][1]); }
}

/* pass 1 (sim/ewpass1.c): S(k) = sum_j q_j exp(2 pi i k.r_j/L); each
   thread sums a slice of the charges (sim/ewald.c:197-243 PARALLEL==1) */
static void *kspace1_worker(void *arg)
{
  orc_work_t *w = arg;
  int j0 = g_nq * w->ith / w->nth, j1 = g_nq * (w->ith + 1) / w->nth, j, m;
  double *xr = malloc(sizeof(double) * (w->nk + 1)), *xi = malloc(sizeof(double) * (w->nk + 1));
  for (j = j0; j < j1; j++) {
    charge_phases(w->s, w->r, g_qlist + j, w->nk, w->kv, xr, xi);
    for (m = 0; m < w->nk; m++) { w->Sre[m] += xr[m]; w->Sim[m] += xi[m]; }
  }
  free(xr); free(xi);
  return NULL;
}

/* pass 2 (sim/ewpass2m.c + sim/ewaldf.c): F_j += ekk k/L Im(conj(S) q e^{ikr}) */
static void *kspace2_worker(void *arg)
{
  orc_work_t *w = arg;
  const orc_sys_t *s = w->s;
  int j0 = g_nq * w->ith / w->nth, j1 = g_nq * (w->ith + 1) / w->nth, j, m;
  double *xr = malloc(sizeof(double) * (w->nk + 1)), *xi = malloc(sizeof(double) * (w->nk + 1));
  for (j = j0; j < j1; j++) {
    double F[3] = {0, 0, 0};
    const qitem_t *it = g_qlist + j;
    double *fo = w->f + (it->drude ? 3 * s->ns : 0) + 3 * it->site;
    charge_phases(s, w->r, it, w->nk, w->kv, xr, xi);
    for (m = 0; m < w->nk; m++) {
      const int *k = w->kv + 3 * m;
      double FA = w->gre[m] * xi[m] - w->gim[m] * xr[m], e = w->ekk[m];
      F[0] += e * (k[0] / s->L[0]) * FA;
      F[1] += e * (k[1] / s->L[1]) * FA;
      F[2] += e * (k[2] / s->L[2]) * FA;
    }
    fo[0] += F[0]; fo[1] += F[1]; fo[2] += F[2];
  }
  free(xr); free(xi);
  return NULL;
}

/* ---------------------------------------------------------- orc_forces --- */

int orc_forces(const orc_sys_t *s, const double *r, double *f, orc_en_t *en, int nthreads)
{
  int ns = s->ns, nf = is_polar(s) ? 6 * ns : 3 * ns, t, i, m;
  int measure = en != NULL;
  orc_work_t *w;
  int *kv, nk, nc[3], usecells = 1;
  double kappa = s->kappa, V = s->L[0] * s->L[1] * s->L[2];
  double Energy = 0, PVIR[6] = {0, 0, 0, 0, 0, 0}, M[3] = {0, 0, 0}, sumq = 0;
  double *Sre, *Sim, *ekk;
  int *cellhead = NULL, *cellnext = NULL;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 64) nthreads = 64;
  g_measure = measure;
  memset(f, 0, sizeof(double) * nf);
  w = calloc(nthreads, sizeof(orc_work_t));

  /* charges in the order of the reference qtab */
  g_qlist = malloc(sizeof(qitem_t) * 2 * ns);
  g_nq = 0;
  for (i = 0; i < ns; i++) {
    if (s->q[i] != 0) { g_qlist[g_nq].site = i; g_qlist[g_nq].q = s->q[i]; g_qlist[g_nq].drude = 0; g_nq++; }
    if (is_polar(s) && s->qpol[i] != 0) {
      g_qlist[g_nq].site = i; g_qlist[g_nq].q = s->qpol[i]; g_qlist[g_nq].drude = 1; g_nq++;
    }
    /* self term uses the total charge of the site (sim/ewald.c:395-410) */
    sumq += SQ(s->q[i] + (is_polar(s) ? s->qpol[i] : 0));
  }

  /* cells for the r-space sum */
  for (m = 0; m < 3; m++) {
    nc[m] = (int)(s->L[m] / s->cutoff);
    if (nc[m] < 3) usecells = 0;
  }
  if (usecells) {
    int ncell = nc[0] * nc[1] * nc[2];
    cellhead = malloc(sizeof(int) * ncell);
    cellnext = malloc(sizeof(int) * ns);
    for (i = 0; i < ncell; i++) cellhead[i] = -1;
    for (i = ns - 1; i >= 0; i--) {
      int c = (cell_of(s->L, nc, r + 3 * i, 0) * nc[1] + cell_of(s->L, nc, r + 3 * i, 1)) * nc[2] +
              cell_of(s->L, nc, r + 3 * i, 2);
      cellnext[i] = cellhead[c];
      cellhead[c] = i;
    }
  }

  /* k-vectors (count + list), ekk (sim/ewald.c:565-600) */
  nk = orc_kvectors(s->L, &kappa, 0, NULL);
  kv = malloc(sizeof(int) * 3 * (nk > 0 ? nk : 1));
  kappa = s->kappa;
  orc_kvectors(s->L, &kappa, nk, kv);
  ekk = malloc(sizeof(double) * (nk + 1));
  g_kmax[0] = g_kmax[1] = g_kmax[2] = 0;
  for (m = 0; m < nk; m++) {
    int d;
    for (d = 0; d < 3; d++)
      if (abs(kv[3 * m + d]) > g_kmax[d]) g_kmax[d] = abs(kv[3 * m + d]);
  }
  Sre = calloc(nk + 1, sizeof(double));
  Sim = calloc(nk + 1, sizeof(double));
  {
    double PIaq = -SQ(M_PI / s->alpha);
    for (m = 0; m < nk; m++) {
      double kk = SQ(kv[3 * m + 2] / s->L[2]) + (SQ(kv[3 * m + 1] / s->L[1]) + SQ(kv[3 * m] / s->L[0]));
      ekk[m] = 4 / (kk * V) * exp(PIaq * kk);
    }
  }

  for (t = 0; t < nthreads; t++) {
    w[t].s = s; w[t].r = r; w[t].ith = t; w[t].nth = nthreads;
    w[t].f = calloc(nf, sizeof(double));
    w[t].nk = nk; w[t].kv = kv; w[t].ekk = ekk;
    w[t].Sre = calloc(nk + 1, sizeof(double));
    w[t].Sim = calloc(nk + 1, sizeof(double));
    w[t].cellhead = cellhead; w[t].cellnext = cellnext;
    memcpy(w[t].nc, nc, sizeof(nc));
  }

  /* Ewald pass 1 */
  run_threads(kspace1_worker, w, nthreads);
  for (t = 0; t < nthreads; t++)
    for (m = 0; m < nk; m++) { Sre[m] += w[t].Sre[m]; Sim[m] += w[t].Sim[m]; }
  for (t = 0; t < nthreads; t++) { w[t].gre = Sre; w[t].gim = Sim; }

  /* pass 2 energy and k-space virial (sim/ewpass2m.c measure branch) */
  if (measure) {
    double PIaq = -SQ(M_PI / s->alpha);
    for (m = 0; m < nk; m++) {
      double kx = kv[3 * m] / s->L[0], ky = kv[3 * m + 1] / s->L[1], kz = kv[3 * m + 2] / s->L[2];
      double kk = SQ(kx) + SQ(ky) + SQ(kz), E1 = (SQ(Sre[m]) + SQ(Sim[m])) * ekk[m];
      double ptf = 1 / kk - PIaq;
      Energy += E1;
      PVIR[0] += E1 * ptf * SQ(kx);
      PVIR[1] += E1 * ptf * SQ(ky);
      PVIR[2] += E1 * ptf * SQ(kz);
      PVIR[3] += E1 * ptf * ky * kz;
      PVIR[4] += E1 * ptf * kx * kz;
      PVIR[5] += E1 * ptf * kx * ky;
    }
    Energy /= 4 * M_PI;
  }
  run_threads(kspace2_worker, w, nthreads);

  /* r-space */
  run_threads(rspace_worker, w, nthreads);

  for (t = 0; t < nthreads; t++)
    for (i = 0; i < nf; i++) f[i] += w[t].f[i];

  /* dipole (epsinf) term and forces, sim/ewald.c:865-887 + sim/ewaldf.c */
  {
    double c, ek[3], Edip;
    for (i = 0; i < g_nq; i++) {
      double p[3];
      charge_pos(s, r, g_qlist + i, p);
      for (m = 0; m < 3; m++) M[m] += g_qlist[i].q * p[m];
    }
    if (s->elcorr) {
      /* Yeh-Berkowitz: the selected axes only (sim/ewald.c:869-882) */
      c = 4 * M_PI / V;
      Edip = 0;
      for (m = 0; m < 3; m++) {
        ek[m] = 0;
        if (s->elcorr & 1 << m) {
          if (!(s->elcorr & 8)) ek[m] = -c * M[m];
          Edip += c / 2 * SQ(M[m]);
        }
      }
    } else {
      c = 4 * M_PI / (2 * s->epsinf + 1) / V;
      for (m = 0; m < 3; m++) ek[m] = -c * M[m];
      Edip = c / 2 * (SQ(M[0]) + SQ(M[1]) + SQ(M[2]));
    }
    for (i = 0; i < g_nq; i++) {
      const qitem_t *it = g_qlist + i;
      double *fo = f + (it->drude ? 3 * ns : 0) + 3 * it->site, p[3];
      for (m = 0; m < 3; m++) fo[m] += it->q * ek[m];
      if (measure) {
        charge_pos(s, r, it, p);
        /* aux*ek*R (diagonal) and off-diagonal terms of ewaldf ADDFORCES */
        w[0].Pvir[0] += it->q * ek[0] * p[0];
        w[0].Pvir[1] += it->q * ek[1] * p[1];
        w[0].Pvir[2] += it->q * ek[2] * p[2];
        w[0].Pvir[3] += it->q * ek[1] * p[2];
        w[0].Pvir[4] += it->q * ek[2] * p[0];
        w[0].Pvir[5] += it->q * ek[0] * p[1];
      }
    }
    if (measure) {
      double el = 0, lj = 0, vir = 0, Pv[6] = {0, 0, 0, 0, 0, 0};
      memset(en, 0, sizeof(*en));
      for (t = 0; t < nthreads; t++) {
        el += w[t].el; lj += w[t].lj; vir += w[t].vir;
        for (m = 0; m < 6; m++) Pv[m] += w[t].Pvir[m];
      }
      en->er = el;
      en->ek = Energy;
      en->eself = -s->alpha / SQRTPI * sumq;
      en->edip = Edip;
      en->el = Energy - s->alpha / SQRTPI * sumq + Edip + el;
      en->lj = lj;
      en->vir = vir;
      /* k-space tensor: +Energy on the diagonal, -2/(4 pi) PVIR (sim/ewald.c:852-856) */
      for (m = 0; m < 3; m++) Pv[m] += Energy + Edip;
      for (m = 0; m < 6; m++) Pv[m] -= 2 / (4 * M_PI) * PVIR[m];
      memcpy(en->Pvir, Pv, sizeof(Pv));
    }
  }

  for (t = 0; t < nthreads; t++) { free(w[t].f); free(w[t].Sre); free(w[t].Sim); }
  free(w); free(kv); free(ekk); free(Sre); free(Sim); free(g_qlist);
  free(cellhead); free(cellnext);
  return 0;
}

/* ---------------------------------------------------------------- SHAKE --- */

/* sim/constrd.c:767-839 (SHAKE=1 sweeps) with sim/verlet.c:101-104 (no
   thermostat) and the VERLET=3 kinetic energy of sim/shakev3.c */
int orc_shake_step_dp(int ns, double *r, double *r1, const double *f, const double *mass,
                      int nmol, const int *mol_first, const int *mol_nc, const int *cfirst,
                      const int *ci, const int *cj, const double *bondq,
                      double h, double eps, double omega, int maxit, const double *dp,
                      double *ekin);

int orc_shake_step(int ns, double *r, double *r1, const double *f, const double *mass,
                   int nmol, const int *mol_first, const int *mol_nc, const int *cfirst,
                   const int *ci, const int *cj, const double *bondq,
                   double h, double eps, double omega, int maxit, double *ekin)
{
  return orc_shake_step_dp(ns, r, r1, f, mass, nmol, mol_first, mol_nc, cfirst, ci, cj, bondq,
                           h, eps, omega, maxit, NULL, ekin);
}

/* the same step with dp[] added to the unconstrained positions: the
   Nose-Hoover friction term -Vfactor v_pred of sim/verlet.c:22-37 */
int orc_shake_step_dp(int ns, double *r, double *r1, const double *f, const double *mass,
                      int nmol, const int *mol_first, const int *mol_nc, const int *cfirst,
                      const int *ci, const int *cj, const double *bondq,
                      double h, double eps, double omega, int maxit, const double *dp,
                      double *ekin)
{
  return orc_shake_step_meas(ns, r, r1, f, mass, nmol, mol_first, mol_nc, cfirst, ci, cj,
                             bondq, h, eps, omega, maxit, dp, ekin, NULL);
}

/* the step of a measured cycle: with meas != NULL also cook's constraint
   virial (sim/virc.c, accumulated in the sweep at sim/constrd.c:833 and
   divided by h^2 at sim/constrd.c:1038-1040) and the VERLET=3 kinetic
   tensor (sim/shakev3.c:20-32 scaled by hscale = 0.5/h^2,
   sim/constrd.c:1012-1017): meas[0] = En.virc, meas[1..6] = PTvirc,
   meas[7..12] = En.Pkin before the division by V (xx yy zz yz zx xy) */
int orc_shake_step_meas(int ns, double *r, double *r1, const double *f, const double *mass,
                        int nmol, const int *mol_first, const int *mol_nc, const int *cfirst,
                        const int *ci, const int *cj, const double *bondq,
                        double h, double eps, double omega, int maxit, const double *dp,
                        double *ekin, double *meas)
{
  double hh = h * h, kin = 0, virc = 0, PT[6] = {0, 0, 0, 0, 0, 0}, PK[6] = {0, 0, 0, 0, 0, 0};
  int n, worst = 0;
  double *p = malloc(sizeof(double) * 3 * ns);
  for (n = 0; n < nmol; n++) {
    int i0 = mol_first[n], i1 = mol_first[n + 1], i, k, it = 0, al;
    int c0 = cfirst[n], nc = mol_nc[n];
    double maxsq;
    for (i = i0; i < i1; i++)
      for (k = 0; k < 3; k++)
        /* a massless site is a dependant, placed by depend_r after the step;
           the friction term joins h^2 f/m before r and r1 are added, as in
           sim/verlet.c:35-36 */
        p[3 * i + k] = f[3 * i + k] * (mass[i] > 0 ? hh / mass[i] : 0) +
                       (dp ? dp[3 * i + k] : 0) + r[3 * i + k] + r1[3 * i + k];
    if (nc > 0) {
      do {
        it++;
        maxsq = 0;
        for (al = c0; al < c0 + nc; al++) {
          int a = ci[al], b = cj[al];
          double pij[3], rij[3], sq = bondq[al], mi = 1 / mass[a], mj = 1 / mass[b];
          for (k = 0; k < 3; k++) pij[k] = p[3 * a + k] - p[3 * b + k];
          sq -= SQ(pij[0]) + SQ(pij[1]) + SQ(pij[2]);
          if (fabs(sq / bondq[al]) > maxsq) maxsq = fabs(sq / bondq[al]);
          for (k = 0; k < 3; k++) rij[k] = r[3 * a + k] - r[3 * b + k];
          sq *= omega / (mi + mj);
          if (meas) {
            double sb = sq / bondq[al];
            PT[0] += sb * (rij[0] * rij[0]);
            PT[1] += sb * (rij[1] * rij[1]);
            PT[2] += sb * (rij[2] * rij[2]);
            PT[3] += sb * (rij[1] * rij[2]);
            PT[4] += sb * (rij[2] * rij[0]);
            PT[5] += sb * (rij[0] * rij[1]);
            virc += sq;
          }
          sq /= bondq[al];
          for (k = 0; k < 3; k++) {
            rij[k] *= sq;
            p[3 * a + k] += mi * rij[k];
            p[3 * b + k] -= mj * rij[k];
          }
        }
      } while (maxsq > eps && it < maxit);
      if (it >= maxit && maxsq > eps) { free(p); return -1; }
    }
    if (it > worst) worst = it;
    for (i = i0; i < i1; i++) {
      double V2[3], V1[3];
      for (k = 0; k < 3; k++) {
        V1[k] = r1[3 * i + k];
        V2[k] = p[3 * i + k] - r[3 * i + k];
      }
      kin += (SQ(V1[0]) + SQ(V1[1]) + SQ(V1[2]) + SQ(V2[0]) + SQ(V2[1]) + SQ(V2[2])) * mass[i];
      PK[0] += (V1[0] * V1[0] + V2[0] * V2[0]) * mass[i];
      PK[1] += (V1[1] * V1[1] + V2[1] * V2[1]) * mass[i];
      PK[2] += (V1[2] * V1[2] + V2[2] * V2[2]) * mass[i];
      PK[3] += (V1[1] * V1[2] + V2[1] * V2[2]) * mass[i];
      PK[4] += (V1[2] * V1[0] + V2[2] * V2[0]) * mass[i];
      PK[5] += (V1[0] * V1[1] + V2[0] * V2[1]) * mass[i];
      for (k = 0; k < 3; k++) { r1[3 * i + k] = V2[k]; r[3 * i + k] = p[3 * i + k]; }
    }
  }
  free(p);
  if (ekin) *ekin = kin / hh / 4;
  if (meas) {
    meas[0] = virc / hh;
    for (n = 0; n < 6; n++) {
      meas[1 + n] = PT[n] / hh;
      meas[7 + n] = PK[n] * (0.5 / hh);
    }
  }
  return worst;
}

/* ------------------------------------------------------------- Drude --- */

/* sim/scf.c:12-300 selffield (POLAR=0, no saturation): Ewald correction of
   the centre-Drude pair of each site (exacterud_sqrt_1), relaxation
   rpol <- (1-omega) rpol + omega alpha_qq fpol, Drude force folded into the
   centre, spring energy and virial.  Returns the max |rpol change|/omega. */
double orc_selffield(const orc_sys_t *s, double *r, double *f, orc_en_t *en, double omega)
{
  int ns = s->ns, i, k;
  double self = 0, maxd = 0;
  for (i = 0; i < ns; i++) {
    double *rp = r + 3 * ns + 3 * i, *fp = f + 3 * ns + 3 * i, *fc = f + 3 * i;
    double rr, byerd, fq, old[3], dd = 0;
    if (s->qpol[i] == 0) continue;
    rr = SQ(rp[0]) + SQ(rp[1]) + SQ(rp[2]);
    fq = s->q[i] * s->qpol[i];
    {
      double e = orc_exacterud_sqrt_1(rr, s->alpha, &byerd);
      double ff = fq * byerd;
      if (en) en->el += fq * e;
      for (k = 0; k < 3; k++) {
        double fdr = ff * rp[k];
        fp[k] += fdr;
        fc[k] -= fdr;
      }
      if (en) {
        en->Pvir[0] += rp[0] * ff * rp[0]; en->Pvir[1] += rp[1] * ff * rp[1];
        en->Pvir[2] += rp[2] * ff * rp[2]; en->Pvir[3] += rp[2] * ff * rp[1];
        en->Pvir[4] += rp[0] * ff * rp[2]; en->Pvir[5] += rp[1] * ff * rp[0];
      }
    }
    for (k = 0; k < 3; k++) {
      old[k] = rp[k];
      rp[k] = (1 - omega) * rp[k] + omega * s->alphaqq[i] * fp[k];
      dd += SQ(old[k] - rp[k]);
      fc[k] += fp[k];
    }
    if (dd > maxd) maxd = dd;
    self += rp[0] * fp[0] + rp[1] * fp[1] + rp[2] * fp[2];
    if (en) {
      en->Pvir[0] -= rp[0] * fp[0]; en->Pvir[1] -= rp[1] * fp[1]; en->Pvir[2] -= rp[2] * fp[2];
      en->Pvir[3] -= rp[1] * fp[2]; en->Pvir[4] -= rp[2] * fp[0]; en->Pvir[5] -= rp[0] * fp[1];
    }
  }
  if (en) en->self = self / 2;
  return sqrt(maxd) / omega;
}

/* ASPC coefficients of sim/pred2.c:70-97 (Kolafa 2004) for predictor length
   k: B[0..k+1] and the stabilizing mixing omega=(k+2)/(2k+3); k=0 gives the
   linear predictor {2,-1} */
void orc_aspc_coef(int k, double *B, double *omega)
{
  int i;
  if (k == 0) { B[0] = 2; B[1] = -1; *omega = 2.0 / 3.0; return; }
  {
    double o = (double)(4 * k + 6) / (double)(k + 3);
    for (i = 0; i < k + 2; i++) {
      B[i] = o * (i + 1);
      o *= (double)(i - k - 1) / (double)(k + i + 4);
    }
  }
  *omega = (k + 2) / (double)(2 * k + 3);
}

/* --------------------------------------------------------------- Widom --- */

/* The insertion stream.  The reference draws rnd() (gen/rndgen.h); the
   insertion points are inputs of the method, so the oracle and the GPU path
   share one counter-based stream instead: word c of insertion k is the
   SplitMix64 output function (Steele, Lea and Flood, "Fast splittable
   pseudorandom number generators", OOPSLA 2014) of seed + (8k+c+1)*gamma. */
static uint64_t mix64(uint64_t z)
{
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

unsigned long long orc_widom_word(unsigned long long seed, long long k, int c)
{
  return mix64(seed + (uint64_t)(8 * k + c + 1) * 0x9E3779B97F4A7C15ULL);
}

/* probe sites of insertion k: the point is (w_c >> 32)/2^32 * L_c for words
   c = 0,1,2; for more than one site the geometry is turned by the uniform
   random rotation of Shoemake ("Uniform random rotations", Graphics Gems
   III, 1992) from u_c = (w_c >> 11)/2^53, c = 3,4,5 (cook/simils.c
   rndorientation plays this part in the reference) */
void orc_widom_sites(unsigned long long seed, long long k, const double L[3], int nps, const double *geom,
                     double *out)
{
  double p[3], R[9];
  int c, i;
  for (c = 0; c < 3; c++)
    p[c] = (double)(uint32_t)(orc_widom_word(seed, k, c) >> 32) * (1.0 / 4294967296.0) * L[c];
  if (nps > 1) {
    double u1 = (double)(orc_widom_word(seed, k, 3) >> 11) * (1.0 / 9007199254740992.0);
    double u2 = (double)(orc_widom_word(seed, k, 4) >> 11) * (1.0 / 9007199254740992.0);
    double u3 = (double)(orc_widom_word(seed, k, 5) >> 11) * (1.0 / 9007199254740992.0);
    double a = sqrt(1 - u1), b = sqrt(u1);
    double x = a * sin(2 * M_PI * u2), y = a * cos(2 * M_PI * u2);
    double z = b * sin(2 * M_PI * u3), w = b * cos(2 * M_PI * u3);
    R[0] = 1 - 2 * (y * y + z * z); R[1] = 2 * (x * y - z * w);     R[2] = 2 * (x * z + y * w);
    R[3] = 2 * (x * y + z * w);     R[4] = 1 - 2 * (x * x + z * z); R[5] = 2 * (y * z - x * w);
    R[6] = 2 * (x * z - y * w);     R[7] = 2 * (y * z + x * w);     R[8] = 1 - 2 * (x * x + y * y);
  } else {
    R[0] = R[4] = R[8] = 1;
    R[1] = R[2] = R[3] = R[5] = R[6] = R[7] = 0;
  }
  for (i = 0; i < nps; i++)
    for (c = 0; c < 3; c++)
      out[3 * i + c] = p[c] + R[3 * c] * geom[3 * i] + R[3 * c + 1] * geom[3 * i + 1] +
                       R[3 * c + 2] * geom[3 * i + 2];
}

/* Einsert (cook/widom.c:175-288): energy of a ghost molecule with sites at
   ppos against every site of the box within the cutoff (nearest image):
   the pair function of cook/ljqqnp.c (LJ with the smooth cutoff + q q eru,
   r-space only); no intramolecular exclusion applies to the ghost
   (lsloc.n = No.s, cook/widom.c:195) */
double orc_einsert(const orc_sys_t *s, const double *r, int nps, const int *ptype,
                   const double *pq, const double *ppos)
{
  double U = 0, El = 0;
  const double cq = SQ(s->cutoff);
  int a, j;
  for (a = 0; a < nps; a++)
    for (j = 0; j < s->ns; j++) {
      double dr[3], rr, x, y;
      const orc_ss_t *ss = s->ss + ptype[a] * s->ntypes + s->type[j];
      const double qq = (pq ? pq[a] : 0) * s->q[j];
      nearest(s->L, ppos + 3 * a, r + 3 * j, dr);
      rr = SQ(dr[0]) + SQ(dr[1]) + SQ(dr[2]);
      if (rr >= cq) continue;
      if (rr < ss->C2q) {
        if (rr < ss->C1q) {
          x = ss->Sq / rr;
          y = x * x * x;
          U += ss->E4 * (y * y - y);
        } else {
          x = rr - ss->C2q;
          U += x * x * ss->A;
        }
      }
      if (qq != 0) {
        const double *p = s->ertab + 6 * (int)(rr * s->sgrid);
        El += (p[1] / (p[2] + rr) + p[0]) * qq;
      }
    }
  return U + El;
}

/* cook/widom.c:16-170 (Eidchange) and sim/simmeas.c:1961-2003 (XWidom):
   for each listed molecule, the r-space energy change (smoothed LJ + erfc
   spline) of giving its sites the types vtype[] and charges vq[], summed
   over every site of the other molecules within the cutoff (the molecule
   itself is taken out of the cell list first); returns the sum of
   exp(-dU/T) (a term with -dU/T <= -700 counts 0); dU[] per molecule */
double orc_xwidom(const orc_sys_t *s, const double *r, int nlist, const int *mols,
                  const int *mol_first, const int *vtype, const double *vq, double T,
                  double *dU)
{
  const double cq = SQ(s->cutoff);
  double sum = 0;
  int l, i, j;
  for (l = 0; l < nlist; l++) {
    const int n = mols[l], i0 = mol_first[n], i1 = mol_first[n + 1];
    double Ur = 0, Uv = 0, El = 0, e;
    for (i = i0; i < i1; i++) {
      const int k = i - i0;
      for (j = 0; j < s->ns; j++) {
        double dr[3], rr, x, y;
        const orc_ss_t *sr, *sv;
        if (s->mol[j] == s->mol[i]) continue;
        nearest(s->L, r + 3 * i, r + 3 * j, dr);
        rr = SQ(dr[0]) + SQ(dr[1]) + SQ(dr[2]);
        if (rr >= cq) continue;
        sr = s->ss + s->type[i] * s->ntypes + s->type[j];
        sv = s->ss + vtype[k] * s->ntypes + s->type[j];
        if (rr < sr->C2q) {
          if (rr < sr->C1q) {
            x = sr->Sq / rr;
            y = x * x * x;
            Ur += sr->E4 * (y * y - y);
          } else {
            x = rr - sr->C2q;
            Ur += x * x * sr->A;
          }
        }
        if (rr < sv->C2q) {
          if (rr < sv->C1q) {
            x = sv->Sq / rr;
            y = x * x * x;
            Uv += sv->E4 * (y * y - y);
          } else {
            x = rr - sv->C2q;
            Uv += x * x * sv->A;
          }
        }
        if (s->q[j] != 0 && vq[k] != s->q[i]) {
          const double *p = s->ertab + 6 * (int)(rr * s->sgrid);
          El += (p[1] / (p[2] + rr) + p[0]) * (vq[k] - s->q[i]) * s->q[j];
        }
      }
    }
    if (dU) dU[l] = Uv - Ur + El;
    e = -(Uv - Ur + El) / T;
    if (e > -700) sum += exp(e);
  }
  return sum;
}

typedef struct {
  const orc_sys_t *s;
  const double *r, *geom, *pq;
  const int *ptype;
  int nps;
  long long k0, k1;
  uint64_t seed;
  double T, sum;
  double *U;
} widom_work_t;

static void *widom_worker(void *arg)
{
  widom_work_t *w = (widom_work_t *)arg;
  double pos[3 * 16];
  long long k;
  w->sum = 0;
  for (k = w->k0; k < w->k1; k++) {
    double U, e;
    orc_widom_sites(w->seed, k, w->s->L, w->nps, w->geom, pos);
    U = orc_einsert(w->s, w->r, w->nps, w->ptype, w->pq, pos);
    if (w->U) w->U[k] = U;
    e = -U / w->T;
    if (e > -700) w->sum += exp(e);
  }
  return NULL;
}

/* Widom (sim/simmeas.c:1821-1958): sum over n insertions of exp(-U/T),
   a term skipped when -U/T <= -700; per-insertion energies into U when
   U != NULL.  The caller divides by n and applies exp(-corr/(V T)). */
double orc_widom(const orc_sys_t *s, const double *r, int nps, const int *ptype,
                 const double *pq, const double *geom, long long n, unsigned long long seed, double T,
                 double *U, int nthreads)
{
  widom_work_t w[64];
  pthread_t th[64];
  double sum = 0;
  int t;
  if (nps > 16) return -1;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 64) nthreads = 64;
  for (t = 0; t < nthreads; t++) {
    w[t].s = s; w[t].r = r; w[t].geom = geom; w[t].pq = pq; w[t].ptype = ptype;
    w[t].nps = nps; w[t].seed = seed; w[t].T = T; w[t].U = U;
    w[t].k0 = n * t / nthreads;
    w[t].k1 = n * (t + 1) / nthreads;
    pthread_create(&th[t], NULL, widom_worker, &w[t]);
  }
  for (t = 0; t < nthreads; t++) {
    pthread_join(th[t], NULL);
    sum += w[t].sum;
  }
  return sum;
}

/* Widomcutcorr (sim/siminit.c:762-808): sum of the pair cutoff corrections
   (setss, sim/setss.c:454-500) over the ghost's sites x every box site */
double orc_widom_corr(const orc_sys_t *s, int nps, const int *ptype)
{
  double c = 0;
  int a, j;
  for (a = 0; a < nps; a++)
    for (j = 0; j < s->ns; j++) c += s->ss[ptype[a] * s->ntypes + s->type[j]].corr;
  return c;
}

/* ------------------------------------------------------------- adjoint --- */

/* d/d sigma of the smoothed LJ pair terms: u = E4 (y^2 - y), y = (Sq/r^2)^3
   below C1 (sigma^2 = Sq), u = A (r^2 - C2^2)^2 above; f = -2 du/d(r^2).
   dA[0], dA[1]: dA/dsigma, dA4/dsigma of the smoothing constants. */
static void lj_terms(const orc_ss_t *ss, const double *dA, double rr, double *u, double *f,
                     double *du, double *df)
{
  *u = *f = *du = *df = 0;
  if (rr >= ss->C2q || ss->E4 == 0) return;
  if (rr < ss->C1q) {
    double sig = sqrt(ss->Sq), y = ss->Sq / rr;
    y = y * y * y;
    *u = ss->E4 * (y * y - y);
    *f = 6 * ss->E4 * (2 * y * y - y) / rr;
    *du = ss->E4 / sig * (12 * y * y - 6 * y);
    *df = 36 * ss->E4 * y * (4 * y - 1) / (sig * rr);
  } else {
    double x = rr - ss->C2q;
    *u = ss->A * x * x;
    *f = ss->A4 * x;
    *du = dA[0] * x * x;
    *df = dA[1] * x;
  }
}

/* Gradients of the energy E, the scalar virial W = sum r.f (LJ) + E_el, and
   (with g = dLoss/dF, [3 ns]) of a loss of the forces, with respect to the
   LJ parameters of every type pair (epsilon > 0 and sigma of
   4 eps [(sigma/r)^12 - (sigma/r)^6]) and to every site charge.  The
   restatement of the adjoint: all pairs by nearest image, k-space by direct
   sums over the k set of orc_forces, tin-foil boundary (no dipole term).
   Per type pair (a <= b) arrays [nt*nt*2]: (d/d eps_ab, d/d sigma_ab). */
int orc_adjoint(const orc_sys_t *s, const double *r, const double *g, const double *dA,
                double *E, double *W, double *dEp, double *dWp, double *dLp, double *dEq,
                double *dLq)
{
  const int ns = s->ns, nt = s->ntypes;
  int i, j, m, d, nk;
  int *kv;
  double kappa = s->kappa, V = s->L[0] * s->L[1] * s->L[2], cq = SQ(s->cutoff);
  double Elj = 0, Eel = 0, vir = 0;
  double *ekk, *Sre, *Sim, *Tre, *Tim, *pr, *pi;
  if (is_polar(s)) return -1;
  memset(dEp, 0, sizeof(double) * nt * nt * 2);
  memset(dWp, 0, sizeof(double) * nt * nt * 2);
  memset(dLp, 0, sizeof(double) * nt * nt * 2);
  memset(dEq, 0, sizeof(double) * ns);
  memset(dLq, 0, sizeof(double) * ns);
  /* r-space pairs */
  for (i = 0; i < ns; i++)
    for (j = i + 1; j < ns; j++) {
      double dr[3], rr, qq = s->q[i] * s->q[j], phi = 0, e = 0, gd = 0;
      nearest(s->L, r + 3 * i, r + 3 * j, dr);
      rr = SQ(dr[0]) + SQ(dr[1]) + SQ(dr[2]);
      if (rr >= cq) continue;
      if (g)
        for (d = 0; d < 3; d++) gd += (g[3 * i + d] - g[3 * j + d]) * dr[d];
      if (s->mol[i] == s->mol[j]) {
        phi = orc_exacterud_sqrt(rr, s->alpha, &e);
      } else {
        int a = s->type[i], b = s->type[j], lo = a < b ? a : b, hi = a < b ? b : a;
        const orc_ss_t *ss = s->ss + a * nt + b;
        double u, f, du, df, eps = -ss->eps;
        lj_terms(ss, dA + 2 * (a * nt + b), rr, &u, &f, &du, &df);
        Elj += u;
        vir += rr * f;
        if (eps > 0) {
          dEp[2 * (lo * nt + hi)] += u / eps;
          dWp[2 * (lo * nt + hi)] += rr * f / eps;
          dLp[2 * (lo * nt + hi)] += gd * f / eps;
        }
        dEp[2 * (lo * nt + hi) + 1] += du;
        dWp[2 * (lo * nt + hi) + 1] += rr * df;
        dLp[2 * (lo * nt + hi) + 1] += gd * df;
        if (qq != 0 || s->q[i] != 0 || s->q[j] != 0) {
          const double *p = s->ertab + 6 * (int)(rr * s->sgrid);
          phi = p[1] / (p[2] + rr) + p[0];
          e = p[4] / (p[5] + rr) + p[3];
        }
      }
      Eel += qq * phi;
      dEq[i] += s->q[j] * phi;
      dEq[j] += s->q[i] * phi;
      dLq[i] += gd * e * s->q[j];
      dLq[j] += gd * e * s->q[i];
    }
  /* k-space: S, T_d = sum_j q_j g_jd Phi_j, then per charge */
  nk = orc_kvectors(s->L, &kappa, 0, NULL);
  kv = malloc(sizeof(int) * 3 * (nk > 0 ? nk : 1));
  kappa = s->kappa;
  orc_kvectors(s->L, &kappa, nk, kv);
  ekk = malloc(sizeof(double) * (nk + 1));
  Sre = calloc(nk + 1, sizeof(double)); Sim = calloc(nk + 1, sizeof(double));
  Tre = calloc(nk + 1, sizeof(double)); Tim = calloc(nk + 1, sizeof(double));
  pr = malloc(sizeof(double) * (nk + 1)); pi = malloc(sizeof(double) * (nk + 1));
  g_kmax[0] = g_kmax[1] = g_kmax[2] = 0;
  for (m = 0; m < nk; m++)
    for (d = 0; d < 3; d++)
      if (abs(kv[3 * m + d]) > g_kmax[d]) g_kmax[d] = abs(kv[3 * m + d]);
  {
    double PIaq = -SQ(M_PI / s->alpha);
    for (m = 0; m < nk; m++) {
      double kk = SQ(kv[3 * m + 2] / s->L[2]) + (SQ(kv[3 * m + 1] / s->L[1]) + SQ(kv[3 * m] / s->L[0]));
      ekk[m] = 4 / (kk * V) * exp(PIaq * kk);
    }
  }
  for (j = 0; j < ns; j++) {
    qitem_t it = {j, s->q[j], 0};
    if (s->q[j] == 0) continue;
    charge_phases(s, r, &it, nk, kv, pr, pi);       /* q_j Phi_j(k) */
    for (m = 0; m < nk; m++) {
      double w = 0;
      Sre[m] += pr[m]; Sim[m] += pi[m];
      if (g)
        for (d = 0; d < 3; d++) w += g[3 * j + d] * kv[3 * m + d] / s->L[d];
      Tre[m] += w * pr[m]; Tim[m] += w * pi[m];
    }
  }
  {
    double Ek = 0;
    for (m = 0; m < nk; m++) Ek += ekk[m] * (SQ(Sre[m]) + SQ(Sim[m]));
    Eel += Ek / (4 * M_PI);
  }
  for (j = 0; j < ns; j++) {
    qitem_t it = {j, 1.0, 0};
    double psi = 0, fk[3] = {0, 0, 0}, kl = 0;
    if (s->q[j] == 0) continue;
    charge_phases(s, r, &it, nk, kv, pr, pi);       /* Phi_j(k) */
    for (m = 0; m < nk; m++) {
      /* conj(S) Phi and conj(Phi) T */
      double re = Sre[m] * pr[m] + Sim[m] * pi[m], im = Sre[m] * pi[m] - Sim[m] * pr[m];
      double tim = pr[m] * Tim[m] - pi[m] * Tre[m];
      psi += ekk[m] * re;
      for (d = 0; d < 3; d++) fk[d] += ekk[m] * kv[3 * m + d] / s->L[d] * im;
      kl += ekk[m] * tim;
    }
    dEq[j] += psi / (2 * M_PI) - 2 * s->alpha / SQRTPI * s->q[j];
    if (g) dLq[j] += g[3 * j] * fk[0] + g[3 * j + 1] * fk[1] + g[3 * j + 2] * fk[2] + kl;
  }
  {
    double sq2 = 0;
    for (j = 0; j < ns; j++) sq2 += SQ(s->q[j]);
    Eel += -s->alpha / SQRTPI * sq2;
  }
  /* the electrostatic virial equals the electrostatic energy */
  for (i = 0; i < nt * nt * 2; i++) dWp[i] += 0;
  *E = Elj + Eel;
  *W = vir + Eel;
  free(kv); free(ekk); free(Sre); free(Sim); free(Tre); free(Tim); free(pr); free(pi);
  return 0;
}

/* ---------------------------------------------------------- thermostats --- */

/* Gaussian number i of step `step` of the thermostat stream: Box-Muller on
   the SplitMix64 words 2i, 2i+1 of seed + (step*2^40 + n + 1)*gamma (the
   stream of the GPU path; the reference draws rndgauss()) */
double orc_thermo_gauss(unsigned long long seed, long long step, long long i)
{
  unsigned long long base = (unsigned long long)step << 40;
  double u1 = ((double)(mix64(seed + (base + 2 * i + 1) * 0x9E3779B97F4A7C15ULL) >> 11) + 1.0) /
              9007199254740992.0;
  double u2 = (double)(mix64(seed + (base + 2 * i + 2) * 0x9E3779B97F4A7C15ULL) >> 11) /
              9007199254740992.0;
  return sqrt(-2.0 * log(u1)) * cos(2 * M_PI * u2);
}

/* the velocity factor of sim/thermo.c after a SHAKE step: kin2 = sum m
   (V1^2 + V2^2) (V = h v), En.T = kin2/(2 h^2)/f; kind 1 Berendsen
   (:157-163, blogT of sim/constrd.c:98-107), kind 2 Bussi (:165-179) */
double orc_thermostat(int kind, double kin2, double h, double nf, double T, double tau,
                      unsigned long long seed, long long step)
{
  double ET = kin2 / (2 * h * h) / nf;
  if (kind == 1) {
    const double e2 = 7.38905609893065022723;
    double bl = ET > T * e2 ? 1 : (ET * e2 < T ? -1 : log(ET / T) / 2);
    return exp(bl * -h / tau);
  }
  if (kind == 2) {
    double e = exp(-h / tau), c = T / (nf * ET), u1 = orc_thermo_gauss(seed, step, 0), uf = 0;
    long long i;
    for (i = 1; i < (long long)nf; i++) {
      double g = orc_thermo_gauss(seed, step, i);
      uf += g * g;
    }
    return sqrt(e + c * (1 - e) * (u1 * u1 + uf) + 2 * e * sqrt(c * (1 - e)) * u1);
  }
  return 1;
}
