/*
 * cookoracle -- CPU restatement of MACSIMUS cook's per-step force path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity oracle: the tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it to check
 * or time the GPU path.  The product path never links, loads or calls it.
 *
 * It restates, in plain C99 double precision, the reference algorithms:
 *   smoothed LJ cutoff              sim/setss.c:137-300, sim/lj/sitesite.c:66-112
 *   erfc hyperbolic splines         sim/erfc.c:119-191, sim/splines.c:23-158
 *   exact Ewald exclusion term      sim/erexact.c:25-75
 *   pair kernel (non-polar)         cook/ljqqnp.c:43-259, sim/intermac.h:47-76
 *   k-vector set + ekk              sim/ewald.c:334-612
 *   Ewald passes 1, 2, M/self terms sim/ewpass1.c, sim/ewpass2m.c, sim/ewaldf.c,
 *                                   sim/ewald.c:865-999
 *   leap-frog + SHAKE               sim/constrd.c:622-1081, sim/verlet.c:101-104,
 *                                   sim/shakev3.c:1-33
 *   Drude SCF + ASPC                sim/scf.c:12-393, sim/pred2.c:26-100,
 *                                   cook/ljqqpol.c:15-698
 *   Widom insertions                cook/widom.c:175-288, sim/simmeas.c:1821-1958,
 *                                   sim/siminit.c:762-808
 * Parity is pinned against dumps of the reference binary (tests/golden).
 */
#ifndef COOKORACLE_H
#define COOKORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* site-site constants of one type pair (cook: sitesite_t, sim/lj/sitesite.h:44-52) */
typedef struct {
  double C1q, C2q;        /* smoothing start^2, LJ cutoff^2 */
  double A, A4;           /* u=A*(r^2-C2^2)^2, f/r=A4*(r^2-C2^2) on C1<r<C2 */
  double Sq, E4, E24, E48;/* LJ constants (E24,E48 already divided by Sq) */
  double corr;            /* normalized cutoff correction */
  double eps, sig;        /* pair parameters: eps<0 (minimum), sig = vdW diameter */
} orc_ss_t;

/* energies of one force evaluation (program units, K) */
typedef struct {
  double el;        /* electrostatic energy (r + k + self + dipole) = En.el */
  double lj;        /* Lennard-Jones energy (added to En.pot) */
  double vir;       /* LJ virial sum r*f (En.vir contribution of the pair kernel) */
  double Pvir[6];   /* virial tensor xx yy zz yz zx xy */
  double ek;        /* k-space part (Ewald pass 2 energy) */
  double er;        /* r-space part incl. exclusion corrections */
  double eself;     /* -alpha/sqrt(pi) sum q^2 */
  double edip;      /* dipole (epsinf) term */
  double self;      /* Drude spring energy En.self (POLAR) */
} orc_en_t;

/* combining rule of sim/lj/sitesite.c:66-93 (EvdW<0 in K, RvdW in A) */
void orc_combrule(double E0, double R0, double alpha0, double E1, double R1, double alpha1,
                  int comb_rule, double *eps, double *sig);
/* sim/setss.c:137-300 (LJ only, no NBFIX, no SHARPCUTOFF) */
int orc_setss(double eps, double sig, double C2, orc_ss_t *ss);

/* erfc hyperbolic-spline table: number of intervals, and the table itself
   (6 doubles per interval: Au Bu Cu Ad Bd Cd); sgrid returned */
int orc_erfc_ntab(int grid, double maxr, double alpha);
void orc_erfc_build(int grid, double maxr, double cutoff, double alpha, int shift,
                    double *tab, double *sgrid);
double orc_eru(const double *tab, double sgrid, double rr);
double orc_erd(const double *tab, double sgrid, double rr);
/* exacterud_sqrt / exacterud_sqrt_1 (SUBGRID==1 variants) */
double orc_exacterud_sqrt(double rr, double alpha, double *erd);
double orc_exacterud_sqrt_1(double rr, double alpha, double *erd);

/* k-vector enumeration (sim/ewald.c:334-560).  kappa is adjusted in place
   exactly as the reference does for rounding problems.  Fills up to maxk
   half-space vectors (kx,ky,kz) in the reference order (sign combos
   +++,++-,+-+,+-- of each octant entry) when kv!=NULL; returns Q->N. */
int orc_kvectors(const double L[3], double *kappa, int maxk, int *kv);

/* the system */
typedef struct {
  int ns;               /* number of sites */
  const int *type;      /* [ns] LJ site type */
  const double *q;      /* [ns] charge (program units); POLAR: central charge */
  const int *mol;       /* [ns] molecule id; all intramolecular pairs excluded */
  int ntypes;
  const orc_ss_t *ss;   /* [ntypes*ntypes] */
  double L[3];
  double cutoff;        /* r-space cutoff */
  double alpha;         /* Ewald separation parameter */
  double kappa;         /* k-space cutoff (already adjusted by orc_kvectors) */
  double epsinf;        /* dielectric of the surroundings (3e33 = tin foil) */
  const double *ertab;  /* erfc table */
  int ntab;
  double sgrid;
  /* Drude (POLAR); NULL if non-polar */
  const double *qpol;   /* [ns] Drude charge */
  const double *alphaqq;/* [ns] 1/(Drude spring constant) = alphapol/qpol^2 in p.u. */
  /* cook's el.corr (sim/simglob.h:828): bits 1, 2, 4 select the
     Yeh-Berkowitz dipole term along x, y, z in place of the isotropic
     epsinf term; bit 8 keeps its energy and virial but applies no force */
  int elcorr;
} orc_sys_t;

/* forces(B,A) of cook: f (3*ns, or 6*ns with Drude) is overwritten; energies
   filled when en != NULL.  r: 3*ns (+3*ns Drude displacements).
   nthreads >= 1 (pthreads). returns 0 */
int orc_forces(const orc_sys_t *s, const double *r, double *f, orc_en_t *en, int nthreads);

/* Verlet/leap-frog + SHAKE of rigid molecules (sim/constrd.c Shake, SHAKE=1,
   VERLET=3).  r, r1 updated in place (r1 = r(t)-r(t-h)); f = forces at r.
   Constraints: nc pairs (ci,cj) with squared lengths bondq; imass per site.
   omega = half of cook's omegac.  Returns the number of sweeps of the worst
   molecule (or -1 when maxit is exceeded).  ekin: sum m (V1^2+V2^2)/(4 h^2), the kinetic energy */
int orc_shake_step(int ns, double *r, double *r1, const double *f, const double *mass,
                   int nmol, const int *mol_first, const int *mol_nc, const int *cfirst,
                   const int *ci, const int *cj, const double *bondq,
                   double h, double eps, double omega, int maxit, double *ekin);
/* orc_shake_step with dp[] added to the unconstrained positions (NULL: none) */
int orc_shake_step_dp(int ns, double *r, double *r1, const double *f, const double *mass,
                      int nmol, const int *mol_first, const int *mol_nc, const int *cfirst,
                      const int *ci, const int *cj, const double *bondq,
                      double h, double eps, double omega, int maxit, const double *dp,
                      double *ekin);

/* orc_shake_step_dp of a measured cycle: meas[13] gets cook's En.virc,
   PTvirc[6] (sim/virc.c / h^2) and En.Pkin[6] (m (V1 V1 + V2 V2) / (2 h^2),
   before the division by V) of the step */
int orc_shake_step_meas(int ns, double *r, double *r1, const double *f, const double *mass,
                        int nmol, const int *mol_first, const int *mol_nc, const int *cfirst,
                        const int *ci, const int *cj, const double *bondq,
                        double h, double eps, double omega, int maxit, const double *dp,
                        double *ekin, double *meas);

/* one Drude relaxation iteration (sim/scf.c selffield): r and f hold 2*ns
   vectors (sites, then Drude displacements / Drude forces); energies added
   to *en (el, self, Pvir) when en != NULL; returns max |d rpol|/omega */
double orc_selffield(const orc_sys_t *s, double *r, double *f, orc_en_t *en, double omega);
/* ASPC predictor B[0..k+1] and mixing omega (sim/pred2.c:70-97) */
void orc_aspc_coef(int k, double *B, double *omega);

/* Widom insertions (cook/widom.c:175-288 Einsert, sim/simmeas.c:1821-1958
   Widom, sim/siminit.c:762-808 Widomcutcorr).  The insertion points come
   from a counter-based stream shared with the GPU path (orc_widom_word). */
unsigned long long orc_widom_word(unsigned long long seed, long long k, int c);
void orc_widom_sites(unsigned long long seed, long long k, const double L[3], int nps,
                     const double *geom, double *out);
double orc_einsert(const orc_sys_t *s, const double *r, int nps, const int *ptype,
                   const double *pq, const double *ppos);
double orc_widom(const orc_sys_t *s, const double *r, int nps, const int *ptype,
                 const double *pq, const double *geom, long long n, unsigned long long seed,
                 double T, double *U, int nthreads);
double orc_widom_corr(const orc_sys_t *s, int nps, const int *ptype);
double orc_xwidom(const orc_sys_t *s, const double *r, int nlist, const int *mols,
                  const int *mol_first, const int *vtype, const double *vq, double T,
                  double *dU);

/* Adjoint: gradients of E, W = LJ sum r.f + E_el and (g = dLoss/dF) of a
   force loss with respect to the LJ (epsilon, sigma) of every type pair a<=b
   ([nt*nt*2]) and to every site charge ([ns]); dA: [nt*nt*2] dA/dsigma,
   dA4/dsigma of the smoothing constants.  Non-polar, tin-foil. */
int orc_adjoint(const orc_sys_t *s, const double *r, const double *g, const double *dA,
                double *E, double *W, double *dEp, double *dWp, double *dLp, double *dEq,
                double *dLq);

/* thermostats of sim/thermo.c (Berendsen 1, Bussi 2): the velocity factor
   after a SHAKE step from kin2 = sum m (V1^2+V2^2), V = h v */
double orc_thermo_gauss(unsigned long long seed, long long step, long long i);
double orc_thermostat(int kind, double kin2, double h, double nf, double T, double tau,
                      unsigned long long seed, long long step);

#ifdef __cplusplus
}
#endif
#endif
