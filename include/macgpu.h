/*
 * macgpu.h -- C ABI of the GB300 force path for MACSIMUS cook.
 *
 * The library replaces cook's per-step force routine and its integrator:
 *
 *   mg_forces()   replaces  void forces(ToIntPtr B, ToIntPtr A)
 *                           (cook/forces.h:1, cook/forces.c:93-224): B (forces)
 *                           is overwritten, energies/virial are returned only
 *                           when measure != 0, exactly as cook fills En.el,
 *                           En.pot, En.vir, En.Pvir (sim/simglob.h:436-577).
 *   mg_ewald()    replaces  double Ewald(int pass, vector *frp, vector *rp)
 *                           (sim/ewald.h:60, sim/ewald.c:258) passes 1+2.
 *   mg_md_steps() replaces  the step loop around void Shake(double eps,double prob)
 *                           (sim/constrd.h:5, sim/constrd.c:622-1081) with
 *                           coordinates kept on the device between steps.
 *
 * Arrays are cook's ``rp`` layout: contiguous site vectors in molecule order
 * (species by species, molecule by molecule, site by site), double[3] each,
 * Angstrom, program units (energy in K, charge e*408.779826922048, mass in
 * g/mol/0.831446261815324).  With Drude charges (chargepol != NULL) the site
 * vectors are followed by the Drude displacement vectors (cook's polar_off
 * half, sim/simglob.h:912-913), so r and f hold 2*ns vectors.
 *
 * Errors: every call returns an int status (MG_OK = 0); mg_last_error()
 * gives the message.  A context is used by one host thread at a time.
 */
#ifndef MACGPU_H
#define MACGPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mg_ctx mg_ctx;

enum mg_status {
  MG_OK = 0,
  MG_ERR_ARG = 1,          /* invalid argument */
  MG_ERR_CUDA = 2,         /* CUDA runtime error */
  MG_ERR_SHAKE = 3,        /* SHAKE did not converge (cook: "too many iterations") */
  MG_ERR_NONFINITE = 4,    /* non-finite position or force */
  MG_ERR_SETUP = 5,        /* force-field setup failed (smooth cutoff, k-vectors) */
  MG_ERR_SIZE = 6,         /* size beyond a compiled or stated maximum */
  MG_ERR_SCF = 7,          /* Drude displacement beyond el.minqq (sim/scf.c:142,253) */
  MG_ERR_LIST = 8          /* a site moved more than skin/2 between neighbour-list builds */
};

enum mg_precision {
  MG_FP64 = 0,   /* plain double precision everywhere */
  MG_MIXED = 1   /* FP32 pair/k-space arithmetic, FP64 accumulation and reductions;
                    SHAKE sweeps of three-site molecules in float-float
                    arithmetic (about 48 bits), their set-up and the rest FP64 */
};

/* The molecular topology and force-field tables cook builds in
   cook/simdef.c (readblend) and sim/siminit.c. */
typedef struct {
  int ns;                     /* number of sites (No.s) */
  int nmol;                   /* number of molecules (No.N) */
  const int *mol_first;       /* [nmol+1] first site of each molecule */
  const int *site_type;       /* [ns] LJ site type (siteinfo_t.st) */
  const double *charge;       /* [ns] site charge (Drude builds: central charge) */
  const double *mass;         /* [ns] site mass */
  int ntypes;                 /* number of LJ site types (nsites of the .ble) */
  const double *type_EvdW;    /* [ntypes] LJ well depth, K, <= 0 (sitedef.LJ.EvdW) */
  const double *type_RvdW;    /* [ntypes] van der Waals radius, A (sitedef.LJ.RvdW) */
  const double *type_alpha;   /* [ntypes] combining-rule polarizability (sitedef.LJ.alpha) */
  int comb_rule;              /* combining rule of the .ble (sim/lj/sitesite.c:66-93) */
  int nc;                     /* number of bond constraints */
  const int *cons;            /* [2*nc] constrained site pairs (global site indices) */
  const double *cons_len;     /* [nc] constraint lengths, A */
  const int *mol_cfirst;      /* [nmol+1] first constraint of each molecule */
  const double *chargepol;    /* [ns] Drude charge or NULL (siteinfo_t.chargepol) */
  const double *alphapol;     /* [ns] Drude polarizability volume, A^3, or NULL */
  /* linear ("Middle") dependants, cook's depend_t of type DEP_M
     (cook/simdef.c:322-432): massless site dep_site[k] at
     sum_p dep_w[p] r[dep_parent[p]], p in [dep_first[k], dep_first[k+1]);
     mg_md_steps places them before and redistributes their forces after
     every force evaluation (sim/norm.c:1161-1276 depend_r / depend_f, as
     sim/constrd.c:722,747 call them); mg_forces returns the raw forces like
     cook's forces().  ndep = 0: none. */
  int ndep;
  const int *dep_site;        /* [ndep], dependants of a molecule consecutive */
  const int *dep_first;       /* [ndep+1] */
  const int *dep_parent;      /* [dep_first[ndep]] */
  const double *dep_w;        /* [dep_first[ndep]] */
  /* the kind of each dependant (NULL: all linear): 0 "Middle" (DEP_M),
     1 "Rowlinson" (DEP_R: at D0 + wz n / |n|, n = (D1 - D0) x (D2 - D0),
     sim/norm.c:1196-1214, forces sim/norm.c:1304-1336), 2 "Lone" (DEP_L:
     at sum_p w_p D_p + wz z / |z|, z = (sum x_p D_p) x (sum y_p D_p),
     sim/norm.c:1216-1231, forces sim/norm.c:1338-1360); Rowlinson and Lone
     dependants have exactly 3 parents D0, D1, D2 */
  const int *dep_type;
  /* [13 ndep] per dependant (NULL when all are linear): wz, x[3], y[3],
     tx[3], ty[3] (cook's d->wz, d->x, d->y, d->tx, d->ty; zeros where the
     kind does not use them).  A measured MD step adds the virial and
     pressure-tensor terms cook's depend_f adds for these two kinds
     (sim/norm.c:1335-1338, 1363-1368) to mg_energy's vir and Pvir. */
  const double *dep_par;
} mg_topology;

/* Run parameters (cook's box, el, cutoff, h, epsc ... globals). */
typedef struct {
  double L[3];       /* box (box.L) */
  double cutoff;     /* r-space cutoff (box.cutoff) */
  double LJcutoff;   /* LJ smooth cutoff C2 (LJcutoff); <=0 means cutoff */
  double alpha;      /* Ewald separation parameter (el.alpha) */
  double kappa;      /* k-space cutoff K/L (el.kappa) */
  int grid;          /* erfc spline grid (el.grid, default 256) */
  int rshift;        /* spline shift flags (el.rshift, default 3) */
  double rplus;      /* spline table margin (el.rplus, default 2.5) */
  double epsinf;     /* dielectric constant of surroundings (el.epsinf, 3e33 = tin foil) */
  int precision;     /* enum mg_precision */
  double h;          /* time step, ps */
  double epsc;       /* SHAKE relative tolerance (epsc) */
  double omegac;     /* SHAKE over-relaxation (cook's omegac; <=0 selects 1.2) */
  int shake_maxit;   /* SHAKE sweep limit per molecule (<=0 selects 1000) */
  int cells_per_cutoff; /* linked-cell subdivision (0 = automatic) */
  /* Drude builds (cook option -p2K0 and scf.eps<=-1, sim/pred2.c, sim/scf.c) */
  int aspc_k;        /* ASPC predictor length k (0..9; cook -p2K0) */
  int scf_iter;      /* force evaluations + SCF iterations per step (|scf.eps|, >=1) */
  double scf_omega;  /* SCF mixing when aspc_k == 0 (ASPC sets (k+2)/(2k+3) itself) */
  double minqq;      /* largest allowed Drude displacement (el.minqq, default 1 A) */
  /* pair search: skin <= 0 re-bins the linked cells at every force
     evaluation as cook does (cook/lc.c); skin > 0 selects per-site Verlet
     lists of radius cutoff+skin, rebuilt at every mg_forces call and, in MD,
     once a site has moved skin/4 since the build (or after nl_every steps) */
  double skin;       /* A */
  int nl_every;      /* most MD steps between list builds; <=0 selects 50 */
  /* Ewald pass 1 work split: charge chunks sized for this many CTAs per SM;
     <=0 selects 10 (FP32) / 8 (FP64).  mg_autotune picks it. */
  int kspace_ctas_per_sm;
  /* FP32 pair kernel: 8 = the group kernel (a warp per group of 8 home
     sites; neighbours pruned against the group's bounding box; needs a grid
     of at least 2 cdiv + 1 cells per edge, else the cell kernel runs);
     9 = the group kernel with Newton's third law (every pair once, over a
     half-shell stencil; forces, of the shells too, summed in 64-bit fixed
     point, 2^-32 K/A, by integer atomics, so still reproducible bit for
     bit), lanes on the home sites; 10 = the same with lanes on the
     neighbours (each lane runs one neighbour against the group's home
     sites; with Drude shells 9 runs);
     otherwise the cell kernel with bit 0 = 8 warps per home cell (else 4),
     bit 2 = 16 warps per home cell (over bit 0), bit 1 = the erfc force
     spline in shared memory (else read through L1).  mg_autotune picks it. */
  int pair_variant;
  /* thermostat (sim/thermo.c): 0 none, 1 Berendsen, 2 Bussi (stochastic
     velocity rescaling), both applied after every SHAKE step; 3 Nose-Hoover
     in cook's Verlet+SHAKE form (cook's thermostat=2, T_NOSE: friction
     -Vfactor vpred inside the step with the time-reversible velocity
     predictor of nose_pred steps, sim/trvpscale.c, sim/verlet.c:22-37,
     sim/thermo.c:180-212); temperature T (K), time constant tau_T (ps),
     degrees of freedom thermo_f (<=0: cook's No.f, 3 (ns - ndep) - nc - 3),
     seed of the Bussi stream */
  int thermostat;
  double T, tau_T, thermo_f;
  unsigned long long seed;
  /* molecule wrapping after every MD step, cook's normalize(-1)
     (sim/norm.c:356-447, called at sim/main.c:1607): a molecule whose lowest
     coordinate over its massive sites leaves [r0, r0 + L) moves by one box
     length.  box_rmin as cook's box.rmin (cook/linklist.c:363-377): > 0 sets
     r0, < 0 gives r0 = 0, 0 gives cook's Verlet/SHAKE choice r0 = 0.15 A.
     no_normalize != 0 leaves the positions unwrapped. */
  double box_rmin;
  int no_normalize;
  /* Ewald k-space engine of the FP32 path: 0 = each pass on the tensor
     cores when its shared-memory tiles fit (else on the FP32 cores); 1 =
     both passes on the FP32 cores; 2 = pass 2 on the tensor cores, pass 1 on
     the FP32 cores; 3 = both passes on the tensor cores.  The tensor-core
     passes run TF32 split into three products with FP32 accuracy. */
  int kspace_engine;
  /* Nose-Hoover predictor length k (cook's No.pred = option -p % 10,
     sim/main.c:404-405), 1..8; <=0 selects 2 */
  int nose_pred;
  /* dipole term of Ewald(2) (sim/ewald.c:865-887), cook's el.corr
     (sim/simglob.h:828): 0 = the isotropic term of epsinf (none for
     epsinf >= 1e20, tin foil); bits 1, 2, 4 = the Yeh-Berkowitz slab term
     along x, y, z instead; + 8 = its energy and virial without the force */
  int dipole_corr;
  /* cook's drmax (sim/main.c:140) for its bounddr step limiter
     (sim/norm.c:1513-1560): 0 = off; otherwise, after every MD step and its
     thermostat, the displacement r1 of a site longer than |drmax| (A) is
     scaled to that length (cook applies a positive drmax only to thermostatted
     runs that start with init > 2; the caller decides) */
  double drmax;
  /* drift_step != 0: the momentum drift is removed after every step (after
     bounddr), cook's removedrifts with its momentum bits and DRIFT_STEP
     (sim/norm.c:677-705, sim/main.c:1626); cook's default removes it once
     per cycle, which a host loop does with mg_remove_drift */
  int drift_step;
  /* FP32 path: 0 runs the Ewald k-space chain on a second stream beside the
     r-space chain, 1 after it on one stream (mg_set_overlap changes it
     later); mg_autotune picks it.  No reference counterpart. */
  int kspace_serial;
} mg_params;

/* Energies of one force evaluation (program units, K).
   cook: En.el = el; En.pot += lj; En.vir += vir; En.Pvir[] += Pvir[]. */
typedef struct {
  double el;        /* electrostatic energy: r + k + self + dipole */
  double lj;        /* Lennard-Jones energy */
  double vir;       /* LJ virial sum r*f */
  double Pvir[6];   /* virial tensor xx yy zz yz zx xy */
  double ek;        /* k-space part */
  double er;        /* r-space part incl. Ewald exclusion corrections */
  double eself;     /* -alpha/sqrt(pi) sum q^2 */
  double edip;      /* dipole term (finite epsinf or Yeh-Berkowitz; part of el) */
  double self;      /* Drude spring energy (En.self) */
  double ekin;      /* kinetic energy (mg_md_steps only) */
  /* pressure of the last step of mg_md_steps (zero after mg_forces), as
     cook's measurePconstraints assembles it (sim/constrd.c:115-265) with
     No.Pkinq = 1; tensors xx yy zz yz zx xy in K/A^3 (times 13806490 =
     cook's Punit gives Pa) */
  double virc;      /* constraint virial En.virc: sum of the SHAKE factors / h^2 (sim/virc.c) */
  double Pkin[6];   /* kinetic tensor sum m v v / V, leap-frog v of sim/shakev3.c */
  double Ptens[6];  /* (Pvir + constraint virial tensor PTvirc) / V + Pkin */
  double P;         /* cook's Pevir: (2 ekin + vir + virc + el - 2 self) / (3 V) */
} mg_energy;

/* Create a context on the current CUDA device.  Builds the smooth-cutoff LJ
   tables (setss), the erfc spline table (initerfc) and the k-vector set
   (Ewald(0)) from the topology and parameters; allocates device buffers.
   Returns NULL on failure with *status set. */
mg_ctx *mg_create(const mg_topology *top, const mg_params *par, int *status);
int mg_destroy(mg_ctx *ctx);
const char *mg_last_error(const mg_ctx *ctx);
/* the k-space cutoff after cook's rounding-problem adjustment (sim/ewald.c:485-506) */
double mg_kappa(const mg_ctx *ctx);
/* number of k-vectors Q->N */
int mg_nkvec(const mg_ctx *ctx);

/* cook's forces(B,A): r = A->rp (host, ns or 2*ns vectors), f = B->rp
   (host, overwritten).  measure != 0 fills *en (may be NULL otherwise). */
int mg_forces(mg_ctx *ctx, const double *r, double *f, int measure, mg_energy *en);
/* the same with device pointers; the call is ordered on the context stream
   and returns after the forces are complete */
int mg_forces_device(mg_ctx *ctx, const double *r_dev, double *f_dev, int measure,
                     mg_energy *en);
/* Ewald(1,...)+Ewald(2,...): k-space forces only (added to f), returns the
   k-space + self + dipole energy in *energy when energy != NULL */
int mg_ewald(mg_ctx *ctx, const double *r, double *f, double *energy);

/* One SCF iteration of the Drude displacements, cook's
   int selffield(ToIntPtr B, ToIntPtr A, eps, omega, run) (sim/scf.c:12,
   sim/constrd.h:8): on host arrays r (2*ns vectors, Drude half updated) and
   f (2*ns vectors as returned by mg_forces; the Drude force is folded into
   the centre); with measure, *en gets the self-pair Ewald term added to el,
   the spring energy in self and its virial added to Pvir (*en must hold the
   energies of the forces call). */
int mg_selffield(mg_ctx *ctx, double *r, double *f, double omega, int measure, mg_energy *en);

/* Device-resident MD (leap-frog Verlet + SHAKE, sim/constrd.c Shake with
   SHAKE=1, VERLET=3, no thermostat): state r = r(t), r1 = r(t)-r(t-h).
   Drude builds: r holds the Drude displacements after the sites, r1 the
   displacements of the previous step (cook's cfg[0], cfg[1] polar halves);
   every step runs the ASPC predictor, scf_iter force + SCF iterations and
   SHAKE (sim/constrd.c:726-736). */
int mg_md_set_state(mg_ctx *ctx, const double *r, const double *r1);
int mg_md_get_state(mg_ctx *ctx, double *r, double *r1);

/* One playback frame of the MD state as cook's writeplayback writes it
   (sim/simils.c:1646-1697): frame[0..2] = L, then ns float triples of
     what = MG_PLB_POS:   r                  (.plb)
            MG_PLB_VEL:   r1 / h             (.vlb, leap-frog v(t - h/2))
            MG_PLB_DRUDE: r + Drude offset   (.dlb, Drude builds only)
   flags are cook's option -n bits for positions: 2 = r - r1/2 (t - h/2),
   4 = centred, r - L/2.  The file layout (float header ns, -3 or -6 when
   centred, then the frames) is the caller's; the Python package writes it. */
enum { MG_PLB_POS = 0, MG_PLB_VEL = 1, MG_PLB_DRUDE = 2 };

/* Diagnostic: C[128 x n] = A[128 x k] B[n x k]^T (row-major FP32 host
   arrays) on the tensor cores in TF32 with the descriptors, TMEM accumulator
   and completion protocol of the tensor-core Ewald kernels; n a multiple of
   16 in 16..256, k a multiple of 8 up to 64. */
int mg_tc_selftest(const float *A, const float *B, float *C, int n, int k);
int mg_playback_frame(mg_ctx *ctx, int what, int flags, float *frame);
/* advance nsteps; energies of the last step in *en when en != NULL */
int mg_md_steps(mg_ctx *ctx, int nsteps, mg_energy *en);
/* what the drmax limiter did since the last report (cook prints "dr in 1
   step reduced for N site(s), min Q x"): sites reduced (summed over steps)
   and the smallest factor (1 if none); resets both (a synchronising call) */
int mg_bounddr_report(mg_ctx *ctx, long long *nreduced, double *minfactor);
/* cook's removedrifts for the linear momentum (sim/norm.c:677-705, called
   once per cycle at sim/maincps.c:65): the mass-weighted mean of r1 is
   subtracted from every site of the MD state; vdrift (or NULL) gets the
   removed drift velocity, A/ps */
int mg_remove_drift(mg_ctx *ctx, double vdrift[3]);

/* number of kernels launched by the last call (diagnostics) */
int mg_last_launches(const mg_ctx *ctx);

/* Run the context's work on the given CUDA stream (a cudaStream_t of the
   caller, e.g. a framework's current stream); NULL selects the context's own
   stream again.  No counterpart in the reference (cook has no device). */
/* factor by which the last thermostat call scaled the velocities (1 if
   none); a synchronising read */
double mg_thermostat_factor(mg_ctx *ctx);

/* Nose-Hoover state after the last step (thermostat 3): state[0] = logs,
   state[1] = h dlogs/dt (cook's cfg[0]->logs and cfg[1]->logs), state[2] =
   the thermostat's part of the conserved energy of that step (cook's Eext
   of VERLET=3, sim/thermo.c:205-212), in K; a synchronising read.
   mg_md_set_state starts the thermostat from logs = 0 with no history. */
int mg_nose_state(mg_ctx *ctx, double state[3]);

/* FP32 path: run the Ewald k-space chain on a second stream beside the
   r-space chain (on by default; off serialises them, e.g. to time kernels
   one by one).  No reference counterpart. */
int mg_set_overlap(mg_ctx *ctx, int on);
/* mg_md_steps of a non-polar box with cells re-binned: replay one captured
   CUDA graph per step (on, the default) or launch the kernels one by one.
   No reference counterpart. */
int mg_set_graph(mg_ctx *ctx, int on);
int mg_set_stream(mg_ctx *ctx, void *stream);

/* Per-kernel timing with CUDA events recorded on the context stream around
   every launch while enabled (diagnostics; no counterpart in the reference).
   mg_profile_entry(ctx, i, ...) returns 0 and fills name / total ms / count
   of entry i, or MG_ERR_ARG past the last entry. */
int mg_profile_enable(mg_ctx *ctx, int on);
int mg_profile_reset(mg_ctx *ctx);
int mg_profile_entry(mg_ctx *ctx, int i, const char **name, double *ms, long *count);

/* Measured FP32 FMA throughput of the current device in TFLOP/s: a long
   chain of independent fused multiply-adds on every SM, timed with CUDA
   events (the FP32 roofline denominator; no counterpart in the reference). */
int mg_probe_fp32_tflops(double *tflops);

/* k-space Ewald forces and energy without any memory allocation.
   No counterpart in the reference (cook allocates its Ewald tables per call).
   For callers that cannot allocate device memory -- a host program that hands
   all device memory out from its own fixed pool, or a time-critical loop that
   cannot afford cudaMalloc/cudaFree and the device-wide synchronization they
   can imply -- this variant keeps all of its scratch in a fixed array inside
   the library: every GPU that loads the library holds it (about 4.6 MB) until
   the process exits.  Inputs and outputs stay the caller's: r_dev [3*nq]
   charge positions and q_dev [nq] charges (device), f_dev [3*nq] forces
   (device, overwritten), *energy (host: k-space + self term, may be NULL);
   L, alpha, kappa as in mg_params; stream is a cudaStream_t (NULL: default
   stream); the call returns after the work is done.  Limits: at most
   MG_NOALLOC_MAX_CHARGES charges, MG_NOALLOC_MAX_KVEC k-vectors, phase rows
   of at most MG_NOALLOC_MAX_ROW entries ((Kx+1)+(2Ky+1)+(Kz+1), Kx, Ky, Kz
   the largest |kx|, |ky|, |kz| of the k set); larger inputs return
   MG_ERR_SIZE.  Every call looks up the array's address on the current
   device.  All calls share the array and keep the last call's data in it:
   calls that overlap on the GPU (or run concurrently from several host
   threads) race. */
#define MG_NOALLOC_MAX_CHARGES 4096
#define MG_NOALLOC_MAX_KVEC 4096
#define MG_NOALLOC_MAX_ROW 96
int mg_ewald_kspace_noalloc(const double *r_dev, const double *q_dev, int nq, const double L[3],
                            double alpha, double kappa, double *f_dev, double *energy,
                            void *stream);

/* ---- Widom test-particle insertion ----
   Replaces Einsert (cook/forces.h:3, cook/widom.c:175-288) and the averaging
   of Widom (sim/simmeas.c:1821-1958) with the cutoff correction of
   Widomcutcorr (sim/siminit.c:762-808).  ninsert ghost molecules are placed
   at random into the configuration of the last force evaluation (mg_forces,
   mg_forces_device or the last step of mg_md_steps -- cook's "last cell
   list"); each one's energy U against the box (LJ with the smooth cutoff +
   q q erfc r-space terms within the cutoff; the ghost is not part of the
   box) enters exp(-U/T), a term skipped when -U/T <= -700.  Insertion k
   takes its point and (for more than one site) a uniform rotation from a
   counter-based stream of `seed`, so the result is reproducible and does
   not depend on the launch.  Not available for Drude systems. */
#define MG_WIDOM_MAX_SITES 8
typedef struct {
  int ns;                  /* ghost sites, 1..MG_WIDOM_MAX_SITES */
  const int *site_type;    /* LJ type of each site (index into the topology's types) */
  const double *charge;    /* site charges in program units, or NULL (neutral) */
  const double *geometry;  /* [3*ns] site offsets from the insertion point, A */
} mg_probe;

typedef struct {
  double sum;     /* sum of exp(-U/T) */
  double raw;     /* sum / ninsert (cook's "Widom raw") */
  double corr;    /* cutoff correction numerator (cook's widom.corr), K A^3 */
  double factor;  /* exp(-corr/(V T)) */
  double widom;   /* raw * factor (cook's "Widom") */
  double mu;      /* -T ln(widom): residual chemical potential, K */
} mg_widom_result;

/* U (optional, [ninsert]) receives every insertion energy (K) */
int mg_widom(mg_ctx *ctx, const mg_probe *probe, long long ninsert, unsigned long long seed,
             double T, mg_widom_result *out, double *U);

/* Identity change, cook's XWidom (sim/simmeas.c:1961-2003, with Eidchange
   of cook/widom.c:16-170): the r-space energy change dU (smoothed LJ and
   the erfc spline) of giving the sites of each listed molecule the types
   vtype[] and charges vcharge[] (program units), against the other
   molecules in the cell list of the last force evaluation.  The listed
   molecules share one structure (1..8 sites, the same site kinds).  out:
   sum of exp(-dU/T), raw = sum / nlist (cook's "XWidom"), mu = -T ln raw;
   no cutoff correction (cook applies none).  dU (optional) per molecule. */
int mg_xwidom(mg_ctx *ctx, int nlist, const int *mols, const int *vtype, const double *vcharge,
              double T, mg_widom_result *out, double *dU);

/* ---- autotuner ----
   No reference counterpart.  Times the force evaluation of the configuration
   r for every cell subdivision (cells_per_cutoff 1..3) and Ewald pass-1
   split (kspace_ctas_per_sm 6, 10, 16) and writes the fastest pair into
   *par, then the fastest of the 8 cell-kernel pair_variant values at that
   choice, of the group kernel (pair_variant 8) at every subdivision and,
   on the FP32 path, of its half-shell forms (pair_variant 9 and 10) at
   every subdivision, each timed (FP32 path) with
   kspace_serial 0 and 1, the pair chosen together.  Builds and frees its
   own trial contexts; ms[28] (optional) gets the time per evaluation of
   each trial (the best of three blocks of nrep evaluations; cdiv-major,
   then the 8 cell-kernel variants, the group
   kernel at cdiv 1..3 and the half-shell group kernel (9) at cdiv 1..3, the
   faster of the two kspace_serial settings each, then the chosen variant
   with kspace_serial 0 and 1, then pair_variant 10 at cdiv 1..3; -1 if that
   grid is not possible or the trial did not run). */
int mg_autotune(const mg_topology *top, mg_params *par, const double *r, int nrep, double *ms);

/* ---- adjoint ----
   No reference counterpart.  Gradients, at the configuration r, of the
   energy E, the scalar virial W = LJ sum r.f + electrostatic energy, and of
   a loss of the forces through its weights g = dLoss/dF ([3 ns], or NULL),
   with respect to the LJ parameters (epsilon > 0 and sigma of
   4 eps[(sigma/r)^12 - (sigma/r)^6], combined as in the topology) of every
   pair of types and to every site charge.  FP64 contexts without Drude
   shells, cells re-binned (skin <= 0); tin-foil boundary.  Pair terms are
   recomputed (nothing stored but S(k)); the type-pair sums use shared-memory
   atomics, so their last bits may vary between calls. */
typedef struct {
  double E, W;        /* energy, scalar virial at r (K) */
  double *dE_pair;    /* [ntypes*ntypes*2] or NULL: (d/d eps, d/d sigma) of the */
  double *dW_pair;    /*   type pair (a, b), a <= b, at 2*(a*ntypes + b)        */
  double *dL_pair;
  double *dE_dq;      /* [ns] or NULL: dE/dq_i (= dW/dq_i) */
  double *dL_dq;      /* [ns] or NULL: dLoss/dq_i */
} mg_adjoint_out;

int mg_adjoint(mg_ctx *ctx, const double *r, const double *g, mg_adjoint_out *out);

/* ---- batches of independent boxes ----
   No reference counterpart (cook runs one box per process).  A batch owns
   nbox contexts whose kernels run on nlanes streams; mg_batch_md_steps
   replays one captured CUDA graph per MD step of all boxes (non-polar boxes
   with cells re-binned at every step); mg_batch_widom inserts into every
   box in one kernel launch (box i draws from seed + i * 0x632BE59BD9B4E019).
   Per-box state, forces and single-box calls go through mg_batch_box(). */
typedef struct mg_batch mg_batch;

mg_batch *mg_batch_create(int nbox, const mg_topology *tops, const mg_params *params,
                          int nlanes, int *status);
int mg_batch_destroy(mg_batch *b);
const char *mg_batch_last_error(const mg_batch *b);
int mg_batch_size(const mg_batch *b);
mg_ctx *mg_batch_box(mg_batch *b, int i);
/* kernels launched by the last batch call (graph nodes counted per step) */
int mg_batch_last_launches(const mg_batch *b);
/* en: NULL or [nbox] energies of the last step.  When every box runs the
   FP32 path with both Ewald passes on the FP32 cores or both on the tensor
   cores (kspace_engine 1 or 0; under 0 a box whose tiles do not fit runs on
   the FP32 cores), the cell pair kernel with 4 warps (pair_variant 0),
   cells re-binned every step and no Drude charges, dependants, thermostat,
   drmax, drift removal or dipole term, a step is one launch per kernel over
   all boxes (blockIdx.y = box, each box with its single-launch arguments,
   so its results are those of the box run alone); otherwise one graph node
   per box kernel. */
int mg_batch_md_steps(mg_batch *b, int nsteps, mg_energy *en);
/* 1 once mg_batch_md_steps has chosen the one-launch-per-kernel form */
int mg_batch_fused(const mg_batch *b);
/* No reference counterpart.  nrep further MD steps of a fused batch (no
   energies), each timed stage by stage with CUDA events; ms[7] gets the
   mean time per step of: the cell lists; the pair and exclusion terms (with
   the FP32-core phase rows); the tensor-core phase rows and operand tiles;
   Ewald pass 1; the S(k) sums; pass 2; the step (SHAKE).  The events sit
   between launches, so the stages add up to a little more than a step. */
int mg_batch_profile(mg_batch *b, int nrep, double ms[7]);
/* probes: one ghost for all boxes (probe_per_box = 0) or [nbox];
   out: [nbox] */
int mg_batch_widom(mg_batch *b, const mg_probe *probes, int probe_per_box, long long ninsert,
                   unsigned long long seed, double T, mg_widom_result *out);

#ifdef __cplusplus
}
#endif
#endif
