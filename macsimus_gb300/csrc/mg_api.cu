// C ABI of the GB300 force path (include/macgpu.h): context set-up and the
// per-call orchestration of the kernels in mg_kernels.cu.
#include "../../include/macgpu.h"
#include "mg_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <tuple>
#include <string>
#include <vector>


using namespace mg;

// length of the reduction-output block d_sums / h_sums (doubles)
constexpr int NSUMS = 56;

struct mg_ctx {
  std::string err;
  int precision = MG_MIXED;
  int ns = 0, nmol = 0, nc = 0, nq = 0, nk = 0, nkind = 0, launches = 0;
  double L[3] = {0, 0, 0};
  double cutoff = 0, alpha = 0, kappa = 0, sgrid = 0, eself = 0, epsinf = 3e33;
  // dipole term of Ewald(2) (finite epsinf or Yeh-Berkowitz): force factors
  // c_d (force q (-c_d M_d)), energy factors e_d (E = sum e_d M_d^2)
  bool dipole = false;
  int elcorr = 0;
  double dipc[3] = {0, 0, 0}, dipe[3] = {0, 0, 0};
  double* d_dippart = nullptr;
  // cook's bounddr after every MD step (drmax != 0): sites reduced, float
  // bits of the smallest factor
  double drmax = 0;
  unsigned int* d_bdrep = nullptr;
  // momentum drift removal (cook's removedrifts, momentum bits): after every
  // step with drift_step, else on request; total mass of the sites
  bool drift_step = false;
  double total_mass = 0;
  double *d_driftpart = nullptr, *d_drift = nullptr;  // [blocks*3], [6]: P, removed drift
  double h = 0.002, epsc = 1e-7, omega = 0.6;
  int shake_maxit = 1000;
  int ncx = 0, ncy = 0, ncz = 0, ncell = 0, nstencil = 0;
  bool allpairs = false;
  int ntab = 0;
  int Kx = 0, Ky = 0, Kz = 0, row = 0, ntask = 0, ncol = 0, nchunk = 1;
  cudaStream_t stream = nullptr;
  // host copies
  std::vector<int> h_kind, h_mol, h_mol_first;
  // device buffers
  double *d_r = nullptr, *d_f = nullptr, *d_r1 = nullptr, *d_p = nullptr;
  double *d_rs = nullptr, *d_fs = nullptr;  // staging of the host-array calls
  int *d_kind = nullptr, *d_mol = nullptr;
  int *d_key = nullptr, *d_idx = nullptr, *d_key_s = nullptr, *d_order = nullptr;
  int4* d_pfix = nullptr;  // fixed-point site records in site order (cell list scratch)
  int* d_cell_start = nullptr;
  int *d_ccount = nullptr, *d_ccursor = nullptr;  // cell counts (kept zero), cursors
  int4* d_pj = nullptr;
  double4* d_pd = nullptr;
  int4* d_stencil = nullptr;
  // group pair kernel: the stencil as z-runs, first group and cell of every
  // group, its grid; nprows = energy rows of the pair kernel (cell or group)
  int4* d_spans = nullptr;
  int nspans = 0, ngroup_grid = 0, nprows = 0;
  // its half-shell forms (pair_variant 9, 10): the half stencil as z-runs and the
  // 64-bit fixed-point force sums (sorted order, zero between evaluations)
  int4* d_hspans = nullptr;
  int nhspans = 0;
  long long* d_facc = nullptr;
  int *d_gstart = nullptr, *d_gcell = nullptr;
  PairF* d_ptabf = nullptr;
  PairD* d_ptabd = nullptr;
  float4 *d_erd = nullptr, *d_eru = nullptr;
  double* d_ert = nullptr;
  double* d_epart = nullptr;
  // k-space
  int* d_qsite = nullptr;
  double* d_qval = nullptr;
  KTask* d_task = nullptr;
  KCol* d_col = nullptr;
  int4* d_kvec = nullptr;
  double* d_ekk = nullptr;
  double* d_S = nullptr;
  float2* d_Wf = nullptr;
  double2* d_Wd = nullptr;
  void* d_tab = nullptr;   // float2 or double2 rows
  uint4* d_qfix = nullptr; // FP32 path: fixed-point coordinates of the charges
  void* d_part = nullptr;  // float2 or double2 partials
  double* d_ekpart = nullptr;
  int nkblocks = 0;
  KRow* d_krows = nullptr;
  KTile* d_tiles = nullptr;
  int2* d_p1job = nullptr;
  int ntile = 0, np1job = 0;
  // pass 2 on the tensor cores (FP32 path): operand tiles
  int nkrows = 0;
  bool kspace_tc = false;
  float *d_za = nullptr, *d_vb = nullptr;
  TcRow* d_tcrows = nullptr;
  KRow* d_tckrows = nullptr;   // the k rows in (kx, ky) order
  // pass 1 on the tensor cores
  bool sk_tc = false;
  float* d_zb = nullptr;
  int sk_nch = 1, sk_gpc = 1;
  // SHAKE
  int* d_mol_first = nullptr;
  int* d_mol_cfirst = nullptr;
  int2* d_cons = nullptr;
  double *d_bondq = nullptr, *d_imass = nullptr, *d_mass = nullptr;
  double* d_kinpart = nullptr;
  double* d_meas = nullptr;  // [nblocks * 13] constraint virial and kinetic tensor sums
  int* d_status = nullptr;
  // linear dependant sites
  int ndep = 0;
  int *d_dep_site = nullptr, *d_dep_first = nullptr, *d_dep_parent = nullptr;
  double* d_dep_w = nullptr;
  int* d_dep_type = nullptr;    // null: all linear
  // with Rowlinson or Lone dependants: per dependant the virial and virial
  // tensor rows of a measured depend_f, reduced into d_sums + 48
  double* d_deppart = nullptr;
  double* d_dep_par = nullptr;
  // intramolecular (excluded) charge pairs of the mixed cell path
  int* d_xfirst = nullptr;
  int2* d_xpair = nullptr;
  double4* d_xq = nullptr;
  int nxblocks = 0;
  float* d_plb = nullptr;  // playback frame staging
  // reduction outputs
  // [0..9] pair, [10..16] k-space, [17] kinetic, [20..27] Drude,
  // [31] status word (host copy), [32..44] SHAKE measurement
  double* d_sums = nullptr;
  double* h_sums = nullptr;  // pinned
  bool have_state = false;
  // neighbour lists
  bool use_list = true, need_build = true;
  double skin = 1.5;
  int nl_every = 5, since_build = 0, nl_cap = 0;
  long nl_pitch = 0;
  int *d_nlist = nullptr, *d_ncount = nullptr;
  double* d_rbuild = nullptr;
  int* d_dmax = nullptr;        // max squared displacement since the build (float bits)
  int* h_dmax = nullptr;        // pinned copy, read before the next step
  cudaEvent_t ev_dmax = nullptr;
  bool dmax_pending = false;
  int nepart = 0;
  int pair_variant = 0;
  // thermostat
  int normalize = 1;
  double box_r0 = 0.15;
  int thermostat = 0, nchi = 0;
  double T = 298, tau_T = 0.1, thermo_f = 0;
  unsigned long long seed = 0;
  long long* d_step = nullptr;
  double *d_chi = nullptr, *d_zth = nullptr;
  // Nose-Hoover: state (NoseSlot) and the r1 history [nose_pred][3 ns]
  int nose_pred = 0;
  double *d_nh = nullptr, *d_vhist = nullptr;
  // Widom: the type table, the site kinds, sites per type; cell data of the
  // last force evaluation (cook's lastlist)
  int ntypes = 0, comb_rule = 1;
  double C2 = 0;
  std::vector<double> h_tE, h_tR, h_tA;
  std::vector<int> kind_type;
  std::vector<double> kind_q;
  std::vector<long> type_count;
  bool have_cells = false;
  const double* last_r = nullptr;   // positions of the last force evaluation (device)
  PairF* d_wtabf = nullptr;
  PairD* d_wtabd = nullptr;
  double *d_wgeom = nullptr, *d_wpart = nullptr;
  WidomBox* d_wbox = nullptr;
  // adjoint scratch (FP64 contexts)
  AdjPair* d_adjtab = nullptr;
  double *d_ag = nullptr, *d_aq = nullptr, *d_apart = nullptr, *d_adEq = nullptr,
         *d_adLq = nullptr;
  double4* d_ags = nullptr;
  double2 *d_atpart = nullptr, *d_aT = nullptr;
  int adj_ntch = 0;
  std::vector<PairF> h_wtabf;
  std::vector<PairD> h_wtabd;
  std::vector<double> h_wgeom;
  // Drude
  bool polar = false;
  int nd = 0, ndblocks = 0, aspc_k = 2, aspc_kk = 0, scf_iter = 1, hist_h = 0;
  double scf_omega = 0.6, cur_omega = 0.6, minqq = 1.0;
  int *d_dsite = nullptr, *d_qdrude = nullptr;
  double *d_qc = nullptr, *d_qp = nullptr, *d_aqq = nullptr, *d_hist = nullptr,
         *d_drpart = nullptr;
  float4* d_pdj = nullptr;
  double4* d_pdd = nullptr;
  // stream ownership and per-kernel event timing
  cudaStream_t own_stream = nullptr;
  // FP32 path: the Ewald k-space chain runs on kstream beside the r-space
  // chain (forks and joins on events, k-space forces into d_fk, added at the join)
  bool overlap = true;
  cudaStream_t kstream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  double* d_fk = nullptr;
  // the tensor-core passes' arguments (TcBox) for the position and force
  // buffers of the context's own calls: slot 3 ri + fi for r = (d_r, d_rs)[ri],
  // f = (d_f, d_fs, d_fk)[fi]; slot 6 for a caller's buffers
  TcBox* d_tcb = nullptr;
  TcBox h_tcb[7];
  bool prof_on = false;
  // one MD step (force-only / measured) captured as a CUDA graph
  cudaGraphExec_t g_step = nullptr, g_meas = nullptr;
  int graph_launches = 0, graph_launches_meas = 0;
  bool use_graph = true;
  struct Rec { int id; cudaEvent_t a, b; };
  std::vector<std::string> pnames;
  std::vector<double> pms;
  std::vector<long> pcnt;
  std::vector<Rec> pending;
  std::vector<cudaEvent_t> evpool;
  size_t evused = 0;
};

namespace {

int fail(mg_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return fail(ctx, MG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

cudaEvent_t prof_event(mg_ctx* c) {
  if (c->evused == c->evpool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    c->evpool.push_back(e);
  }
  return c->evpool[c->evused++];
}

int prof_id(mg_ctx* c, const char* name) {
  for (size_t i = 0; i < c->pnames.size(); i++)
    if (c->pnames[i] == name) return (int)i;
  c->pnames.push_back(name);
  c->pms.push_back(0);
  c->pcnt.push_back(0);
  return (int)c->pnames.size() - 1;
}

// fold the recorded event pairs into the per-kernel totals (after a sync)
void prof_resolve(mg_ctx* c) {
  for (auto& r : c->pending) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      c->pms[r.id] += ms;
      c->pcnt[r.id] += 1;
    }
  }
  c->pending.clear();
  c->evused = 0;
}

// launch `call` on stream `strm`; with profiling on, bracket it by events
// on that stream
#define PROFS(name, strm, call)                                       \
  do {                                                                \
    cudaEvent_t a_ = nullptr;                                         \
    if (ctx->prof_on) {                                               \
      a_ = prof_event(ctx);                                           \
      cudaEventRecord(a_, strm);                                      \
    }                                                                 \
    CK(call);                                                         \
    if (ctx->prof_on) {                                               \
      cudaEvent_t b_ = prof_event(ctx);                               \
      cudaEventRecord(b_, strm);                                      \
      ctx->pending.push_back(mg_ctx::Rec{prof_id(ctx, name), a_, b_}); \
    }                                                                 \
  } while (0)
#define PROF(name, call) PROFS(name, ctx->stream, call)

template <typename T>
cudaError_t dalloc(T** p, size_t n) {
  return cudaMalloc((void**)p, sizeof(T) * (n ? n : 1));
}
template <typename T>
cudaError_t upload(T** p, const T* h, size_t n) {
  cudaError_t e = dalloc(p, n);
  if (e != cudaSuccess || n == 0) return e;
  return cudaMemcpy(*p, h, sizeof(T) * n, cudaMemcpyHostToDevice);
}

int setup(mg_ctx* ctx, const mg_topology* t, const mg_params* p) {
  if (!t || !p || t->ns <= 0 || t->nmol <= 0 || !t->mol_first || !t->site_type || !t->charge ||
      !t->mass || t->ntypes <= 0 || !t->type_EvdW || !t->type_RvdW)
    return fail(ctx, MG_ERR_ARG, "incomplete topology");
  if (t->chargepol && !t->alphapol)
    return fail(ctx, MG_ERR_ARG, "Drude charges need alphapol");
  if (p->precision != MG_FP64 && p->precision != MG_MIXED)
    return fail(ctx, MG_ERR_ARG, "precision must be MG_FP64 or MG_MIXED");
  if (!(p->cutoff > 0) || !(p->alpha > 0) || !(p->kappa > 0))
    return fail(ctx, MG_ERR_ARG, "cutoff, alpha and kappa must be positive");
  for (int d = 0; d < 3; d++)
    if (!(p->L[d] > 2 * p->cutoff))
      return fail(ctx, MG_ERR_ARG, "the cutoff must be shorter than half the box");
  if (!(p->epsinf >= 1) || p->dipole_corr < 0 || p->dipole_corr > 15)
    return fail(ctx, MG_ERR_ARG, "epsinf must be >= 1, dipole_corr 0..15");
  if (t->nmol >= (1 << 23)) return fail(ctx, MG_ERR_SIZE, "too many molecules (limit 2^23-1)");

  ctx->precision = p->precision;
  ctx->ns = t->ns;
  ctx->nmol = t->nmol;
  std::memcpy(ctx->L, p->L, sizeof(ctx->L));
  ctx->cutoff = p->cutoff;
  ctx->alpha = p->alpha;
  ctx->epsinf = p->epsinf;
  ctx->elcorr = p->dipole_corr;
  {
    // sim/ewald.c:869-887; the tin-foil term (epsinf >= 1e20) is below 1e-30 K
    const double V = p->L[0] * p->L[1] * p->L[2];
    if (ctx->elcorr & 7) {
      for (int d = 0; d < 3; d++)
        if (ctx->elcorr & (1 << d)) {
          ctx->dipe[d] = 2 * M_PI / V;
          ctx->dipc[d] = (ctx->elcorr & 8) ? 0 : 4 * M_PI / V;
        }
      ctx->dipole = true;
    } else if (p->epsinf < 1e20) {
      const double c = 4 * M_PI / (2 * p->epsinf + 1) / V;
      for (int d = 0; d < 3; d++) {
        ctx->dipc[d] = c;
        ctx->dipe[d] = c / 2;
      }
      ctx->dipole = true;
    }
  }
  ctx->h = p->h > 0 ? p->h : 0.002;
  ctx->epsc = p->epsc > 0 ? p->epsc : 1e-7;
  ctx->omega = 0.5 * (p->omegac > 0 ? p->omegac : 1.2);
  ctx->shake_maxit = p->shake_maxit > 0 ? p->shake_maxit : 1000;
  ctx->polar = t->chargepol != nullptr;
  ctx->aspc_k = p->aspc_k;
  if (ctx->aspc_k < 0 || ctx->aspc_k > 9) return fail(ctx, MG_ERR_ARG, "aspc_k must be 0..9");
  ctx->scf_iter = p->scf_iter > 0 ? p->scf_iter : 1;
  ctx->scf_omega = p->scf_omega > 0 ? p->scf_omega : 0.6;
  ctx->minqq = p->minqq > 0 ? p->minqq : 1.0;
  ctx->use_list = p->skin > 0;
  ctx->pair_variant = p->pair_variant;
  if (ctx->pair_variant < 0 || ctx->pair_variant > 10)
    return fail(ctx, MG_ERR_ARG, "pair_variant must be 0..10");
  ctx->thermostat = p->thermostat;
  if (ctx->thermostat < 0 || ctx->thermostat > 3)
    return fail(ctx, MG_ERR_ARG, "thermostat: 0 none, 1 Berendsen, 2 Bussi, 3 Nose-Hoover");
  ctx->nose_pred = p->nose_pred > 0 ? p->nose_pred : 2;
  if (ctx->nose_pred > MG_NOSE_MAXPRED)
    return fail(ctx, MG_ERR_ARG, "nose_pred must be at most 8");
  if (ctx->thermostat && !(p->T > 0 && p->tau_T > 0))
    return fail(ctx, MG_ERR_ARG, "thermostat needs T > 0 and tau_T > 0");
  ctx->T = p->T;
  ctx->tau_T = p->tau_T;
  ctx->seed = p->seed;
  ctx->skin = p->skin > 0 ? p->skin : 0;
  ctx->drmax = std::fabs(p->drmax);
  ctx->drift_step = p->drift_step != 0;
  ctx->overlap = p->kspace_serial == 0;
  ctx->normalize = p->no_normalize ? 0 : 1;
  ctx->box_r0 = p->box_rmin > 0 ? p->box_rmin : (p->box_rmin < 0 ? 0.0 : 0.15);
  ctx->nl_every = p->nl_every > 0 ? p->nl_every : 50;
  CK(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
  ctx->stream = ctx->own_stream;
  CK(cudaStreamCreateWithFlags(&ctx->kstream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
  const int ns = t->ns;

  // ---- site kinds: distinct (LJ type, charge, Drude charge) combinations
  std::map<std::tuple<int, double, double>, int> kinds;
  std::vector<int> kind_type;
  std::vector<double> kind_q, kind_qp;
  ctx->h_kind.resize(ns);
  ctx->h_mol.resize(ns);
  for (int n = 0; n < t->nmol; n++)
    for (int i = t->mol_first[n]; i < t->mol_first[n + 1]; i++) ctx->h_mol[i] = n;
  double sumq2 = 0;
  for (int i = 0; i < ns; i++) {
    if (t->site_type[i] < 0 || t->site_type[i] >= t->ntypes)
      return fail(ctx, MG_ERR_ARG, "site type out of range");
    const double qp = ctx->polar ? t->chargepol[i] : 0.0;
    auto key = std::make_tuple(t->site_type[i], t->charge[i], qp);
    auto it = kinds.find(key);
    if (it == kinds.end()) {
      int k = (int)kind_type.size();
      kinds[key] = k;
      kind_type.push_back(t->site_type[i]);
      kind_q.push_back(t->charge[i]);
      kind_qp.push_back(qp);
      ctx->h_kind[i] = k;
    } else {
      ctx->h_kind[i] = it->second;
    }
    // the self term takes the total charge of the site (sim/ewald.c:395-410)
    sumq2 += (t->charge[i] + qp) * (t->charge[i] + qp);
  }
  ctx->nkind = (int)kind_type.size();
  if (ctx->nkind > MAX_KINDS) return fail(ctx, MG_ERR_SIZE, "more than 16 site kinds");
  ctx->kind_type = kind_type;
  ctx->kind_q = kind_q;
  ctx->ntypes = t->ntypes;
  ctx->comb_rule = t->comb_rule;
  ctx->h_tE.assign(t->type_EvdW, t->type_EvdW + t->ntypes);
  ctx->h_tR.assign(t->type_RvdW, t->type_RvdW + t->ntypes);
  ctx->h_tA.assign(t->ntypes, 0.0);
  if (t->type_alpha) ctx->h_tA.assign(t->type_alpha, t->type_alpha + t->ntypes);
  ctx->type_count.assign(t->ntypes, 0);
  for (int i = 0; i < ns; i++) ctx->type_count[t->site_type[i]]++;
  ctx->eself = -p->alpha / 1.772453850905516 * sumq2;

  // ---- LJ pair tables (combining rule + smooth cutoff), per pair of kinds
  double C2 = p->LJcutoff > 0 ? p->LJcutoff : p->cutoff;
  ctx->C2 = C2;
  std::vector<PairLJ> tp(t->ntypes * t->ntypes);
  std::vector<double> ta(t->ntypes, 0.0);
  for (int a = 0; a < t->ntypes; a++)
    for (int b = 0; b < t->ntypes; b++) {
      double eps, sig;
      double aa = t->type_alpha ? t->type_alpha[a] : 0, ab = t->type_alpha ? t->type_alpha[b] : 0;
      combining_rule(t->type_EvdW[a], t->type_RvdW[a], aa, t->type_EvdW[b], t->type_RvdW[b], ab,
                     t->comb_rule, &eps, &sig);
      if (smooth_lj(eps, sig, C2, &tp[a * t->ntypes + b]))
        return fail(ctx, MG_ERR_SETUP, "smooth LJ cutoff cannot be determined");
    }
  int nk2 = ctx->nkind * ctx->nkind;
  std::vector<PairF> pf(nk2);
  std::vector<PairD> pd(nk2);
  for (int a = 0; a < ctx->nkind; a++)
    for (int b = 0; b < ctx->nkind; b++) {
      const PairLJ& P = tp[kind_type[a] * t->ntypes + kind_type[b]];
      const double qq = kind_q[a] * kind_q[b], qpc = kind_qp[a] * kind_q[b],
                   qcp = kind_q[a] * kind_qp[b], qpp = kind_qp[a] * kind_qp[b];
      pd[a * ctx->nkind + b] =
          PairD{P.C1q, P.C2q, P.A4, P.E24, P.Sq, qq, P.A, P.E4, qpc, qcp, qpp, 0.0};
      pf[a * ctx->nkind + b] = PairF{(float)P.C1q, (float)P.C2q, (float)P.A4, (float)P.E24,
                                     (float)P.Sq,  (float)qq,    (float)P.A,  (float)P.E4,
                                     (float)qpc,   (float)qcp,   (float)qpp,  0.f,
                                     qq,           qpc,          qcp,         qpp};
    }

  // ---- erfc spline table over [0, cutoff + rplus)
  std::vector<double> ert;
  double rplus = p->rplus > 0 ? p->rplus : 2.5;
  int grid = p->grid > 0 ? p->grid : 256;
  erfc_table(grid, p->cutoff + rplus, p->cutoff, p->alpha, p->rshift, &ert, &ctx->sgrid);
  int ntab = (int)(ert.size() / 6);

  // ---- cells: size >= cutoff/cdiv and at least 2*cdiv+1 cells per edge.
  // Automatic cdiv: about 24 sites per cell (a warp's lanes own the sites of
  // a home cell), i.e. cdiv = cutoff (rho/24)^(1/3): 2 for water at a 10-12 A
  // cutoff, 1 for dilute ionic fluids
  int cdivv = p->cells_per_cutoff;
  if (cdivv <= 0) {
    const double rho = ns / (p->L[0] * p->L[1] * p->L[2]);
    cdivv = (int)std::lround((ctx->use_list ? p->cutoff + ctx->skin : p->cutoff) *
                             std::cbrt(rho / 24.0));
    cdivv = std::max(1, std::min(cdivv, 3));
  }
  // cells cover the list radius cutoff+skin (or the cutoff without lists)
  const double rgrid = ctx->use_list ? p->cutoff + ctx->skin : p->cutoff;
  int nc3[3] = {1, 1, 1};
  bool allpairs = false;
  for (;; cdivv++) {
    if (cdivv > 8) {
      // box barely larger than twice the cutoff: one cell holding every
      // site, pairs taken with the nearest image
      allpairs = true;
      nc3[0] = nc3[1] = nc3[2] = 1;
      break;
    }
    bool ok = true;
    for (int d = 0; d < 3; d++) {
      nc3[d] = (int)(p->L[d] * cdivv / rgrid);
      if (nc3[d] < 2 * cdivv + 1) ok = false;
    }
    if (ok) break;
  }
  ctx->allpairs = allpairs;
  ctx->ntab = (int)(ert.size() / 6);
  ctx->ncx = nc3[0];
  ctx->ncy = nc3[1];
  ctx->ncz = nc3[2];
  ctx->ncell = nc3[0] * nc3[1] * nc3[2];
  std::vector<int4> st;
  if (allpairs) {
    st.push_back(make_int4(0, 0, 0, 0));
  } else {
    for (int dx = -cdivv; dx <= cdivv; dx++)
      for (int dy = -cdivv; dy <= cdivv; dy++)
        for (int dz = -cdivv; dz <= cdivv; dz++) {
          double g[3] = {(double)std::max(std::abs(dx) - 1, 0) * p->L[0] / nc3[0],
                         (double)std::max(std::abs(dy) - 1, 0) * p->L[1] / nc3[1],
                         (double)std::max(std::abs(dz) - 1, 0) * p->L[2] / nc3[2]};
          double dmin2 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
          // margin: a site's cell comes from its 32-bit fixed-point
          // coordinate, within 2^-32 L of the cell's bounds
          if (dmin2 < rgrid * rgrid * (1 + 1e-6)) st.push_back(make_int4(dx, dy, dz, 0));
        }
  }
  ctx->nstencil = (int)st.size();
  // z-runs of the stencil: its entries come (dx, dy)-major with dz running
  std::vector<int4> spans;
  for (size_t k = 0; k < st.size();) {
    size_t e = k + 1;
    while (e < st.size() && st[e].x == st[k].x && st[e].y == st[k].y && st[e].z == st[e - 1].z + 1)
      e++;
    spans.push_back(make_int4(st[k].x, st[k].y, st[k].z, st[e - 1].z));
    k = e;
  }
  ctx->nspans = (int)spans.size();
  // the half shell: columns with dx > 0, or dx = 0 and dy > 0, whole; the
  // column (0, 0) from the home cell up (dz >= 0)
  std::vector<int4> hspans;
  for (const int4& sp : spans) {
    if (sp.x > 0 || (sp.x == 0 && sp.y > 0)) {
      hspans.push_back(sp);
    } else if (sp.x == 0 && sp.y == 0 && sp.w >= 0) {
      hspans.push_back(make_int4(0, 0, std::max(sp.z, 0), sp.w));
    }
  }
  ctx->nhspans = (int)hspans.size();
  // work items of the group kernel: at most ns / GROUP_SITES + ncell
  ctx->ngroup_grid = (int)(((long)ns / GROUP_SITES + ctx->ncell + GROUP_WARPS) / GROUP_WARPS);
  ctx->nprows = std::max(ctx->ncell, ctx->ngroup_grid);

  // ---- k-vectors (cook's set), sorted into (kx,ky) columns of consecutive kz
  double kappa = p->kappa;
  std::vector<int> kv;
  int nk = kvector_set(p->L, &kappa, &kv);
  if (nk <= 0) return fail(ctx, MG_ERR_SETUP, "k-vector set is empty or ill-defined");
  ctx->kappa = kappa;
  ctx->nk = nk;
  std::vector<int> ordk(nk);
  for (int i = 0; i < nk; i++) ordk[i] = i;
  std::sort(ordk.begin(), ordk.end(), [&](int a, int b) {
    for (int d = 0; d < 3; d++)
      if (kv[3 * a + d] != kv[3 * b + d]) return kv[3 * a + d] < kv[3 * b + d];
    return false;
  });
  std::vector<int4> kvec(nk);
  std::vector<double> ekk(nk);
  double V = p->L[0] * p->L[1] * p->L[2], PIaq = -std::pow(M_PI / p->alpha, 2);
  for (int i = 0; i < nk; i++) {
    int a = ordk[i];
    kvec[i] = make_int4(kv[3 * a], kv[3 * a + 1], kv[3 * a + 2], 0);
    double kk = std::pow(kvec[i].z / p->L[2], 2) +
                (std::pow(kvec[i].y / p->L[1], 2) + std::pow(kvec[i].x / p->L[0], 2));
    ekk[i] = 4 / (kk * V) * std::exp(PIaq * kk);
    ctx->Kx = std::max(ctx->Kx, std::abs(kvec[i].x));
    ctx->Ky = std::max(ctx->Ky, std::abs(kvec[i].y));
    ctx->Kz = std::max(ctx->Kz, std::abs(kvec[i].z));
  }
  std::vector<KCol> cols;
  std::vector<KTask> tasks;
  for (int i = 0; i < nk;) {
    int j = i + 1;
    while (j < nk && kvec[j].x == kvec[i].x && kvec[j].y == kvec[i].y &&
           kvec[j].z == kvec[j - 1].z + 1)
      j++;
    cols.push_back(KCol{kvec[i].x, kvec[i].y, kvec[i].z, j - i, i, {0, 0, 0}});
    for (int s = i; s < j; s += KZT)
      tasks.push_back(KTask{kvec[s].x, kvec[s].y, kvec[s].z, std::min(KZT, j - s), s, {0, 0, 0}});
    i = j;
  }
  ctx->ncol = (int)cols.size();
  ctx->ntask = (int)tasks.size();
  // rows of the tiled k-space kernels: sorted by kz extent, KTR per tile
  std::vector<KRow> krows;
  for (const KCol& c : cols) krows.push_back(KRow{c.kx, c.ky, c.kz0, c.kz0 + c.n - 1, c.k0, {0, 0, 0}});
  auto extent = [](const KRow& r) { return std::max(std::abs(r.kzlo), std::abs(r.kzhi)); };
  std::stable_sort(krows.begin(), krows.end(),
                   [&](const KRow& x, const KRow& y) { return extent(x) > extent(y); });
  std::vector<KTile> tiles;
  std::vector<int2> p1job;
  for (int r0 = 0; r0 < (int)krows.size(); r0 += KTR) {
    int n = std::min(KTR, (int)krows.size() - r0), R = 0;
    for (int i = r0; i < r0 + n; i++) R = std::max(R, extent(krows[i]));
    // pass-1 jobs: |kz| chunks of KZC_MIXED over [0, R] (FP32 kernel, both
    // signs at once) or kz chunks of 16 over [-R, R] (FP64 kernel)
    if (ctx->precision == MG_MIXED)
      for (int kz0 = 0; kz0 <= R; kz0 += KZC_MIXED) p1job.push_back(make_int2((int)tiles.size(), kz0));
    else
      for (int kz0 = -R; kz0 <= R; kz0 += 16) p1job.push_back(make_int2((int)tiles.size(), kz0));
    tiles.push_back(KTile{r0, n, R, 0});
  }
  ctx->ntile = (int)tiles.size();
  ctx->np1job = (int)p1job.size();
  ctx->row = ctx->precision == MG_MIXED ? phase_row_mixed(ctx->Kx, ctx->Ky, ctx->Kz)
                                         : (ctx->Kx + 1) + (2 * ctx->Ky + 1) + (2 * ctx->Kz + 1);

  // ---- charges of the Ewald sums: centres, then the site's Drude charge
  std::vector<int> qsite, qdrude, dsite;
  std::vector<double> qval, dqc, dqp, daqq;
  for (int i = 0; i < ns; i++) {
    if (t->charge[i] != 0) {
      qsite.push_back(i);
      qval.push_back(t->charge[i]);
      qdrude.push_back(0);
    }
    if (ctx->polar && t->chargepol[i] != 0) {
      qsite.push_back(i);
      qval.push_back(t->chargepol[i]);
      qdrude.push_back(1);
      dsite.push_back(i);
      dqc.push_back(t->charge[i]);
      dqp.push_back(t->chargepol[i]);
      // cook: si->alpha_qq = alphapol / chargepol^2 (cook/simdef.c:1008-1010)
      daqq.push_back(t->alphapol[i] / (t->chargepol[i] * t->chargepol[i]));
    }
  }
  ctx->nq = (int)qsite.size();
  ctx->nd = (int)dsite.size();
  ctx->ndblocks = (ctx->nd + 127) / 128;
  // charge chunks of pass 1: about 8 (FP64 kernel) or 10 (FP32 kernel) CTAs
  // per SM of a GB300, at least 512 charges each.  Smaller chunks fill the
  // GPU with one small box but multiply the partial sums the reduction
  // reads (nk x nchunk): a batch of 256 boxes of 500-4000 ions spent more
  // time reducing 64-charge chunks than in pass 1 itself.  The split is
  // fixed by the box, not by the device, so results do not depend on it.
  const int p1ctas = (p->kspace_ctas_per_sm > 0 ? p->kspace_ctas_per_sm
                                                : (ctx->precision == MG_MIXED ? 10 : 8)) *
                     PARTITION_SMS;
  ctx->nchunk = std::max(1, std::min(std::max(1, ctx->nq / 512),
                                     (p1ctas + ctx->np1job - 1) / ctx->np1job));
  ctx->nkblocks = (nk + 255) / 256;

  // ---- constraints
  ctx->nc = t->nc;
  std::vector<int> mcf(t->nmol + 1, 0);
  std::vector<int2> cons(std::max(t->nc, 0));
  std::vector<double> bondq(std::max(t->nc, 0));
  if (t->nc > 0) {
    if (!t->cons || !t->cons_len || !t->mol_cfirst)
      return fail(ctx, MG_ERR_ARG, "constraints need cons, cons_len and mol_cfirst");
    for (int k = 0; k <= t->nmol; k++) mcf[k] = t->mol_cfirst[k];
    for (int k = 0; k < t->nc; k++) {
      cons[k] = make_int2(t->cons[2 * k], t->cons[2 * k + 1]);
      bondq[k] = t->cons_len[k] * t->cons_len[k];
    }
  }
  std::vector<double> imass(ns), mass(ns);
  for (int i = 0; i < ns; i++) {
    mass[i] = t->mass[i];
    imass[i] = t->mass[i] > 0 ? 1 / t->mass[i] : 0;
  }

  // ---- device buffers (Drude builds: 2*ns vectors, cook's polar half)
  const size_t nvec = 3 * (size_t)ns * (ctx->polar ? 2 : 1);
  CK(dalloc(&ctx->d_r, nvec));
  CK(dalloc(&ctx->d_f, nvec));
  CK(dalloc(&ctx->d_r1, nvec));
  CK(dalloc(&ctx->d_rs, nvec));
  CK(dalloc(&ctx->d_fs, nvec));
  CK(dalloc(&ctx->d_p, 3 * (size_t)ns));
  if (ctx->polar) {
    CK(upload(&ctx->d_dsite, dsite.data(), dsite.size()));
    CK(upload(&ctx->d_qc, dqc.data(), dqc.size()));
    CK(upload(&ctx->d_qp, dqp.data(), dqp.size()));
    CK(upload(&ctx->d_aqq, daqq.data(), daqq.size()));
    CK(upload(&ctx->d_qdrude, qdrude.data(), qdrude.size()));
    CK(dalloc(&ctx->d_hist, (size_t)(ctx->aspc_k + 2) * 3 * std::max(ctx->nd, 1)));
    CK(dalloc(&ctx->d_drpart, (size_t)std::max(ctx->ndblocks, 1) * 8));
    if (p->precision == MG_MIXED) CK(dalloc(&ctx->d_pdj, ns));
    else CK(dalloc(&ctx->d_pdd, ns));
  }
  CK(upload(&ctx->d_kind, ctx->h_kind.data(), ns));
  CK(upload(&ctx->d_mol, ctx->h_mol.data(), ns));
  CK(dalloc(&ctx->d_key, ns));
  CK(dalloc(&ctx->d_pfix, ns));
  CK(dalloc(&ctx->d_idx, ns));
  CK(dalloc(&ctx->d_key_s, ns));
  CK(dalloc(&ctx->d_order, ns));
  CK(dalloc(&ctx->d_cell_start, ctx->ncell + 1));
  {
    const size_t nc4 = ((size_t)ctx->ncell + 3) / 4 * 4;
    CK(dalloc(&ctx->d_ccount, nc4));
    CK(cudaMemset(ctx->d_ccount, 0, nc4 * sizeof(int)));
    CK(dalloc(&ctx->d_ccursor, ctx->ncell));
  }
  CK(upload(&ctx->d_stencil, st.data(), st.size()));
  CK(upload(&ctx->d_spans, spans.data(), spans.size()));
  CK(upload(&ctx->d_hspans, hspans.data(), hspans.size()));
  if (ctx->pair_variant >= 9) {
    // centres, then (Drude builds) shells
    const size_t nfix = 3 * (size_t)ns * (t->chargepol ? 2 : 1);
    CK(dalloc(&ctx->d_facc, nfix));
    CK(cudaMemset(ctx->d_facc, 0, nfix * sizeof(long long)));
  }
  CK(dalloc(&ctx->d_gstart, (size_t)ctx->ncell + 1));
  CK(dalloc(&ctx->d_gcell, (size_t)ns / GROUP_SITES + ctx->ncell + 1));
  ctx->nxblocks = (t->nmol + EXCL_THREADS - 1) / EXCL_THREADS;
  ctx->nepart = std::max(ctx->nprows + ctx->nxblocks,
                         std::max(list_blocks(ns, true), list_blocks(ns, false)));
  CK(dalloc(&ctx->d_epart, (size_t)ctx->nepart * 10));
  // rows a pair kernel does not write stay zero
  CK(cudaMemset(ctx->d_epart, 0, (size_t)ctx->nepart * 10 * sizeof(double)));
  if (ctx->use_list) {
    // capacity: the largest expected count in a sphere of the list radius at
    // 1.5 times the mean site density, in multiples of 32 (grown on overflow)
    const double V = p->L[0] * p->L[1] * p->L[2], rl = p->cutoff + ctx->skin;
    ctx->nl_cap = ((int)(1.5 * ns / V * 4.18879 * rl * rl * rl) + 64 + 31) / 32 * 32;
    ctx->nl_cap = (std::min(ctx->nl_cap, ns) + 7) / 8 * 8;  // rows 16-byte aligned
    ctx->nl_pitch = ctx->nl_cap;
    CK(dalloc(&ctx->d_nlist, (size_t)ctx->nl_cap * ns));
    CK(dalloc(&ctx->d_ncount, ns));
    CK(dalloc(&ctx->d_rbuild, 3 * (size_t)ns));
    CK(dalloc(&ctx->d_dmax, 1));
    CK(cudaMemset(ctx->d_dmax, 0, sizeof(int)));
    CK(cudaMallocHost((void**)&ctx->h_dmax, sizeof(int)));
    *ctx->h_dmax = 0;
    CK(cudaEventCreateWithFlags(&ctx->ev_dmax, cudaEventDisableTiming));
    if (p->precision != MG_MIXED) CK(dalloc(&ctx->d_pj, ns));
  }
  CK(upload(&ctx->d_qsite, qsite.data(), qsite.size()));
  CK(upload(&ctx->d_qval, qval.data(), qval.size()));
  if (ctx->dipole) CK(dalloc(&ctx->d_dippart, 3 * (size_t)dipole_blocks(std::max(ctx->nq, 1))));
  CK(upload(&ctx->d_task, tasks.data(), tasks.size()));
  CK(upload(&ctx->d_col, cols.data(), cols.size()));
  CK(upload(&ctx->d_kvec, kvec.data(), kvec.size()));
  CK(upload(&ctx->d_krows, krows.data(), krows.size()));
  ctx->nkrows = (int)krows.size();
  if (p->kspace_engine < 0 || p->kspace_engine > 3)
    return fail(ctx, MG_ERR_ARG,
                "kspace_engine: 0 auto, 1 FP32 cores, 2 tensor-core pass 2, 3 tensor cores");
  if (ctx->precision == MG_MIXED && p->kspace_engine != 1) {
    KArgs kd;
    kd.Kx = ctx->Kx;
    kd.Ky = ctx->Ky;
    kd.Kz = ctx->Kz;
    kd.nq = ctx->nq;
    kd.row = ctx->row;
    const bool fits = kf_tc_fits(kd, ctx->nkrows);
    if (!fits && p->kspace_engine >= 2)
      return fail(ctx, MG_ERR_SIZE, "the k set is too large for the tensor-core tiles");
    ctx->kspace_tc = fits && ctx->nq > 0;
    if (ctx->kspace_tc) {
      CK(dalloc(&ctx->d_za, kf_tc_za_floats(kd)));
      CK(dalloc(&ctx->d_vb, kf_tc_vb_floats(kd, ctx->nkrows)));
      std::vector<TcRow> tr;
      std::vector<KRow> tck = krows;
      std::sort(tck.begin(), tck.end(), [](const KRow& x, const KRow& y) {
        return x.kx != y.kx ? x.kx < y.kx : x.ky < y.ky;
      });
      kf_tc_rows(kd, tck, &tr);
      CK(upload(&ctx->d_tcrows, tr.data(), tr.size()));
      CK(upload(&ctx->d_tckrows, tck.data(), tck.size()));
      if (p->kspace_engine == 3 && !sk_tc_fits(kd))
        return fail(ctx, MG_ERR_SIZE, "the k set is too large for the tensor-core pass 1");
      ctx->sk_tc = p->kspace_engine == 3 || (p->kspace_engine == 0 && sk_tc_fits(kd));
      if (ctx->sk_tc) {
        const size_t nzb = sk_tc_zb_floats(kd);
        CK(dalloc(&ctx->d_zb, nzb));
        CK(cudaMemset(ctx->d_zb, 0, nzb * sizeof(float)));
        sk_tc_split(kd, ctx->nkrows, &ctx->sk_nch, &ctx->sk_gpc);
      }
    }
  }
  CK(upload(&ctx->d_tiles, tiles.data(), tiles.size()));
  CK(upload(&ctx->d_p1job, p1job.data(), p1job.size()));
  CK(upload(&ctx->d_ekk, ekk.data(), ekk.size()));
  CK(dalloc(&ctx->d_S, 2 * (size_t)nk));
  CK(dalloc(&ctx->d_ekpart, (size_t)ctx->nkblocks * 7));
  if (ctx->precision == MG_MIXED) {
    CK(dalloc(&ctx->d_pj, ns));
    CK(upload(&ctx->d_ptabf, pf.data(), pf.size()));
    std::vector<float4> erd(ntab), eru(ntab);
    for (int i = 0; i < ntab; i++) {
      erd[i] = make_float4((float)ert[6 * i + 3], (float)ert[6 * i + 4], (float)ert[6 * i + 5], 0);
      eru[i] = make_float4((float)ert[6 * i], (float)ert[6 * i + 1], (float)ert[6 * i + 2], 0);
    }
    CK(upload(&ctx->d_erd, erd.data(), ntab));
    CK(upload(&ctx->d_eru, eru.data(), ntab));
    {
      // phase rows zero-padded to whole groups of 32 charges (tensor-core pass 1)
      const size_t ntab = (size_t)((ctx->nq + 31) / 32 * 32) * ctx->row;
      CK(dalloc((float2**)&ctx->d_tab, ntab));
      CK(cudaMemset(ctx->d_tab, 0, ntab * sizeof(float2)));
    }
    CK(dalloc(&ctx->d_qfix, std::max(1, ctx->nq)));
    CK(dalloc(&ctx->d_fk, 3 * (size_t)ns * (ctx->polar ? 2 : 1)));
    CK(dalloc((float2**)&ctx->d_part, (size_t)std::max(ctx->nchunk, ctx->sk_nch) * nk));
    CK(dalloc(&ctx->d_Wf, nk));
  } else {
    CK(dalloc(&ctx->d_pd, ns));
    CK(upload(&ctx->d_ptabd, pd.data(), pd.size()));
    CK(upload(&ctx->d_ert, ert.data(), ert.size()));
    CK(dalloc((double2**)&ctx->d_tab, (size_t)ctx->nq * ctx->row));
    CK(dalloc((double2**)&ctx->d_part, (size_t)ctx->nchunk * nk));
    CK(dalloc(&ctx->d_Wd, nk));
  }
  CK(upload(&ctx->d_mol_first, t->mol_first, t->nmol + 1));
  ctx->h_mol_first.assign(t->mol_first, t->mol_first + t->nmol + 1);
  {
    // every pair of sites of one molecule with a charge product is an Ewald
    // exclusion (the r-space term of a rigid molecule is not counted)
    std::vector<int> xfirst(t->nmol + 1, 0);
    std::vector<int2> xpair;
    std::vector<double4> xq;
    for (int n = 0; n < t->nmol; n++) {
      for (int i = t->mol_first[n]; i < t->mol_first[n + 1]; i++)
        for (int j = i + 1; j < t->mol_first[n + 1]; j++) {
          const PairD& P = pd[ctx->h_kind[i] * ctx->nkind + ctx->h_kind[j]];
          if (P.qq == 0 && P.qpc == 0 && P.qcp == 0 && P.qpp == 0) continue;
          xpair.push_back(make_int2(i, j));
          xq.push_back(make_double4(P.qq, P.qpc, P.qcp, P.qpp));
        }
      xfirst[n + 1] = (int)xpair.size();
    }
    CK(upload(&ctx->d_xfirst, xfirst.data(), xfirst.size()));
    CK(upload(&ctx->d_xpair, xpair.data(), xpair.size()));
    CK(upload(&ctx->d_xq, xq.data(), xq.size()));
  }
  CK(upload(&ctx->d_mol_cfirst, mcf.data(), mcf.size()));
  CK(upload(&ctx->d_cons, cons.data(), cons.size()));
  CK(upload(&ctx->d_bondq, bondq.data(), bondq.size()));
  CK(upload(&ctx->d_imass, imass.data(), ns));
  CK(upload(&ctx->d_mass, mass.data(), ns));
  CK(dalloc(&ctx->d_kinpart, (size_t)(t->nmol + 127) / 128 + 1));
  CK(dalloc(&ctx->d_meas, 13 * ((size_t)(t->nmol + 127) / 128 + 1)));
  // dependants: parents and dependants of one molecule, consecutive per
  // molecule, no dependant a parent, weights summing to 1 (cook fixes
  // other sums with a warning, cook/simdef.c:390)
  if (t->ndep < 0) return fail(ctx, MG_ERR_ARG, "ndep < 0");
  ctx->ndep = t->ndep;
  if (t->ndep > 0) {
    if (!t->dep_site || !t->dep_first || !t->dep_parent || !t->dep_w)
      return fail(ctx, MG_ERR_ARG, "incomplete dependant tables");
    std::vector<char> isdep(ns, 0);
    for (int k = 0; k < t->ndep; k++) {
      const int d = t->dep_site[k];
      if (d < 0 || d >= ns || isdep[d]) return fail(ctx, MG_ERR_ARG, "bad dependant site");
      isdep[d] = 1;
      if (t->mass[d] != 0) return fail(ctx, MG_ERR_ARG, "a dependant site must be massless");
      if (k > 0 && ctx->h_mol[t->dep_site[k - 1]] > ctx->h_mol[d])
        return fail(ctx, MG_ERR_ARG, "dependants must be ordered by molecule");
    }
    if (t->dep_first[0] != 0) return fail(ctx, MG_ERR_ARG, "dep_first[0] must be 0");
    for (int k = 0; k < t->ndep; k++) {
      if (t->dep_first[k + 1] <= t->dep_first[k])
        return fail(ctx, MG_ERR_ARG, "a dependant without parents");
      double sw = 0;
      for (int q = t->dep_first[k]; q < t->dep_first[k + 1]; q++) {
        const int a = t->dep_parent[q];
        if (a < 0 || a >= ns || isdep[a] || ctx->h_mol[a] != ctx->h_mol[t->dep_site[k]])
          return fail(ctx, MG_ERR_ARG, "a dependant's parent must be a site of its molecule");
        sw += t->dep_w[q];
      }
      if (std::fabs(sw - 1) > 1e-5) return fail(ctx, MG_ERR_ARG, "dependant weights must sum to 1");
      if (t->dep_type) {
        const int ty = t->dep_type[k];
        if (ty < 0 || ty > 2) return fail(ctx, MG_ERR_ARG, "dependant kind must be 0, 1 or 2");
        if (ty > 0 && t->dep_first[k + 1] - t->dep_first[k] != 3)
          return fail(ctx, MG_ERR_ARG, "a Rowlinson or Lone dependant needs 3 parents");
        if (ty > 0 && !t->dep_par)
          return fail(ctx, MG_ERR_ARG, "Rowlinson or Lone dependants need dep_par");
      }
    }
    const int npar = t->dep_first[t->ndep];
    CK(upload(&ctx->d_dep_site, t->dep_site, t->ndep));
    CK(upload(&ctx->d_dep_first, t->dep_first, t->ndep + 1));
    CK(upload(&ctx->d_dep_parent, t->dep_parent, npar));
    CK(upload(&ctx->d_dep_w, t->dep_w, npar));
    if (t->dep_type) {
      CK(upload(&ctx->d_dep_type, t->dep_type, t->ndep));
      CK(upload(&ctx->d_dep_par, t->dep_par, 13 * (size_t)t->ndep));
      CK(dalloc(&ctx->d_deppart, 7 * (size_t)t->ndep));
    }
  }
  // cook's No.f: 3 per site less constraints, dependants and the conserved
  // momentum (sim/siminit.c:518-530)
  ctx->thermo_f = p->thermo_f > 0 ? p->thermo_f : 3.0 * (ns - t->ndep) - t->nc - 3;
  ctx->nchi = 2 * PARTITION_SMS;
  CK(dalloc(&ctx->d_chi, (size_t)ctx->nchi));
  CK(dalloc(&ctx->d_zth, 1));
  CK(dalloc(&ctx->d_step, 1));
  CK(cudaMemset(ctx->d_step, 0, sizeof(long long)));
  if (ctx->thermostat == 3) {
    CK(dalloc(&ctx->d_nh, NH_HIST + MG_NOSE_MAXPRED));
    CK(cudaMemset(ctx->d_nh, 0, sizeof(double) * (NH_HIST + MG_NOSE_MAXPRED)));
    CK(dalloc(&ctx->d_vhist, (size_t)ctx->nose_pred * 3 * ns));
    CK(cudaMemset(ctx->d_vhist, 0, sizeof(double) * ctx->nose_pred * 3 * (size_t)ns));
  }
  {
    const double one = 1;
    CK(cudaMemcpy(ctx->d_zth, &one, sizeof(double), cudaMemcpyHostToDevice));
  }
  CK(dalloc(&ctx->d_status, 1));
  CK(cudaMemset(ctx->d_status, 0, sizeof(int)));
  if (ctx->drmax > 0) {
    const unsigned int rep0[2] = {0u, 0x3f800000u};  // no site, factor 1.0f
    CK(upload(&ctx->d_bdrep, rep0, 2));
  }
  ctx->total_mass = 0;
  for (int i = 0; i < ns; i++) ctx->total_mass += t->mass[i];
  CK(dalloc(&ctx->d_driftpart, 3 * (size_t)drift_blocks(ns)));
  CK(dalloc(&ctx->d_drift, 6));
  CK(dalloc(&ctx->d_sums, NSUMS));
  CK(cudaMemset(ctx->d_sums, 0, NSUMS * sizeof(double)));
  CK(cudaMallocHost((void**)&ctx->h_sums, NSUMS * sizeof(double)));
  return MG_OK;
}

Launch launch(mg_ctx* ctx) { return Launch{ctx->stream, &ctx->launches}; }

// forces of the positions in r_dev (device, cook layout) into f_dev; the
// energies are reduced into d_sums when measure
ListArgs list_args(mg_ctx* ctx) {
  ListArgs l;
  l.ncx = ctx->ncx;
  l.ncy = ctx->ncy;
  l.ncz = ctx->ncz;
  l.nstencil = ctx->nstencil;
  l.cell_start = ctx->d_cell_start;
  l.stencil = ctx->d_stencil;
  l.sx = (float)(ctx->L[0] / 4294967296.0);
  l.sy = (float)(ctx->L[1] / 4294967296.0);
  l.sz = (float)(ctx->L[2] / 4294967296.0);
  const double rl = ctx->cutoff + ctx->skin;
  l.rlist2 = (float)(rl * rl);
  l.cap = ctx->nl_cap;
  l.pitch = ctx->nl_pitch;
  l.nlist = ctx->d_nlist;
  l.ncount = ctx->d_ncount;
  l.status = ctx->d_status;
  return l;
}

// Verlet lists of the positions r_dev (cells binned and sorted here): the
// build is followed by a synchronous overflow check that grows the lists
int build_lists(mg_ctx* ctx, const double* r_dev) {
  Launch L = launch(ctx);
  for (int attempt = 0; attempt < 4; attempt++) {
    ListArgs l = list_args(ctx);
    if (ctx->allpairs)
      PROF("list_build", k_build_list(L, l, ctx->ns, ctx->d_key_s, ctx->d_pj));
    else
      PROF("list_build", k_build_list_cells(L, l, ctx->d_pj));
    PROF("neighbour_list", k_save_build(L, ctx->ns, r_dev, ctx->d_rbuild));
    int st = 0;
    CK(cudaMemcpyAsync(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (!(st & 16)) {
      ctx->need_build = false;
      ctx->since_build = 0;
      CK(cudaMemsetAsync(ctx->d_dmax, 0, sizeof(int), ctx->stream));
      ctx->dmax_pending = false;
      return MG_OK;
    }
    st &= ~16;
    CK(cudaMemcpyAsync(ctx->d_status, &st, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaFree(ctx->d_nlist));
    ctx->d_nlist = nullptr;
    ctx->nl_cap = (std::min(ctx->ns, ctx->nl_cap * 3 / 2 + 32) + 7) / 8 * 8;
    ctx->nl_pitch = ctx->nl_cap;
    CK(dalloc(&ctx->d_nlist, (size_t)ctx->nl_cap * ctx->ns));
  }
  return fail(ctx, MG_ERR_SIZE, "neighbour list capacity");
}

// the arguments of the context's tensor-core Ewald passes (r: the positions,
// needed by the phase kernel only)
TcBox tc_args(mg_ctx* ctx, const KArgs& a, const double* r) {
  TcBox b;
  tc_box(a, ctx->nkrows, ctx->sk_nch, ctx->sk_gpc, ctx->d_tckrows, ctx->d_tcrows, r,
         (float2*)ctx->d_tab, ctx->d_za, ctx->sk_tc ? ctx->d_zb : nullptr, ctx->d_vb,
         (float2*)ctx->d_part, &b);
  return b;
}

// the device copy of the tensor-core arguments for positions r (NULL: any;
// only the phase kernel reads them) and the forces of a; *h gets the host
// copy.  Buffers other than the context's own go to the last slot, uploaded
// before the launch (not while the stream is being captured).
const TcBox* tc_slot(mg_ctx* ctx, const Launch& L, const KArgs& a, const double* r,
                     const TcBox** h) {
  const double* rs[2] = {ctx->d_r, ctx->d_rs};
  const double* fs[3] = {ctx->d_f, ctx->d_fs, ctx->d_fk};
  int ri = -1, fi = -1;
  for (int i = 0; i < 2; i++)
    if (!r || r == rs[i]) {
      ri = i;
      break;
    }
  for (int i = 0; i < 3; i++)
    if (a.f == fs[i]) fi = i;
  if (ri >= 0 && fi >= 0) {
    *h = &ctx->h_tcb[3 * ri + fi];
    return ctx->d_tcb + 3 * ri + fi;
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(L.s, &cs) != cudaSuccess ||
      cs != cudaStreamCaptureStatusNone)
    return nullptr;
  ctx->h_tcb[6] = tc_args(ctx, a, r);
  if (cudaMemcpyAsync(ctx->d_tcb + 6, &ctx->h_tcb[6], sizeof(TcBox), cudaMemcpyHostToDevice,
                      L.s) != cudaSuccess ||
      cudaStreamSynchronize(L.s) != cudaSuccess)
    return nullptr;
  *h = &ctx->h_tcb[6];
  return ctx->d_tcb + 6;
}

// phase rows of the FP32 path; with the tensor-core passes the same kernel
// builds their operand tiles
cudaError_t phase_mixed(mg_ctx* ctx, const Launch& L, const KArgs& a, const double* r) {
  if (ctx->kspace_tc) {
    const TcBox* h = nullptr;
    const TcBox* d = tc_slot(ctx, L, a, r, &h);
    if (!d) return cudaErrorInvalidValue;
    return k_batch_tc_phase(L, d, 1, h->g_phase, h->smem_phase);
  }
  return k_phase_tables_mixed(L, a, r, (float2*)ctx->d_tab, ctx->d_qfix);
}

// Ewald pass 1 of the FP32 path (structure factor partials, then their FP64
// sum): tensor cores or FP32 cores
cudaError_t sk_mixed(mg_ctx* ctx, const Launch& L, const KArgs& a, bool measure) {
  const float2* tab = (const float2*)ctx->d_tab;
  float2* part = (float2*)ctx->d_part;
  if (!ctx->sk_tc) {
    cudaError_t e = k_sk_gemm_mixed(L, a, tab, part);
    if (e != cudaSuccess) return e;
    return k_sk_reduce_mixed(L, a, part, measure);
  }
  const TcBox* h = nullptr;
  const TcBox* d = tc_slot(ctx, L, a, nullptr, &h);
  if (!d) return cudaErrorInvalidValue;
  cudaError_t e = k_batch_sk_tc(L, d, 1, h->g_sk, h->smem_sk);
  if (e != cudaSuccess) return e;
  KArgs b = a;
  b.nchunk = ctx->sk_nch;
  return k_sk_reduce_mixed(L, b, part, measure);
}

// Ewald pass 2 of the FP32 path: tensor cores or FP32 cores
cudaError_t kf_mixed(mg_ctx* ctx, const Launch& L, const KArgs& a) {
  if (!ctx->kspace_tc) return k_kf_gemm_mixed(L, a, (const float2*)ctx->d_tab);
  const TcBox* h = nullptr;
  const TcBox* d = tc_slot(ctx, L, a, nullptr, &h);
  if (!d) return cudaErrorInvalidValue;
  return k_batch_kf_tc(L, d, 1, h->g_vb, h->g_kf, h->smem_kf);
}

ExclArgs excl_args(mg_ctx* ctx, const double* r_dev, double* f) {
  ExclArgs a;
  a.nmol = ctx->nmol;
  a.ns = ctx->ns;
  a.xfirst = ctx->d_xfirst;
  a.xpair = ctx->d_xpair;
  a.xq = ctx->d_xq;
  a.Lx = ctx->L[0];
  a.Ly = ctx->L[1];
  a.Lz = ctx->L[2];
  a.iLx = 1 / ctx->L[0];
  a.iLy = 1 / ctx->L[1];
  a.iLz = 1 / ctx->L[2];
  a.cutoff_sq = ctx->cutoff * ctx->cutoff;
  a.alpha = (float)ctx->alpha;
  a.r = r_dev;
  a.f = f;
  // energy rows after the pair kernel's
  a.epart = ctx->d_epart + (size_t)ctx->nprows * 10;
  return a;
}

// the arguments of the pair kernels and of the Ewald passes of a force
// evaluation into f_dev
PairArgs make_pair_args(mg_ctx* ctx, double* f_dev) {
  PairArgs pa{};
  pa.ns = ctx->ns;
  pa.ncx = ctx->ncx;
  pa.ncy = ctx->ncy;
  pa.ncz = ctx->ncz;
  pa.nstencil = ctx->nstencil;
  pa.allpairs = ctx->allpairs ? 1 : 0;
  pa.nkind = ctx->nkind;
  pa.cell_start = ctx->d_cell_start;
  pa.order = ctx->d_order;
  pa.stencil = ctx->d_stencil;
  pa.Lx = ctx->L[0];
  pa.Ly = ctx->L[1];
  pa.Lz = ctx->L[2];
  pa.cutoff_sq = ctx->cutoff * ctx->cutoff;
  pa.sgrid = ctx->sgrid;
  pa.alpha = ctx->alpha;
  pa.f = f_dev;
  pa.epart = ctx->d_epart;
  pa.ntab = ctx->ntab;
  pa.pdj = ctx->d_pdj;
  pa.pdd = ctx->d_pdd;
  pa.pair_warps = (ctx->pair_variant & 4) ? 16 : ((ctx->pair_variant & 1) ? 8 : 4);
  pa.spline_smem = (ctx->pair_variant & 2) && ctx->ntab * 16 <= 200 * 1024 ? 1 : 0;
  pa.group = (ctx->pair_variant & 8) ? 1 : 0;
  // half shell: 1 lanes on the home sites, 2 lanes on the neighbours
  pa.newton = ctx->pair_variant == 9 ? 1 : (ctx->pair_variant == 10 ? 2 : 0);
  pa.hspans = ctx->d_hspans;
  pa.nhspans = ctx->nhspans;
  pa.facc = ctx->d_facc;
  pa.gstart = ctx->d_gstart;
  pa.gcell = ctx->d_gcell;
  pa.spans = ctx->d_spans;
  pa.nspans = ctx->nspans;
  pa.ngrid = ctx->ngroup_grid;
  return pa;
}

KArgs make_kargs(mg_ctx* ctx, double* f_dev) {
  KArgs ka{};
  ka.nq = ctx->nq;
  ka.nk = ctx->nk;
  ka.ntask = ctx->ntask;
  ka.ncol = ctx->ncol;
  ka.nchunk = ctx->nchunk;
  ka.Kx = ctx->Kx;
  ka.Ky = ctx->Ky;
  ka.Kz = ctx->Kz;
  ka.row = ctx->row;
  set_box(ka, ctx->L);
  ka.alpha = ctx->alpha;
  ka.qsite = ctx->d_qsite;
  ka.qval = ctx->d_qval;
  ka.task = ctx->d_task;
  ka.col = ctx->d_col;
  ka.kvec = ctx->d_kvec;
  ka.ekk = ctx->d_ekk;
  ka.S = ctx->d_S;
  ka.Wf = ctx->d_Wf;
  ka.Wd = ctx->d_Wd;
  ka.f = f_dev;
  ka.ek_part = ctx->d_ekpart;
  ka.krows = ctx->d_krows;
  ka.tiles = ctx->d_tiles;
  ka.ntile = ctx->ntile;
  ka.p1job = ctx->d_p1job;
  ka.np1job = ctx->np1job;
  ka.qdrude = ctx->d_qdrude;
  ka.ns = ctx->ns;
  ka.status = ctx->d_status;
  return ka;
}

// the tensor-core arguments for the context's own buffer pairs, on the
// device once (a context with the Ewald passes on the tensor cores)
int tc_upload_slots(mg_ctx* ctx) {
  if (!ctx->kspace_tc) return MG_OK;
  double* rs[2] = {ctx->d_r, ctx->d_rs};
  double* fs[3] = {ctx->d_f, ctx->d_fs, ctx->d_fk};
  for (int ri = 0; ri < 2; ri++)
    for (int fi = 0; fi < 3; fi++) {
      const KArgs ka = make_kargs(ctx, fs[fi]);
      ctx->h_tcb[3 * ri + fi] = tc_args(ctx, ka, rs[ri]);
    }
  ctx->h_tcb[6] = ctx->h_tcb[0];
  CK(dalloc(&ctx->d_tcb, 7));
  CK(cudaMemcpy(ctx->d_tcb, ctx->h_tcb, 7 * sizeof(TcBox), cudaMemcpyHostToDevice));
  return MG_OK;
}

int forces_async(mg_ctx* ctx, const double* r_dev, double* f_dev, bool measure) {
  Launch L = launch(ctx);
  const int ns = ctx->ns;
  ctx->last_r = r_dev;
  // fork point of the concurrent k-space chain (FP32 path): everything
  // queued before, nothing of this evaluation's r-space work
  if (ctx->precision == MG_MIXED && ctx->overlap && ctx->nq > 0)
    CK(cudaEventRecord(ctx->ev_fork, ctx->stream));
  const bool rebuild = !ctx->use_list || ctx->need_build || ctx->since_build >= ctx->nl_every;
  const double iL[3] = {1.0 / ctx->L[0], 1.0 / ctx->L[1], 1.0 / ctx->L[2]};
  if (rebuild) {
    // linked cells, with the fixed-point records of the sorted sites (d_pj,
    // when the context has them) and the work items of the group kernel
    PROF("cell_list", k_cell_list(L, ns, r_dev, ctx->d_status, iL, ctx->ncx, ctx->ncy, ctx->ncz,
                                  ctx->d_kind, ctx->d_mol, ctx->d_pfix, ctx->d_key, ctx->d_ccount,
                                  ctx->d_ccursor, ctx->d_idx, ctx->d_order, ctx->d_key_s,
                                  ctx->d_cell_start, ctx->d_gstart, ctx->d_pj, ctx->d_gcell));
  }
  PairArgs pa = make_pair_args(ctx, f_dev);
  KArgs ka = make_kargs(ctx, f_dev);
  ListArgs la = list_args(ctx);
  int nerows = ctx->nprows;
  if (ctx->precision == MG_MIXED) {
    // the k-space chain on kstream, concurrent with the r-space chain below;
    // its forces go to d_fk and are added at the join
    const bool fork = ctx->overlap && ctx->nq > 0;
    const size_t nf = 3 * (size_t)ns * (ctx->polar ? 2 : 1);
    if (fork) {
      cudaStream_t ks = ctx->kstream;
      Launch LK{ks, &ctx->launches};
      KArgs kk = ka;
      kk.f = ctx->d_fk;
      CK(cudaStreamWaitEvent(ks, ctx->ev_fork, 0));
      CK(cudaMemsetAsync(ctx->d_fk, 0, nf * sizeof(double), ks));
      PROFS("phase_tables", ks, phase_mixed(ctx, LK, kk, r_dev));
      PROFS("ewald_sk", ks, sk_mixed(ctx, LK, kk, measure));
      PROFS("ewald_kforce", ks, kf_mixed(ctx, LK, kk));
      CK(cudaEventRecord(ctx->ev_join, ks));
    }
    // new positions with the order of an earlier build (lists kept)
    if (!rebuild)
      PROF("gather", k_gather_mixed(L, ns, r_dev, ctx->d_order, ctx->d_kind, ctx->d_mol, iL,
                                    ctx->d_pj));
    if (ctx->polar) PROF("gather", k_gather_drude(L, ns, r_dev, ctx->d_order, ctx->d_pdj, nullptr));
    if (ctx->use_list) {
      if (rebuild) {
        int rc = build_lists(ctx, r_dev);
        if (rc) return rc;
        la = list_args(ctx);
      }
      PROF("pair_mixed", k_pair_list_mixed(L, pa, la, ctx->d_pj, ctx->d_ptabf, ctx->d_erd,
                                           ctx->d_eru, measure, ctx->polar));
      nerows = list_blocks(ns, true);
    } else {
      PROF("pair_mixed", k_pair_mixed(L, pa, ctx->d_pj, ctx->d_ptabf, ctx->d_erd, ctx->d_eru,
                                      measure, ctx->polar));
      // after the pair kernel, before the k-space forces are added: the same
      // summation order with and without the concurrent k-space chain
      ExclArgs xa = excl_args(ctx, r_dev, f_dev);
      PROF("exclusions", k_excl_mixed(L, xa, measure, ctx->polar));
      nerows = ctx->nprows + ctx->nxblocks;
    }
    if (fork) {
      CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0));
      PROF("ewald_kforce", k_add_forces(L, nf, ctx->d_fk, f_dev));
    } else if (ctx->nq > 0) {
      PROF("phase_tables", phase_mixed(ctx, L, ka, r_dev));
      PROF("ewald_sk", sk_mixed(ctx, L, ka, measure));
      PROF("ewald_kforce", kf_mixed(ctx, L, ka));
    }
  } else {
    PROF("gather", k_gather_fp64(L, ns, r_dev, ctx->d_order, ctx->d_kind, ctx->d_mol, ctx->L[0],
                                 ctx->L[1], ctx->L[2], ctx->d_pd));
    if (ctx->polar) PROF("gather", k_gather_drude(L, ns, r_dev, ctx->d_order, nullptr, ctx->d_pdd));
    if (ctx->use_list) {
      if (rebuild) {
        // the fixed-point records came with the cell list
        int rc = build_lists(ctx, r_dev);
        if (rc) return rc;
        la = list_args(ctx);
      }
      PROF("pair_fp64", k_pair_list_fp64(L, pa, la, ctx->d_pd, ctx->d_ptabd, ctx->d_ert, measure,
                                         ctx->polar));
      nerows = list_blocks(ns, false);
    } else {
      PROF("pair_fp64", k_pair_fp64(L, pa, ctx->d_pd, ctx->d_ptabd, ctx->d_ert, measure,
                                    ctx->polar));
    }
    if (ctx->nq > 0) {
      PROF("phase_tables", k_phase_tables_fp64(L, ka, r_dev, (double2*)ctx->d_tab));
      PROF("ewald_sk", k_sk_gemm_fp64(L, ka, (const double2*)ctx->d_tab, (double2*)ctx->d_part));
      PROF("ewald_sk_reduce", k_sk_reduce_fp64(L, ka, (const double2*)ctx->d_part, measure));
      PROF("ewald_kforce", k_kf_gemm_fp64(L, ka, (const double2*)ctx->d_tab));
    }
  }
  // the dipole term (finite epsinf or Yeh-Berkowitz), after the k-space forces
  if (ctx->dipole && ctx->nq > 0)
    PROF("ewald_dipole", k_dipole(L, ka, r_dev, ctx->d_dippart, ctx->d_sums + 45, ctx->dipc,
                                  f_dev));
  ctx->have_cells = true;
  if (measure) {
    PROF("reduce", k_reduce_sum(L, ctx->d_epart, nerows, 10, ctx->d_sums));
    if (ctx->nq > 0) PROF("reduce", k_reduce_sum(L, ctx->d_ekpart, ctx->nkblocks, 7, ctx->d_sums + 10));
  }
  return MG_OK;
}

DrudeArgs drude_args(mg_ctx* ctx) {
  DrudeArgs d;
  d.nd = ctx->nd;
  d.ns = ctx->ns;
  d.dsite = ctx->d_dsite;
  d.qc = ctx->d_qc;
  d.qp = ctx->d_qp;
  d.aqq = ctx->d_aqq;
  d.alpha = ctx->alpha;
  d.part = ctx->d_drpart;
  d.minqq2 = ctx->minqq * ctx->minqq;
  d.status = ctx->d_status;
  return d;
}

// one SCF iteration on the device arrays r, f; with measure its energy
// partials are reduced into d_sums[20..27] (el, 2*self, Pvir)
int selffield_async(mg_ctx* ctx, double* r, double* f, double omega, bool measure,
                    double* hist_out) {
  Launch L = launch(ctx);
  DrudeArgs d = drude_args(ctx);
  PROF("drude_scf", k_selffield(L, d, omega, r, f, hist_out));
  if (measure) PROF("reduce", k_reduce_sum(L, ctx->d_drpart, ctx->ndblocks, 8, ctx->d_sums + 20));
  return MG_OK;
}

void add_drude_energy(mg_ctx* ctx, mg_energy* en) {
  const double* s = ctx->h_sums;
  en->el += s[20];
  en->self = s[21] / 2;
  for (int m = 0; m < 6; m++) en->Pvir[m] += s[22 + m];
}

// the dipole term's energy from the reduced moment M (h_sums[45..47]) and,
// with Pv != NULL, its virial tensor added to Pv (sim/ewald.c:888-890: Edip on
// the diagonal; the ADDFORCES terms q ek R of sim/ewaldf.c summed over the
// charges give ek_a M_b)
double dipole_energy(mg_ctx* ctx, double* Pv) {
  if (!ctx->dipole) return 0;
  const double* M = ctx->h_sums + 45;
  double E = 0, ek[3];
  for (int d = 0; d < 3; d++) {
    E += ctx->dipe[d] * M[d] * M[d];
    ek[d] = -ctx->dipc[d] * M[d];
  }
  if (Pv) {
    for (int d = 0; d < 3; d++) Pv[d] += E + ek[d] * M[d];
    Pv[3] += ek[1] * M[2];
    Pv[4] += ek[2] * M[0];
    Pv[5] += ek[0] * M[1];
  }
  return E;
}

// energies from the reduced sums (host, after the stream has been synchronized)
void fill_energy(mg_ctx* ctx, mg_energy* en) {
  const double* s = ctx->h_sums;
  std::memset(en, 0, sizeof(*en));
  double Ek = ctx->nq > 0 ? s[10] / (4 * M_PI) : 0;
  en->er = s[0];
  en->lj = s[1];
  en->vir = s[2];
  en->ek = Ek;
  en->eself = ctx->eself;
  en->edip = 0;
  en->el = s[0] + Ek + ctx->eself;
  for (int m = 0; m < 6; m++) en->Pvir[m] = s[3 + m];
  if (ctx->nq > 0) {
    for (int m = 0; m < 3; m++) en->Pvir[m] += Ek;
    for (int m = 0; m < 6; m++) en->Pvir[m] -= 2 / (4 * M_PI) * s[11 + m];
    en->edip = dipole_energy(ctx, en->Pvir);
    en->el += en->edip;
  }
}

// after a measured SHAKE step (energies and ekin already filled): cook's
// measurePconstraints (sim/constrd.c:115-265) with the constraint virial of
// the sweeps divided by h^2 (sim/constrd.c:1038-1040), the VERLET=3 kinetic
// tensor scaled by 1/(2 h^2) (sim/constrd.c:1012-1017), No.Pkinq = 1 (cook's
// corr without bit 4): Pvir = (force virial + constraint virial)/V,
// Pkin = kinetic tensor/V, Ptens = Pvir + Pkin, and the pressure from the
// scalar virial En.vir + En.virc + En.el (- 2 En.self with Drude charges),
// cook's Pevir
void fill_pressure(mg_ctx* ctx, mg_energy* en) {
  const double* s = ctx->h_sums + 32;
  const double hh = ctx->h * ctx->h, V = ctx->L[0] * ctx->L[1] * ctx->L[2];
  en->virc = s[0] / hh;
  for (int m = 0; m < 6; m++) {
    en->Pkin[m] = s[7 + m] * (0.5 / hh) / V;
    en->Ptens[m] = (en->Pvir[m] + s[1 + m] / hh) / V + en->Pkin[m];
  }
  const double vir = en->vir + en->virc + en->el - 2 * en->self;
  en->P = (2 * en->ekin + vir) / (3 * V);
}

ShakeArgs shake_args(mg_ctx* ctx, bool measure) {
  ShakeArgs sa;
  sa.meas_part = measure ? ctx->d_meas : nullptr;
  sa.nmol = ctx->nmol;
  sa.mol_first = ctx->d_mol_first;
  sa.mol_cfirst = ctx->d_mol_cfirst;
  sa.cons = ctx->d_cons;
  sa.bondq = ctx->d_bondq;
  sa.imass = ctx->d_imass;
  sa.mass = ctx->d_mass;
  sa.hh = ctx->h * ctx->h;
  sa.eps = ctx->epsc;
  sa.omega = ctx->omega;
  sa.maxit = ctx->shake_maxit;
  sa.ffsweep = ctx->precision == MG_MIXED ? 1 : 0;
  sa.r = ctx->d_r;
  sa.r1 = ctx->d_r1;
  sa.f = ctx->d_f;
  sa.p = ctx->d_p;
  sa.kin_part = ctx->d_kinpart;
  sa.status = ctx->d_status;
  sa.normalize = ctx->normalize;
  sa.r0 = ctx->box_r0;
  for (int d = 0; d < 3; d++) sa.Lb[d] = ctx->L[d];
  sa.nh = ctx->d_nh;
  sa.vhist = ctx->thermostat == 3 ? ctx->d_vhist : nullptr;
  sa.nh_pred = ctx->nose_pred;
  sa.nstride = 3LL * ctx->ns;
  return sa;
}

DependArgs depend_args(mg_ctx* ctx, bool measure = false) {
  DependArgs a;
  a.ndep = ctx->ndep;
  a.site = ctx->d_dep_site;
  a.first = ctx->d_dep_first;
  a.parent = ctx->d_dep_parent;
  a.w = ctx->d_dep_w;
  a.mol = ctx->d_mol;
  a.type = ctx->d_dep_type;
  a.par = ctx->d_dep_par;
  a.vpart = measure ? ctx->d_deppart : nullptr;
  return a;
}

// the dependants' forces onto their parents; on a measured step with
// Rowlinson or Lone dependants also their virial and tensor terms, summed
// into d_sums + 48 (scalar) and + 49 (xx yy zz yz zx xy)
cudaError_t depend_f_enqueue(mg_ctx* ctx, const Launch& L, bool measure) {
  const DependArgs a = depend_args(ctx, measure);
  cudaError_t e = k_depend_f(L, a, ctx->d_r, ctx->d_f);
  if (e == cudaSuccess && a.vpart) e = k_reduce_sum(L, a.vpart, a.ndep, 7, ctx->d_sums + 48);
  return e;
}

// cook adds those terms to En.vir and En.Pvir (sim/norm.c:1335-1338,
// 1363-1368) after the force evaluation; a measured MD step's energies carry
// them
void add_depend_virial(mg_ctx* ctx, mg_energy* en) {
  if (!ctx->d_deppart) return;
  const double* s = ctx->h_sums + 48;
  en->vir += s[0];
  for (int m = 0; m < 6; m++) en->Pvir[m] += s[1 + m];
}

ThermoArgs thermo_args(mg_ctx* ctx) {
  ThermoArgs t;
  t.kind = ctx->thermostat;
  t.ns = ctx->ns;
  t.nkin = (ctx->nmol + 127) / 128;
  t.nchi = ctx->nchi;
  t.nf = ctx->thermo_f;
  t.T = ctx->T;
  t.tau = ctx->tau_T;
  t.h = ctx->h;
  t.seed = ctx->seed;
  t.step = ctx->d_step;
  t.zout = ctx->d_zth;
  t.nh = ctx->d_nh;
  t.pred = ctx->nose_pred;
  return t;
}

// one leap-frog + SHAKE step of a non-polar box with cells re-binned at the
// force evaluation: kernels only, no host synchronisation (graph capture)
int md_step_enqueue(mg_ctx* ctx, bool measure) {
  Launch L = launch(ctx);
  int rc = forces_async(ctx, ctx->d_r, ctx->d_f, measure);
  if (rc) return rc;
  CK(depend_f_enqueue(ctx, L, measure));
  CK(k_shake(L, shake_args(ctx, measure)));
  CK(k_depend_r(L, depend_args(ctx), ctx->d_r));
  if (measure) {
    CK(k_reduce_sum(L, ctx->d_kinpart, (ctx->nmol + 127) / 128, 1, ctx->d_sums + 17));
    CK(k_reduce_sum(L, ctx->d_meas, (ctx->nmol + 127) / 128, 13, ctx->d_sums + 32));
  }
  if (ctx->thermostat)
    CK(k_thermostat(L, thermo_args(ctx), ctx->d_kinpart, ctx->d_chi, ctx->d_r1));
  if (ctx->drmax > 0) CK(k_bounddr(L, ctx->ns, ctx->drmax, ctx->d_r1, ctx->d_bdrep));
  if (ctx->drift_step)
    CK(k_remove_drift(L, ctx->ns, ctx->d_mass, ctx->total_mass, ctx->d_r1, ctx->d_driftpart,
                      ctx->d_drift, nullptr));
  return MG_OK;
}

int fetch_sums(mg_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->h_sums, ctx->d_sums, NSUMS * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  return MG_OK;
}

// device status word: bit 0 SHAKE did not converge, bit 1 non-finite position.
// Copied into the pinned block behind the sums; read after the stream sync.
int fetch_status(mg_ctx* ctx) {
  CK(cudaMemcpyAsync(ctx->h_sums + 31, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost,
                     ctx->stream));
  return MG_OK;
}

int check_status(mg_ctx* ctx) {
  int st;
  std::memcpy(&st, ctx->h_sums + 31, sizeof(int));
  if (!st) return MG_OK;
  CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (st & 2) return fail(ctx, MG_ERR_NONFINITE, "non-finite site position");
  if (st & 4) return fail(ctx, MG_ERR_SCF, "Drude displacement beyond el.minqq");
  if (st & 16)
    return fail(ctx, MG_ERR_CUDA, "a tensor-core Ewald pass gave up waiting for its operands");
  if (st & 8)
    return fail(ctx, MG_ERR_LIST,
                "a site moved more than skin/2 between neighbour-list builds (larger skin or "
                "smaller nl_every)");
  return fail(ctx, MG_ERR_SHAKE, "SHAKE: too many iterations");
}

// the steps kernel by kernel (Drude boxes, neighbour lists, profiling)
int md_steps_launched(mg_ctx* ctx, int nsteps, mg_energy* en) {
  Launch L = launch(ctx);
  const int nkin = (ctx->nmol + 127) / 128;
  for (int s = 0; s < nsteps; s++) {
    const bool last = s == nsteps - 1;
    const bool measure = last && en != nullptr;
    if (ctx->use_list && ctx->dmax_pending) {
      // the previous step's largest displacement since the build: rebuild
      // once half of the skin/2 budget is used (one more step cannot spend
      // the other half at any physical speed)
      CK(cudaEventSynchronize(ctx->ev_dmax));
      ctx->dmax_pending = false;
      float d2;
      std::memcpy(&d2, ctx->h_dmax, sizeof(float));
      if (d2 > 0.0625 * ctx->skin * ctx->skin) ctx->need_build = true;
    }
    if (ctx->polar && ctx->nd > 0) {
      // ASPC predictor, then scf_iter force evaluations each followed by one
      // SCF iteration (sim/constrd.c:726-736, sim/pred2.c:56-97)
      const int K2 = ctx->aspc_k + 2;
      const size_t slot = 3 * (size_t)ctx->nd;
      AspcCoef B;
      double om;
      aspc_coefficients(ctx->aspc_kk, B.b, &om);
      B.n = ctx->aspc_kk + 2;
      DrudeArgs d = drude_args(ctx);
      PROF("drude_aspc", k_aspc_predict(L, d, ctx->d_hist, K2, ctx->hist_h, B, ctx->d_r));
      if (ctx->aspc_kk < ctx->aspc_k) {
        ctx->aspc_kk++;
        aspc_coefficients(ctx->aspc_kk, B.b, &om);
        ctx->cur_omega = om;
      }
      const int hn = (ctx->hist_h + 1) % K2;
      for (int it = 0; it < ctx->scf_iter; it++) {
        const bool lastit = it == ctx->scf_iter - 1;
        int rc = forces_async(ctx, ctx->d_r, ctx->d_f, measure && lastit);
        if (rc) return rc;
        rc = selffield_async(ctx, ctx->d_r, ctx->d_f, ctx->cur_omega, measure && lastit,
                             lastit ? ctx->d_hist + slot * hn : nullptr);
        if (rc) return rc;
      }
      ctx->hist_h = hn;
    } else {
      int rc = forces_async(ctx, ctx->d_r, ctx->d_f, measure);
      if (rc) return rc;
    }
    // forces on dependants to their parents (sim/constrd.c:747), the step,
    // and dependant positions for the next force evaluation: the same
    // positions cook's depend_r makes at the start of its next step
    if (ctx->ndep > 0) PROF("depend", depend_f_enqueue(ctx, L, measure));
    PROF("shake", k_shake(L, shake_args(ctx, measure)));
    if (ctx->ndep > 0) PROF("depend", k_depend_r(L, depend_args(ctx), ctx->d_r));
    if (ctx->use_list) {
      ctx->since_build++;
      PROF("neighbour_list", k_check_skin(L, ctx->ns, ctx->d_r, ctx->d_rbuild,
                                          0.25 * ctx->skin * ctx->skin, ctx->L, ctx->d_status,
                                          ctx->d_dmax));
      CK(cudaMemcpyAsync(ctx->h_dmax, ctx->d_dmax, sizeof(int), cudaMemcpyDeviceToHost,
                         ctx->stream));
      CK(cudaEventRecord(ctx->ev_dmax, ctx->stream));
      ctx->dmax_pending = true;
    }
    if (measure) {
      PROF("reduce", k_reduce_sum(L, ctx->d_kinpart, nkin, 1, ctx->d_sums + 17));
      PROF("reduce", k_reduce_sum(L, ctx->d_meas, nkin, 13, ctx->d_sums + 32));
    }
    if (ctx->thermostat)
      PROF("thermostat", k_thermostat(L, thermo_args(ctx), ctx->d_kinpart, ctx->d_chi, ctx->d_r1));
    // cook calls bounddr after Shake (and its thermostat) and normalize
    // (sim/main.c:1607-1623)
    if (ctx->drmax > 0)
      PROF("bounddr", k_bounddr(L, ctx->ns, ctx->drmax, ctx->d_r1, ctx->d_bdrep));
    // then the momentum drift (cook's removedrifts with DRIFT_STEP,
    // sim/main.c:1626)
    if (ctx->drift_step)
      PROF("drift", k_remove_drift(L, ctx->ns, ctx->d_mass, ctx->total_mass, ctx->d_r1,
                                   ctx->d_driftpart, ctx->d_drift, nullptr));
  }
  return MG_OK;
}

void drop_graphs(mg_ctx* ctx) {
  if (ctx->g_step) cudaGraphExecDestroy(ctx->g_step);
  if (ctx->g_meas) cudaGraphExecDestroy(ctx->g_meas);
  ctx->g_step = ctx->g_meas = nullptr;
}

// steps that md_step_enqueue covers (no Drude SCF, cells re-binned every
// step) and that nothing times kernel by kernel run as a captured graph
bool graph_step_ok(const mg_ctx* ctx) {
  return ctx->use_graph && !ctx->polar && !ctx->use_list && !ctx->prof_on;
}

// capture one step on the context's own stream (a caller's stream may be
// the legacy default stream, which cannot capture); the graph is launched
// on whatever stream the context runs on
int capture_md_step(mg_ctx* ctx, bool measure, cudaGraphExec_t* out) {
  cudaStream_t keep = ctx->stream;
  CK(cudaStreamSynchronize(keep));
  ctx->stream = ctx->own_stream;
  const int l0 = ctx->launches;
  cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) {
    ctx->stream = keep;
    return fail(ctx, MG_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  }
  int rc = md_step_enqueue(ctx, measure);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(ctx->stream, &g);
  ctx->stream = keep;
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return fail(ctx, MG_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess)
    return fail(ctx, MG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  (measure ? ctx->graph_launches_meas : ctx->graph_launches) = ctx->launches - l0;
  ctx->launches = l0;
  return MG_OK;
}

}  // namespace

extern "C" {

mg_ctx* mg_create(const mg_topology* top, const mg_params* par, int* status) {
  mg_ctx* ctx = new mg_ctx();
  int rc = setup(ctx, top, par);
  if (rc == MG_OK) rc = tc_upload_slots(ctx);
  if (rc != MG_OK) {
    fprintf(stderr, "mg_create: %s\n", ctx->err.c_str());
    mg_destroy(ctx);
    if (status) *status = rc;
    return nullptr;
  }
  if (status) *status = MG_OK;
  return ctx;
}

int mg_destroy(mg_ctx* ctx) {
  if (!ctx) return MG_OK;
  void* bufs[] = {ctx->d_rs, ctx->d_fs, ctx->d_r,      ctx->d_f,       ctx->d_r1,    ctx->d_p,      ctx->d_kind,
                  ctx->d_mol,    ctx->d_key,     ctx->d_pfix,   ctx->d_idx,   ctx->d_key_s,  ctx->d_order,
                  ctx->d_cell_start, ctx->d_ccount, ctx->d_ccursor, ctx->d_spans, ctx->d_gstart,
                  ctx->d_hspans, ctx->d_facc, ctx->d_tcb,
                  ctx->d_gcell, ctx->d_pj, ctx->d_pd,  ctx->d_stencil,
                  ctx->d_ptabf,  ctx->d_ptabd,   ctx->d_erd,   ctx->d_eru,    ctx->d_ert,
                  ctx->d_epart,  ctx->d_qsite,   ctx->d_qval,  ctx->d_task,   ctx->d_col,
                  ctx->d_kvec,   ctx->d_ekk,     ctx->d_S,     ctx->d_Wf,     ctx->d_Wd,
                  ctx->d_tab,    ctx->d_part,    ctx->d_ekpart, ctx->d_mol_first,
                  ctx->d_mol_cfirst, ctx->d_cons, ctx->d_bondq, ctx->d_imass, ctx->d_mass,
                  ctx->d_kinpart, ctx->d_meas, ctx->d_dippart, ctx->d_bdrep, ctx->d_driftpart,
                  ctx->d_drift, ctx->d_status, ctx->d_sums, ctx->d_krows,
                  ctx->d_tiles, ctx->d_p1job, ctx->d_dsite, ctx->d_qdrude, ctx->d_qc,
                  ctx->d_qp, ctx->d_aqq, ctx->d_hist, ctx->d_drpart, ctx->d_pdj, ctx->d_pdd,
                  ctx->d_nlist, ctx->d_ncount, ctx->d_rbuild, ctx->d_dmax,
                  ctx->d_wtabf, ctx->d_wtabd, ctx->d_wgeom, ctx->d_wpart, ctx->d_wbox,
                  ctx->d_qfix, ctx->d_adjtab, ctx->d_ag, ctx->d_aq, ctx->d_apart, ctx->d_adEq,
                  ctx->d_adLq, ctx->d_ags, ctx->d_atpart, ctx->d_aT, ctx->d_fk,
                  ctx->d_chi, ctx->d_zth, ctx->d_step, ctx->d_nh, ctx->d_vhist, ctx->d_dep_site, ctx->d_dep_first,
                  ctx->d_dep_parent, ctx->d_dep_w, ctx->d_dep_type, ctx->d_dep_par, ctx->d_deppart, ctx->d_plb, ctx->d_xfirst, ctx->d_xpair,
                  ctx->d_xq, ctx->d_za, ctx->d_vb, ctx->d_tcrows, ctx->d_zb, ctx->d_tckrows};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (ctx->h_sums) cudaFreeHost(ctx->h_sums);
  if (ctx->h_dmax) cudaFreeHost(ctx->h_dmax);
  if (ctx->ev_dmax) cudaEventDestroy(ctx->ev_dmax);
  for (cudaEvent_t e : ctx->evpool) cudaEventDestroy(e);
  if (ctx->g_step) cudaGraphExecDestroy(ctx->g_step);
  if (ctx->g_meas) cudaGraphExecDestroy(ctx->g_meas);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  if (ctx->kstream) cudaStreamDestroy(ctx->kstream);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  delete ctx;
  return MG_OK;
}

const char* mg_last_error(const mg_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }
double mg_kappa(const mg_ctx* ctx) { return ctx ? ctx->kappa : 0; }
int mg_nkvec(const mg_ctx* ctx) { return ctx ? ctx->nk : 0; }
int mg_last_launches(const mg_ctx* ctx) { return ctx ? ctx->launches : 0; }

int mg_forces_device(mg_ctx* ctx, const double* r_dev, double* f_dev, int measure,
                     mg_energy* en) {
  if (!ctx || !r_dev || !f_dev) return fail(ctx, MG_ERR_ARG, "null argument");
  ctx->launches = 0;
  ctx->need_build = true;
  int rc = forces_async(ctx, r_dev, f_dev, measure != 0);
  if (rc) return rc;
  if (measure) {
    rc = fetch_sums(ctx);
    if (rc) return rc;
  }
  rc = fetch_status(ctx);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  prof_resolve(ctx);
  rc = check_status(ctx);
  if (rc) return rc;
  ctx->need_build = true;  // the lists now describe these positions, not the MD state
  if (measure && en) fill_energy(ctx, en);
  return MG_OK;
}

int mg_forces(mg_ctx* ctx, const double* r, double* f, int measure, mg_energy* en) {
  if (!ctx || !r || !f) return fail(ctx, MG_ERR_ARG, "null argument");
  ctx->launches = 0;
  ctx->need_build = true;
  const size_t nb = 3 * (size_t)ctx->ns * (ctx->polar ? 2 : 1) * sizeof(double);
  CK(cudaMemcpyAsync(ctx->d_rs, r, nb, cudaMemcpyHostToDevice, ctx->stream));
  int rc = forces_async(ctx, ctx->d_rs, ctx->d_fs, measure != 0);
  if (rc) return rc;
  CK(cudaMemcpyAsync(f, ctx->d_fs, nb, cudaMemcpyDeviceToHost, ctx->stream));
  if (measure) {
    rc = fetch_sums(ctx);
    if (rc) return rc;
  }
  rc = fetch_status(ctx);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  prof_resolve(ctx);
  rc = check_status(ctx);
  if (rc) return rc;
  ctx->need_build = true;  // the lists now describe these positions, not the MD state
  if (measure && en) fill_energy(ctx, en);
  return MG_OK;
}

int mg_ewald(mg_ctx* ctx, const double* r, double* f, double* energy) {
  if (!ctx || !r || !f) return fail(ctx, MG_ERR_ARG, "null argument");
  // full forces minus the r-space part is not separable cheaply here: run
  // the k-space kernels alone on a zeroed force buffer
  ctx->launches = 0;
  const size_t nb = 3 * (size_t)ctx->ns * (ctx->polar ? 2 : 1) * sizeof(double);
  Launch L = launch(ctx);
  CK(cudaMemcpyAsync(ctx->d_rs, r, nb, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemsetAsync(ctx->d_fs, 0, nb, ctx->stream));
  KArgs ka;
  std::memset(&ka, 0, sizeof(ka));
  ka.nq = ctx->nq;
  ka.nk = ctx->nk;
  ka.ntask = ctx->ntask;
  ka.ncol = ctx->ncol;
  ka.nchunk = ctx->nchunk;
  ka.Kx = ctx->Kx;
  ka.Ky = ctx->Ky;
  ka.Kz = ctx->Kz;
  ka.row = ctx->row;
  set_box(ka, ctx->L);
  ka.alpha = ctx->alpha;
  ka.qsite = ctx->d_qsite;
  ka.qval = ctx->d_qval;
  ka.task = ctx->d_task;
  ka.col = ctx->d_col;
  ka.kvec = ctx->d_kvec;
  ka.ekk = ctx->d_ekk;
  ka.S = ctx->d_S;
  ka.Wf = ctx->d_Wf;
  ka.Wd = ctx->d_Wd;
  ka.f = ctx->d_fs;
  ka.ek_part = ctx->d_ekpart;
  ka.krows = ctx->d_krows;
  ka.tiles = ctx->d_tiles;
  ka.ntile = ctx->ntile;
  ka.p1job = ctx->d_p1job;
  ka.np1job = ctx->np1job;
  ka.qdrude = ctx->d_qdrude;
  ka.ns = ctx->ns;
  ka.status = ctx->d_status;
  if (ctx->nq > 0) {
    if (ctx->precision == MG_MIXED) {
      CK(phase_mixed(ctx, L, ka, ctx->d_rs));
      CK(sk_mixed(ctx, L, ka, true));
      CK(kf_mixed(ctx, L, ka));
    } else {
      CK(k_phase_tables_fp64(L, ka, ctx->d_rs, (double2*)ctx->d_tab));
      CK(k_sk_gemm_fp64(L, ka, (const double2*)ctx->d_tab, (double2*)ctx->d_part));
      CK(k_sk_reduce_fp64(L, ka, (const double2*)ctx->d_part, true));
      CK(k_kf_gemm_fp64(L, ka, (const double2*)ctx->d_tab));
    }
    CK(k_reduce_sum(L, ctx->d_ekpart, ctx->nkblocks, 7, ctx->d_sums + 10));
    if (ctx->dipole)
      CK(k_dipole(L, ka, ctx->d_rs, ctx->d_dippart, ctx->d_sums + 45, ctx->dipc, ctx->d_fs));
  }
  std::vector<double> fk(nb / sizeof(double));
  CK(cudaMemcpyAsync(fk.data(), ctx->d_fs, nb, cudaMemcpyDeviceToHost, ctx->stream));
  int rc = fetch_sums(ctx);
  if (rc) return rc;
  rc = fetch_status(ctx);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  rc = check_status(ctx);
  if (rc) return rc;
  for (size_t i = 0; i < fk.size(); i++) f[i] += fk[i];
  if (energy)
    *energy = (ctx->nq > 0 ? ctx->h_sums[10] / (4 * M_PI) + dipole_energy(ctx, nullptr) : 0) +
              ctx->eself;
  return MG_OK;
}

int mg_md_set_state(mg_ctx* ctx, const double* r, const double* r1) {
  if (!ctx || !r || !r1) return fail(ctx, MG_ERR_ARG, "null argument");
  const size_t nb = 3 * (size_t)ctx->ns * (ctx->polar ? 2 : 1) * sizeof(double);
  CK(cudaMemcpyAsync(ctx->d_r, r, nb, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_r1, r1, nb, cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->ndep > 0) {
    // dependant positions from their parents, as cook's depend_r before the
    // first force evaluation (sim/constrd.c:722)
    Launch L = launch(ctx);
    CK(k_depend_r(L, depend_args(ctx), ctx->d_r));
  }
  if (ctx->polar && ctx->nd > 0) {
    // ASPC history as cook starts it (sim/pred2.c:45-55): the latest slot is
    // rpol(t) from r, the previous one rpol(t-h) from r1, older slots zero
    Launch L = launch(ctx);
    DrudeArgs d = drude_args(ctx);
    const int K2 = ctx->aspc_k + 2;
    const size_t slot = 3 * (size_t)ctx->nd;
    CK(cudaMemsetAsync(ctx->d_hist, 0, sizeof(double) * slot * K2, ctx->stream));
    CK(k_drude_take(L, d, ctx->d_r, ctx->d_hist));
    CK(k_drude_take(L, d, ctx->d_r1, ctx->d_hist + slot * (K2 - 1)));
    ctx->hist_h = 0;
    ctx->aspc_kk = 0;
    ctx->cur_omega = ctx->scf_omega;
  }
  if (ctx->thermostat == 3) {
    // Nose-Hoover from logs = 0 and h dlogs/dt = 0 with no predictor
    // history (cook's k = 0 at the first step, sim/trvpscale.c:28)
    CK(cudaMemsetAsync(ctx->d_nh, 0, sizeof(double) * (NH_HIST + MG_NOSE_MAXPRED),
                       ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->have_state = true;
  ctx->need_build = true;
  return MG_OK;
}

int mg_md_get_state(mg_ctx* ctx, double* r, double* r1) {
  if (!ctx || !ctx->have_state) return fail(ctx, MG_ERR_ARG, "no MD state");
  const size_t nb = 3 * (size_t)ctx->ns * (ctx->polar ? 2 : 1) * sizeof(double);
  if (ctx->polar && ctx->nd > 0) {
    // cook keeps rpol(t-h) in cfg[1]'s polar half: the previous corrected
    // shells, so that a get/set round trip restarts ASPC from them
    Launch L = launch(ctx);
    DrudeArgs d = drude_args(ctx);
    const int K2 = ctx->aspc_k + 2;
    const size_t slot = 3 * (size_t)ctx->nd;
    CK(k_drude_put(L, d, ctx->d_hist + slot * ((ctx->hist_h - 1 + K2) % K2), ctx->d_r1));
  }
  if (r) CK(cudaMemcpyAsync(r, ctx->d_r, nb, cudaMemcpyDeviceToHost, ctx->stream));
  if (r1) CK(cudaMemcpyAsync(r1, ctx->d_r1, nb, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return MG_OK;
}

int mg_remove_drift(mg_ctx* ctx, double vdrift[3]) {
  if (!ctx || !ctx->have_state) return fail(ctx, MG_ERR_ARG, "no MD state");
  Launch L = launch(ctx);
  CK(k_remove_drift(L, ctx->ns, ctx->d_mass, ctx->total_mass, ctx->d_r1, ctx->d_driftpart,
                    ctx->d_drift, ctx->d_drift + 3));
  double v[3];
  CK(cudaMemcpyAsync(v, ctx->d_drift + 3, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (vdrift)
    for (int d = 0; d < 3; d++) vdrift[d] = v[d] / ctx->h;
  return MG_OK;
}

int mg_bounddr_report(mg_ctx* ctx, long long* nreduced, double* minfactor) {
  if (!ctx) return MG_ERR_ARG;
  unsigned int rep[2] = {0u, 0x3f800000u};
  if (ctx->d_bdrep) {
    CK(cudaMemcpyAsync(rep, ctx->d_bdrep, sizeof(rep), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const unsigned int rep0[2] = {0u, 0x3f800000u};
    CK(cudaMemcpyAsync(ctx->d_bdrep, rep0, sizeof(rep0), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  float q;
  std::memcpy(&q, rep + 1, sizeof(q));
  if (nreduced) *nreduced = rep[0];
  if (minfactor) *minfactor = q;
  return MG_OK;
}

int mg_playback_frame(mg_ctx* ctx, int what, int flags, float* frame) {
  if (!ctx || !frame) return fail(ctx, MG_ERR_ARG, "null argument");
  if (!ctx->have_state) return fail(ctx, MG_ERR_ARG, "no MD state");
  if (what < MG_PLB_POS || what > MG_PLB_DRUDE || (flags & ~6))
    return fail(ctx, MG_ERR_ARG, "what: MG_PLB_POS/VEL/DRUDE; flags: bits 2 and 4");
  if (what == MG_PLB_DRUDE && !ctx->polar)
    return fail(ctx, MG_ERR_ARG, "Drude playback of a build without Drude charges");
  if (!ctx->d_plb) CK(dalloc(&ctx->d_plb, 3 * (size_t)ctx->ns));
  Launch L = launch(ctx);
  CK(k_playback_frame(L, ctx->ns, what, flags, ctx->d_r, ctx->d_r1, 1. / ctx->h, ctx->L,
                      ctx->d_plb));
  for (int d = 0; d < 3; d++) frame[d] = (float)ctx->L[d];
  CK(cudaMemcpyAsync(frame + 3, ctx->d_plb, 3 * sizeof(float) * (size_t)ctx->ns,
                     cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return MG_OK;
}

int mg_md_steps(mg_ctx* ctx, int nsteps, mg_energy* en) {
  if (!ctx || !ctx->have_state || nsteps < 0) return fail(ctx, MG_ERR_ARG, "no MD state");
  ctx->launches = 0;
  if (graph_step_ok(ctx)) {
    // the step as one captured graph per kind (force-only, measured)
    for (int s = 0; s < nsteps; s++) {
      const bool measure = s == nsteps - 1 && en != nullptr;
      cudaGraphExec_t& g = measure ? ctx->g_meas : ctx->g_step;
      if (!g) {
        int rc = capture_md_step(ctx, measure, &g);
        if (rc) return rc;
      }
      CK(cudaGraphLaunch(g, ctx->stream));
      ctx->launches += measure ? ctx->graph_launches_meas : ctx->graph_launches;
    }
    if (nsteps > 0) {
      // what the captured force evaluation leaves behind, as a launched one
      ctx->last_r = ctx->d_r;
      ctx->have_cells = true;
    }
  } else {
    int rc = md_steps_launched(ctx, nsteps, en);
    if (rc) return rc;
  }
  if (en) {
    int rc = fetch_sums(ctx);
    if (rc) return rc;
  }
  int rc = fetch_status(ctx);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  prof_resolve(ctx);
  rc = check_status(ctx);
  if (rc) return rc;
  if (en) {
    fill_energy(ctx, en);
    if (ctx->polar && ctx->nd > 0) add_drude_energy(ctx, en);
    add_depend_virial(ctx, en);
    en->ekin = ctx->h_sums[17] / (ctx->h * ctx->h) / 4;
    fill_pressure(ctx, en);
  }
  return MG_OK;
}

namespace {

// Widom set-up of one box: checks, the ghost-site x site-kind pair table and
// the ghost geometry uploaded (on the context's stream), the cutoff
// correction, and the launch descriptor
int widom_prepare(mg_ctx* ctx, const mg_probe* probe, long long ninsert, unsigned long long seed,
                  double T, double* d_U, WidomBox* box, double* corr_out) {
  if (!ctx || !probe) return fail(ctx, MG_ERR_ARG, "null argument");
  const int nps = probe->ns;
  if (nps < 1 || nps > MG_WIDOM_MAX_SITES || !probe->site_type || !probe->geometry)
    return fail(ctx, MG_ERR_ARG, "the ghost needs 1..8 sites with types and geometry");
  if (ninsert < 1 || !(T > 0)) return fail(ctx, MG_ERR_ARG, "ninsert >= 1 and T > 0 required");
  if (ctx->polar)
    return fail(ctx, MG_ERR_ARG, "Widom insertion into a Drude system is not supported");
  if (!ctx->have_cells)
    return fail(ctx, MG_ERR_ARG, "no cell list yet: evaluate forces first");
  const double Lmin = std::min(ctx->L[0], std::min(ctx->L[1], ctx->L[2]));
  for (int s = 0; s < nps; s++) {
    if (probe->site_type[s] < 0 || probe->site_type[s] >= ctx->ntypes)
      return fail(ctx, MG_ERR_ARG, "ghost site type out of range");
    const double* g = probe->geometry + 3 * s;
    if (!(std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) < Lmin / 4))
      return fail(ctx, MG_ERR_ARG, "ghost geometry larger than a quarter of the box");
  }
  // pair constants of every ghost site with every site kind of the box, and
  // the cutoff correction over all (ghost site, box site) pairs
  std::vector<PairF>& tf = ctx->h_wtabf;
  std::vector<PairD>& td = ctx->h_wtabd;
  tf.assign(MAX_WPROBE * MAX_KINDS, PairF{});
  td.assign(MAX_WPROBE * MAX_KINDS, PairD{});
  double corr = 0;
  for (int s = 0; s < nps; s++) {
    const int ta = probe->site_type[s];
    const double qs = probe->charge ? probe->charge[s] : 0.0;
    for (int tb = 0; tb < ctx->ntypes; tb++) {
      if (!ctx->type_count[tb]) continue;
      double eps, sig;
      PairLJ P;
      combining_rule(ctx->h_tE[ta], ctx->h_tR[ta], ctx->h_tA[ta], ctx->h_tE[tb], ctx->h_tR[tb],
                     ctx->h_tA[tb], ctx->comb_rule, &eps, &sig);
      if (smooth_lj(eps, sig, ctx->C2, &P))
        return fail(ctx, MG_ERR_SETUP, "smooth LJ cutoff cannot be determined");
      corr += ctx->type_count[tb] * lj_tail_correction(eps, sig, P);
    }
    for (int b = 0; b < ctx->nkind; b++) {
      const int tb = ctx->kind_type[b];
      double eps, sig;
      PairLJ P;
      combining_rule(ctx->h_tE[ta], ctx->h_tR[ta], ctx->h_tA[ta], ctx->h_tE[tb], ctx->h_tR[tb],
                     ctx->h_tA[tb], ctx->comb_rule, &eps, &sig);
      smooth_lj(eps, sig, ctx->C2, &P);
      const double qq = qs * ctx->kind_q[b];
      td[s * ctx->nkind + b] = PairD{P.C1q, P.C2q, P.A4, P.E24, P.Sq, qq, P.A, P.E4, 0, 0, 0, 0};
      tf[s * ctx->nkind + b] = PairF{(float)P.C1q, (float)P.C2q, (float)P.A4, (float)P.E24,
                                     (float)P.Sq,  (float)qq,    (float)P.A,  (float)P.E4,
                                     0.f, 0.f, 0.f, 0.f, qq, 0, 0, 0};
    }
  }
  if (!ctx->d_wgeom) {
    CK(dalloc(&ctx->d_wgeom, 3 * MAX_WPROBE));
    CK(dalloc(&ctx->d_wpart, PARTITION_SMS * 8));
    CK(dalloc(&ctx->d_wtabf, MAX_WPROBE * MAX_KINDS));
    CK(dalloc(&ctx->d_wtabd, MAX_WPROBE * MAX_KINDS));
    CK(dalloc(&ctx->d_wbox, 1));
  }
  ctx->h_wgeom.assign(probe->geometry, probe->geometry + 3 * nps);
  CK(cudaMemcpyAsync(ctx->d_wgeom, ctx->h_wgeom.data(), sizeof(double) * 3 * nps,
                     cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->precision == MG_MIXED)
    CK(cudaMemcpyAsync(ctx->d_wtabf, tf.data(), sizeof(PairF) * tf.size(), cudaMemcpyHostToDevice,
                       ctx->stream));
  else
    CK(cudaMemcpyAsync(ctx->d_wtabd, td.data(), sizeof(PairD) * td.size(), cudaMemcpyHostToDevice,
                       ctx->stream));
  WidomArgs& w = box->a;
  w.n = ninsert;
  w.seed = seed;
  w.T = T;
  w.nps = nps;
  w.nkind = ctx->nkind;
  w.ncx = ctx->ncx;
  w.ncy = ctx->ncy;
  w.ncz = ctx->ncz;
  w.nstencil = ctx->nstencil;
  w.lanes_sites = ctx->nstencil < 16 ? 1 : 0;
  w.ntab = ctx->ntab;
  w.cell_start = ctx->d_cell_start;
  w.stencil = ctx->d_stencil;
  w.Lx = ctx->L[0];
  w.Ly = ctx->L[1];
  w.Lz = ctx->L[2];
  w.cutoff_sq = ctx->cutoff * ctx->cutoff;
  w.sgrid = ctx->sgrid;
  w.geom = ctx->d_wgeom;
  w.U = d_U;
  w.part = ctx->d_wpart;
  box->pj = ctx->d_pj;
  box->pd = ctx->d_pd;
  box->tabf = ctx->d_wtabf;
  box->tabd = ctx->d_wtabd;
  box->eru = ctx->d_eru;
  box->ert = ctx->d_ert;
  *corr_out = corr;
  return MG_OK;
}

void widom_result(const mg_ctx* ctx, const double* part, int nblk, long long n, double T,
                  double corr, mg_widom_result* out) {
  double sum = 0;
  for (int b = 0; b < nblk; b++) sum += part[b];
  const double V = ctx->L[0] * ctx->L[1] * ctx->L[2];
  out->sum = sum;
  out->raw = sum / (double)n;
  out->corr = corr;
  out->factor = std::exp(-corr / (V * T));
  out->widom = out->raw * out->factor;
  out->mu = -T * std::log(out->widom);
}

}  // namespace

int mg_widom(mg_ctx* ctx, const mg_probe* probe, long long ninsert, unsigned long long seed,
             double T, mg_widom_result* out, double* U) {
  if (!ctx || !out) return fail(ctx, MG_ERR_ARG, "null argument");
  double* d_U = nullptr;
  if (U) CK(cudaMalloc((void**)&d_U, sizeof(double) * std::max(ninsert, 1LL)));
  WidomBox box;
  double corr = 0;
  int rc = widom_prepare(ctx, probe, ninsert, seed, T, d_U, &box, &corr);
  if (rc) {
    if (d_U) cudaFree(d_U);
    return rc;
  }
  const int nblk = widom_blocks(ninsert);
  CK(cudaMemcpyAsync(ctx->d_wbox, &box, sizeof(WidomBox), cudaMemcpyHostToDevice, ctx->stream));
  Launch L = launch(ctx);
  cudaError_t e = k_widom(L, ctx->d_wbox, 1, ninsert, ctx->precision != MG_MIXED);
  if (e != cudaSuccess) {
    if (d_U) cudaFree(d_U);
    return fail(ctx, MG_ERR_CUDA, std::string("widom: ") + cudaGetErrorString(e));
  }
  std::vector<double> part(nblk);
  CK(cudaMemcpyAsync(part.data(), ctx->d_wpart, sizeof(double) * nblk, cudaMemcpyDeviceToHost,
                     ctx->stream));
  if (U) CK(cudaMemcpyAsync(U, d_U, sizeof(double) * ninsert, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (d_U) CK(cudaFree(d_U));
  widom_result(ctx, part.data(), nblk, ninsert, T, corr, out);
  return MG_OK;
}

int mg_xwidom(mg_ctx* ctx, int nlist, const int* mols, const int* vtype, const double* vcharge,
              double T, mg_widom_result* out, double* dU) {
  if (!ctx || !mols || !vtype || !vcharge || !out) return fail(ctx, MG_ERR_ARG, "null argument");
  if (nlist < 1 || !(T > 0)) return fail(ctx, MG_ERR_ARG, "nlist >= 1 and T > 0 required");
  if (ctx->polar) return fail(ctx, MG_ERR_ARG, "identity change in a Drude system is not supported");
  if (!ctx->have_cells || !ctx->last_r)
    return fail(ctx, MG_ERR_ARG, "no cell list yet: evaluate forces first");
  if (ctx->use_list)
    return fail(ctx, MG_ERR_ARG, "identity change needs the cell path (skin <= 0)");
  // every listed molecule has the sites and site kinds of the first
  const std::vector<int>& mf = ctx->h_mol_first;
  for (int l = 0; l < nlist; l++)
    if (mols[l] < 0 || mols[l] >= ctx->nmol) return fail(ctx, MG_ERR_ARG, "molecule out of range");
  const int i0 = mf[mols[0]], nps = mf[mols[0] + 1] - i0;
  if (nps < 1 || nps > MAX_WPROBE) return fail(ctx, MG_ERR_ARG, "molecules of 1..8 sites");
  for (int l = 1; l < nlist; l++) {
    const int j0 = mf[mols[l]];
    if (mf[mols[l] + 1] - j0 != nps) return fail(ctx, MG_ERR_ARG, "molecules differ in sites");
    for (int s = 0; s < nps; s++)
      if (ctx->h_kind[j0 + s] != ctx->h_kind[i0 + s])
        return fail(ctx, MG_ERR_ARG, "molecules differ in site kinds");
  }
  for (int s = 0; s < nps; s++)
    if (vtype[s] < 0 || vtype[s] >= ctx->ntypes) return fail(ctx, MG_ERR_ARG, "type out of range");
  // constants of the real (h = 0) and the virtual (h = 1) sites with every kind
  std::vector<PairF> tf(2 * MAX_WPROBE * MAX_KINDS, PairF{});
  std::vector<PairD> td(2 * MAX_WPROBE * MAX_KINDS, PairD{});
  for (int h = 0; h < 2; h++)
    for (int s = 0; s < nps; s++) {
      const int k = ctx->h_kind[i0 + s];
      const int ta = h ? vtype[s] : ctx->kind_type[k];
      const double qs = h ? vcharge[s] : ctx->kind_q[k];
      for (int b = 0; b < ctx->nkind; b++) {
        const int tb = ctx->kind_type[b];
        double eps, sig;
        PairLJ P;
        combining_rule(ctx->h_tE[ta], ctx->h_tR[ta], ctx->h_tA[ta], ctx->h_tE[tb], ctx->h_tR[tb],
                       ctx->h_tA[tb], ctx->comb_rule, &eps, &sig);
        if (smooth_lj(eps, sig, ctx->C2, &P))
          return fail(ctx, MG_ERR_SETUP, "smooth LJ cutoff cannot be determined");
        const double qq = qs * ctx->kind_q[b];
        const size_t o = ((size_t)h * MAX_WPROBE + s) * MAX_KINDS + b;
        td[o] = PairD{P.C1q, P.C2q, P.A4, P.E24, P.Sq, qq, P.A, P.E4, 0, 0, 0, 0};
        tf[o] = PairF{(float)P.C1q, (float)P.C2q, (float)P.A4, (float)P.E24,
                      (float)P.Sq,  (float)qq,    (float)P.A,  (float)P.E4,
                      0.f, 0.f, 0.f, 0.f, qq, 0, 0, 0};
      }
    }
  const int nblk = widom_blocks(nlist);
  int* d_list = nullptr;
  double *d_U = nullptr, *d_part = nullptr;
  PairF* d_tf = nullptr;
  PairD* d_td = nullptr;
  auto release = [&]() {
    cudaFree(d_list);
    cudaFree(d_U);
    cudaFree(d_part);
    cudaFree(d_tf);
    cudaFree(d_td);
  };
  cudaError_t e = cudaMalloc((void**)&d_list, sizeof(int) * nlist);
  if (e == cudaSuccess) e = cudaMalloc((void**)&d_part, sizeof(double) * nblk);
  if (e == cudaSuccess && dU) e = cudaMalloc((void**)&d_U, sizeof(double) * nlist);
  if (e == cudaSuccess) e = cudaMalloc((void**)&d_tf, sizeof(PairF) * tf.size());
  if (e == cudaSuccess) e = cudaMalloc((void**)&d_td, sizeof(PairD) * td.size());
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_list, mols, sizeof(int) * nlist, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_tf, tf.data(), sizeof(PairF) * tf.size(), cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_td, td.data(), sizeof(PairD) * td.size(), cudaMemcpyHostToDevice,
                        ctx->stream);
  XWidomArgs a;
  a.nlist = nlist;
  a.nps = nps;
  a.nkind = ctx->nkind;
  a.ncx = ctx->ncx;
  a.ncy = ctx->ncy;
  a.ncz = ctx->ncz;
  a.nstencil = ctx->nstencil;
  a.lanes_sites = ctx->nstencil < 16 ? 1 : 0;
  a.ntab = ctx->ntab;
  a.list = d_list;
  a.mol_first = ctx->d_mol_first;
  a.r = ctx->last_r;
  a.cell_start = ctx->d_cell_start;
  a.stencil = ctx->d_stencil;
  a.Lx = ctx->L[0];
  a.Ly = ctx->L[1];
  a.Lz = ctx->L[2];
  a.cutoff_sq = ctx->cutoff * ctx->cutoff;
  a.sgrid = ctx->sgrid;
  a.T = T;
  a.U = d_U;
  a.part = d_part;
  a.pj = ctx->d_pj;
  a.pd = ctx->d_pd;
  a.tabf = d_tf;
  a.tabd = d_td;
  a.eru = ctx->d_eru;
  a.ert = ctx->d_ert;
  Launch L = launch(ctx);
  if (e == cudaSuccess) e = k_xwidom(L, a, ctx->precision != MG_MIXED);
  std::vector<double> part(nblk);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(part.data(), d_part, sizeof(double) * nblk, cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess && dU)
    e = cudaMemcpyAsync(dU, d_U, sizeof(double) * nlist, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  release();
  if (e != cudaSuccess) return fail(ctx, MG_ERR_CUDA, std::string("xwidom: ") + cudaGetErrorString(e));
  // no cutoff correction: cook's XWidom applies none
  widom_result(ctx, part.data(), nblk, nlist, T, 0.0, out);
  return MG_OK;
}

namespace {

PairArgs pair_args(mg_ctx* ctx) {
  PairArgs pa{};
  pa.ns = ctx->ns;
  pa.ncx = ctx->ncx;
  pa.ncy = ctx->ncy;
  pa.ncz = ctx->ncz;
  pa.nstencil = ctx->nstencil;
  pa.allpairs = ctx->allpairs ? 1 : 0;
  pa.nkind = ctx->nkind;
  pa.cell_start = ctx->d_cell_start;
  pa.order = ctx->d_order;
  pa.stencil = ctx->d_stencil;
  pa.Lx = ctx->L[0];
  pa.Ly = ctx->L[1];
  pa.Lz = ctx->L[2];
  pa.cutoff_sq = ctx->cutoff * ctx->cutoff;
  pa.sgrid = ctx->sgrid;
  pa.alpha = ctx->alpha;
  pa.f = nullptr;
  pa.epart = nullptr;
  pa.ntab = ctx->ntab;
  pa.pdj = nullptr;
  pa.pdd = nullptr;
  pa.pair_warps = 4;
  pa.spline_smem = 0;
  return pa;
}

KArgs kspace_args(mg_ctx* ctx) {
  KArgs ka;
  std::memset(&ka, 0, sizeof(ka));
  ka.nq = ctx->nq;
  ka.nk = ctx->nk;
  ka.nchunk = ctx->nchunk;
  ka.Kx = ctx->Kx;
  ka.Ky = ctx->Ky;
  ka.Kz = ctx->Kz;
  ka.row = ctx->row;
  set_box(ka, ctx->L);
  ka.alpha = ctx->alpha;
  ka.qsite = ctx->d_qsite;
  ka.qval = ctx->d_qval;
  ka.kvec = ctx->d_kvec;
  ka.ekk = ctx->d_ekk;
  ka.S = ctx->d_S;
  ka.ns = ctx->ns;
  ka.status = ctx->d_status;
  return ka;
}

}  // namespace

int mg_adjoint(mg_ctx* ctx, const double* r, const double* g, mg_adjoint_out* out) {
  if (!ctx || !r || !out) return fail(ctx, MG_ERR_ARG, "null argument");
  if (ctx->precision != MG_FP64 || ctx->polar || ctx->use_list || ctx->dipole)
    return fail(ctx, MG_ERR_ARG,
                "the adjoint needs an FP64, non-polar, tin-foil context with cells re-binned "
                "(skin <= 0)");
  const int ns = ctx->ns, nk2 = ctx->nkind * ctx->nkind, nt = ctx->ntypes;
  if (!ctx->d_adjtab) {
    // per pair of kinds: the smoothed-LJ constants, their sigma derivatives
    // (central differences of the set-up, step 1e-5 sigma) and eps, sigma
    std::vector<AdjPair> tab(nk2);
    const double c6 = 1.122462048309373;  // 2^(1/6): r_min = c6 sigma
    for (int ka = 0; ka < ctx->nkind; ka++)
      for (int kb = 0; kb < ctx->nkind; kb++) {
        const int ta = ctx->kind_type[ka], tb = ctx->kind_type[kb];
        double eps, sig;
        PairLJ P{}, Pp{}, Pm{};
        combining_rule(ctx->h_tE[ta], ctx->h_tR[ta], ctx->h_tA[ta], ctx->h_tE[tb], ctx->h_tR[tb],
                       ctx->h_tA[tb], ctx->comb_rule, &eps, &sig);
        smooth_lj(eps, sig, ctx->C2, &P);
        AdjPair& A = tab[ka * ctx->nkind + kb];
        A = AdjPair{P.C1q, P.C2q, P.Sq, P.E4, P.A, P.A4, 0, 0, 1, 1};
        if (eps != 0) {
          const double h = 1e-5 * sig;
          smooth_lj(eps, sig + h, ctx->C2, &Pp);
          smooth_lj(eps, sig - h, ctx->C2, &Pm);
          A.dA = (Pp.A - Pm.A) / (2 * h) * c6;
          A.dA4 = (Pp.A4 - Pm.A4) / (2 * h) * c6;
          A.eps = -eps;
          A.sig = sig / c6;
        }
      }
    CK(upload(&ctx->d_adjtab, tab.data(), tab.size()));
    std::vector<double> q(ns);
    for (int i = 0; i < ns; i++) q[i] = ctx->kind_q[ctx->h_kind[i]];
    CK(upload(&ctx->d_aq, q.data(), q.size()));
    CK(dalloc(&ctx->d_ag, 3 * (size_t)ns));
    CK(dalloc(&ctx->d_ags, (size_t)ns));
    CK(dalloc(&ctx->d_apart, (size_t)ctx->ncell * nk2 * 6));
    CK(dalloc(&ctx->d_adEq, (size_t)ns));
    CK(dalloc(&ctx->d_adLq, (size_t)ns));
    ctx->adj_ntch = std::max(1, std::min(64, ctx->nq / 256));
    CK(dalloc(&ctx->d_atpart, (size_t)ctx->adj_ntch * std::max(1, ctx->nk) * 3));
    CK(dalloc(&ctx->d_aT, (size_t)std::max(1, ctx->nk)));
  }
  ctx->launches = 0;
  const size_t nb = 3 * (size_t)ns * sizeof(double);
  CK(cudaMemcpyAsync(ctx->d_rs, r, nb, cudaMemcpyHostToDevice, ctx->stream));
  if (g) CK(cudaMemcpyAsync(ctx->d_ag, g, nb, cudaMemcpyHostToDevice, ctx->stream));
  int rc = forces_async(ctx, ctx->d_rs, ctx->d_fs, true);
  if (rc) return rc;
  ctx->need_build = true;
  Launch L = launch(ctx);
  CK(k_adjoint(L, pair_args(ctx), kspace_args(ctx), ctx->d_pd, ctx->d_adjtab, ctx->d_ert,
               (const double2*)ctx->d_tab, g ? ctx->d_ag : nullptr, ctx->d_aq, ctx->d_ags,
               ctx->d_apart, ctx->d_adEq, ctx->d_adLq, ctx->d_atpart, ctx->adj_ntch, ctx->d_aT));
  std::vector<double> part((size_t)ctx->ncell * nk2 * 6);
  CK(cudaMemcpyAsync(part.data(), ctx->d_apart, sizeof(double) * part.size(),
                     cudaMemcpyDeviceToHost, ctx->stream));
  if (out->dE_dq)
    CK(cudaMemcpyAsync(out->dE_dq, ctx->d_adEq, sizeof(double) * ns, cudaMemcpyDeviceToHost,
                       ctx->stream));
  if (out->dL_dq)
    CK(cudaMemcpyAsync(out->dL_dq, ctx->d_adLq, sizeof(double) * ns, cudaMemcpyDeviceToHost,
                       ctx->stream));
  rc = fetch_sums(ctx);
  if (rc) return rc;
  rc = fetch_status(ctx);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  rc = check_status(ctx);
  if (rc) return rc;
  mg_energy en;
  fill_energy(ctx, &en);
  out->E = en.el + en.lj;
  out->W = en.vir + en.el;
  // kind pairs (both orders, halves from the kernel) -> type pairs a <= b,
  // summed over the cell CTAs in a fixed order
  std::vector<double> kp((size_t)nk2 * 6, 0.0);
  for (int c = 0; c < ctx->ncell; c++)
    for (int t = 0; t < nk2 * 6; t++) kp[t] += part[(size_t)c * nk2 * 6 + t];
  double* dst[3] = {out->dE_pair, out->dW_pair, out->dL_pair};
  for (int m = 0; m < 3; m++)
    if (dst[m]) std::memset(dst[m], 0, sizeof(double) * nt * nt * 2);
  for (int ka = 0; ka < ctx->nkind; ka++)
    for (int kb = 0; kb < ctx->nkind; kb++) {
      const int ta = ctx->kind_type[ka], tb = ctx->kind_type[kb];
      const int lo = std::min(ta, tb), hi = std::max(ta, tb);
      const double* v = kp.data() + 6 * (ka * ctx->nkind + kb);
      for (int m = 0; m < 3; m++)
        if (dst[m]) {
          dst[m][2 * (lo * nt + hi)] += v[2 * m];
          dst[m][2 * (lo * nt + hi) + 1] += v[2 * m + 1];
        }
    }
  return MG_OK;
}

int mg_selffield(mg_ctx* ctx, double* r, double* f, double omega, int measure, mg_energy* en) {
  if (!ctx || !r || !f) return fail(ctx, MG_ERR_ARG, "null argument");
  if (!ctx->polar) return fail(ctx, MG_ERR_ARG, "no Drude charges in this context");
  ctx->launches = 0;
  const size_t nb = 6 * (size_t)ctx->ns * sizeof(double);
  CK(cudaMemcpyAsync(ctx->d_rs, r, nb, cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_fs, f, nb, cudaMemcpyHostToDevice, ctx->stream));
  int rc = selffield_async(ctx, ctx->d_rs, ctx->d_fs, omega, measure && en, nullptr);
  if (rc) return rc;
  CK(cudaMemcpyAsync(r, ctx->d_rs, nb, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(f, ctx->d_fs, nb, cudaMemcpyDeviceToHost, ctx->stream));
  if (measure && en) {
    rc = fetch_sums(ctx);
    if (rc) return rc;
  }
  rc = fetch_status(ctx);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  prof_resolve(ctx);
  rc = check_status(ctx);
  if (rc) return rc;
  if (measure && en) add_drude_energy(ctx, en);
  return MG_OK;
}

double mg_thermostat_factor(mg_ctx* ctx) {
  if (!ctx) return 0;
  double z = 1;
  cudaMemcpyAsync(&z, ctx->d_zth, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  return z;
}

int mg_nose_state(mg_ctx* ctx, double state[3]) {
  if (!ctx || !state) return fail(ctx, MG_ERR_ARG, "null argument");
  if (ctx->thermostat != 3) return fail(ctx, MG_ERR_ARG, "no Nose-Hoover thermostat");
  double h[NH_HIST];
  CK(cudaMemcpyAsync(h, ctx->d_nh, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  state[0] = h[NH_LOGS];
  state[1] = h[NH_LOGSV];
  state[2] = h[NH_EXT];
  return MG_OK;
}

int mg_set_overlap(mg_ctx* ctx, int on) {
  if (!ctx) return MG_ERR_ARG;
  if (ctx->overlap != (on != 0)) drop_graphs(ctx);
  ctx->overlap = on != 0;
  return MG_OK;
}

int mg_set_graph(mg_ctx* ctx, int on) {
  if (!ctx) return MG_ERR_ARG;
  ctx->use_graph = on != 0;
  return MG_OK;
}

int mg_set_stream(mg_ctx* ctx, void* stream) {
  if (!ctx) return MG_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return MG_OK;
}

int mg_profile_enable(mg_ctx* ctx, int on) {
  if (!ctx) return MG_ERR_ARG;
  ctx->prof_on = on != 0;
  return MG_OK;
}

int mg_profile_reset(mg_ctx* ctx) {
  if (!ctx) return MG_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  prof_resolve(ctx);
  for (size_t i = 0; i < ctx->pms.size(); i++) {
    ctx->pms[i] = 0;
    ctx->pcnt[i] = 0;
  }
  return MG_OK;
}

int mg_profile_entry(mg_ctx* ctx, int i, const char** name, double* ms, long* count) {
  if (!ctx || i < 0 || i >= (int)ctx->pnames.size()) return MG_ERR_ARG;
  if (name) *name = ctx->pnames[i].c_str();
  if (ms) *ms = ctx->pms[i];
  if (count) *count = ctx->pcnt[i];
  return MG_OK;
}

int mg_probe_fp32_tflops(double* tflops) {
  mg_ctx* ctx = nullptr;
  if (!tflops) return MG_ERR_ARG;
  int dev = 0, nsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  float* buf = nullptr;
  cudaStream_t s;
  cudaEvent_t a, b;
  CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  const int blocks = nsm * 8, threads = 256, iters = 1 << 14;
  CK(cudaMalloc(&buf, sizeof(float) * blocks * threads));
  double best = 0;
  for (int rep = 0; rep < 4; rep++) {
    CK(cudaEventRecord(a, s));
    CK(k_fma_probe(s, blocks, threads, iters, buf));
    CK(cudaEventRecord(b, s));
    CK(cudaEventSynchronize(b));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, a, b));
    double fl = 2.0 * 8 * (double)iters * blocks * threads;
    if (rep > 0 && ms > 0) best = std::max(best, fl / (ms * 1e-3) / 1e12);
  }
  cudaFree(buf);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaStreamDestroy(s);
  *tflops = best;
  return MG_OK;
}

}  // extern "C"

// ------------------------------------------------------------- batches --

struct mg_batch {
  std::string err;
  std::vector<mg_ctx*> box;
  cudaStream_t main = nullptr;
  std::vector<cudaStream_t> lanes;
  std::vector<cudaEvent_t> ev_join;
  cudaEvent_t ev_fork = nullptr;
  cudaGraphExec_t g_step = nullptr, g_meas = nullptr;
  int launches_step = 0, launches = 0;
  WidomBox* d_wbox = nullptr;
  int wcap = 0;
  // one launch per kernel over all boxes, when every box qualifies
  // (fused_ok): the boxes' kernel arguments on the device, the largest
  // grids, one captured graph per kind of step
  int fused_ok = -1;
  BoxStep* d_steps = nullptr;
  TcBox* d_tc = nullptr;
  BatchGrid grid{};
  // the boxes' status words, gathered into one array after unmeasured steps
  int** d_statp = nullptr;
  int* d_stat = nullptr;
  int* h_stat = nullptr;
  cudaGraphExec_t gf_step = nullptr, gf_meas = nullptr;
  int launches_fused = 0;
};

namespace {

int bfail(mg_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}

#define BCK(call)                                                                     \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return bfail(b, MG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// one MD step of every box as a graph: fork from the main stream onto the
// lanes (boxes round-robin), each box's kernels on its lane, join
int capture_step(mg_batch* b, bool measure, cudaGraphExec_t* out) {
  BCK(cudaStreamBeginCapture(b->main, cudaStreamCaptureModeRelaxed));
  int rc = MG_OK;
  cudaEventRecord(b->ev_fork, b->main);
  for (cudaStream_t s : b->lanes) cudaStreamWaitEvent(s, b->ev_fork, 0);
  int nl = 0;
  for (size_t i = 0; i < b->box.size() && !rc; i++) {
    mg_ctx* c = b->box[i];
    c->launches = 0;
    rc = md_step_enqueue(c, measure);
    if (rc) b->err = "box " + std::to_string(i) + ": " + c->err;
    nl += c->launches;
  }
  for (size_t l = 0; l < b->lanes.size(); l++) {
    cudaEventRecord(b->ev_join[l], b->lanes[l]);
    cudaStreamWaitEvent(b->main, b->ev_join[l], 0);
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->main, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return bfail(b, MG_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess)
    return bfail(b, MG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  b->launches_step = nl;
  return MG_OK;
}

}  // namespace

mg_batch* mg_batch_create(int nbox, const mg_topology* tops, const mg_params* params, int nlanes,
                          int* status) {
  int dummy;
  int* st = status ? status : &dummy;
  if (nbox < 1 || !tops || !params) {
    *st = MG_ERR_ARG;
    return nullptr;
  }
  mg_batch* b = new mg_batch;
  const int nl = std::max(1, std::min(nlanes > 0 ? nlanes : 16, nbox));
  if (cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess) {
    *st = MG_ERR_CUDA;
    mg_batch_destroy(b);
    return nullptr;
  }
  b->lanes.resize(nl);
  b->ev_join.resize(nl);
  for (int l = 0; l < nl; l++) {
    if (cudaStreamCreateWithFlags(&b->lanes[l], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_join[l], cudaEventDisableTiming) != cudaSuccess) {
      *st = MG_ERR_CUDA;
      mg_batch_destroy(b);
      return nullptr;
    }
  }
  for (int i = 0; i < nbox; i++) {
    int s = 0;
    mg_ctx* c = mg_create(&tops[i], &params[i], &s);
    if (!c) {
      *st = s ? s : MG_ERR_SETUP;
      mg_batch_destroy(b);
      return nullptr;
    }
    c->stream = b->lanes[i % nl];
    c->overlap = false;
    b->box.push_back(c);
  }
  *st = MG_OK;
  return b;
}

int mg_batch_destroy(mg_batch* b) {
  if (!b) return MG_OK;
  if (b->main) cudaStreamSynchronize(b->main);
  for (mg_ctx* c : b->box) {
    cudaStreamSynchronize(c->stream);
    c->stream = c->own_stream;
    mg_destroy(c);
  }
  if (b->g_step) cudaGraphExecDestroy(b->g_step);
  if (b->g_meas) cudaGraphExecDestroy(b->g_meas);
  if (b->gf_step) cudaGraphExecDestroy(b->gf_step);
  if (b->gf_meas) cudaGraphExecDestroy(b->gf_meas);
  if (b->d_steps) cudaFree(b->d_steps);
  if (b->d_tc) cudaFree(b->d_tc);
  if (b->d_statp) cudaFree(b->d_statp);
  if (b->d_stat) cudaFree(b->d_stat);
  if (b->h_stat) cudaFreeHost(b->h_stat);
  if (b->d_wbox) cudaFree(b->d_wbox);
  for (cudaEvent_t e : b->ev_join)
    if (e) cudaEventDestroy(e);
  for (cudaStream_t s : b->lanes)
    if (s) cudaStreamDestroy(s);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->main) cudaStreamDestroy(b->main);
  delete b;
  return MG_OK;
}

const char* mg_batch_last_error(const mg_batch* b) { return b ? b->err.c_str() : "null batch"; }
int mg_batch_size(const mg_batch* b) { return b ? (int)b->box.size() : 0; }
mg_ctx* mg_batch_box(mg_batch* b, int i) {
  return (b && i >= 0 && i < (int)b->box.size()) ? b->box[i] : nullptr;
}
int mg_batch_last_launches(const mg_batch* b) { return b ? b->launches : 0; }

namespace {

// a box the batched kernels take: the FP32 path without Drude charges,
// dependants, thermostat, step limiter or drift removal, cells re-binned
// at every step on a grid of at least 3 cells per edge, the cell pair kernel
// with 4 warps, both Ewald passes on the FP32 cores or both on the tensor
// cores, no dipole term
bool fusable(const mg_ctx* c) {
  return c->precision == MG_MIXED && !c->polar && !c->use_list && !c->allpairs &&
         c->pair_variant == 0 && c->kspace_tc == c->sk_tc && c->thermostat == 0 &&
         c->ndep == 0 && !c->dipole && c->drmax == 0 && !c->drift_step && c->nq > 0 &&
         !c->prof_on;
}

// the boxes' arguments for the batched kernels, exactly those of their
// single launches in forces_async / md_step_enqueue
int build_fused(mg_batch* b) {
  const int nbox = (int)b->box.size();
  std::vector<BoxStep> h(nbox);
  std::vector<TcBox> tc(nbox);
  BatchGrid& g = b->grid;
  g = BatchGrid{};
  for (int i = 0; i < nbox; i++) {
    mg_ctx* c = b->box[i];
    BoxStep& e = h[i];
    std::memset(&e, 0, sizeof(e));
    e.ns = c->ns;
    e.ncx = c->ncx;
    e.ncy = c->ncy;
    e.ncz = c->ncz;
    for (int d = 0; d < 3; d++) e.iL[d] = 1.0 / c->L[d];
    e.r = c->d_r;
    e.status = c->d_status;
    e.kind = c->d_kind;
    e.mol = c->d_mol;
    e.pfix = c->d_pfix;
    e.key = c->d_key;
    e.count = c->d_ccount;
    e.cursor = c->d_ccursor;
    e.slot_site = c->d_idx;
    e.order = c->d_order;
    e.key_s = c->d_key_s;
    e.start = c->d_cell_start;
    e.gstart = c->d_gstart;
    e.pj = c->d_pj;
    e.gcell = c->d_gcell;
    e.pa = make_pair_args(c, c->d_f);
    e.ptab = c->d_ptabf;
    e.erd = c->d_erd;
    e.eru = c->d_eru;
    e.sx = (float)(c->L[0] / 4294967296.0);
    e.sy = (float)(c->L[1] / 4294967296.0);
    e.sz = (float)(c->L[2] / 4294967296.0);
    e.cq = (float)(c->cutoff * c->cutoff);
    e.sg = (float)c->sgrid;
    e.al = (float)c->alpha;
    e.xa = excl_args(c, c->d_r, c->d_f);
    e.ka = make_kargs(c, c->d_f);
    e.tab = (float2*)c->d_tab;
    e.qf = c->d_qfix;
    e.part = (float2*)c->d_part;
    e.sa = shake_args(c, true);
    const int nkin = (c->nmol + 127) / 128;
    e.rpart[0] = c->d_epart;
    e.rrows[0] = c->nprows + c->nxblocks;
    e.rwidth[0] = 10;
    e.rout[0] = c->d_sums;
    e.rpart[1] = c->d_ekpart;
    e.rrows[1] = c->nkblocks;
    e.rwidth[1] = 7;
    e.rout[1] = c->d_sums + 10;
    e.rpart[2] = c->d_kinpart;
    e.rrows[2] = nkin;
    e.rwidth[2] = 1;
    e.rout[2] = c->d_sums + 17;
    e.rpart[3] = c->d_meas;
    e.rrows[3] = nkin;
    e.rwidth[3] = 13;
    e.rout[3] = c->d_sums + 32;
    e.g_site = cell_site_blocks(c->ns);
    e.g_order = cell_order_blocks(c->ncell);
    e.g_pair = c->ncell;
    e.g_excl = c->nmol > 0 ? (c->nmol + EXCL_THREADS - 1) / EXCL_THREADS : 0;
    e.g_charge = (c->nq + 255) / 256;
    e.g_phase = (int)(((long)c->nq * c->row + 255) / 256);
    e.g_p1x = c->np1job;
    e.g_p1y = c->nchunk;
    e.g_skr = (c->nk + 255) / 256;
    e.g_kf = kf_mixed_blocks(c->nq);
    e.g_shake = (c->nmol + 127) / 128;
    TcBox& t = tc[i];
    if (c->kspace_tc) {
      // the tensor-core passes, with the arguments of the box's single
      // launches (tc_args); its pass 1 reduces sk_nch chunks
      t = tc_args(c, e.ka, c->d_r);
      e.ka.nchunk = c->sk_nch;
      e.g_charge = e.g_phase = e.g_p1x = e.g_p1y = e.g_kf = 0;
      g.any_tc = true;
    } else {
      t = TcBox{};
      g.any_fp32 = true;
    }
    g.tc_phase = std::max(g.tc_phase, t.g_phase);
    g.tc_sk = std::max(g.tc_sk, t.g_sk);
    g.tc_vb = std::max(g.tc_vb, t.g_vb);
    g.tc_kf = std::max(g.tc_kf, t.g_kf);
    g.tc_phase_smem = std::max(g.tc_phase_smem, t.smem_phase);
    g.tc_sk_smem = std::max(g.tc_sk_smem, t.smem_sk);
    g.tc_kf_smem = std::max(g.tc_kf_smem, t.smem_kf);
    g.site = std::max(g.site, e.g_site);
    g.order = std::max(g.order, e.g_order);
    g.pair = std::max(g.pair, e.g_pair);
    g.excl = std::max(g.excl, e.g_excl);
    g.charge = std::max(g.charge, e.g_charge);
    g.phase = std::max(g.phase, e.g_phase);
    g.p1x = std::max(g.p1x, e.g_p1x);
    g.p1y = std::max(g.p1y, e.g_p1y);
    g.skr = std::max(g.skr, e.g_skr);
    g.kf = std::max(g.kf, e.g_kf);
    g.shake = std::max(g.shake, e.g_shake);
    g.pair_smem = std::max(g.pair_smem, sizeof(PairFS) * (size_t)c->nkind * c->nkind);
    if (!c->kspace_tc) g.kf_smem = std::max(g.kf_smem, kf_mixed_smem(e.ka));
  }
  if (cudaMalloc(&b->d_steps, sizeof(BoxStep) * (size_t)nbox) != cudaSuccess ||
      cudaMemcpy(b->d_steps, h.data(), sizeof(BoxStep) * (size_t)nbox, cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMalloc(&b->d_tc, sizeof(TcBox) * (size_t)nbox) != cudaSuccess ||
      cudaMemcpy(b->d_tc, tc.data(), sizeof(TcBox) * (size_t)nbox, cudaMemcpyHostToDevice) !=
          cudaSuccess)
    return bfail(b, MG_ERR_CUDA, "batch: uploading the boxes' kernel arguments");
  return MG_OK;
}

// one MD step of every box with the batched kernels, on the batch stream
// with ev (profiling, not captured): an event recorded after each of the
// seven stages (cell list; pair terms; phase rows and operand tiles; pass 1;
// S(k) sums; pass 2; the step) and one before them
int fused_step_enqueue(mg_batch* b, bool measure, cudaEvent_t* ev = nullptr) {
  const int nbox = (int)b->box.size();
  Launch L{b->main, &b->launches_fused};
  const BatchGrid& g = b->grid;
  auto mark = [&](int k) { return ev ? cudaEventRecord(ev[k], b->main) : cudaSuccess; };
  // the order of a single box's serial chain: cell list, pair and
  // exclusion terms, phase rows (with the operand tiles), pass 1, its sum,
  // pass 2, the step
  BCK(mark(0));
  BCK(k_batch_cells(L, b->d_steps, nbox, g));
  BCK(mark(1));
  BCK(k_batch_pairs(L, b->d_steps, nbox, g, measure));
  BCK(mark(2));
  if (g.any_tc) BCK(k_batch_tc_phase(L, b->d_tc, nbox, g.tc_phase, g.tc_phase_smem));
  BCK(mark(3));
  if (g.any_fp32) BCK(k_batch_pass1(L, b->d_steps, nbox, g));
  if (g.any_tc) BCK(k_batch_sk_tc(L, b->d_tc, nbox, g.tc_sk, g.tc_sk_smem));
  BCK(mark(4));
  BCK(k_batch_sk_reduce(L, b->d_steps, nbox, g, measure));
  BCK(mark(5));
  if (g.any_fp32) BCK(k_batch_pass2(L, b->d_steps, nbox, g));
  if (g.any_tc) BCK(k_batch_kf_tc(L, b->d_tc, nbox, g.tc_vb, g.tc_kf, g.tc_kf_smem));
  BCK(mark(6));
  BCK(k_batch_step(L, b->d_steps, nbox, g, measure));
  BCK(mark(7));
  return MG_OK;
}

int capture_fused(mg_batch* b, bool measure, cudaGraphExec_t* out) {
  BCK(cudaStreamBeginCapture(b->main, cudaStreamCaptureModeRelaxed));
  b->launches_fused = 0;
  int rc = fused_step_enqueue(b, measure);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(b->main, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return bfail(b, MG_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess)
    return bfail(b, MG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  b->launches_step = b->launches_fused;
  return MG_OK;
}

}  // namespace

int mg_batch_fused(const mg_batch* b) { return b && b->fused_ok == 1 ? 1 : 0; }

int mg_batch_profile(mg_batch* b, int nrep, double ms[7]) {
  if (!b || !ms || nrep < 1) return bfail(b, MG_ERR_ARG, "bad arguments");
  if (b->fused_ok != 1) return bfail(b, MG_ERR_ARG, "the batch does not run the fused step");
  for (int k = 0; k < 7; k++) ms[k] = 0;
  cudaEvent_t ev[8] = {};
  for (int k = 0; k < 8; k++)
    if (cudaEventCreate(&ev[k]) != cudaSuccess) {
      for (int j = 0; j < k; j++) cudaEventDestroy(ev[j]);
      return bfail(b, MG_ERR_CUDA, "profile events");
    }
  int rc = MG_OK;
  for (int r = 0; r < nrep && rc == MG_OK; r++) {
    rc = fused_step_enqueue(b, false, ev);
    if (rc == MG_OK && cudaEventSynchronize(ev[7]) != cudaSuccess)
      rc = bfail(b, MG_ERR_CUDA, "profile step");
    for (int k = 0; k < 7 && rc == MG_OK; k++) {
      float t = 0;
      cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      ms[k] += t / nrep;
    }
  }
  for (int k = 0; k < 8; k++) cudaEventDestroy(ev[k]);
  if (rc == MG_OK) {
    for (mg_ctx* c : b->box) {
      c->last_r = c->d_r;
      c->have_cells = true;
    }
  }
  return rc;
}

int mg_batch_md_steps(mg_batch* b, int nsteps, mg_energy* en) {
  if (!b || nsteps < 0) return bfail(b, MG_ERR_ARG, "bad arguments");
  for (size_t i = 0; i < b->box.size(); i++) {
    const mg_ctx* c = b->box[i];
    if (!c->have_state) return bfail(b, MG_ERR_ARG, "box " + std::to_string(i) + ": no MD state");
    if (c->polar || c->use_list || c->prof_on)
      return bfail(b, MG_ERR_ARG, "box " + std::to_string(i) +
                                      ": batched MD needs non-polar boxes, cells re-binned "
                                      "every step and profiling off");
  }
  // the lanes must have finished what the per-box calls queued on them
  for (cudaStream_t s : b->lanes) BCK(cudaStreamSynchronize(s));
  if (b->fused_ok < 0) {
    bool ok = true;
    for (const mg_ctx* c : b->box) ok = ok && fusable(c);
    b->fused_ok = ok ? 1 : 0;
    if (ok) {
      int rc = build_fused(b);
      if (rc) return rc;
    }
  }
  b->launches = 0;
  for (int s = 0; s < nsteps; s++) {
    const bool meas = en && s == nsteps - 1;
    if (b->fused_ok == 1) {
      cudaGraphExec_t& g = meas ? b->gf_meas : b->gf_step;
      if (!g) {
        int rc = capture_fused(b, meas, &g);
        if (rc) return rc;
      }
      BCK(cudaGraphLaunch(g, b->main));
      b->launches += b->launches_step;
      continue;
    }
    cudaGraphExec_t& g = meas ? b->g_meas : b->g_step;
    if (!g) {
      int rc = capture_step(b, meas, &g);
      if (rc) return rc;
    }
    BCK(cudaGraphLaunch(g, b->main));
    b->launches += b->launches_step;
  }
  if (b->fused_ok == 1 && nsteps > 0)
    for (mg_ctx* c : b->box) {
      // what a launched force evaluation leaves behind (Widom's cell list)
      c->last_r = c->d_r;
      c->have_cells = true;
    }
  if (!en) {
    // unmeasured: the boxes' status words in one copy (every box's work ran
    // on the batch stream or joined it)
    const int nbox = (int)b->box.size();
    if (!b->d_statp) {
      std::vector<int*> sp(nbox);
      for (int i = 0; i < nbox; i++) sp[i] = b->box[i]->d_status;
      if (cudaMalloc(&b->d_statp, sizeof(int*) * nbox) != cudaSuccess ||
          cudaMalloc(&b->d_stat, sizeof(int) * nbox) != cudaSuccess ||
          cudaMallocHost(&b->h_stat, sizeof(int) * nbox) != cudaSuccess ||
          cudaMemcpy(b->d_statp, sp.data(), sizeof(int*) * nbox, cudaMemcpyHostToDevice) !=
              cudaSuccess)
        return bfail(b, MG_ERR_CUDA, "batch: status buffers");
    }
    BCK(k_gather_status(b->main, b->d_statp, nbox, b->d_stat));
    BCK(cudaMemcpyAsync(b->h_stat, b->d_stat, sizeof(int) * nbox, cudaMemcpyDeviceToHost,
                        b->main));
    BCK(cudaStreamSynchronize(b->main));
    for (int i = 0; i < nbox; i++) {
      if (!b->h_stat[i]) continue;
      mg_ctx* c = b->box[i];
      std::memcpy(c->h_sums + 31, &b->h_stat[i], sizeof(int));
      const int rc = check_status(c);
      if (rc) return bfail(b, rc, "box " + std::to_string(i) + ": " + c->err);
    }
    return MG_OK;
  }
  BCK(cudaStreamSynchronize(b->main));
  for (size_t i = 0; i < b->box.size(); i++) {
    mg_ctx* c = b->box[i];
    int rc = fetch_status(c);
    if (!rc && en) rc = fetch_sums(c);
    if (!rc) {
      cudaError_t e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) rc = fail(c, MG_ERR_CUDA, cudaGetErrorString(e));
    }
    if (!rc) rc = check_status(c);
    if (rc) return bfail(b, rc, "box " + std::to_string(i) + ": " + c->err);
    if (en) {
      fill_energy(c, &en[i]);
      en[i].ekin = c->h_sums[17] / (c->h * c->h) / 4;
      fill_pressure(c, &en[i]);
    }
  }
  return MG_OK;
}

int mg_batch_widom(mg_batch* b, const mg_probe* probes, int probe_per_box, long long ninsert,
                   unsigned long long seed, double T, mg_widom_result* out) {
  if (!b || !probes || !out) return bfail(b, MG_ERR_ARG, "null argument");
  const int nbox = (int)b->box.size();
  std::vector<WidomBox> desc(nbox);
  std::vector<double> corr(nbox);
  for (int i = 0; i < nbox; i++) {
    mg_ctx* c = b->box[i];
    int rc = widom_prepare(c, probe_per_box ? &probes[i] : probes, ninsert,
                           seed + 0x632BE59BD9B4E019ULL * (unsigned long long)i, T, nullptr,
                           &desc[i], &corr[i]);
    if (rc) return bfail(b, rc, "box " + std::to_string(i) + ": " + c->err);
    if (c->precision != b->box[0]->precision)
      return bfail(b, MG_ERR_ARG, "all boxes of a batch need the same precision");
  }
  for (cudaStream_t s : b->lanes) BCK(cudaStreamSynchronize(s));
  if (b->wcap < nbox) {
    if (b->d_wbox) cudaFree(b->d_wbox);
    b->d_wbox = nullptr;
    BCK(cudaMalloc((void**)&b->d_wbox, sizeof(WidomBox) * nbox));
    b->wcap = nbox;
  }
  BCK(cudaMemcpyAsync(b->d_wbox, desc.data(), sizeof(WidomBox) * nbox, cudaMemcpyHostToDevice,
                      b->main));
  int cnt = 0;
  Launch L{b->main, &cnt};
  BCK(k_widom(L, b->d_wbox, nbox, ninsert, b->box[0]->precision != MG_MIXED));
  b->launches = cnt;
  const int nblk = widom_blocks(ninsert);
  std::vector<double> part((size_t)nblk * nbox);
  for (int i = 0; i < nbox; i++)
    BCK(cudaMemcpyAsync(part.data() + (size_t)i * nblk, b->box[i]->d_wpart, sizeof(double) * nblk,
                        cudaMemcpyDeviceToHost, b->main));
  BCK(cudaStreamSynchronize(b->main));
  for (int i = 0; i < nbox; i++)
    widom_result(b->box[i], part.data() + (size_t)i * nblk, nblk, ninsert, T, corr[i], &out[i]);
  return MG_OK;
}

// ------------------------------------------------------------- autotuner --

int mg_autotune(const mg_topology* top, mg_params* par, const double* r, int nrep, double* ms) {
  if (!top || !par || !r) return MG_ERR_ARG;
  const int cd[3] = {1, 2, 3}, kc[3] = {6, 10, 16};
  nrep = std::max(1, nrep);
  const bool polar = top->chargepol != nullptr;
  const size_t nv = 3 * (size_t)top->ns * (polar ? 2 : 1);
  double *r_dev = nullptr, *f_dev = nullptr;
  if (cudaMalloc((void**)&r_dev, nv * sizeof(double)) != cudaSuccess) return MG_ERR_CUDA;
  if (cudaMalloc((void**)&f_dev, nv * sizeof(double)) != cudaSuccess) {
    cudaFree(r_dev);
    return MG_ERR_CUDA;
  }
  cudaMemcpy(r_dev, r, nv * sizeof(double), cudaMemcpyHostToDevice);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int rc = MG_OK;
  // time per force evaluation of one trial context (-1: not possible): the
  // best of three blocks of nrep evaluations (choices within a few per cent
  // of each other, such as the Ewald chain beside or after the r-space
  // chain, flipped between runs on single blocks)
  auto trial = [&](const mg_params& p2) -> double {
    int st = 0;
    mg_ctx* c = mg_create(top, &p2, &st);
    if (!c) return -1;
    double t = -1;
    int e = mg_forces_device(c, r_dev, f_dev, 0, nullptr);  // warm-up
    for (int blk = 0; blk < 3 && !e; blk++) {
      cudaEventRecord(e0, c->stream);
      for (int k = 0; k < nrep && !e; k++) e = mg_forces_device(c, r_dev, f_dev, 0, nullptr);
      cudaEventRecord(e1, c->stream);
      cudaEventSynchronize(e1);
      float f = 0;
      cudaEventElapsedTime(&f, e0, e1);
      if (!e && (t < 0 || f / nrep < t)) t = f / nrep;
    }
    if (e) {
      rc = e;
      t = -1;
    }
    mg_destroy(c);
    return t;
  };
  double best = 1e300;
  int bc = 0, bk = 0;
  for (int a = 0; a < 3 && rc == MG_OK; a++)
    for (int b = 0; b < 3 && rc == MG_OK; b++) {
      mg_params p2 = *par;
      p2.cells_per_cutoff = cd[a];
      p2.kspace_ctas_per_sm = kc[b];
      const double t = trial(p2);
      if (ms) ms[3 * a + b] = t;
      if (t > 0 && t < best) {
        best = t;
        bc = cd[a];
        bk = kc[b];
      }
    }
  // the pair-kernel variants at the best split, each with the Ewald chain
  // beside the r-space chain and after it (FP32 path): which is faster
  // depends on how the kernels share the SMs, so the two are chosen together
  int bv = par->pair_variant, bser = par->kspace_serial;
  const int nser = par->precision == MG_MIXED ? 2 : 1;
  double tser[2] = {-1, -1};
  if (!rc && bc) {
    double bestv = 1e300;
    auto consider = [&](int v, int cdv, double* slot) {
      double tv = -1, ts[2] = {-1, -1};
      for (int ser = 0; ser < nser && rc == MG_OK; ser++) {
        mg_params p2 = *par;
        p2.cells_per_cutoff = cdv;
        p2.kspace_ctas_per_sm = bk;
        p2.pair_variant = v;
        p2.kspace_serial = nser == 2 ? ser : par->kspace_serial;
        ts[ser] = trial(p2);
        if (ts[ser] > 0 && (tv < 0 || ts[ser] < tv)) tv = ts[ser];
        if (ts[ser] > 0 && ts[ser] < bestv) {
          bestv = ts[ser];
          bv = v;
          bc = cdv;
          bser = p2.kspace_serial;
          tser[0] = ts[0];
          tser[1] = ts[1];
        }
      }
      if (slot) *slot = tv;
    };
    const int cbest = bc;
    for (int v = 0; v < 8 && rc == MG_OK; v++) consider(v, cbest, ms ? ms + 9 + v : nullptr);
    // the group pair kernel (variant 8) at every cell subdivision: its
    // pruning favours other cells than the cell kernel does
    for (int a = 0; a < 3 && rc == MG_OK; a++) consider(8, cd[a], ms ? ms + 17 + a : nullptr);
    // and its half-shell forms (Newton's third law; FP32 path): lanes on the
    // home sites, and lanes on the neighbours
    if (par->precision == MG_MIXED) {
      for (int a = 0; a < 3 && rc == MG_OK; a++) consider(9, cd[a], ms ? ms + 20 + a : nullptr);
      for (int a = 0; a < 3 && rc == MG_OK; a++) consider(10, cd[a], ms ? ms + 25 + a : nullptr);
    }
  }
  if (ms) {
    ms[23] = tser[0];
    ms[24] = tser[1];
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(r_dev);
  cudaFree(f_dev);
  if (rc) return rc;
  if (bc == 0) return MG_ERR_SETUP;
  par->cells_per_cutoff = bc;
  par->kspace_ctas_per_sm = bk;
  par->pair_variant = bv;
  par->kspace_serial = bser;
  return MG_OK;
}
