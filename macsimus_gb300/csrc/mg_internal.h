// Internal declarations shared by the host tables, the kernels and the C ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace mg {

// smoothed LJ constants of one type pair (cook's sitesite_t)
struct PairLJ {
  double C1q, C2q, A, A4, Sq, E4, E24, E48;
};

void combining_rule(double E0, double R0, double a0, double E1, double R1, double a1,
                    int comb_rule, double* eps, double* sig);
int smooth_lj(double eps, double sig, double C2, PairLJ* p);
double lj_tail_correction(double eps, double sig, const PairLJ& p);
int erfc_table_size(int grid, double maxr, double alpha);
void erfc_table(int grid, double maxr, double cutoff, double alpha, int shift,
                std::vector<double>* tab, double* sgrid);
int kvector_set(const double L[3], double* kappa, std::vector<int>* kv);
void aspc_coefficients(int k, double* B, double* omega);

// ---------------------------------------------------------------- device --

// per pair-of-kinds constants (kind = LJ type x charge class); FP32 copy
// charge products: qq centre-centre, qpc Drude(i)-centre(j), qcp centre(i)-
// Drude(j), qpp Drude-Drude (zero without Drude charges)
struct PairF {
  float C1q, C2q, A4, E24;        // LJ force
  float Sq, qq, A, E4;            // LJ energy, centre-centre charge product
  float qpc, qcp, qpp, pad;
  double qqd, qpcd, qcpd, qppd;   // the charge products in FP64 (exclusions)
};
struct PairD {
  double C1q, C2q, A4, E24, Sq, qq, A, E4, qpc, qcp, qpp, pad;
};
// the FP32 fields of PairF alone (the first 48 bytes), as the cell pair
// kernel keeps them in shared memory
struct PairFS {
  float C1q, C2q, A4, E24;
  float Sq, qq, A, E4;
  float qpc, qcp, qpp, pad;
};
static_assert(sizeof(PairF) == 80 && sizeof(PairFS) == 48, "PairFS is the head of PairF");

// one k-space task: a run of <=KZT consecutive kz of one (kx,ky) column
struct KTask {
  int kx, ky, kz0, n;   // first kz and count
  int k0;               // index of (kx,ky,kz0) in the k list
  int pad[3];
};
// a (kx,ky) column of the k list
struct KCol {
  int kx, ky, kz0, n, k0, pad[3];
};

// a (kx,ky) row of the k set: kz in [kzlo,kzhi], k index kstart+(kz-kzlo)
struct KRow {
  int kx, ky, kzlo, kzhi, kstart, pad[3];
};
// KTR rows sharing the kz span [-R,R]
struct KTile {
  int row0, nrows, R, pad;
};
constexpr int KTR = 64;         // rows per k-space tile
// FP32 path: phase rows [X(0..Kx) | Y(-Ky..Ky) | Z(0..Kz)] (Z(-kz) is the
// conjugate of Z(kz), so one product serves +kz and -kz); pass-1 jobs cover
// kz in [kz0, kz0+KZC_MIXED) of [0, R]
constexpr int KZC_MIXED = 32;
inline int phase_row_mixed(int Kx, int Ky, int Kz) { return (Kx + 1) + (2 * Ky + 1) + (Kz + 1); }

// The body of a kernel that has a single-box launch and a batched launch
// (blockIdx.y = box): compiled once, not inlined, so that both launches run
// the same machine code.  Inlined into two kernels, the compiler may fuse a
// multiply and an add into an FMA in one and not in the other, and a box of
// a batch would no longer get its single-launch results bit for bit.  It
// runs once per CTA, so the call costs nothing measurable.
#ifdef __CUDACC__
#define MG_BODY __device__ __noinline__
#endif

// the SM count of a GB300, used to size fixed partitions of sums (pass-1
// charge chunks, Widom and Bussi partials): fixed rather than queried, so
// that the summation order, and with it the last bits, do not depend on the
// device
constexpr int PARTITION_SMS = 152;

constexpr int KZT = 4;          // kz per pass-1 thread
constexpr int PAIR_THREADS = 128;
constexpr int MAX_KINDS = 16;

struct Launch {
  cudaStream_t s;
  int* counter;  // number of kernel launches (diagnostics)
};

// kernels (mg_kernels.cu); each returns cudaGetLastError()
// the linked-cell list as a counting sort (four kernels): key [ns] cell of
// every site; count [ncell rounded up to 4] zero on entry and on return;
// cursor [ncell], slot_site [ns] scratch; out: order [ns] sorted -> site
// (by z, then site index, within a cell), key_s [ns] the sorted cells, start [ncell+1]
// pfix [ns] scratch: the fixed-point site records in site order; pj (or
// null) gets them in cell order: {x, y, z as 32-bit fractions of the box,
// (molecule << 8) | kind} (kind, mol: [ns] site tables).  gstart
// [ncell+1]: first group of each cell (groups: its sites in runs of
// GROUP_SITES, in cell order); gcell [ns / GROUP_SITES + ncell] (or null):
// the cell of every group
cudaError_t k_cell_list(const Launch& L, int ns, const double* r, int* status, const double iL[3],
                        int ncx, int ncy, int ncz, const int* kind, const int* mol, int4* pfix,
                        int* key, int* count, int* cursor, int* slot_site, int* order,
                        int* key_s, int* start, int* gstart, int4* pj, int* gcell);
// sites per work item (group) of the group pair kernel, its warps per CTA
constexpr int GROUP_SITES = 8;
constexpr int GROUP_WARPS = 4;
// the fixed-point records of the sorted sites for new positions and an
// unchanged order (neighbour lists kept from an earlier build)
cudaError_t k_gather_mixed(const Launch& L, int ns, const double* r, const int* order,
                           const int* kind, const int* mol, const double iL[3], int4* pj);
cudaError_t k_gather_fp64(const Launch& L, int ns, const double* r, const int* order,
                          const int* kind, const int* mol, double Lx, double Ly, double Lz,
                          double4* pd);
// Drude builds: sorted Drude displacements (second half of r)
cudaError_t k_gather_drude(const Launch& L, int ns, const double* r, const int* order,
                           float4* pdj, double4* pdd);

struct PairArgs {
  int ns, ncx, ncy, ncz, nstencil, nkind;
  int allpairs;             // one cell: nearest image taken per pair (FP64 path)
  const int* cell_start;
  const int* order;         // sorted -> site
  const int4* stencil;      // dx,dy,dz
  double Lx, Ly, Lz;
  double cutoff_sq;
  double sgrid;
  double alpha;
  double* f;                // [3*ns] output (original order), overwritten
  double* epart;            // [nblocks*10] partial energies (measure)
  int ntab;                 // erfc spline intervals (lookups are clamped)
  const float4* pdj;        // mixed, Drude builds: sorted Drude displacements
  int pair_warps;           // mixed cell kernel: warps per CTA (4 or 8)
  int spline_smem;          // mixed cell kernel: force spline in shared memory
  const double4* pdd;       // FP64, Drude builds: sorted Drude displacements
  // group pair kernel (FP32 path, grids with the nearest image per cell):
  // work items = groups of GROUP_SITES sites of a home cell (gstart, gcell),
  // the stencil as z-runs (dx, dy, dzlo, dzhi) of consecutive cells
  int group;
  const int* gstart;
  const int* gcell;
  const int4* spans;
  int nspans;
  int ngrid;                // CTAs of the group kernel (its energy rows)
  // the group kernel with Newton's third law (pair_variant 9: 1, lanes on
  // the home sites; pair_variant 10: 2, lanes on the neighbours, shells as
  // 1): the half-shell z-runs, and the 64-bit fixed-point force sums (2^-32
  // K/A units, sorted order, kept zero between evaluations)
  int newton;
  const int4* hspans;
  int nhspans;
  long long* facc;
};
cudaError_t k_pair_mixed(const Launch& L, const PairArgs& a, const int4* pj,
                         const PairF* ptab, const float4* erd, const float4* eru,
                         bool measure, bool polar);
cudaError_t k_pair_fp64(const Launch& L, const PairArgs& a, const double4* pd,
                        const PairD* ptab, const double* ertab, bool measure, bool polar);

struct KArgs {
  int nq, nk, ntask, ncol, nchunk;
  int Kx, Ky, Kz, row;      // table extents; row = (Kx+1)+(2Ky+1)+(2Kz+1)
  double Lx, Ly, Lz;
  double iLx, iLy, iLz;     // 1 / box edges (set_box)
  double alpha;
  const int* qsite;         // [nq] site of each charge
  const double* qval;       // [nq]
  const KTask* task;
  const KCol* col;
  const int4* kvec;         // [nk] kx,ky,kz
  const double* ekk;        // [nk]
  double* S;                // [2*nk] structure factor (FP64)
  float2* Wf;               // [nk] ekk conj(S) for the mixed back-transform (or NULL)
  double2* Wd;              // [nk] the same in FP64 (or NULL)
  double* f;                // forces (added)
  double* ek_part;          // [nk-blocks * 7] energy + virial partials
  const KRow* krows;        // rows sorted by kz extent
  const KTile* tiles;
  int ntile;
  const int2* p1job;        // pass-1 CTA jobs: (tile, first kz)
  int np1job;
  const int* qdrude;        // [nq] 1 if the charge is a Drude charge (or NULL)
  int ns;
  int* status;              // device status word (tensor-core waits that give up: 16)
};
inline void set_box(KArgs& a, const double L[3]) {
  a.Lx = L[0];
  a.Ly = L[1];
  a.Lz = L[2];
  a.iLx = 1.0 / L[0];
  a.iLy = 1.0 / L[1];
  a.iLz = 1.0 / L[2];
}
cudaError_t k_add_forces(const Launch& L, size_t n, const double* fk, double* f);
// qf: [nq] scratch for the charges' fixed-point coordinates
cudaError_t k_phase_tables_mixed(const Launch& L, const KArgs& a, const double* r, float2* tab,
                                 uint4* qf);
cudaError_t k_phase_tables_fp64(const Launch& L, const KArgs& a, const double* r, double2* tab);
cudaError_t k_sk_mixed(const Launch& L, const KArgs& a, const float2* tab, float2* part);
cudaError_t k_sk_fp64(const Launch& L, const KArgs& a, const double2* tab, double2* part);
cudaError_t k_sk_reduce_mixed(const Launch& L, const KArgs& a, const float2* part, bool measure);
cudaError_t k_sk_reduce_fp64(const Launch& L, const KArgs& a, const double2* part, bool measure);
cudaError_t k_kforce_mixed(const Launch& L, const KArgs& a, const float2* tab);
cudaError_t k_kforce_fp64(const Launch& L, const KArgs& a, const double2* tab);
cudaError_t k_sk_gemm_mixed(const Launch& L, const KArgs& a, const float2* tab, float2* part);
cudaError_t k_sk_gemm_fp64(const Launch& L, const KArgs& a, const double2* tab, double2* part);
cudaError_t k_kf_gemm_mixed(const Launch& L, const KArgs& a, const float2* tab);
cudaError_t k_kf_gemm_fp64(const Launch& L, const KArgs& a, const double2* tab);
cudaError_t k_reduce_sum(const Launch& L, const double* part, int nrows, int width, double* out);
// the dipole term of Ewald(2): M = sum q r into M[0..2] (part: [dipole_blocks(nq) * 3]
// scratch), then forces q (-c_d M_d) added to f (none when c is zero)
int dipole_blocks(int nq);
cudaError_t k_dipole(const Launch& L, const KArgs& a, const double* r, double* part, double* M,
                     const double c[3], double* f);
// pass 2 on the tensor cores (mg_kspace_tc.cu); KP = 2 Kz + 1 rounded up
// to 8; per k row (kx, ky) as floats and the offsets of X(kx), Y(ky) in the
// kernel's phase block
struct TcRow {
  float kx, ky;
  int ox, oy;
};
static_assert(sizeof(TcRow) == 16, "pass 2 reads a TcRow as one int4");
// the arguments of the tensor-core pass 2 (one CTA per 128 charges) and
// pass 1 (nrt row tiles x charge chunks) kernels
struct KfTc {
  int nq, ns, KP, ntm, ntn, nrows, nxy;
  const float* za;
  const float* vb;
  const TcRow* rows;
  const int* qsite;
  const int* qdrude;
  double Lx, Ly, Lz;
  double* f;
  int* status;
};
struct SkTc {
  int KP, KN, Kz, nrows, nrt, ngroups, gpc, row, oyl, nk;
  const float2* tab;   // phase rows, zero-padded to whole groups of 32 charges
  const float* zb;     // Z^T tiles
  const KRow* krows;
  float2* part;
  int* status;
};
// every argument of one box's tensor-core Ewald passes, as its single
// launches (k_kf_tc_phase, k_sk_tc, k_kf_tc) take them, with their grids
// and shared-memory sizes; the batched launches take an array of these
struct TcBox {
  KArgs ka;
  const double* r;
  float2* tab;
  float* za;
  float* zb;
  int KP, nxy, KN;
  SkTc sk;
  KfTc kf;
  const KRow* tckrows;   // the V-tile builder's rows and output
  float* vb;
  int g_phase, g_sk, g_vb, g_kf;
  size_t smem_phase, smem_sk, smem_kf;
};
// zb (and with it pass 1) may be NULL; part: pass 1's partial sums
void tc_box(const KArgs& a, int nrows, int nch, int gpc, const KRow* tckrows, const TcRow* rows,
            const double* r, float2* tab, float* za, float* zb, float* vb, float2* part,
            TcBox* out);
int kf_tc_kp(const KArgs& a);
bool kf_tc_fits(const KArgs& a, int nrows);
size_t kf_tc_za_floats(const KArgs& a);
size_t kf_tc_vb_floats(const KArgs& a, int nrows);
void kf_tc_rows(const KArgs& a, const std::vector<KRow>& krows, std::vector<TcRow>* out);
// the operand tiles of both passes from the phase rows (zb may be NULL)
cudaError_t k_kf_tc_za(const Launch& L, const KArgs& a, const float2* tab, float* za, float* zb);

// pass 1 on the tensor cores: KN = 2 Kz + 1 rounded up to 16 (at most 64);
// the phase rows must be zero-padded to whole groups of 32 charges
int sk_tc_kn(const KArgs& a);
bool sk_tc_fits(const KArgs& a);
size_t sk_tc_zb_floats(const KArgs& a);
// charge chunks of pass 1 (of PARTITION_SMS CTAs over the row tiles, at
// least 64 groups of 32 charges each: a CTA's set-up and pipeline drain
// cost about as much as 15 groups): a split fixed by the box
void sk_tc_split(const KArgs& a, int nrows, int* nch, int* gpc);

// the tensor-core passes of nbox boxes (d: device array of their TcBox;
// grid: the largest box grid; smem: the largest box's shared memory); a
// single box is a list of one.  Phase rows and operand tiles; pass 1;
// the V tiles from W (in the order of the tensor-core tiles, (kx, ky)
// order) and pass 2
cudaError_t k_batch_tc_phase(const Launch& L, const TcBox* d, int nbox, int grid, size_t smem);
cudaError_t k_batch_sk_tc(const Launch& L, const TcBox* d, int nbox, int grid, size_t smem);
cudaError_t k_batch_kf_tc(const Launch& L, const TcBox* d, int nbox, int gvb, int gkf,
                          size_t smem);

struct ShakeArgs {
  int nmol;
  const int* mol_first;
  const int* mol_cfirst;
  const int2* cons;
  const double* bondq;
  const double* imass;
  const double* mass;
  double hh, eps, omega;
  int maxit;
  // 1: the three-site sweeps in float-float arithmetic on the FP32 pipe
  // (mixed path); 0: FP64
  int ffsweep;
  double* r;
  double* r1;
  const double* f;
  double* p;           // scratch [3*ns]
  double* kin_part;    // [nblocks]
  // measured step (or null): per CTA [nblocks * 13] the constraint virial
  // sum, its tensor (xx yy zz yz zx xy) and the kinetic tensor sum
  double* meas_part;
  int* status;         // set to 1 on non-convergence
  // molecule wrapping after the step (cook's normalize): a molecule whose
  // lowest massive-site coordinate is outside [r0, r0 + L) moves by L
  int normalize;
  double r0, Lb[3];
  // Nose-Hoover (vhist != null): the friction displacement -Vfactor vpred
  // joins the unconstrained positions; vpred and Vfactor come from the
  // thermostat state nh (NoseSlot) and the history of r1 (nh_pred slots of
  // nstride doubles), which the kernel shifts by one step
  const double* nh;
  double* vhist;
  int nh_pred;
  long long nstride;
};
cudaError_t k_shake(const Launch& L, const ShakeArgs& a);

// Nose-Hoover thermostat state on the device: logs, h dlogs/dt, the
// predictor length k reached so far, the extended energy of the last step,
// then the history of h dlogs/dt (newest first)
enum NoseSlot { NH_LOGS = 0, NH_LOGSV = 1, NH_K = 2, NH_EXT = 3, NH_HIST = 4 };
constexpr int MG_NOSE_MAXPRED = 8;

// Ewald exclusion corrections of the intramolecular pairs, one thread per
// molecule (mixed cell path: the pair kernel skips these pairs)
struct ExclArgs {
  int nmol, ns;
  const int* xfirst;    // [nmol+1] pair range of each molecule
  const int2* xpair;    // (i, j), i < j, sites of one molecule
  const double4* xq;    // charge products: centre-centre, Drude(i)-centre(j),
                        // centre(i)-Drude(j), Drude-Drude
  double Lx, Ly, Lz, iLx, iLy, iLz, cutoff_sq;
  float alpha;
  const double* r;      // positions (+ Drude offsets in the second half)
  double* f;            // forces, added to
  double* epart;        // [nblocks * 10] energy rows (measure)
};
constexpr int EXCL_THREADS = 128;
cudaError_t k_excl_mixed(const Launch& L, const ExclArgs& a, bool measure, bool polar);

// ---- batches: one launch per kernel over all boxes ----
// One box of a batched MD step (non-polar boxes on the FP32 path whose
// Ewald passes run on the FP32 cores, cells re-binned at every step): the
// arguments of every kernel of its step and the CTAs each would be launched
// with.  The batched kernels take blockIdx.y (pass 1: blockIdx.z) as the
// box; CTAs beyond a box's own grid return at once.
struct BoxStep {
  // cell list
  int ns, ncx, ncy, ncz;
  double iL[3];
  const double* r;
  int* status;
  const int* kind;
  const int* mol;
  int4* pfix;
  int* key;
  int* count;
  int* cursor;
  int* slot_site;
  int* order;
  int* key_s;
  int* start;
  int* gstart;
  int4* pj;
  int* gcell;
  // r-space (the cell pair kernel, 4 warps per home cell)
  PairArgs pa;
  const PairF* ptab;
  const float4* erd;
  const float4* eru;
  float sx, sy, sz, cq, sg, al;
  ExclArgs xa;
  // k-space on the FP32 cores (the tensor-core passes take a TcBox; ka
  // serves both, its nchunk the chunk count of the box's pass 1)
  KArgs ka;
  float2* tab;
  uint4* qf;
  float2* part;
  // integrator
  ShakeArgs sa;
  // sums of a measured step: rows of part -> out, four of them
  const double* rpart[4];
  int rrows[4], rwidth[4];
  double* rout[4];
  // CTAs of each kernel
  int g_site, g_order, g_pair, g_excl, g_charge, g_phase, g_p1x, g_p1y, g_skr, g_kf, g_shake;
};
// the largest grid and shared memory of each kernel over the boxes (the
// FP32-core k-space kernels have zero grids for boxes on the tensor cores
// and the other way round; tc: the TcBox grids and shared memory)
struct BatchGrid {
  int site, order, pair, excl, charge, phase, p1x, p1y, skr, kf, shake;
  size_t pair_smem, kf_smem;
  int tc_phase, tc_sk, tc_vb, tc_kf;
  size_t tc_phase_smem, tc_sk_smem, tc_kf_smem;
  bool any_fp32, any_tc;
};
// the force evaluation up to Ewald pass 1 (the cell list; the pair and
// exclusion kernels and the FP32-core phase rows), then pass 1
// (mg_kspace.cu), then the S(k) sums and pass 2; then the step (SHAKE and,
// measured, the sums)
// out[i] = *p[i] for the n status words of a batch's boxes
cudaError_t k_gather_status(cudaStream_t s, const int* const* p, int n, int* out);
cudaError_t k_batch_cells(const Launch& L, const BoxStep* d, int nbox, const BatchGrid& g);
cudaError_t k_batch_pairs(const Launch& L, const BoxStep* d, int nbox, const BatchGrid& g,
                          bool measure);
cudaError_t k_batch_pass1(const Launch& L, const BoxStep* d, int nbox, const BatchGrid& g);
cudaError_t k_batch_sk_reduce(const Launch& L, const BoxStep* d, int nbox, const BatchGrid& g,
                              bool measure);
cudaError_t k_batch_pass2(const Launch& L, const BoxStep* d, int nbox, const BatchGrid& g);
cudaError_t k_batch_step(const Launch& L, const BoxStep* d, int nbox, const BatchGrid& g,
                         bool measure);
size_t kf_mixed_smem(const KArgs& a);
int kf_mixed_blocks(int nq);
int cell_site_blocks(int ns);
int cell_order_blocks(int ncell);


// neighbour lists (mg_nlist.cu)
struct ListArgs {
  int ncx, ncy, ncz, nstencil;   // build grid (cells >= (cutoff+skin)/cdiv)
  const int* cell_start;
  const int4* stencil;
  float sx, sy, sz;              // fixed-point -> A
  float rlist2;                  // (cutoff+skin)^2
  int cap;                       // list capacity per site
  long pitch;                    // row stride of nlist (= cap)
  int* nlist;                    // [ns*cap]: entry k of sorted site t at t*cap + k
  int* ncount;                   // [ns]
  int* status;                   // bit 4: capacity exceeded
};
// cell_of: [ns] cell of every sorted site (the sorted cell keys)
cudaError_t k_build_list(const Launch& L, const ListArgs& a, int ns, const int* cell_of,
                         const int4* pj);
// the same by warp per home cell with staged appends (grids of >= 2 cdiv + 1
// cells per edge; cap a multiple of 8)
cudaError_t k_build_list_cells(const Launch& L, const ListArgs& a, const int4* pj);
cudaError_t k_save_build(const Launch& L, int ns, const double* r, double* rb);
cudaError_t k_check_skin(const Launch& L, int ns, const double* r, const double* rb, double lim2,
                         const double Lb[3], int* status, int* dmax);
cudaError_t k_pair_list_mixed(const Launch& L, const PairArgs& a, const ListArgs& l,
                              const int4* pj, const PairF* ptab, const float4* erd,
                              const float4* eru, bool measure, bool polar);
cudaError_t k_pair_list_fp64(const Launch& L, const PairArgs& a, const ListArgs& l,
                             const double4* pd, const PairD* ptab, const double* ertab,
                             bool measure, bool polar);
int list_blocks(int ns, bool mixed);  // CTAs of the list pair kernels

// Drude sites (mg_drude.cu)
struct DrudeArgs {
  int nd, ns;
  const int* dsite;    // [nd] sites carrying a Drude charge
  const double* qc;    // [nd] central charge of the site
  const double* qp;    // [nd] Drude charge
  const double* aqq;   // [nd] alpha_qq = alphapol/qp^2
  double alpha;        // Ewald alpha
  double* part;        // [nblocks*8] el, self, Pvir0..5
  double minqq2;       // squared limit of the Drude displacement
  int* status;         // bit 2 set when a displacement reaches it
};
struct AspcCoef {
  int n;
  double b[12];
};
cudaError_t k_selffield(const Launch& L, const DrudeArgs& a, double omega, double* r, double* f,
                        double* hist_out);
cudaError_t k_aspc_predict(const Launch& L, const DrudeArgs& a, const double* hist, int K2, int h,
                           const AspcCoef& B, double* r);
// Widom insertions: nps ghost sites against the cell list of the last force
// evaluation; per-CTA sums of exp(-U/T) into part[], energies into U[]
constexpr int MAX_WPROBE = 8;
struct WidomArgs {
  long long n;
  unsigned long long seed;
  double T;
  int nps, nkind, ncx, ncy, ncz, nstencil, lanes_sites, ntab;
  const int* cell_start;
  const int4* stencil;
  double Lx, Ly, Lz, cutoff_sq, sgrid;
  const double* geom;  // [3*nps] site offsets of the ghost
  double* U;           // [n] or null
  double* part;        // [nblocks]
};
// thermostat after SHAKE (mg_thermo.cu)
struct ThermoArgs {
  int kind;              // 1 Berendsen, 2 Bussi, 3 Nose-Hoover
  int ns, nkin, nchi;    // sites, SHAKE kinetic partials, Bussi chi^2 partials
  double nf;             // degrees of freedom
  double T, tau, h;
  unsigned long long seed;
  long long* step;       // device step counter (Bussi stream), advanced per call
  double* zout;          // the factor of the step, or null
  double* nh;            // Nose-Hoover state (NoseSlot), kind 3
  int pred;              // Nose-Hoover predictor length
};
// cook's bounddr: r1 of every site limited to length drmax; rep[0] counts
// the sites reduced, rep[1] keeps the float bits of the smallest factor
cudaError_t k_bounddr(const Launch& L, int ns, double drmax, double* r1, unsigned int* rep);
// momentum drift removal: part [drift_blocks(ns) * 3] scratch, P [3] the
// summed momentum, vout [3] (or null) the drift per step that was removed
int drift_blocks(int ns);
cudaError_t k_remove_drift(const Launch& L, int ns, const double* mass, double total_mass,
                           double* r1, double* part, double* P, double* vout);
cudaError_t k_thermostat(const Launch& L, const ThermoArgs& a, const double* kin_part,
                         double* chi_part, double* r1);

// adjoint constants of one pair of site kinds (FP64)
struct AdjPair {
  double C1q, C2q, Sq, E4, A, A4;
  double dA, dA4;   // d/dsigma of the smoothing constants
  double eps, sig;  // epsilon > 0 (1 when the pair has no LJ), sigma
};
// per cell CTA: kind-pair sums [ncell][nkind^2][6]; per site dE/dq, dLoss/dq;
// k-space: tpart [ntch][nk][3], T [nk]
cudaError_t k_adjoint(const Launch& L, const PairArgs& pa, const KArgs& ka, const double4* pd,
                      const AdjPair* tab, const double* ert, const double2* ptab, const double* g,
                      const double* q, double4* gs, double* part, double* dEq, double* dLq,
                      double2* tpart, int ntch, double2* T);

// one box of a Widom launch (blockIdx.y): its arguments and data
struct WidomBox {
  WidomArgs a;
  const int4* pj;       // mixed: sorted fixed-point sites
  const double4* pd;    // FP64: sorted sites
  const PairF* tabf;    // [nps*nkind] ghost-site x site-kind constants
  const PairD* tabd;
  const float4* eru;    // erfc energy spline (mixed)
  const double* ert;    // erfc splines (FP64)
};
int widom_blocks(long long n);
// identity change of whole molecules (cook's XWidom): per listed molecule the
// r-space energy of its sites with the real and with the virtual constants,
// against the other molecules in the cell list of the last force evaluation
struct XWidomArgs {
  int nlist, nps, nkind, ncx, ncy, ncz, nstencil, lanes_sites, ntab;
  const int* list;        // [nlist] molecules
  const int* mol_first;
  const double* r;        // positions of the last force evaluation (site order)
  const int* cell_start;
  const int4* stencil;
  double Lx, Ly, Lz, cutoff_sq, sgrid, T;
  double* U;              // [nlist] energy changes, or null
  double* part;           // [nblocks] sums of exp(-dU/T)
  const int4* pj;
  const double4* pd;
  const PairF* tabf;      // [2][MAX_WPROBE][MAX_KINDS]: real site constants, then virtual
  const PairD* tabd;
  const float4* eru;
  const double* ert;
};
cudaError_t k_xwidom(const Launch& L, const XWidomArgs& a, bool fp64);
cudaError_t k_widom(const Launch& L, const WidomBox* boxes, int nbox, long long n, bool fp64);

cudaError_t k_drude_take(const Launch& L, const DrudeArgs& a, const double* r, double* out);
cudaError_t k_drude_put(const Launch& L, const DrudeArgs& a, const double* in, double* r);
cudaError_t k_fma_probe(cudaStream_t s, int blocks, int threads, int iters, float* out);

// linear dependant sites (r_d = sum_p w_p r_p; f_p += w_p f_d)
struct DependArgs {
  int ndep;
  const int* site;    // [ndep] dependant site, those of a molecule consecutive
  const int* first;   // [ndep+1] parent range
  const int* parent;  // parent sites
  const double* w;    // parent weights
  const int* mol;     // [ns] molecule of each site
  const int* type;    // [ndep] 0 Middle, 1 Rowlinson, 2 Lone (or null: all Middle)
  const double* par;  // [13 ndep] wz, x[3], y[3], tx[3], ty[3]
  // or null; else [7 ndep] per dependant row: the virial and the virial
  // tensor (xx yy zz yz zx xy) its redistribution adds (the out-of-plane
  // kinds), written by the thread of the molecule's first dependant, zero
  // in the other rows
  double* vpart;
};
cudaError_t k_depend_r(const Launch& L, const DependArgs& a, double* r);
// the dependants' forces onto their parents at positions r
cudaError_t k_depend_f(const Launch& L, const DependArgs& a, const double* r, double* f);
// one playback frame (float triples of ns sites) from the MD state
cudaError_t k_playback_frame(const Launch& L, int ns, int what, int flags, const double* r,
                             const double* r1, double ih, const double Lb[3], float* out);

}  // namespace mg
