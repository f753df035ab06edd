// k-space Ewald forces and energy for callers that cannot allocate device
// memory.
//
// Everything the Ewald kernels need besides the caller's inputs and outputs
// lives in one file-scope __device__ array (g_noalloc_scratch below): the
// per-charge phase rows, the FP32 partial structure factors, S(k), W(k), the
// k tables and the reduction slots.  The array is sized for at most
// MG_NOALLOC_MAX_CHARGES charges, MG_NOALLOC_MAX_KVEC k-vectors and phase rows
// of at most MG_NOALLOC_MAX_ROW entries; every GPU that loads the library
// keeps it resident until the process exits.  Host-side k tables are built in
// static host buffers, so no call allocates on the host either.
//
// The host cannot use the array's name as a device address: every call asks
// the runtime for the current device's address of the array
// (cudaGetSymbolAddress, with that device current; the lookup is cheap and
// stays right when the device's context is reset and the module reloaded),
// together with the device's SM count, which sizes the pass-1 split.
#include "../../include/macgpu.h"
#include "mg_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

using namespace mg;

namespace {

constexpr int MAXQ = MG_NOALLOC_MAX_CHARGES;
constexpr int MAXK = MG_NOALLOC_MAX_KVEC;
constexpr int MAXROW = MG_NOALLOC_MAX_ROW;
constexpr int MAXCHUNK = 32;
constexpr int MAXTILE = MAXK / KTR + 2;
constexpr int MAXJOB = MAXTILE * 8;
constexpr int MAXKB = MAXK / 256 + 1;

// byte offsets inside the scratch array (each part 256-byte aligned)
constexpr size_t al(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t OFF_TAB = 0;
constexpr size_t OFF_PART = OFF_TAB + al(sizeof(float2) * (size_t)MAXQ * MAXROW);
constexpr size_t OFF_S = OFF_PART + al(sizeof(float2) * (size_t)MAXCHUNK * MAXK);
constexpr size_t OFF_W = OFF_S + al(sizeof(double) * 2 * MAXK);
constexpr size_t OFF_EKK = OFF_W + al(sizeof(float2) * MAXK);
constexpr size_t OFF_KVEC = OFF_EKK + al(sizeof(double) * MAXK);
constexpr size_t OFF_ROWS = OFF_KVEC + al(sizeof(int4) * MAXK);
constexpr size_t OFF_TILES = OFF_ROWS + al(sizeof(KRow) * MAXK);
constexpr size_t OFF_JOBS = OFF_TILES + al(sizeof(KTile) * MAXTILE);
constexpr size_t OFF_QSITE = OFF_JOBS + al(sizeof(int2) * MAXJOB);
constexpr size_t OFF_EKPART = OFF_QSITE + al(sizeof(int) * MAXQ);
constexpr size_t OFF_SUMS = OFF_EKPART + al(sizeof(double) * 7 * MAXKB);
constexpr size_t OFF_QFIX = OFF_SUMS + al(sizeof(double) * 32);
constexpr size_t SCRATCH_BYTES = OFF_QFIX + al(sizeof(uint4) * MAXQ);

}  // namespace

// the scratch: shared by every call on a device; holds the last call's data
static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

namespace {

// errors are returned as status codes and described on stderr
int fail_na(int code, const char* msg) {
  fprintf(stderr, "%s\n", msg);
  return code;
}

// static host copies of the tables of one call
int4 h_kvec[MAXK];
double h_ekk[MAXK];
KRow h_rows[MAXK];
KTile h_tiles[MAXTILE];
int2 h_jobs[MAXJOB];
int h_kv[3 * MAXK];

bool near_integer(double x) {
  x -= (int)x;
  return std::fabs(0.5 - std::fabs(x - 0.5)) < 1e-9;
}

// cook's half-space k set (as kvector_set) into the static buffer; -1 if
// ill-defined, -2 if it exceeds MAXK
int kset_static(const double L[3], double* kappa) {
  double dK = 2e-9;
  for (int again = 0; again <= 25; again++) {
    bool retry = false;
    int n = 0;
    double Kk = (*kappa) * (*kappa);
    int kxmax = (int)(L[0] * *kappa);
    for (int kx = 0; kx <= kxmax && !retry; kx++) {
      double kxq = Kk - (kx / L[0]) * (kx / L[0]);
      double aux = L[1] * std::sqrt(kxq);
      if (near_integer(aux)) { retry = true; break; }
      int kymax = (int)aux;
      for (int ky = 0; ky <= kymax && !retry; ky++) {
        double kyq = kxq - (ky / L[1]) * (ky / L[1]);
        aux = L[2] * std::sqrt(kyq);
        if (near_integer(aux)) { retry = true; break; }
        int kzmax = (int)aux;
        for (int kz = !(kx + ky); kz <= kzmax; kz++) {
          int nz = (kx > 0) + (ky > 0) + (kz > 0);
          int c[4][3] = {{kx, ky, kz}, {kx, ky, -kz}, {kx, -ky, kz}, {kx, -ky, -kz}};
          int use[4] = {1, nz == 3 || (nz == 2 && kz != 0), nz == 3 || (nz == 2 && kz == 0), nz == 3};
          for (int m = 0; m < 4; m++) {
            if (!use[m]) continue;
            if (n >= MAXK) return -2;
            h_kv[3 * n] = c[m][0];
            h_kv[3 * n + 1] = c[m][1];
            h_kv[3 * n + 2] = c[m][2];
            n++;
          }
        }
      }
    }
    if (!retry) return n;
    *kappa += *kappa * dK;
    dK *= 1.4;
  }
  return -1;
}

__global__ void iota_kernel(int n, int* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = i;
}

// sum of q^2 over the charges in a fixed order (one CTA; the self term)
constexpr int SQ_THREADS = 256;
__global__ void sumq2_kernel(int n, const double* __restrict__ q, double* __restrict__ out) {
  __shared__ double red[SQ_THREADS];
  double s = 0;
  for (int i = threadIdx.x; i < n; i += SQ_THREADS) s += q[i] * q[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = SQ_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

}  // namespace

extern "C" int mg_ewald_kspace_noalloc(const double* r_dev, const double* q_dev, int nq,
                                       const double L[3], double alpha, double kappa,
                                       double* f_dev, double* energy, void* stream) {
  if (!r_dev || !q_dev || !f_dev || !L || nq <= 0 || !(alpha > 0) || !(kappa > 0))
    return fail_na(MG_ERR_ARG, "mg_ewald_kspace_noalloc: invalid argument");
  if (nq > MAXQ)
    return fail_na(MG_ERR_SIZE, "mg_ewald_kspace_noalloc: more charges than MG_NOALLOC_MAX_CHARGES");
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1)
    return fail_na(MG_ERR_CUDA, "mg_ewald_kspace_noalloc: no usable current device");
  // the current device's address of the scratch array (the current device
  // is the one the kernels below run on)
  void* sym = nullptr;
  if (cudaGetSymbolAddress(&sym, g_noalloc_scratch) != cudaSuccess || !sym)
    return fail_na(MG_ERR_CUDA, "mg_ewald_kspace_noalloc: cudaGetSymbolAddress failed");
  unsigned char* base = (unsigned char*)sym;

  // ---- k tables on the host (static buffers)
  double kap = kappa;
  int nk = kset_static(L, &kap);
  if (nk == -2)
    return fail_na(MG_ERR_SIZE, "mg_ewald_kspace_noalloc: more k-vectors than MG_NOALLOC_MAX_KVEC");
  if (nk <= 0) return fail_na(MG_ERR_ARG, "mg_ewald_kspace_noalloc: empty k-vector set");
  // k list sorted by (kx,ky,kz) so that each (kx,ky) row has consecutive kz
  {
    int idx[MAXK];
    for (int i = 0; i < nk; i++) idx[i] = i;
    std::sort(idx, idx + nk, [](int a, int b) {
      for (int d = 0; d < 3; d++)
        if (h_kv[3 * a + d] != h_kv[3 * b + d]) return h_kv[3 * a + d] < h_kv[3 * b + d];
      return false;
    });
    const double V = L[0] * L[1] * L[2], PIaq = -(M_PI / alpha) * (M_PI / alpha);
    for (int i = 0; i < nk; i++) {
      const int a = idx[i];
      h_kvec[i] = make_int4(h_kv[3 * a], h_kv[3 * a + 1], h_kv[3 * a + 2], 0);
      const double kk = (h_kvec[i].z / L[2]) * (h_kvec[i].z / L[2]) +
                        ((h_kvec[i].y / L[1]) * (h_kvec[i].y / L[1]) +
                         (h_kvec[i].x / L[0]) * (h_kvec[i].x / L[0]));
      h_ekk[i] = 4 / (kk * V) * std::exp(PIaq * kk);
    }
  }
  int Kx = 0, Ky = 0, Kz = 0;
  for (int i = 0; i < nk; i++) {
    Kx = std::max(Kx, std::abs(h_kvec[i].x));
    Ky = std::max(Ky, std::abs(h_kvec[i].y));
    Kz = std::max(Kz, std::abs(h_kvec[i].z));
  }
  const int rowlen = phase_row_mixed(Kx, Ky, Kz);
  if (rowlen > MAXROW)
    return fail_na(MG_ERR_SIZE, "mg_ewald_kspace_noalloc: phase row longer than MG_NOALLOC_MAX_ROW");
  int nrows = 0;
  for (int i = 0; i < nk;) {
    int j = i + 1;
    while (j < nk && h_kvec[j].x == h_kvec[i].x && h_kvec[j].y == h_kvec[i].y &&
           h_kvec[j].z == h_kvec[j - 1].z + 1)
      j++;
    h_rows[nrows++] = KRow{h_kvec[i].x, h_kvec[i].y, h_kvec[i].z, h_kvec[j - 1].z, i, {0, 0, 0}};
    i = j;
  }
  auto ext = [](const KRow& r) { return std::max(std::abs(r.kzlo), std::abs(r.kzhi)); };
  // rows by decreasing kz extent, stable: a counting sort over the extents
  // (std::stable_sort may take a temporary buffer from the heap)
  {
    static KRow tmp[MAXK];
    static int cnt[MAXK + 2];
    int emax = 0;
    for (int i = 0; i < nrows; i++) emax = std::max(emax, ext(h_rows[i]));
    if (emax > MAXK) return fail_na(MG_ERR_SIZE, "mg_ewald_kspace_noalloc: k set too long in z");
    std::fill(cnt, cnt + emax + 2, 0);
    for (int i = 0; i < nrows; i++) cnt[emax - ext(h_rows[i]) + 1]++;
    for (int e = 1; e <= emax + 1; e++) cnt[e] += cnt[e - 1];
    for (int i = 0; i < nrows; i++) tmp[cnt[emax - ext(h_rows[i])]++] = h_rows[i];
    std::copy(tmp, tmp + nrows, h_rows);
  }
  int ntile = 0, njob = 0;
  for (int r0 = 0; r0 < nrows; r0 += KTR) {
    const int n = std::min(KTR, nrows - r0);
    int R = 0;
    for (int i = r0; i < r0 + n; i++) R = std::max(R, ext(h_rows[i]));
    for (int kz0 = 0; kz0 <= R; kz0 += KZC_MIXED) {
      if (njob >= MAXJOB) return fail_na(MG_ERR_SIZE, "mg_ewald_kspace_noalloc: k tiling too large");
      h_jobs[njob++] = make_int2(ntile, kz0);
    }
    h_tiles[ntile++] = KTile{r0, n, R, 0};
  }
  const int nchunk = std::max(1, std::min(std::min(MAXCHUNK, std::max(1, nq / 64)),
                                          (8 * nsm + njob - 1) / njob));

  // ---- pointers into the scratch
  float2* tab = (float2*)(base + OFF_TAB);
  float2* part = (float2*)(base + OFF_PART);
  double* S = (double*)(base + OFF_S);
  float2* Wf = (float2*)(base + OFF_W);
  double* ekk = (double*)(base + OFF_EKK);
  int4* kvec = (int4*)(base + OFF_KVEC);
  KRow* rows = (KRow*)(base + OFF_ROWS);
  KTile* tiles = (KTile*)(base + OFF_TILES);
  int2* jobs = (int2*)(base + OFF_JOBS);
  int* qsite = (int*)(base + OFF_QSITE);
  double* ekpart = (double*)(base + OFF_EKPART);
  double* sums = (double*)(base + OFF_SUMS);
  uint4* qfix = (uint4*)(base + OFF_QFIX);

#define NA_CK(call)                                                     \
  do {                                                                  \
    if ((call) != cudaSuccess)                                          \
      return fail_na(MG_ERR_CUDA, "mg_ewald_kspace_noalloc: " #call);   \
  } while (0)
  NA_CK(cudaMemcpyAsync(kvec, h_kvec, sizeof(int4) * nk, cudaMemcpyHostToDevice, s));
  NA_CK(cudaMemcpyAsync(ekk, h_ekk, sizeof(double) * nk, cudaMemcpyHostToDevice, s));
  NA_CK(cudaMemcpyAsync(rows, h_rows, sizeof(KRow) * nrows, cudaMemcpyHostToDevice, s));
  NA_CK(cudaMemcpyAsync(tiles, h_tiles, sizeof(KTile) * ntile, cudaMemcpyHostToDevice, s));
  NA_CK(cudaMemcpyAsync(jobs, h_jobs, sizeof(int2) * njob, cudaMemcpyHostToDevice, s));
  // the output is overwritten: the back-transform adds to it
  NA_CK(cudaMemsetAsync(f_dev, 0, sizeof(double) * 3 * (size_t)nq, s));
  iota_kernel<<<(nq + 255) / 256, 256, 0, s>>>(nq, qsite);
  NA_CK(cudaGetLastError());

  int launches = 0;
  Launch Lc{s, &launches};
  KArgs ka;
  std::memset(&ka, 0, sizeof(ka));
  ka.nq = nq;
  ka.nk = nk;
  ka.nchunk = nchunk;
  ka.Kx = Kx;
  ka.Ky = Ky;
  ka.Kz = Kz;
  ka.row = rowlen;
  set_box(ka, L);
  ka.alpha = alpha;
  ka.qsite = qsite;
  ka.qval = q_dev;
  ka.kvec = kvec;
  ka.ekk = ekk;
  ka.S = S;
  ka.Wf = Wf;
  ka.Wd = nullptr;
  ka.f = f_dev;
  ka.ek_part = ekpart;
  ka.krows = rows;
  ka.tiles = tiles;
  ka.ntile = ntile;
  ka.p1job = jobs;
  ka.np1job = njob;
  ka.qdrude = nullptr;
  ka.ns = nq;
  NA_CK(k_phase_tables_mixed(Lc, ka, r_dev, tab, qfix));
  NA_CK(k_sk_gemm_mixed(Lc, ka, tab, part));
  NA_CK(k_sk_reduce_mixed(Lc, ka, part, true));
  NA_CK(k_kf_gemm_mixed(Lc, ka, tab));
  NA_CK(k_reduce_sum(Lc, ekpart, (nk + 255) / 256, 7, sums));
  // sums[0] = sum_k ekk |S|^2, sums[8] = sum q^2; both read in one copy
  // on the caller's stream
  sumq2_kernel<<<1, SQ_THREADS, 0, s>>>(nq, q_dev, sums + 8);
  NA_CK(cudaGetLastError());
  double e[9];
  NA_CK(cudaMemcpyAsync(e, sums, sizeof(e), cudaMemcpyDeviceToHost, s));
  NA_CK(cudaStreamSynchronize(s));
#undef NA_CK
  // k-space energy sum_k ekk |S|^2 / (4 pi) plus the self term
  if (energy) *energy = e[0] / (4 * M_PI) - alpha / 1.772453850905516 * e[8];
  return MG_OK;
}
