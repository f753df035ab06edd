// Classical Ewald k-space sums as register-tiled complex products on the
// FP32 (or FP64) pipes.
//
// The half-space k set of cook (sim/ewald.c:410-510) is organised in "rows":
// one row per (kx,ky) with its contiguous kz range [kzlo,kzhi].  Rows are
// sorted by kz extent and grouped in tiles of TR rows; a tile spans
// kz in [-R,R] with R its largest |kz| (entries outside a row's range are
// padding).  With A_j(row) = q_j e^{2 pi i (kx x_j/Lx + ky y_j/Ly)} and
// Z_j(kz) = e^{2 pi i kz z_j/Lz} (per-charge phase rows built by
// k_phase_tables_*):
//
//   pass 1   S(row,kz)  = sum_j A_j(row) Z_j(kz)                 (split over j)
//   pass 2   H_j(row)   = sum_kz W(row,kz) Z_j(kz),  Hz_j = sum_kz kz W Z_j
//            F_j        = sum_row [kx/Lx, ky/Ly, 1/Lz] Im(A_j H_j | A_j Hz_j)
//
// with W = ekk conj(S) (sim/ewpass2.c: force = ekk k Im(conj(S) q e^{ikr})).
// Pass 1 partial sums are FP32 over a chunk of charges and reduced in FP64
// (k_sk_reduce_*); pass 2 sums a row tile in FP32 and folds it into FP64.
#include "mg_internal.h"

namespace mg {

template <typename T2>
struct Cx;
template <>
struct Cx<float2> {
  typedef float T;
  static __device__ __forceinline__ float2 zero() { return make_float2(0.f, 0.f); }
};
template <>
struct Cx<double2> {
  typedef double T;
  static __device__ __forceinline__ double2 zero() { return make_double2(0.0, 0.0); }
};

// a += b*c
template <typename T2>
__device__ __forceinline__ void cmac(T2& a, const T2 b, const T2 c) {
  a.x = fma(b.x, c.x, a.x);
  a.x = fma(-b.y, c.y, a.x);
  a.y = fma(b.x, c.y, a.y);
  a.y = fma(b.y, c.x, a.y);
}
template <typename T2>
__device__ __forceinline__ T2 cmul(const T2 b, const T2 c) {
  T2 r;
  r.x = b.x * c.x - b.y * c.y;
  r.y = b.x * c.y + b.y * c.x;
  return r;
}

// s + c += v, c carrying the low-order part lost by s (Kahan summation); the
// FP64 path adds directly
__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}
__device__ __forceinline__ void kahan_add(double& s, double&, double v) { s += v; }

// ------------------------------------------------------------ pass 1 --

constexpr int P1_THREADS = 128;
constexpr int P1_KC = 32;  // charges per shared-memory stage
constexpr int P1_NZ = 16;  // kz per CTA tile

// grid.x: (tile, kz chunk) pairs, grid.y: charge chunks.  Thread (tr, tz):
// rows tr+16i (i<4) of the tile, kz = kz0 + tz + 8m (m<2).
template <typename T2>
__global__ void __launch_bounds__(P1_THREADS)
    sk_gemm_kernel(KArgs a, const T2* __restrict__ tab, T2* __restrict__ part) {
  __shared__ T2 As[P1_KC][KTR];
  __shared__ T2 Bs[P1_KC][P1_NZ];
  __shared__ KRow rows[KTR];
  const int2 job = a.p1job[blockIdx.x];  // (tile, first kz)
  const KTile tile = a.tiles[job.x];
  const int kz0 = job.y;
  const int ch = blockIdx.y;
  const int j0 = (int)((long)a.nq * ch / a.nchunk), j1 = (int)((long)a.nq * (ch + 1) / a.nchunk);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tz = lane & 7, tr = (lane >> 3) + 4 * warp;
  const int oy = a.Kx + 1 + a.Ky, oz = a.Kx + 2 * a.Ky + 2 + a.Kz;
  for (int t = tid; t < KTR; t += P1_THREADS)
    rows[t] = t < tile.nrows ? a.krows[tile.row0 + t] : KRow{0, 0, 1, 0, 0, 0, 0, 0};
  T2 acc[4][2];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int m = 0; m < 2; m++) acc[i][m] = Cx<T2>::zero();
  __syncthreads();
  for (int js = j0; js < j1; js += P1_KC) {
    const int nst = min(P1_KC, j1 - js);
    for (int t = tid; t < P1_KC * KTR; t += P1_THREADS) {
      const int jj = t / KTR, rr = t % KTR;
      T2 v = Cx<T2>::zero();
      if (jj < nst && rr < tile.nrows) {
        const T2* R = tab + (long)(js + jj) * a.row;
        v = cmul(R[rows[rr].kx], R[oy + rows[rr].ky]);
      }
      As[jj][rr] = v;
    }
    for (int t = tid; t < P1_KC * P1_NZ; t += P1_THREADS) {
      const int jj = t / P1_NZ, zz = t % P1_NZ, kz = kz0 + zz;
      T2 v = Cx<T2>::zero();
      if (jj < nst && kz >= -a.Kz && kz <= a.Kz) v = tab[(long)(js + jj) * a.row + oz + kz];
      Bs[jj][zz] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int jj = 0; jj < P1_KC; jj++) {
      T2 av[4], bv[2];
#pragma unroll
      for (int i = 0; i < 4; i++) av[i] = As[jj][tr + 16 * i];
#pragma unroll
      for (int m = 0; m < 2; m++) bv[m] = Bs[jj][tz + 8 * m];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int m = 0; m < 2; m++) cmac(acc[i][m], av[i], bv[m]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int rr = tr + 16 * i;
    if (rr >= tile.nrows) continue;
    const KRow rw = rows[rr];
#pragma unroll
    for (int m = 0; m < 2; m++) {
      const int kz = kz0 + tz + 8 * m;
      if (kz >= rw.kzlo && kz <= rw.kzhi) part[(long)ch * a.nk + rw.kstart + (kz - rw.kzlo)] = acc[i][m];
    }
  }
}

template <typename T2>
static cudaError_t launch_sk_gemm(const Launch& L, const KArgs& a, const T2* tab, T2* part) {
  dim3 grid(a.np1job, a.nchunk);
  sk_gemm_kernel<T2><<<grid, P1_THREADS, 0, L.s>>>(a, tab, part);
  ++*L.counter;
  return cudaGetLastError();
}

// ---------------------------------------------- pass 1, FP32 pipelined --
//
// Z(-kz) = conj(Z(kz)), so with A = X(kx) Y(ky) = (ax, ay) and Z(kz) = (c, s)
//   S(row, kz) = sum (ax c - ay s, ax s + ay c),  S(row,-kz) = sum (ax c + ay s, ay c - ax s)
// share the four sums P = (sum ax c, sum ax s), Q = (sum ay s, sum ay c):
// two FFMA2 per (row, |kz|) give both signs.  CTA = (tile, |kz| chunk of
// <= 32) x charge chunk; thread (tr, tz) holds rows tr+16i (i<4) x
// |kz| = kz0+tz+8m (m < MZ <= 4).  The A products staged for a block of 16
// charges serve every kz of the tile; the phase values of the next block
// stream into shared memory with cp.async while the current one is
// multiplied (two buffers).  Each thread stages one fixed row rr = tid&63
// (and one fixed kz slot) for charges (tid>>6)+2u, so its gather offsets are
// constants.

constexpr int Q1_THREADS = 128;
constexpr int Q1_KC = 16;
constexpr int Q1_NZ = KZC_MIXED;

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, bool valid) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? 8 : 0;  // 0: nothing is read, the 8 bytes are zero-filled
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(gmem), "r"(n)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

struct SkSmem {
  float2 X[2][Q1_KC][KTR];
  float2 Y[2][Q1_KC][KTR];
  float2 Z[2][Q1_KC][Q1_NZ];
};

// the multiply loop of one stage for MZ kz groups (no per-group branches, so
// the compiler interleaves all 4 x MZ accumulator chains)
template <int MZ>
__device__ __forceinline__ void sk_stage_mac(const float2 (*X)[KTR], const float2 (*Z)[Q1_NZ],
                                             int tr, int tz, float2 (&P)[4][4],
                                             float2 (&Q)[4][4]) {
#pragma unroll 2
  for (int jj = 0; jj < Q1_KC; jj++) {
    float2 ax[4], ay[4], zv[MZ], zs[MZ];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const float2 v = X[jj][tr + 16 * i];
      ax[i] = make_float2(v.x, v.x);
      ay[i] = make_float2(v.y, v.y);
    }
#pragma unroll
    for (int m = 0; m < MZ; m++) {
      zv[m] = Z[jj][tz + 8 * m];
      zs[m] = make_float2(zv[m].y, zv[m].x);
    }
#pragma unroll
    for (int m = 0; m < MZ; m++)
#pragma unroll
      for (int i = 0; i < 4; i++) {
        P[i][m] = __ffma2_rn(ax[i], zv[m], P[i][m]);
        Q[i][m] = __ffma2_rn(ay[i], zs[m], Q[i][m]);
      }
  }
}

template <int MZ>
__device__ __forceinline__ void sk_gemm_mixed_body(const KArgs& a, const float2* __restrict__ tab,
                                                   float2* __restrict__ part, const KTile& tile,
                                                   int kz0, int nz, SkSmem& sm, const int ch) {
  auto& Xs = sm.X;
  auto& Ys = sm.Y;
  auto& Zs = sm.Z;
  const int j0 = (int)((long)a.nq * ch / a.nchunk), j1 = (int)((long)a.nq * (ch + 1) / a.nchunk);
  const int tid = threadIdx.x, tr = tid >> 3, tz = tid & 7;
  const int oy = a.Kx + 1 + a.Ky, oz = a.Kx + 2 * a.Ky + 2;
  // this thread's staging slots: row rr for charges jb + 2u; kz slot zz for
  // charges zb + 4u
  const int rr = tid & (KTR - 1), jb = tid >> 6;
  const int zz = tid & (Q1_NZ - 1), zb = tid / Q1_NZ;
  const bool vr = rr < tile.nrows, vz = zz < nz;
  const KRow myrow = vr ? a.krows[tile.row0 + rr] : KRow{0, 0, 1, 0, 0, 0, 0, 0};
  const int xoff = myrow.kx, yoff = oy + myrow.ky, zoff = oz + kz0 + zz;
  const int nstage = (j1 - j0 + Q1_KC - 1) / Q1_KC;
  auto issue = [&](int st, int buf) {
    const int js = j0 + st * Q1_KC;
#pragma unroll
    for (int u = 0; u < Q1_KC / 2; u++) {
      const int jj = jb + 2 * u;
      const bool vj = js + jj < j1;
      const float2* base = vj ? tab + (long)(js + jj) * a.row : tab;
      cp_async8(&Xs[buf][jj][rr], base + (vj && vr ? xoff : 0), vj && vr);
      cp_async8(&Ys[buf][jj][rr], base + (vj && vr ? yoff : 0), vj && vr);
    }
#pragma unroll
    for (int u = 0; u < Q1_KC * Q1_NZ / Q1_THREADS; u++) {
      const int jj = zb + (Q1_THREADS / Q1_NZ) * u;
      const bool vj = js + jj < j1;
      const float2* base = vj ? tab + (long)(js + jj) * a.row : tab;
      cp_async8(&Zs[buf][jj][zz], base + (vj && vz ? zoff : 0), vj && vz);
    }
    cp_async_commit();
  };
  float2 P[4][4], Q[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int m = 0; m < 4; m++) P[i][m] = Q[i][m] = make_float2(0.f, 0.f);
  if (nstage > 0) issue(0, 0);
  for (int st = 0; st < nstage; st++) {
    const int buf = st & 1;
    if (st + 1 < nstage) {
      issue(st + 1, buf ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    // A = X Y for the entries this thread staged (its own copies are complete)
#pragma unroll
    for (int u = 0; u < Q1_KC / 2; u++) {
      const int jj = jb + 2 * u;
      const float2 x = Xs[buf][jj][rr], y = Ys[buf][jj][rr];
      Xs[buf][jj][rr] = make_float2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
    }
    __syncthreads();
    sk_stage_mac<MZ>(Xs[buf], Zs[buf], tr, tz, P, Q);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int r = tr + 16 * i;
    if (r >= tile.nrows) continue;
    const KRow rw = a.krows[tile.row0 + r];
#pragma unroll
    for (int m = 0; m < MZ; m++) {
      const int kz = kz0 + tz + 8 * m;
      if (tz + 8 * m >= nz) continue;
      const float2 p = P[i][m], q = Q[i][m];
      if (kz >= rw.kzlo && kz <= rw.kzhi)
        part[(long)ch * a.nk + rw.kstart + (kz - rw.kzlo)] = make_float2(p.x - q.x, p.y + q.y);
      if (kz > 0 && -kz >= rw.kzlo && -kz <= rw.kzhi)
        part[(long)ch * a.nk + rw.kstart + (-kz - rw.kzlo)] = make_float2(p.x + q.x, q.y - p.y);
    }
  }
}

MG_BODY void sk_gemm_mixed_kernel_body(const KArgs& a,
    const float2* __restrict__ tab,
    float2* __restrict__ part,
    const int bx_,
    const int by_) {
  __shared__ __align__(16) SkSmem sm;
  const int2 job = a.p1job[bx_];
  const KTile tile = a.tiles[job.x];
  const int kz0 = job.y;
  const int nz = min(Q1_NZ, tile.R - kz0 + 1);
  switch ((nz + 7) >> 3) {
    case 1: sk_gemm_mixed_body<1>(a, tab, part, tile, kz0, nz, sm, by_); break;
    case 2: sk_gemm_mixed_body<2>(a, tab, part, tile, kz0, nz, sm, by_); break;
    case 3: sk_gemm_mixed_body<3>(a, tab, part, tile, kz0, nz, sm, by_); break;
    default: sk_gemm_mixed_body<4>(a, tab, part, tile, kz0, nz, sm, by_); break;
  }
}

__global__ void __launch_bounds__(Q1_THREADS)
    sk_gemm_mixed_kernel(const __grid_constant__ KArgs a, const float2* __restrict__ tab, float2* __restrict__ part) {
  sk_gemm_mixed_kernel_body(a, tab, part, blockIdx.x, blockIdx.y);
}

cudaError_t k_sk_gemm_mixed(const Launch& L, const KArgs& a, const float2* tab, float2* part) {
  dim3 grid(a.np1job, a.nchunk);
  sk_gemm_mixed_kernel<<<grid, Q1_THREADS, 0, L.s>>>(a, tab, part);
  ++*L.counter;
  return cudaGetLastError();
}
cudaError_t k_sk_gemm_fp64(const Launch& L, const KArgs& a, const double2* tab, double2* part) {
  return launch_sk_gemm<double2>(L, a, tab, part);
}

// ------------------------------------------------------------ pass 2 --

constexpr int P2_THREADS = 256;
constexpr int P2_NJ = 64;  // charges per CTA

// Thread (tj, tw): charges 4tj..4tj+3 of the CTA, rows tw+16i (i<4) of the
// current tile.  Z of the CTA's charges stays in shared memory for the
// whole kernel; W of one tile at a time.
template <typename T2>
__global__ void __launch_bounds__(P2_THREADS)
    kf_gemm_kernel(KArgs a, const T2* __restrict__ tab, const T2* __restrict__ W) {
  typedef typename Cx<T2>::T T;
  extern __shared__ unsigned char smem_raw[];
  const int nz = 2 * a.Kz + 1;
  T2* Zs = reinterpret_cast<T2*>(smem_raw);            // [nz][P2_NJ]
  T2* Ws = Zs + (size_t)nz * P2_NJ;                     // [nz][KTR]
  KRow* rows = reinterpret_cast<KRow*>(Ws + (size_t)nz * KTR);  // [KTR]
  float2* kxy = reinterpret_cast<float2*>(rows + KTR);  // [KTR] (kx, ky) as floats
  double* red = reinterpret_cast<double*>(kxy + KTR);   // [P2_THREADS][12]
  const int tid = threadIdx.x;
  const int tw = tid & 15, tj = tid >> 4;
  const int jbase = blockIdx.x * P2_NJ;
  const int oy = a.Kx + 1 + a.Ky, oz = a.Kx + 2 * a.Ky + 2 + a.Kz;
  for (int t = tid; t < nz * P2_NJ; t += P2_THREADS) {
    const int z = t / P2_NJ, c = t % P2_NJ, j = jbase + c;
    Zs[t] = j < a.nq ? tab[(long)j * a.row + oz - a.Kz + z] : Cx<T2>::zero();
  }
  // per-charge force sums over the tiles: compensated (Kahan) in the FP32
  // path, so that the fold costs FP32 and not FP64 instructions
  T F[4][3], Fc[4][3];
#pragma unroll
  for (int c = 0; c < 4; c++)
#pragma unroll
    for (int d = 0; d < 3; d++) F[c][d] = Fc[c][d] = 0;
  for (int ti = 0; ti < a.ntile; ti++) {
    const KTile tile = a.tiles[ti];
    const int R = tile.R;
    __syncthreads();
    for (int t = tid; t < KTR; t += P2_THREADS) {
      const KRow rw = t < tile.nrows ? a.krows[tile.row0 + t] : KRow{0, 0, 1, 0, 0, 0, 0, 0};
      rows[t] = rw;
      kxy[t] = make_float2((float)rw.kx, (float)rw.ky);
    }
    __syncthreads();
    for (int t = tid; t < (2 * R + 1) * KTR; t += P2_THREADS) {
      const int z = t / KTR, rr = t % KTR, kz = z - R;
      const KRow rw = rows[rr];
      Ws[t] = (kz >= rw.kzlo && kz <= rw.kzhi) ? W[rw.kstart + kz - rw.kzlo] : Cx<T2>::zero();
    }
    __syncthreads();
    T2 H[4][4], Hz[4][4];
#pragma unroll
    for (int c = 0; c < 4; c++)
#pragma unroll
      for (int i = 0; i < 4; i++) H[c][i] = Hz[c][i] = Cx<T2>::zero();
    T kz = (T)(-R);
    for (int z = 0; z < 2 * R + 1; z++, kz += (T)1) {
      const T2* Zrow = Zs + (size_t)(z - R + a.Kz) * P2_NJ + 4 * tj;
      const T2* Wrow = Ws + (size_t)z * KTR + tw;
      T2 zv[4], wv[4];
#pragma unroll
      for (int c = 0; c < 4; c++) zv[c] = Zrow[c];
#pragma unroll
      for (int i = 0; i < 4; i++) wv[i] = Wrow[16 * i];
#pragma unroll
      for (int c = 0; c < 4; c++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const T2 p = cmul(wv[i], zv[c]);
          H[c][i].x += p.x;
          H[c][i].y += p.y;
          Hz[c][i].x = fma(kz, p.x, Hz[c][i].x);
          Hz[c][i].y = fma(kz, p.y, Hz[c][i].y);
        }
    }
    // epilogue: A_j(row) from the phase rows, Im(A H) weighted by k
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int j = jbase + 4 * tj + c;
      if (j >= a.nq) continue;
      const T2* Rj = tab + (long)j * a.row;
      T g3[3] = {0, 0, 0};
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const int rr = tw + 16 * i;
        if (rr >= tile.nrows) continue;
        const KRow rw = rows[rr];
        const float2 kf = kxy[rr];
        const T2 A = cmul(Rj[rw.kx], Rj[oy + rw.ky]);
        const T g = A.x * H[c][i].y + A.y * H[c][i].x;
        g3[0] = fma((T)kf.x, g, g3[0]);
        g3[1] = fma((T)kf.y, g, g3[1]);
        g3[2] += A.x * Hz[c][i].y + A.y * Hz[c][i].x;
      }
#pragma unroll
      for (int d = 0; d < 3; d++) kahan_add(F[c][d], Fc[c][d], g3[d]);
    }
  }
  // sum over the 16 row slots of each charge
#pragma unroll
  for (int c = 0; c < 4; c++)
#pragma unroll
    for (int d = 0; d < 3; d++) red[tid * 12 + c * 3 + d] = (double)F[c][d] + (double)Fc[c][d];
  __syncthreads();
  if (tw == 0) {
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int j = jbase + 4 * tj + c;
      if (j >= a.nq) continue;
      double s[3] = {0, 0, 0};
      for (int w = 0; w < 16; w++)
        for (int d = 0; d < 3; d++) s[d] += red[(tj * 16 + w) * 12 + c * 3 + d];
      const int site = a.qsite[j];
      double* fo = a.f + 3 * (long)site + (a.qdrude && a.qdrude[j] ? 3 * (long)a.ns : 0);
      fo[0] += s[0] / a.Lx;
      fo[1] += s[1] / a.Ly;
      fo[2] += s[2] / a.Lz;
    }
  }
}

template <typename T2>
static cudaError_t launch_kf_gemm(const Launch& L, const KArgs& a, const T2* tab, const T2* W) {
  const int nz = 2 * a.Kz + 1;
  size_t smem = (size_t)nz * P2_NJ * sizeof(T2) + (size_t)nz * KTR * sizeof(T2) +
                KTR * (sizeof(KRow) + sizeof(float2)) + (size_t)P2_THREADS * 12 * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(kf_gemm_kernel<T2>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int grid = (a.nq + P2_NJ - 1) / P2_NJ;
  kf_gemm_kernel<T2><<<grid, P2_THREADS, smem, L.s>>>(a, tab, W);
  ++*L.counter;
  return cudaGetLastError();
}

// ---------------------------------------------- pass 2, FP32 pipelined --
//
// CTA = 32 charges; thread (tj, tw) = (warp, lane): charges 4tj..4tj+3,
// rows tw and tw+32 of the current tile.  With W+- = W(row, +-kz),
// P = W+ + W-, M = W+ - W- and Z(kz) = (c, s):
//   H  = W(row,0) + sum_{kz>0} (P.x c - M.y s,  M.x s + P.y c)
//   Hz =            sum_{kz>0} kz (M.x c - P.y s,  P.x s + M.y c)
// (Z(-kz) = conj Z(kz)): four FFMA2 per (charge, row, |kz|).  Z(0..Kz) and the
// X|Y phase values of the CTA's charges stay in shared memory for the whole
// kernel (the epilogue's A = X(kx) Y(ky) products read them there); W of the
// next tile streams in with cp.async while the current tile is multiplied.
// A warp owns whole charges, so the sum over its 32 row slots is a shuffle
// reduction.

constexpr int Q2_THREADS = 256;
constexpr int Q2_NJ = 32;

int kf_mixed_blocks(int nq) { return (nq + Q2_NJ - 1) / Q2_NJ; }

size_t kf_mixed_smem(const KArgs& a) {
  const int nz = a.Kz + 1, nw = 2 * a.Kz + 1, nxy = a.Kx + 1 + 2 * a.Ky + 1;
  return sizeof(float2) * ((size_t)nz * Q2_NJ + (size_t)Q2_NJ * nxy + 2 * (size_t)nw * KTR);
}

MG_BODY void kf_gemm_mixed_kernel_body(const KArgs& a,
    const float2* __restrict__ tab,
    const float2* __restrict__ W,
    const int bx_,
    const int by_) {
  extern __shared__ __align__(16) unsigned char smem_kf[];
  const int nz = a.Kz + 1, nw = 2 * a.Kz + 1, nxy = a.Kx + 1 + 2 * a.Ky + 1;
  float2* Zs = reinterpret_cast<float2*>(smem_kf);  // [nz][Q2_NJ]: Z(0..Kz)
  float2* XYs = Zs + (size_t)nz * Q2_NJ;            // [Q2_NJ][nxy]
  float2* Ws = XYs + (size_t)Q2_NJ * nxy;           // [2][nw][KTR]: W(kz = z - R)
  const int tid = threadIdx.x, tw = tid & 31, tj = tid >> 5;
  const int jbase = bx_ * Q2_NJ;
  const int oz = a.Kx + 2 * a.Ky + 2, oyl = a.Kx + 1 + a.Ky;
  for (int t = tid; t < nz * Q2_NJ; t += Q2_THREADS) {
    const int z = t / Q2_NJ, c = t % Q2_NJ, j = jbase + c;
    Zs[t] = j < a.nq ? tab[(long)j * a.row + oz + z] : make_float2(0.f, 0.f);
  }
  for (int t = tid; t < Q2_NJ * nxy; t += Q2_THREADS) {
    const int c = t / nxy, e = t % nxy, j = jbase + c;
    XYs[t] = j < a.nq ? tab[(long)j * a.row + e] : make_float2(0.f, 0.f);
  }
  // W staging: this thread copies row wr = tid&63, kz slots (tid>>6)+4u
  const int wr = tid & (KTR - 1), wz = tid >> 6;
  auto issue = [&](int ti, int buf) {
    const KTile tl = a.tiles[ti];
    const KRow rw = wr < tl.nrows ? a.krows[tl.row0 + wr] : KRow{0, 0, 1, 0, 0, 0, 0, 0};
    float2* dst = Ws + (size_t)buf * nw * KTR;
    for (int z = wz; z < 2 * tl.R + 1; z += Q2_THREADS / KTR) {
      const int kz = z - tl.R;
      const bool v = kz >= rw.kzlo && kz <= rw.kzhi;
      cp_async8(dst + z * KTR + wr, v ? W + rw.kstart + (kz - rw.kzlo) : W, v);
    }
    cp_async_commit();
  };
  float F[4][3], Fc[4][3];
#pragma unroll
  for (int c = 0; c < 4; c++)
#pragma unroll
    for (int d = 0; d < 3; d++) F[c][d] = Fc[c][d] = 0.f;
  if (a.ntile > 0) issue(0, 0);
  for (int ti = 0; ti < a.ntile; ti++) {
    const int buf = ti & 1;
    if (ti + 1 < a.ntile) {
      issue(ti + 1, buf ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const KTile tile = a.tiles[ti];
    const int R = tile.R;
    const float2* W0 = Ws + (size_t)buf * nw * KTR + (size_t)R * KTR;  // kz = 0
    float2 H[4][2], Hz[4][2];
#pragma unroll
    for (int i = 0; i < 2; i++) {
      const float2 w0 = W0[tw + 32 * i];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        H[c][i] = w0;
        Hz[c][i] = make_float2(0.f, 0.f);
      }
    }
    float kz = 1.f;
    for (int z = 1; z <= R; z++, kz += 1.f) {
      const float4* zp = reinterpret_cast<const float4*>(Zs + (size_t)z * Q2_NJ + 4 * tj);
      const float4 z01 = zp[0], z23 = zp[1];
      const float2 zv[4] = {make_float2(z01.x, z01.y), make_float2(z01.z, z01.w),
                            make_float2(z23.x, z23.y), make_float2(z23.z, z23.w)};
#pragma unroll
      for (int i = 0; i < 2; i++) {
        const float2 wp = W0[z * KTR + tw + 32 * i], wm = W0[-z * KTR + tw + 32 * i];
        const float Px = wp.x + wm.x, Py = wp.y + wm.y, Mx = wp.x - wm.x, My = wp.y - wm.y;
        const float2 h1 = make_float2(Px, Mx), h2 = make_float2(-My, Py);
        const float2 g1 = make_float2(kz * Mx, kz * Px), g2 = make_float2(-kz * Py, kz * My);
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const float2 zs = make_float2(zv[c].y, zv[c].x);
          H[c][i] = __ffma2_rn(h1, zv[c], H[c][i]);
          H[c][i] = __ffma2_rn(h2, zs, H[c][i]);
          Hz[c][i] = __ffma2_rn(g1, zv[c], Hz[c][i]);
          Hz[c][i] = __ffma2_rn(g2, zs, Hz[c][i]);
        }
      }
    }
    // epilogue: A_j(row) = X(kx) Y(ky) from shared memory, Im(A H) weighted by k
#pragma unroll
    for (int i = 0; i < 2; i++) {
      const int r = tw + 32 * i;
      if (r >= tile.nrows) continue;
      const KRow rw = a.krows[tile.row0 + r];
      const float kxf = (float)rw.kx, kyf = (float)rw.ky;
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const float2* xy = XYs + (size_t)(4 * tj + c) * nxy;
        const float2 X = xy[rw.kx], Y = xy[oyl + rw.ky];
        const float2 A = make_float2(X.x * Y.x - X.y * Y.y, X.x * Y.y + X.y * Y.x);
        const float g = A.x * H[c][i].y + A.y * H[c][i].x;
        kahan_add(F[c][0], Fc[c][0], kxf * g);
        kahan_add(F[c][1], Fc[c][1], kyf * g);
        kahan_add(F[c][2], Fc[c][2], A.x * Hz[c][i].y + A.y * Hz[c][i].x);
      }
    }
    __syncthreads();
  }
  // sum over the 32 row slots of the warp as compensated FP32 pairs (s, e)
  // (Knuth's TwoSum), so that only lane 0 touches the slow FP64 pipe
#pragma unroll
  for (int c = 0; c < 4; c++) {
    double s[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      float hi = F[c][d], lo = -Fc[c][d];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
        const float t = hi + h2, bb = t - hi;
        const float err = (hi - (t - bb)) + (h2 - bb);
        hi = t;
        lo = lo + l2 + err;
      }
      s[d] = (double)hi + (double)lo;
    }
    const int j = jbase + 4 * tj + c;
    if (tw == 0 && j < a.nq) {
      const int site = a.qsite[j];
      double* fo = a.f + 3 * (long)site + (a.qdrude && a.qdrude[j] ? 3 * (long)a.ns : 0);
      // the product rounded on its own (no fused multiply-add with the
      // running force), so that adding to the r-space forces here or in a
      // separate buffer gives the same bits
      fo[0] += __dmul_rn(s[0], 1.0 / a.Lx);
      fo[1] += __dmul_rn(s[1], 1.0 / a.Ly);
      fo[2] += __dmul_rn(s[2], 1.0 / a.Lz);
    }
  }
}

__global__ void __launch_bounds__(Q2_THREADS, 2)
    kf_gemm_mixed_kernel(const __grid_constant__ KArgs a, const float2* __restrict__ tab, const float2* __restrict__ W) {
  kf_gemm_mixed_kernel_body(a, tab, W, blockIdx.x, 0);
}

cudaError_t k_kf_gemm_mixed(const Launch& L, const KArgs& a, const float2* tab) {
  const size_t smem = kf_mixed_smem(a);
  cudaError_t e = cudaFuncSetAttribute(kf_gemm_mixed_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kf_gemm_mixed_kernel<<<(a.nq + Q2_NJ - 1) / Q2_NJ, Q2_THREADS, smem, L.s>>>(a, tab, a.Wf);
  ++*L.counter;
  return cudaGetLastError();
}
cudaError_t k_kf_gemm_fp64(const Launch& L, const KArgs& a, const double2* tab) {
  return launch_kf_gemm<double2>(L, a, tab, a.Wd);
}

// ----------------------------------------------------- the dipole term --
//
// Ewald(2)'s dipole term (sim/ewald.c:865-887, forces through the ADDFORCES
// of sim/ewaldf.c): with M = sum_i q_i r_i over the charges (Drude charges
// at r + rpol), every charge gets the force q_i ek, ek = -c M (isotropic:
// c = 4 pi / ((2 epsinf + 1) V); Yeh-Berkowitz: c = 4 pi / V on the selected
// axes, no force with bit 8).  FP64 throughout, M summed in a fixed order.

__device__ __forceinline__ void charge_position(const KArgs& a, const double* __restrict__ r,
                                                int j, double p[3]) {
  const int site = a.qsite[j];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    p[d] = r[3 * (long)site + d];
    if (a.qdrude && a.qdrude[j]) p[d] += r[3 * (long)a.ns + 3 * (long)site + d];
  }
}

constexpr int DIP_THREADS = 256;
__global__ void __launch_bounds__(DIP_THREADS)
dipole_moment_kernel(KArgs a, const double* __restrict__ r, double* __restrict__ part) {
  __shared__ double red[3][DIP_THREADS];
  const int j = blockIdx.x * DIP_THREADS + threadIdx.x;
  double m[3] = {0, 0, 0};
  if (j < a.nq) {
    double p[3];
    charge_position(a, r, j, p);
    const double q = a.qval[j];
#pragma unroll
    for (int d = 0; d < 3; d++) m[d] = q * p[d];
  }
#pragma unroll
  for (int d = 0; d < 3; d++) red[d][threadIdx.x] = m[d];
  __syncthreads();
  for (int w = DIP_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int d = 0; d < 3; d++) red[d][threadIdx.x] += red[d][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 3) part[3 * (long)blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

// forces q_i ek; ek from the reduced moment M (device) and the factors
__global__ void dipole_force_kernel(KArgs a, const double* __restrict__ M, double c0, double c1,
                                    double c2, double* __restrict__ f) {
  const int j = blockIdx.x * DIP_THREADS + threadIdx.x;
  if (j >= a.nq) return;
  const double q = a.qval[j];
  const int site = a.qsite[j];
  double* fo = f + 3 * (long)site + (a.qdrude && a.qdrude[j] ? 3 * (long)a.ns : 0);
  fo[0] += q * (-c0 * M[0]);
  fo[1] += q * (-c1 * M[1]);
  fo[2] += q * (-c2 * M[2]);
}

int dipole_blocks(int nq) { return (nq + DIP_THREADS - 1) / DIP_THREADS; }

cudaError_t k_dipole(const Launch& L, const KArgs& a, const double* r, double* part, double* M,
                     const double c[3], double* f) {
  const int nb = dipole_blocks(a.nq);
  dipole_moment_kernel<<<nb, DIP_THREADS, 0, L.s>>>(a, r, part);
  ++*L.counter;
  cudaError_t e = k_reduce_sum(L, part, nb, 3, M);
  if (e != cudaSuccess) return e;
  if (c[0] != 0 || c[1] != 0 || c[2] != 0) {
    dipole_force_kernel<<<nb, DIP_THREADS, 0, L.s>>>(a, M, c[0], c[1], c[2], f);
    ++*L.counter;
  }
  return cudaGetLastError();
}

}  // namespace mg

namespace mg {

// Ewald passes 1 and 2 of every box of a batch, one launch each (blockIdx.z
// / blockIdx.y the box; CTAs beyond a box's own grid return at once)
__global__ void __launch_bounds__(Q1_THREADS) batch_sk_gemm_kernel(const BoxStep* __restrict__ B) {
  const BoxStep& e = B[blockIdx.z];
  if ((int)blockIdx.x >= e.g_p1x || (int)blockIdx.y >= e.g_p1y) return;
  sk_gemm_mixed_kernel_body(e.ka, e.tab, e.part, blockIdx.x, blockIdx.y);
}

__global__ void __launch_bounds__(Q2_THREADS) batch_kf_gemm_kernel(const BoxStep* __restrict__ B) {
  const BoxStep& e = B[blockIdx.y];
  if ((int)blockIdx.x >= e.g_kf) return;
  kf_gemm_mixed_kernel_body(e.ka, e.tab, e.ka.Wf, blockIdx.x, 0);
}

cudaError_t k_batch_pass1(const Launch& L, const BoxStep* d, int nbox, const BatchGrid& g) {
  batch_sk_gemm_kernel<<<dim3(g.p1x, g.p1y, nbox), Q1_THREADS, 0, L.s>>>(d);
  ++*L.counter;
  return cudaGetLastError();
}

cudaError_t k_batch_pass2(const Launch& L, const BoxStep* d, int nbox, const BatchGrid& g) {
  cudaError_t e = cudaFuncSetAttribute(batch_kf_gemm_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)g.kf_smem);
  if (e != cudaSuccess) return e;
  batch_kf_gemm_kernel<<<dim3(g.kf, nbox), Q2_THREADS, g.kf_smem, L.s>>>(d);
  ++*L.counter;
  return cudaGetLastError();
}

}  // namespace mg
