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

cudaError_t k_sk_gemm_mixed(const Launch& L, const KArgs& a, const float2* tab, float2* part) {
  return launch_sk_gemm<float2>(L, a, tab, part);
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

cudaError_t k_kf_gemm_mixed(const Launch& L, const KArgs& a, const float2* tab) {
  return launch_kf_gemm<float2>(L, a, tab, a.Wf);
}
cudaError_t k_kf_gemm_fp64(const Launch& L, const KArgs& a, const double2* tab) {
  return launch_kf_gemm<double2>(L, a, tab, a.Wd);
}

}  // namespace mg
