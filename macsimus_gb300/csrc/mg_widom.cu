// Widom test-particle insertions on the device (cook/widom.c:175-288 Einsert,
// sim/simmeas.c:1821-1958 Widom).
//
// One warp per insertion: the ghost's sites are placed from a counter-based
// stream (insertion k, word c: the SplitMix64 output function of
// seed + (8k+c+1)*gamma, Steele, Lea and Flood, OOPSLA 2014), each site's
// energy against the box is summed over the cell stencil of its home cell
// in the cell list of the last force evaluation (cook uses the last cell
// list the same way), and lane 0 adds exp(-U/T) (skipped when -U/T <= -700,
// sim/simmeas.c:1934) to the warp's sum.  Lanes take stencil cells (or, for
// grids of few cells, the sites of one cell).  Sums per CTA in FP64, in a
// fixed order, so the result does not depend on scheduling.  blockIdx.y
// selects the box: one launch serves a whole batch of boxes, each with its
// own cell list, pair table and ghost.
#include "mg_internal.h"

namespace mg {

constexpr int WD_THREADS = 128;
constexpr int WD_WARPS = WD_THREADS / 32;

__device__ __forceinline__ unsigned long long wd_word(unsigned long long seed, long long k, int c) {
  unsigned long long z = seed + (unsigned long long)(8 * k + c + 1) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// uniform random rotation of Shoemake (Graphics Gems III, 1992) from words
// 3..5 of insertion k; identity for a one-site ghost
__device__ void wd_rotation(unsigned long long seed, long long k, int nps, double R[9]) {
  if (nps < 2) {
    R[0] = R[4] = R[8] = 1;
    R[1] = R[2] = R[3] = R[5] = R[6] = R[7] = 0;
    return;
  }
  const double s53 = 1.0 / 9007199254740992.0;
  const double u1 = (double)(wd_word(seed, k, 3) >> 11) * s53;
  const double u2 = (double)(wd_word(seed, k, 4) >> 11) * s53;
  const double u3 = (double)(wd_word(seed, k, 5) >> 11) * s53;
  const double a = sqrt(1 - u1), b = sqrt(u1);
  double s2, c2, s3, c3;
  sincospi(2 * u2, &s2, &c2);
  sincospi(2 * u3, &s3, &c3);
  const double x = a * s2, y = a * c2, z = b * s3, w = b * c3;
  R[0] = 1 - 2 * (y * y + z * z); R[1] = 2 * (x * y - z * w);     R[2] = 2 * (x * z + y * w);
  R[3] = 2 * (x * y + z * w);     R[4] = 1 - 2 * (x * x + z * z); R[5] = 2 * (y * z - x * w);
  R[6] = 2 * (x * z - y * w);     R[7] = 2 * (y * z + x * w);     R[8] = 1 - 2 * (x * x + y * y);
}

__device__ __forceinline__ int wd_wrap(int c, int n) { return c < 0 ? c + n : (c >= n ? c - n : c); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// the end of the kernel: per-warp Boltzmann sums into one FP64 value per CTA
__device__ __forceinline__ void wd_block_sum(double wacc, double* part) {
  __shared__ double ws[WD_WARPS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) ws[warp] = wacc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int w = 0; w < WD_WARPS; w++) s += ws[w];
    part[blockIdx.x] = s;
  }
}

// mixed path: fixed-point ghost sites, FP32 pair energies, FP64 sums per cell
__global__ void __launch_bounds__(WD_THREADS) widom_mixed_kernel(const WidomBox* __restrict__ boxes) {
  __shared__ PairF tab[MAX_WPROBE * MAX_KINDS];
  const WidomBox& B = boxes[blockIdx.y];
  const WidomArgs a = B.a;
  const int4* __restrict__ pj = B.pj;
  const float4* __restrict__ eru = B.eru;
  for (int t = threadIdx.x; t < a.nps * a.nkind; t += WD_THREADS) tab[t] = B.tabf[t];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * WD_WARPS;
  const float sx = (float)(a.Lx * 2.3283064365386963e-10), sy = (float)(a.Ly * 2.3283064365386963e-10),
              sz = (float)(a.Lz * 2.3283064365386963e-10);
  const float cq = (float)a.cutoff_sq, sgrid = (float)a.sgrid;
  double wacc = 0;
  for (long long k = blockIdx.x * (long long)WD_WARPS + (threadIdx.x >> 5); k < a.n; k += nw) {
    double R[9];
    wd_rotation(a.seed, k, a.nps, R);
    const unsigned px = (unsigned)(wd_word(a.seed, k, 0) >> 32),
                   py = (unsigned)(wd_word(a.seed, k, 1) >> 32),
                   pz = (unsigned)(wd_word(a.seed, k, 2) >> 32);
    double U = 0;
    for (int s = 0; s < a.nps; s++) {
      const double g0 = a.geom[3 * s], g1 = a.geom[3 * s + 1], g2 = a.geom[3 * s + 2];
      // site = point + R g, as 32-bit fractions of the box (wrap-around)
      const unsigned ux = px + (unsigned)(int)llrint((R[0] * g0 + R[1] * g1 + R[2] * g2) / a.Lx * 4294967296.0);
      const unsigned uy = py + (unsigned)(int)llrint((R[3] * g0 + R[4] * g1 + R[5] * g2) / a.Ly * 4294967296.0);
      const unsigned uz = pz + (unsigned)(int)llrint((R[6] * g0 + R[7] * g1 + R[8] * g2) / a.Lz * 4294967296.0);
      const int cx = (int)(((unsigned long long)ux * a.ncx) >> 32),
                cy = (int)(((unsigned long long)uy * a.ncy) >> 32),
                cz = (int)(((unsigned long long)uz * a.ncz) >> 32);
      const PairF* T = tab + s * a.nkind;
      const int s0 = a.lanes_sites ? 0 : lane, ds = a.lanes_sites ? 1 : 32;
      for (int st = s0; st < a.nstencil; st += ds) {
        const int4 o = a.stencil[st];
        const int c2 = (wd_wrap(cx + o.x, a.ncx) * a.ncy + wd_wrap(cy + o.y, a.ncy)) * a.ncz +
                       wd_wrap(cz + o.z, a.ncz);
        const int j0 = a.cell_start[c2], j1 = a.cell_start[c2 + 1];
        float u = 0;
        for (int j = j0 + (a.lanes_sites ? lane : 0); j < j1; j += a.lanes_sites ? 32 : 1) {
          const int4 q = pj[j];
          const float dx = (float)(int)(ux - (unsigned)q.x) * sx;
          const float dy = (float)(int)(uy - (unsigned)q.y) * sy;
          const float dz = (float)(int)(uz - (unsigned)q.z) * sz;
          const float rr = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          if (rr >= cq) continue;
          const PairF P = T[q.w & 255];
          if (rr < P.C2q) {
            if (rr < P.C1q) {
              const float x = P.Sq / rr, y = x * x * x;
              u += P.E4 * fmaf(y, y, -y);
            } else {
              const float x = rr - P.C2q;
              u += P.A * x * x;
            }
          }
          if (P.qq != 0.f) {
            const float4 e = __ldg(eru + min((int)(rr * sgrid), a.ntab - 1));
            u += (__fdividef(e.y, e.z + rr) + e.x) * P.qq;
          }
        }
        U += u;
      }
    }
    U = warp_sum(U);
    if (lane == 0) {
      if (a.U) a.U[k] = U;
      const double e = -U / a.T;
      if (e > -700) wacc += exp(e);
    }
  }
  wd_block_sum(wacc, a.part);
}

// FP64 path: the same in double, nearest image by rint
__global__ void __launch_bounds__(WD_THREADS) widom_fp64_kernel(const WidomBox* __restrict__ boxes) {
  __shared__ PairD tab[MAX_WPROBE * MAX_KINDS];
  const WidomBox& B = boxes[blockIdx.y];
  const WidomArgs a = B.a;
  const double4* __restrict__ pd = B.pd;
  const double* __restrict__ ert = B.ert;
  for (int t = threadIdx.x; t < a.nps * a.nkind; t += WD_THREADS) tab[t] = B.tabd[t];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * WD_WARPS;
  const double s32 = 2.3283064365386963e-10;
  double wacc = 0;
  for (long long k = blockIdx.x * (long long)WD_WARPS + (threadIdx.x >> 5); k < a.n; k += nw) {
    double R[9];
    wd_rotation(a.seed, k, a.nps, R);
    const double px = (double)(unsigned)(wd_word(a.seed, k, 0) >> 32) * s32 * a.Lx,
                 py = (double)(unsigned)(wd_word(a.seed, k, 1) >> 32) * s32 * a.Ly,
                 pz = (double)(unsigned)(wd_word(a.seed, k, 2) >> 32) * s32 * a.Lz;
    double U = 0;
    for (int s = 0; s < a.nps; s++) {
      const double g0 = a.geom[3 * s], g1 = a.geom[3 * s + 1], g2 = a.geom[3 * s + 2];
      const double x = px + (R[0] * g0 + R[1] * g1 + R[2] * g2);
      const double y = py + (R[3] * g0 + R[4] * g1 + R[5] * g2);
      const double z = pz + (R[6] * g0 + R[7] * g1 + R[8] * g2);
      const double fx = x / a.Lx - floor(x / a.Lx), fy = y / a.Ly - floor(y / a.Ly),
                   fz = z / a.Lz - floor(z / a.Lz);
      const int cx = min((int)(fx * a.ncx), a.ncx - 1), cy = min((int)(fy * a.ncy), a.ncy - 1),
                cz = min((int)(fz * a.ncz), a.ncz - 1);
      const PairD* T = tab + s * a.nkind;
      const int s0 = a.lanes_sites ? 0 : lane, ds = a.lanes_sites ? 1 : 32;
      for (int st = s0; st < a.nstencil; st += ds) {
        const int4 o = a.stencil[st];
        const int c2 = (wd_wrap(cx + o.x, a.ncx) * a.ncy + wd_wrap(cy + o.y, a.ncy)) * a.ncz +
                       wd_wrap(cz + o.z, a.ncz);
        const int j0 = a.cell_start[c2], j1 = a.cell_start[c2 + 1];
        for (int j = j0 + (a.lanes_sites ? lane : 0); j < j1; j += a.lanes_sites ? 32 : 1) {
          const double4 q = pd[j];
          double dx = x - q.x, dy = y - q.y, dz = z - q.z;
          dx -= a.Lx * rint(dx / a.Lx);
          dy -= a.Ly * rint(dy / a.Ly);
          dz -= a.Lz * rint(dz / a.Lz);
          const double rr = dx * dx + dy * dy + dz * dz;
          if (rr >= a.cutoff_sq) continue;
          const PairD P = T[(int)(__double_as_longlong(q.w) & 255)];
          if (rr < P.C2q) {
            if (rr < P.C1q) {
              const double xx = P.Sq / rr, yy = xx * xx * xx;
              U += P.E4 * (yy * yy - yy);
            } else {
              const double xx = rr - P.C2q;
              U += P.A * xx * xx;
            }
          }
          if (P.qq != 0) {
            const double* e = ert + 6 * min((int)(rr * a.sgrid), a.ntab - 1);
            U += (e[1] / (e[2] + rr) + e[0]) * P.qq;
          }
        }
      }
    }
    U = warp_sum(U);
    if (lane == 0) {
      if (a.U) a.U[k] = U;
      const double e = -U / a.T;
      if (e > -700) wacc += exp(e);
    }
  }
  wd_block_sum(wacc, a.part);
}

// ------------------------------------------------- identity change --
//
// cook/widom.c:16-170 (Eidchange), sim/simmeas.c:1961-2003 (XWidom): a warp
// per listed molecule; each of its sites against every site of the other
// molecules within the cutoff, with the virtual minus the real constants
// (smoothed LJ, erfc spline times the charge change); lane 0 adds
// exp(-dU/T) (skipped for -dU/T <= -700).

__device__ __forceinline__ float xw_lj(const PairF& P, float rr) {
  if (rr >= P.C2q) return 0.f;
  if (rr < P.C1q) {
    const float x = P.Sq / rr, y = x * x * x;
    return P.E4 * fmaf(y, y, -y);
  }
  const float x = rr - P.C2q;
  return P.A * x * x;
}
__device__ __forceinline__ double xw_lj(const PairD& P, double rr) {
  if (rr >= P.C2q) return 0.0;
  if (rr < P.C1q) {
    const double x = P.Sq / rr, y = x * x * x;
    return P.E4 * (y * y - y);
  }
  const double x = rr - P.C2q;
  return P.A * x * x;
}

__device__ __forceinline__ int xw_cell(double x, double L, int n) {
  const double s = x / L - floor(x / L);
  const int c = (int)(s * n);
  return c < 0 ? 0 : (c >= n ? n - 1 : c);
}

template <bool FP64>
__global__ void __launch_bounds__(WD_THREADS) xwidom_kernel(XWidomArgs a) {
  __shared__ PairF tf[FP64 ? 1 : 2 * MAX_WPROBE * MAX_KINDS];
  __shared__ PairD td[FP64 ? 2 * MAX_WPROBE * MAX_KINDS : 1];
  for (int t = threadIdx.x; t < 2 * MAX_WPROBE * MAX_KINDS; t += WD_THREADS) {
    if (FP64) td[t] = a.tabd[t];
    else tf[t] = a.tabf[t];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * WD_WARPS;
  const float sx = (float)(a.Lx * 2.3283064365386963e-10), sy = (float)(a.Ly * 2.3283064365386963e-10),
              sz = (float)(a.Lz * 2.3283064365386963e-10);
  const float cqf = (float)a.cutoff_sq, sgf = (float)a.sgrid;
  double wacc = 0;
  for (int l = blockIdx.x * WD_WARPS + (threadIdx.x >> 5); l < a.nlist; l += nw) {
    const int n = a.list[l], i0 = a.mol_first[n];
    double U = 0;
    for (int s = 0; s < a.nps; s++) {
      const double* ri = a.r + 3 * (long)(i0 + s);
      const double x = ri[0], y = ri[1], z = ri[2];
      const int cx = xw_cell(x, a.Lx, a.ncx), cy = xw_cell(y, a.Ly, a.ncy),
                cz = xw_cell(z, a.Lz, a.ncz);
      // the site as the cell list stores it: 32-bit box fraction (mixed) or
      // the position wrapped into the box (FP64)
      const unsigned ux = (unsigned)llrint((x / a.Lx - floor(x / a.Lx)) * 4294967296.0),
                     uy = (unsigned)llrint((y / a.Ly - floor(y / a.Ly)) * 4294967296.0),
                     uz = (unsigned)llrint((z / a.Lz - floor(z / a.Lz)) * 4294967296.0);
      const double wx = x - a.Lx * floor(x / a.Lx), wy = y - a.Ly * floor(y / a.Ly),
                   wz = z - a.Lz * floor(z / a.Lz);
      const int s0 = a.lanes_sites ? 0 : lane, ds = a.lanes_sites ? 1 : 32;
      for (int st = s0; st < a.nstencil; st += ds) {
        const int4 o = a.stencil[st];
        const int c2 = (wd_wrap(cx + o.x, a.ncx) * a.ncy + wd_wrap(cy + o.y, a.ncy)) * a.ncz +
                       wd_wrap(cz + o.z, a.ncz);
        const int j0 = a.cell_start[c2], j1 = a.cell_start[c2 + 1];
        double u = 0;
        for (int j = j0 + (a.lanes_sites ? lane : 0); j < j1; j += a.lanes_sites ? 32 : 1) {
          if (FP64) {
            const double4 q = a.pd[j];
            const long long w = __double_as_longlong(q.w);
            if ((int)(w >> 8) == n) continue;
            double dx = wx - q.x, dy = wy - q.y, dz = wz - q.z;
            dx -= a.Lx * rint(dx / a.Lx);
            dy -= a.Ly * rint(dy / a.Ly);
            dz -= a.Lz * rint(dz / a.Lz);
            const double rr = dx * dx + dy * dy + dz * dz;
            if (rr >= a.cutoff_sq) continue;
            const PairD& PR = td[s * MAX_KINDS + (int)(w & 255)];
            const PairD& PV = td[(MAX_WPROBE + s) * MAX_KINDS + (int)(w & 255)];
            u += xw_lj(PV, rr) - xw_lj(PR, rr);
            const double dq = PV.qq - PR.qq;
            if (dq != 0) {
              const double* e = a.ert + 6 * min((int)(rr * a.sgrid), a.ntab - 1);
              u += (e[1] / (e[2] + rr) + e[0]) * dq;
            }
          } else {
            const int4 q = a.pj[j];
            if ((q.w >> 8) == n) continue;
            const float dx = (float)(int)(ux - (unsigned)q.x) * sx;
            const float dy = (float)(int)(uy - (unsigned)q.y) * sy;
            const float dz = (float)(int)(uz - (unsigned)q.z) * sz;
            const float rr = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            if (rr >= cqf) continue;
            const PairF& PR = tf[s * MAX_KINDS + (q.w & 255)];
            const PairF& PV = tf[(MAX_WPROBE + s) * MAX_KINDS + (q.w & 255)];
            float du = xw_lj(PV, rr) - xw_lj(PR, rr);
            const float dq = PV.qq - PR.qq;
            if (dq != 0.f) {
              const float4 e = __ldg(a.eru + min((int)(rr * sgf), a.ntab - 1));
              du += (__fdividef(e.y, e.z + rr) + e.x) * dq;
            }
            u += du;
          }
        }
        U += u;
      }
    }
    U = warp_sum(U);
    if (lane == 0) {
      if (a.U) a.U[l] = U;
      const double e = -U / a.T;
      if (e > -700) wacc += exp(e);
    }
  }
  wd_block_sum(wacc, a.part);
}

cudaError_t k_xwidom(const Launch& L, const XWidomArgs& a, bool fp64) {
  const int nb = widom_blocks(a.nlist);
  if (fp64) xwidom_kernel<true><<<nb, WD_THREADS, 0, L.s>>>(a);
  else xwidom_kernel<false><<<nb, WD_THREADS, 0, L.s>>>(a);
  ++*L.counter;
  return cudaGetLastError();
}

int widom_blocks(long long n) {
  long long b = (n + WD_WARPS - 1) / WD_WARPS;
  return (int)(b < PARTITION_SMS * 8 ? (b > 0 ? b : 1) : PARTITION_SMS * 8);
}

cudaError_t k_widom(const Launch& L, const WidomBox* boxes, int nbox, long long n, bool fp64) {
  const dim3 grid(widom_blocks(n), nbox);
  if (fp64)
    widom_fp64_kernel<<<grid, WD_THREADS, 0, L.s>>>(boxes);
  else
    widom_mixed_kernel<<<grid, WD_THREADS, 0, L.s>>>(boxes);
  ++*L.counter;
  return cudaGetLastError();
}

}  // namespace mg
