// sm_103a kernels of the cook force path.
//
//   cell list      k_cell_list: a counting sort of the sites by cell (count,
//                  scan, scatter, per-cell rank) with the fixed-point site
//                  records of the FP32 path; k_gather_* for the FP64 path
//   r-space sum    k_pair_mixed / k_pair_fp64: one CTA per home cell, its warps
//                  split the neighbour-cell stencil; neighbour cells are staged
//                  per warp in shared memory (16-byte loads) and every lane owns
//                  one home-cell site (full shell: each pair is evaluated from
//                  both ends, so no atomics and a fixed summation order).
//   k-space        k_phase_tables_* (per-charge e^{2 pi i n x/L} rows),
//                  k_sk_* (structure factor, FP32 partial sums per charge chunk),
//                  k_sk_reduce_* (FP64 sum of the partials, energy, virial),
//                  k_kforce_* (force back-transform, one thread per charge)
//   integrator     k_shake: leap-frog + SHAKE sweeps, one thread per molecule
//
// Mixed precision: positions enter the pair kernel as 32-bit fixed-point
// fractions of the box, so the nearest-image difference is an exact integer
// subtraction; pair arithmetic is FP32; per-site sums are carried in FP32
// within a neighbour-cell batch and folded into compensated FP32 sums; all
// global reductions are FP64 in a fixed order.
#include "mg_internal.h"
#include "mg_device.cuh"

namespace mg {

#define LAUNCHED(L) (++*(L).counter)

static inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

// ------------------------------------------------------------- cell list --



// ------------------------------------------------------ the cell list --
//
// cook threads the sites of every cell into a linked list
// (cook/linklist.c:38-269).  Here the cells are runs of one array: the sites
// sorted by cell and within a cell by z, then site index (a fixed order, so
// the order and every sum over it are the same run to run), cell c holding
// order[start[c] .. start[c+1]).  A counting sort in four kernels:
//   cell_count    key of every site, sites per cell (atomic increments)
//   cell_scan     one CTA: start = exclusive scan of the counts, cursor =
//                 start, the counts zeroed again for the next list
//   cell_scatter  every site into a free slot of its cell (atomic cursor)
//   cell_order    a warp per cell ranks its sites by z (then site index)
//                 and writes order[] and the sorted keys (the slots of
//                 cell_scatter depend on the timing of the atomics; the ranks
//                 do not)

// the fixed-point record of every site (site order) and its cell, from the
// fixed-point coordinates (so that the cell and the coordinates the pair
// kernels use agree to the last bit); a non-finite coordinate sets bit 1 of
// *status and the site is binned into cell 0 so that every later index
// stays in range
MG_BODY void cell_count_kernel_body(int ns, const double* __restrict__ r, const double* iL,
                                   int ncx, int ncy, int ncz, const int* __restrict__ kind,
                                   const int* __restrict__ mol, int4* __restrict__ pfix,
                                   int* __restrict__ key, int* __restrict__ count,
                                   int* __restrict__ status, const int bx_) {
  const int i = bx_ * blockDim.x + threadIdx.x;
  if (i >= ns) return;
  const double x = r[3 * i], y = r[3 * i + 1], z = r[3 * i + 2];
  int k = 0;
  const int4 q = make_int4(fixed32(x, iL[0]), fixed32(y, iL[1]), fixed32(z, iL[2]),
                           (mol[i] << 8) | kind[i]);
  if (isfinite(x) && isfinite(y) && isfinite(z)) {
    k = (fixed_cell(q.x, ncx) * ncy + fixed_cell(q.y, ncy)) * ncz + fixed_cell(q.z, ncz);
  } else {
    atomicOr(status, 2);
  }
  pfix[i] = q;
  key[i] = k;
  atomicAdd(count + k, 1);
}

struct Inv3 {
  double v[3];
};

__global__ void cell_count_kernel(int ns, const double* __restrict__ r, const __grid_constant__ Inv3 iL, int ncx,
                                  int ncy, int ncz, const int* __restrict__ kind,
                                  const int* __restrict__ mol, int4* __restrict__ pfix,
                                  int* __restrict__ key, int* __restrict__ count,
                                  int* __restrict__ status) {
  cell_count_kernel_body(ns, r, iL.v, ncx, ncy, ncz, kind, mol, pfix, key, count, status,
                         blockIdx.x);
}

// exclusive scan of count[0..ncell) into start[0..ncell] and cursor[], in
// tiles of 4 x 1024 counts (int4 loads; count is padded with zeros to a
// multiple of 4 entries); the counts are cleared for the next list.  With
// gstart the same scan of the group counts ceil(count / GROUP_SITES) (the
// work items of the group pair kernel) goes to gstart[0..ncell].
constexpr int SCAN_THREADS = 1024;
__device__ __forceinline__ int2 add2(int2 a, int2 b) { return make_int2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ int2 shfl_up2(int2 v, int o) {
  return make_int2(__shfl_up_sync(0xffffffffu, v.x, o), __shfl_up_sync(0xffffffffu, v.y, o));
}
__device__ __forceinline__ int ngroups(int n) { return (n + GROUP_SITES - 1) / GROUP_SITES; }

MG_BODY void cell_scan_kernel_body(int ncell,
    int* __restrict__ count,
    int* __restrict__ start,
    int* __restrict__ cursor,
    int* __restrict__ gstart,
    const int bx_,
    const int by_) {
  __shared__ int2 wsum[SCAN_THREADS / 32];
  __shared__ int2 carry_s;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (t == 0) carry_s = make_int2(0, 0);
  __syncthreads();
  const int n4 = (ncell + 3) / 4;
  for (int base = 0; base < n4; base += SCAN_THREADS) {
    const int q = base + t;
    int4 v = make_int4(0, 0, 0, 0);
    if (q < n4) {
      v = reinterpret_cast<int4*>(count)[q];
      reinterpret_cast<int4*>(count)[q] = make_int4(0, 0, 0, 0);
    }
    // (sites, groups) of the four cells
    const int2 tot = make_int2(v.x + v.y + v.z + v.w,
                               ngroups(v.x) + ngroups(v.y) + ngroups(v.z) + ngroups(v.w));
    int2 incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int2 y = shfl_up2(incl, o);
      if (lane >= o) incl = add2(incl, y);
    }
    if (lane == 31) wsum[w] = incl;
    const int2 carry = carry_s;
    __syncthreads();
    if (w == 0) {
      int2 x = wsum[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int2 y = shfl_up2(x, o);
        if (lane >= o) x = add2(x, y);
      }
      wsum[lane] = x;   // inclusive sums of the warps
    }
    __syncthreads();
    const int2 wprev = w ? wsum[w - 1] : make_int2(0, 0);
    const int ex = carry.x + wprev.x + incl.x - tot.x;
    const int gx = carry.y + wprev.y + incl.y - tot.y;
    if (q < n4) {
      const int e[4] = {ex, ex + v.x, ex + v.x + v.y, ex + v.x + v.y + v.z};
      const int g[4] = {gx, gx + ngroups(v.x), gx + ngroups(v.x) + ngroups(v.y),
                        gx + ngroups(v.x) + ngroups(v.y) + ngroups(v.z)};
#pragma unroll
      for (int k = 0; k < 4; k++)
        if (4 * q + k < ncell) {
          start[4 * q + k] = e[k];
          cursor[4 * q + k] = e[k];
          if (gstart) gstart[4 * q + k] = g[k];
        }
    }
    __syncthreads();
    if (t == SCAN_THREADS - 1) carry_s = add2(carry, wsum[31]);
    __syncthreads();
  }
  if (t == 0) {
    start[ncell] = carry_s.x;
    if (gstart) gstart[ncell] = carry_s.y;
  }
}

__global__ void __launch_bounds__(SCAN_THREADS)
cell_scan_kernel(int ncell, int* __restrict__ count, int* __restrict__ start, int* __restrict__ cursor, int* __restrict__ gstart) {
  cell_scan_kernel_body(ncell, count, start, cursor, gstart, blockIdx.x, 0);
}

__global__ void cell_scatter_kernel(int ns, const int* __restrict__ key, int* __restrict__ cursor,
                                    int* __restrict__ slot_site) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns) return;
  slot_site[atomicAdd(cursor + key[i], 1)] = i;
}

constexpr int ORDER_THREADS = 256;
MG_BODY void cell_order_kernel_body(int ncell,
    const int* __restrict__ start,
    const int* __restrict__ slot_site,
    const int4* __restrict__ pfix,
    int* __restrict__ order,
    int* __restrict__ key_s,
    int4* __restrict__ pj,
    const int* __restrict__ gstart,
    int* __restrict__ gcell,
    const int bx_,
    const int by_) {
  const int c = bx_ * (ORDER_THREADS / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= ncell) return;
  const int s0 = start[c], n = start[c + 1] - s0;
  // the cell of each of its groups (work items of the group pair kernel)
  if (gcell)
    for (int g = gstart[c] + lane; g < gstart[c + 1]; g += 32) gcell[g] = c;
  // the sites of a cell in increasing z (ties by site index): runs of
  // consecutive sites are then thin slabs, which the group kernel's
  // bounding boxes prune well
  if (n <= 32) {
    // one site per lane, ranks by shuffles
    const int mine = lane < n ? slot_site[s0 + lane] : 0x7fffffff;
    const unsigned mz = lane < n ? (unsigned)pfix[mine].z : 0xffffffffu;
    int rank = 0;
    for (int j = 0; j < n; j++) {
      const int os = __shfl_sync(0xffffffffu, mine, j);
      const unsigned oz = __shfl_sync(0xffffffffu, mz, j);
      rank += oz < mz || (oz == mz && os < mine);
    }
    if (lane < n) {
      order[s0 + rank] = mine;
      key_s[s0 + rank] = c;
      if (pj) pj[s0 + rank] = pfix[mine];
    }
  } else {
    for (int e = lane; e < n; e += 32) {
      const int mine = slot_site[s0 + e];
      const unsigned mz = (unsigned)pfix[mine].z;
      int rank = 0;
      for (int j = 0; j < n; j++) {
        const int os = slot_site[s0 + j];
        const unsigned oz = (unsigned)pfix[os].z;
        rank += oz < mz || (oz == mz && os < mine);
      }
      order[s0 + rank] = mine;
      key_s[s0 + rank] = c;
      if (pj) pj[s0 + rank] = pfix[mine];
    }
  }
}

__global__ void __launch_bounds__(ORDER_THREADS)
cell_order_kernel(int ncell, const int* __restrict__ start, const int* __restrict__ slot_site, const int4* __restrict__ pfix, int* __restrict__ order, int* __restrict__ key_s, int4* __restrict__ pj, const int* __restrict__ gstart, int* __restrict__ gcell) {
  cell_order_kernel_body(ncell, start, slot_site, pfix, order, key_s, pj, gstart, gcell, blockIdx.x, 0);
}

cudaError_t k_cell_list(const Launch& L, int ns, const double* r, int* status, const double iL[3],
                        int ncx, int ncy, int ncz, const int* kind, const int* mol, int4* pfix,
                        int* key, int* count, int* cursor, int* slot_site, int* order,
                        int* key_s, int* start, int* gstart, int4* pj, int* gcell) {
  const int ncell = ncx * ncy * ncz;
  const Inv3 il{{iL[0], iL[1], iL[2]}};
  cell_count_kernel<<<cdiv(ns, 256), 256, 0, L.s>>>(ns, r, il, ncx, ncy, ncz, kind, mol, pfix, key,
                                                    count, status);
  LAUNCHED(L);
  cell_scan_kernel<<<1, SCAN_THREADS, 0, L.s>>>(ncell, count, start, cursor, gstart);
  LAUNCHED(L);
  cell_scatter_kernel<<<cdiv(ns, 256), 256, 0, L.s>>>(ns, key, cursor, slot_site);
  LAUNCHED(L);
  cell_order_kernel<<<cdiv(ncell, ORDER_THREADS / 32), ORDER_THREADS, 0, L.s>>>(
      ncell, start, slot_site, pfix, order, key_s, pj, gstart, gcell);
  LAUNCHED(L);
  return cudaGetLastError();
}

__global__ void gather_mixed_kernel(int ns, const double* __restrict__ r,
                                    const int* __restrict__ order, const int* __restrict__ kind,
                                    const int* __restrict__ mol, double iLx, double iLy,
                                    double iLz, int4* __restrict__ pj) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ns) return;
  int i = order[t];
  pj[t] = make_int4(fixed32(r[3 * i], iLx), fixed32(r[3 * i + 1], iLy),
                    fixed32(r[3 * i + 2], iLz), (mol[i] << 8) | kind[i]);
}

cudaError_t k_gather_mixed(const Launch& L, int ns, const double* r, const int* order,
                           const int* kind, const int* mol, const double iL[3], int4* pj) {
  gather_mixed_kernel<<<cdiv(ns, 256), 256, 0, L.s>>>(ns, r, order, kind, mol, iL[0], iL[1],
                                                      iL[2], pj);
  LAUNCHED(L);
  return cudaGetLastError();
}

__global__ void gather_fp64_kernel(int ns, const double* __restrict__ r,
                                   const int* __restrict__ order, const int* __restrict__ kind,
                                   const int* __restrict__ mol, double Lx, double Ly, double Lz,
                                   double4* __restrict__ pd) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ns) return;
  int i = order[t];
  double x = r[3 * i], y = r[3 * i + 1], z = r[3 * i + 2];
  x -= Lx * floor(x / Lx);
  y -= Ly * floor(y / Ly);
  z -= Lz * floor(z / Lz);
  pd[t] = make_double4(x, y, z, __longlong_as_double((long long)((mol[i] << 8) | kind[i])));
}

cudaError_t k_gather_fp64(const Launch& L, int ns, const double* r, const int* order,
                          const int* kind, const int* mol, double Lx, double Ly, double Lz,
                          double4* pd) {
  gather_fp64_kernel<<<cdiv(ns, 256), 256, 0, L.s>>>(ns, r, order, kind, mol, Lx, Ly, Lz, pd);
  LAUNCHED(L);
  return cudaGetLastError();
}

// ---------------------------------------------------------- pair kernels --

constexpr int NWARP = PAIR_THREADS / 32;
constexpr int FOLD = 8;   // stencil cells per FP32 force batch before the FP64 fold

// One CTA per home cell; its 4 warps split the neighbour-cell stencil, each
// staging 32 neighbour sites at a time in shared memory; lane = home site.
// Full shell: forces only on the home site.  POLAR adds the Drude terms of
// cook/ljqqpol.c (centre-Drude, Drude-centre, Drude-Drude, each at its own
// separation); Drude forces go to the second half of f.
//
// REL (every grid of at least 2 cdiv + 1 cells per edge): a staged site is
// converted once, as the float offset of its nearest image from the centre
// of the home cell (exact 32-bit fixed-point difference, then one rounding);
// a pair then costs three subtractions and no int-to-float conversion
// (conversions are slow on this GPU).  Every stencil cell lies within half a
// box of the home-cell centre, so the image taken is the nearest one for
// every pair inside the cutoff.  Without REL (one cell: all pairs) each pair
// takes its nearest image from its own fixed-point difference.
// NW warps per CTA (the autotuner picks 4, 8 or 16: more warps per home
// cell finish a cell sooner, which shortens the tail of the grid); STAB: the
// force spline in
// shared memory (dynamic, ntab float4) instead of read through L1.
// Intramolecular pairs are skipped: their Ewald exclusion terms come from
// excl_mixed_kernel, once per pair.  Forces are summed in FP32 per batch of
// FOLD stencil cells and folded into an FP32 sum with a compensation term
// (Knuth's TwoSum): no FP64 instruction in the loop (the FP64 pipe of this
// GPU is narrow and also serves the float/double conversions).
template <bool MEASURE, bool POLAR, bool REL, int NW, bool STAB>
MG_BODY void pair_mixed_kernel_body(const PairArgs& a,
    const int4* __restrict__ pj,
    const PairF* __restrict__ ptab_g,
    const float4* __restrict__ erd_g,
    const float4* __restrict__ eru,
    float sx,
    float sy,
    float sz,
    float cq,
    float sgrid,
    float alpha,
    const int bx_,
    const int by_) {
  constexpr int NT = NW * 32;
  // dynamic shared memory: the nk x nk FP32 pair table, then (STAB) the
  // force spline
  extern __shared__ float4 dyn_smem[];
  __shared__ int4 sj[NW][32];
  __shared__ float4 sjd[POLAR ? NW : 1][32];
  __shared__ double red[NW][32][POLAR ? 6 : 3];
  __shared__ double ered[NT];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = a.nkind, ntab = a.ntab;
  PairFS* ptab = reinterpret_cast<PairFS*>(dyn_smem);
  float4* s_erd = dyn_smem + 3 * nk * nk;
  for (int t = threadIdx.x; t < 3 * nk * nk; t += NT)
    dyn_smem[t] = reinterpret_cast<const float4*>(ptab_g + t / 3)[t % 3];
  if (STAB)
    for (int t = threadIdx.x; t < ntab; t += NT) s_erd[t] = erd_g[t];
  const float4* erd = STAB ? s_erd : erd_g;
  __syncthreads();

  const int c = bx_;
  const int cz = c % a.ncz, cy = (c / a.ncz) % a.ncy, cx = c / (a.ncy * a.ncz);
  const int i0 = a.cell_start[c], ni = a.cell_start[c + 1] - i0;
  // fixed-point centre of the home cell
  const unsigned refx = (unsigned)((((unsigned long long)(2 * cx + 1)) << 31) / a.ncx),
                 refy = (unsigned)((((unsigned long long)(2 * cy + 1)) << 31) / a.ncy),
                 refz = (unsigned)((((unsigned long long)(2 * cz + 1)) << 31) / a.ncz);
  // per-lane energy sums: FP32 per neighbour cell, folded into compensated
  // FP32 sums (the FP64 pipe of this GPU is narrow); FP64 from the CTA sum on
  CSum es[9];

  for (int ib = 0; ib < ni; ib += 32) {
    const bool vi = ib + lane < ni;
    const int ti = i0 + ib + lane;
    const int4 me = vi ? pj[ti] : make_int4(0, 0, 0, 0);
    const float4 md = (POLAR && vi) ? a.pdj[ti] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int kind_i = me.w & 255, mol_i = me.w >> 8;
    const float xi = (float)(int)((unsigned)me.x - refx) * sx,
                yi = (float)(int)((unsigned)me.y - refy) * sy,
                zi = (float)(int)((unsigned)me.z - refz) * sz;
    CSum fx, fy, fz, gx, gy, gz;
    float ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0;
    float e_el = 0, e_lj = 0, e_vir = 0;
    PvF pv;
    pv.zero();
    int nb = 0;
    for (int s = warp; s < a.nstencil; s += NW) {
      const int4 o = a.stencil[s];
      int x2 = cx + o.x, y2 = cy + o.y, z2 = cz + o.z;
      x2 += (x2 < 0) ? a.ncx : (x2 >= a.ncx ? -a.ncx : 0);
      y2 += (y2 < 0) ? a.ncy : (y2 >= a.ncy ? -a.ncy : 0);
      z2 += (z2 < 0) ? a.ncz : (z2 >= a.ncz ? -a.ncz : 0);
      const int c2 = (x2 * a.ncy + y2) * a.ncz + z2;
      const int j0 = a.cell_start[c2], nj = a.cell_start[c2 + 1] - j0;
      for (int jb = 0; jb < nj; jb += 32) {
        if (jb + lane < nj) {
          int4 q = pj[j0 + jb + lane];
          if (REL) {
            // offset of the neighbour's nearest image from the home-cell centre
            const float4 f = make_float4((float)(int)((unsigned)q.x - refx) * sx,
                                         (float)(int)((unsigned)q.y - refy) * sy,
                                         (float)(int)((unsigned)q.z - refz) * sz,
                                         __int_as_float(q.w));
            q = make_int4(__float_as_int(f.x), __float_as_int(f.y), __float_as_int(f.z), q.w);
          }
          sj[warp][lane] = q;
          if (POLAR) sjd[warp][lane] = a.pdj[j0 + jb + lane];
        }
        __syncwarp();
        const int cnt = min(32, nj - jb);
        for (int jj = 0; jj < cnt; jj++) {
          const int4 q = sj[warp][jj];
          float dx, dy, dz;
          if (REL) {
            dx = xi - __int_as_float(q.x);
            dy = yi - __int_as_float(q.y);
            dz = zi - __int_as_float(q.z);
          } else {
            // nearest image: 32-bit wrap-around of the fixed-point difference
            dx = (float)(int)((unsigned)me.x - (unsigned)q.x) * sx;
            dy = (float)(int)((unsigned)me.y - (unsigned)q.y) * sy;
            dz = (float)(int)((unsigned)me.z - (unsigned)q.z) * sz;
          }
          const float rr = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
          // the site itself and its own molecule (exclusions) are skipped
          if (!vi || rr >= cq || (q.w >> 8) == mol_i) continue;
          const PairFS P = ptab[kind_i * nk + (q.w & 255)];
          float4 qd = make_float4(0.f, 0.f, 0.f, 0.f);
          if (POLAR) qd = sjd[warp][jj];
          float f = 0;
          if (rr < P.C2q) {
            float U;
            if (rr < P.C1q) {
              const float x = __fdividef(P.Sq, rr), y = x * x * x;
              f = P.E24 * fmaf(2.f * y, y, -y) * x;
              U = P.E4 * fmaf(y, y, -y);
            } else {
              const float x = rr - P.C2q;
              f = P.A4 * x;
              U = P.A * x * x;
            }
            if (MEASURE) {
              e_lj += U;
              e_vir += rr * f;
            }
          }
          if (P.qq != 0.f) f += spline_any<MEASURE, !STAB>(erd, eru, rr, sgrid, ntab, P.qq, e_el);
          ax = fmaf(f, dx, ax);
          ay = fmaf(f, dy, ay);
          az = fmaf(f, dz, az);
          if (MEASURE) pv.add(dx, dy, dz, f);
          if (POLAR) {
            if (P.qpc != 0.f) {  // Drude(i) - centre(j)
              const float ex = dx + md.x, ey = dy + md.y, ez = dz + md.z;
              const float fp = spline_any<MEASURE, !STAB>(erd, eru, fmaf(ex, ex, fmaf(ey, ey, ez * ez)),
                                                    sgrid, ntab, P.qpc, e_el);
              bx = fmaf(fp, ex, bx);
              by = fmaf(fp, ey, by);
              bz = fmaf(fp, ez, bz);
              if (MEASURE) pv.add(ex, ey, ez, fp);
            }
            if (P.qcp != 0.f) {  // centre(i) - Drude(j)
              const float ex = dx - qd.x, ey = dy - qd.y, ez = dz - qd.z;
              const float fp = spline_any<MEASURE, !STAB>(erd, eru, fmaf(ex, ex, fmaf(ey, ey, ez * ez)),
                                                    sgrid, ntab, P.qcp, e_el);
              ax = fmaf(fp, ex, ax);
              ay = fmaf(fp, ey, ay);
              az = fmaf(fp, ez, az);
              if (MEASURE) pv.add(ex, ey, ez, fp);
            }
            if (P.qpp != 0.f) {  // Drude(i) - Drude(j)
              const float ex = dx + md.x - qd.x, ey = dy + md.y - qd.y, ez = dz + md.z - qd.z;
              const float fp = spline_any<MEASURE, !STAB>(erd, eru, fmaf(ex, ex, fmaf(ey, ey, ez * ez)),
                                                    sgrid, ntab, P.qpp, e_el);
              bx = fmaf(fp, ex, bx);
              by = fmaf(fp, ey, by);
              bz = fmaf(fp, ez, bz);
              if (MEASURE) pv.add(ex, ey, ez, fp);
            }
          }
        }
        __syncwarp();
      }
      // energies fold into the compensated sums after every neighbour cell,
      // forces every FOLD cells
      if (MEASURE) {
        es[0].add(e_el); es[1].add(e_lj); es[2].add(e_vir);
        es[3].add(pv.p0); es[4].add(pv.p1); es[5].add(pv.p2);
        es[6].add(pv.p3); es[7].add(pv.p4); es[8].add(pv.p5);
        e_el = e_lj = e_vir = 0;
        pv.zero();
      }
      if (++nb == FOLD) {
        nb = 0;
        fx.add(ax); fy.add(ay); fz.add(az);
        ax = ay = az = 0;
        if (POLAR) {
          gx.add(bx); gy.add(by); gz.add(bz);
          bx = by = bz = 0;
        }
      }
    }
    fx.add(ax); fy.add(ay); fz.add(az);
    red[warp][lane][0] = fx.value();
    red[warp][lane][1] = fy.value();
    red[warp][lane][2] = fz.value();
    if (POLAR) {
      gx.add(bx); gy.add(by); gz.add(bz);
      red[warp][lane][POLAR ? 3 : 0] = gx.value();
      red[warp][lane][POLAR ? 4 : 0] = gy.value();
      red[warp][lane][POLAR ? 5 : 0] = gz.value();
    }
    __syncthreads();
    if (warp == 0 && vi) {
      double g[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int w = 0; w < NW; w++)
#pragma unroll
        for (int k = 0; k < (POLAR ? 6 : 3); k++) g[k] += red[w][lane][k];
      const int site = a.order[ti];
      a.f[3 * site] = g[0];
      a.f[3 * site + 1] = g[1];
      a.f[3 * site + 2] = g[2];
      if (POLAR) {
        a.f[3 * (long)a.ns + 3 * site] = g[3];
        a.f[3 * (long)a.ns + 3 * site + 1] = g[4];
        a.f[3 * (long)a.ns + 3 * site + 2] = g[5];
      }
    }
    __syncthreads();
  }
  if (MEASURE) {
    // each unordered pair was visited from both ends
    for (int k = 0; k < 9; k++) {
      ered[threadIdx.x] = 0.5 * es[k].value();
      __syncthreads();
      for (int w = NT / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) ered[threadIdx.x] += ered[threadIdx.x + w];
        __syncthreads();
      }
      if (threadIdx.x == 0) a.epart[bx_ * NEN + k] = ered[0];
      __syncthreads();
    }
  }
}

template <bool MEASURE, bool POLAR, bool REL, int NW, bool STAB>
__global__ void __launch_bounds__(NW * 32)
    pair_mixed_kernel(const __grid_constant__ PairArgs a, const int4* __restrict__ pj, const PairF* __restrict__ ptab_g, const float4* __restrict__ erd_g, const float4* __restrict__ eru, float sx, float sy, float sz, float cq, float sgrid, float alpha) {
  pair_mixed_kernel_body<MEASURE, POLAR, REL, NW, STAB>(a, pj, ptab_g, erd_g, eru, sx, sy, sz, cq, sgrid, alpha, blockIdx.x, 0);
}

// ------------------------------------------------- group pair kernel --
//
// The same pair terms as pair_mixed_kernel with the work cut by pruning.
// One warp per group of up to GROUP_SITES = 8 sites of a home cell (the
// group's sites are consecutive in the cell's site order); lane = (i = lane
// & 7, s = lane >> 3).  The neighbour sites come from the stencil's z-runs
// (cells consecutive along z are consecutive in the sorted array, so a run
// is one or, across the periodic edge, two contiguous ranges) in batches of
// 32: every neighbour is tested once against the cutoff sphere around the
// group's bounding box, the kept ones are compacted into shared memory
// (warp ballot, fixed order) and taken four at a time, one per s, each
// against the lane's own site i.  The test keeps every pair within the
// cutoff (the box distance is a lower bound of every pair distance, with the
// same FP32 operations), so the pair set is the cell kernel's.  The pair
// terms are predicated rather than branched (the lanes of a warp hold
// different kinds of pairs, and a branch per kind would run every path one
// after the other).  Forces: FP32 per z-run, folded into compensated sums;
// at the end the four s-lanes of a site are summed in a fixed order.  No
// atomics: results are reproducible.
template <bool MEASURE, bool POLAR, int NW>
__global__ void __launch_bounds__(NW * 32)
    pair_group_mixed_kernel(PairArgs a, const int4* __restrict__ pj,
                            const PairF* __restrict__ ptab_g, const float4* __restrict__ erd,
                            const float4* __restrict__ eru, float sx, float sy, float sz, float cq,
                            float sgrid) {
  constexpr int NT = NW * 32;
  extern __shared__ float4 dyn_smem[];   // the nk x nk FP32 pair table
  __shared__ float4 sj[NW][32];
  __shared__ float4 sjd[POLAR ? NW : 1][32];
  __shared__ double ered[NT];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int il = lane & 7, sl = lane >> 3;
  const int nk = a.nkind, ntab = a.ntab;
  PairFS* ptab = reinterpret_cast<PairFS*>(dyn_smem);
  for (int t = threadIdx.x; t < 3 * nk * nk; t += NT)
    dyn_smem[t] = reinterpret_cast<const float4*>(ptab_g + t / 3)[t % 3];
  __syncthreads();
  const int ncell = a.ncx * a.ncy * a.ncz;
  const int nitems = a.gstart[ncell];
  CSum es[9];

  for (int item = blockIdx.x * NW + warp; item < nitems; item += gridDim.x * NW) {
    const int c = a.gcell[item];
    const int cz = c % a.ncz, cy = (c / a.ncz) % a.ncy, cx = c / (a.ncy * a.ncz);
    const int i0 = a.cell_start[c] + GROUP_SITES * (item - a.gstart[c]);
    const int ni = min(GROUP_SITES, a.cell_start[c + 1] - i0);
    const unsigned refx = (unsigned)((((unsigned long long)(2 * cx + 1)) << 31) / a.ncx),
                   refy = (unsigned)((((unsigned long long)(2 * cy + 1)) << 31) / a.ncy),
                   refz = (unsigned)((((unsigned long long)(2 * cz + 1)) << 31) / a.ncz);
    const bool vi = il < ni;
    const int ti = i0 + il;
    const int4 me = vi ? pj[ti] : make_int4(0, 0, 0, 0);
    const float4 md = (POLAR && vi) ? a.pdj[ti] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int kind_i = me.w & 255, mol_i = me.w >> 8;
    const float xi = (float)(int)((unsigned)me.x - refx) * sx,
                yi = (float)(int)((unsigned)me.y - refy) * sy,
                zi = (float)(int)((unsigned)me.z - refz) * sz;
    // bounding box of the group's sites (the same in all four s-copies)
    float blx = vi ? xi : 3e38f, bly = vi ? yi : 3e38f, blz = vi ? zi : 3e38f;
    float bhx = vi ? xi : -3e38f, bhy = vi ? yi : -3e38f, bhz = vi ? zi : -3e38f;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      blx = fminf(blx, __shfl_xor_sync(0xffffffffu, blx, o));
      bly = fminf(bly, __shfl_xor_sync(0xffffffffu, bly, o));
      blz = fminf(blz, __shfl_xor_sync(0xffffffffu, blz, o));
      bhx = fmaxf(bhx, __shfl_xor_sync(0xffffffffu, bhx, o));
      bhy = fmaxf(bhy, __shfl_xor_sync(0xffffffffu, bhy, o));
      bhz = fmaxf(bhz, __shfl_xor_sync(0xffffffffu, bhz, o));
    }
    CSum fx, fy, fz, gx, gy, gz;
    for (int sp = 0; sp < a.nspans; sp++) {
      const int4 o = a.spans[sp];
      int x2 = cx + o.x, y2 = cy + o.y;
      x2 += (x2 < 0) ? a.ncx : (x2 >= a.ncx ? -a.ncx : 0);
      y2 += (y2 < 0) ? a.ncy : (y2 >= a.ncy ? -a.ncy : 0);
      const int col = (x2 * a.ncy + y2) * a.ncz;
      int za = cz + o.z, zb = cz + o.w;
      if (zb < 0) { za += a.ncz; zb += a.ncz; }
      if (za >= a.ncz) { za -= a.ncz; zb -= a.ncz; }
      // the z-run (at most ncz cells) as one or two contiguous ranges
      int ra0, ra1, rb0 = 0, rb1 = -1;
      if (za < 0) { ra0 = za + a.ncz; ra1 = a.ncz - 1; rb0 = 0; rb1 = zb; }
      else if (zb >= a.ncz) { ra0 = za; ra1 = a.ncz - 1; rb0 = 0; rb1 = zb - a.ncz; }
      else { ra0 = za; ra1 = zb; }
      float ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0;
      float e_el = 0, e_lj = 0, e_vir = 0;
      PvF pv;
      pv.zero();
      for (int part = 0; part < 2; part++) {
        const int z0 = part ? rb0 : ra0, z1 = part ? rb1 : ra1;
        if (z1 < z0) continue;
        const int j0 = a.cell_start[col + z0], j1 = a.cell_start[col + z1 + 1];
        for (int jb = j0; jb < j1; jb += 32) {
          const int j = jb + lane;
          bool keep = false;
          float4 f4 = make_float4(0.f, 0.f, 0.f, 0.f);
          if (j < j1) {
            const int4 q = pj[j];
            f4 = make_float4((float)(int)((unsigned)q.x - refx) * sx,
                             (float)(int)((unsigned)q.y - refy) * sy,
                             (float)(int)((unsigned)q.z - refz) * sz, __int_as_float(q.w));
            const float ddx = fmaxf(fmaxf(blx - f4.x, f4.x - bhx), 0.f),
                        ddy = fmaxf(fmaxf(bly - f4.y, f4.y - bhy), 0.f),
                        ddz = fmaxf(fmaxf(blz - f4.z, f4.z - bhz), 0.f);
            keep = fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz)) < cq;
          }
          const unsigned M = __ballot_sync(0xffffffffu, keep);
          if (keep) {
            const int slot = __popc(M & ((1u << lane) - 1u));
            sj[warp][slot] = f4;
            if (POLAR) sjd[warp][slot] = a.pdj[j];
          }
          __syncwarp();
          const int n = __popc(M);
          for (int t = sl; t < n; t += 4) {
            const float4 q = sj[warp][t];
            const float dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
            const float rr = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
            const int qw = __float_as_int(q.w);
            const bool ok = vi && rr < cq && (qw >> 8) != mol_i;
            const PairFS P = ptab[kind_i * nk + (qw & 255)];
            const float x = __fdividef(P.Sq, rr), y = x * x * x, xt = rr - P.C2q;
            const bool core = rr < P.C1q, tail = rr < P.C2q;
            const float flj = core ? P.E24 * fmaf(2.f * y, y, -y) * x : (tail ? P.A4 * xt : 0.f);
            float e_el_p = 0.f;
            float f = flj + spline_any<MEASURE, true>(erd, eru, rr, sgrid, ntab, P.qq, e_el_p);
            f = ok ? f : 0.f;
            ax = fmaf(f, dx, ax);
            ay = fmaf(f, dy, ay);
            az = fmaf(f, dz, az);
            if (MEASURE && ok) {
              e_lj += core ? P.E4 * fmaf(y, y, -y) : (tail ? P.A * xt * xt : 0.f);
              e_vir += rr * flj;
              e_el += e_el_p;
              pv.add(dx, dy, dz, f);
            }
            if (POLAR) {
              // Drude(i) - centre(j), centre(i) - Drude(j), Drude(i) -
              // Drude(j): zero charge products give zero terms
              const float4 qd = sjd[warp][t];
              float e_p = 0.f;
              const float ex = dx + md.x, ey = dy + md.y, ez = dz + md.z;
              float fp = spline_any<MEASURE, true>(
                  erd, eru, fmaf(ex, ex, fmaf(ey, ey, ez * ez)), sgrid, ntab, P.qpc, e_p);
              fp = ok ? fp : 0.f;
              bx = fmaf(fp, ex, bx);
              by = fmaf(fp, ey, by);
              bz = fmaf(fp, ez, bz);
              const float cx2 = dx - qd.x, cy2 = dy - qd.y, cz2 = dz - qd.z;
              float fc = spline_any<MEASURE, true>(
                  erd, eru, fmaf(cx2, cx2, fmaf(cy2, cy2, cz2 * cz2)), sgrid, ntab, P.qcp, e_p);
              fc = ok ? fc : 0.f;
              ax = fmaf(fc, cx2, ax);
              ay = fmaf(fc, cy2, ay);
              az = fmaf(fc, cz2, az);
              const float px = ex - qd.x, py = ey - qd.y, pz = ez - qd.z;
              float fd = spline_any<MEASURE, true>(
                  erd, eru, fmaf(px, px, fmaf(py, py, pz * pz)), sgrid, ntab, P.qpp, e_p);
              fd = ok ? fd : 0.f;
              bx = fmaf(fd, px, bx);
              by = fmaf(fd, py, by);
              bz = fmaf(fd, pz, bz);
              if (MEASURE && ok) {
                pv.add(ex, ey, ez, fp);
                pv.add(cx2, cy2, cz2, fc);
                pv.add(px, py, pz, fd);
                e_el += e_p;
              }
            }
          }
          __syncwarp();
        }
      }
      // the z-run's FP32 sums into the compensated sums
      fx.add(ax); fy.add(ay); fz.add(az);
      if (POLAR) { gx.add(bx); gy.add(by); gz.add(bz); }
      if (MEASURE) {
        es[0].add(e_el); es[1].add(e_lj); es[2].add(e_vir);
        es[3].add(pv.p0); es[4].add(pv.p1); es[5].add(pv.p2);
        es[6].add(pv.p3); es[7].add(pv.p4); es[8].add(pv.p5);
      }
    }
    // the four s-lanes of a site, summed in a fixed order (xor 8, then 16:
    // every lane holds (s0 + s1) + (s2 + s3))
    double g[6] = {fx.value(), fy.value(), fz.value(), 0, 0, 0};
    if (POLAR) {
      g[3] = gx.value();
      g[4] = gy.value();
      g[5] = gz.value();
    }
#pragma unroll
    for (int k = 0; k < (POLAR ? 6 : 3); k++) {
      g[k] += __shfl_xor_sync(0xffffffffu, g[k], 8);
      g[k] += __shfl_xor_sync(0xffffffffu, g[k], 16);
    }
    if (sl == 0 && vi) {
      const int site = a.order[ti];
      a.f[3 * site] = g[0];
      a.f[3 * site + 1] = g[1];
      a.f[3 * site + 2] = g[2];
      if (POLAR) {
        a.f[3 * (long)a.ns + 3 * site] = g[3];
        a.f[3 * (long)a.ns + 3 * site + 1] = g[4];
        a.f[3 * (long)a.ns + 3 * site + 2] = g[5];
      }
    }
  }
  if (MEASURE) {
    // each unordered pair was visited from both ends; one row per CTA
    for (int k = 0; k < 9; k++) {
      ered[threadIdx.x] = 0.5 * es[k].value();
      __syncthreads();
      for (int w = NT / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) ered[threadIdx.x] += ered[threadIdx.x + w];
        __syncthreads();
      }
      if (threadIdx.x == 0) a.epart[blockIdx.x * NEN + k] = ered[0];
      __syncthreads();
    }
  }
}

// ------------------------------------------- group kernel, half shell --
//
// Newton's third law in the group kernel (pair_variant 9, no Drude shells):
// every unordered pair once.  The stencil is the half shell: the z-runs of
// the columns with dx > 0, or dx = 0 and dy > 0, whole, and the column
// (0, 0) from the home cell up; inside the home cell a pair is taken from
// its site with the lower sorted index (the grid has at least 2 cdiv + 1
// cells per edge, so no cell reaches another by two stencil offsets and no
// pair is found twice).  The pair terms are the group kernel's.  Forces go
// into 64-bit fixed-point sums (FIX_SCALE units per K/A) in sorted order by
// integer atomics; integer addition does not depend on the order, so the
// forces come out the same bit for bit on every run.  The neighbour's force
// of an iteration is summed over the 8 home lanes by a reduce-scatter (three
// shuffle levels: lanes i = 0, 2, 4 end with x, y, z) and added with one
// atomic per component; the home sites' own compensated sums once per
// group.  Every rounding of the force arithmetic is explicit (the `_rn`
// intrinsics and explicit FMAs), so that the measuring and the plain
// instantiation run the same arithmetic: nvcc and ptxas may otherwise fuse
// a product into a following add in one kernel and not in the other, and a
// measured step would move the sites differently.  finish_forces_kernel
// turns the sums into the FP64 forces (site order) and clears them for the
// next evaluation.  Measured on 32768 waters (cells of cutoff/2): 0.37 ms
// against 0.45 ms for the group kernel.  Pairing two iterations on one
// conversion and one atomic, and a float-to-integer conversion in FP32
// arithmetic instead of the one on the FP64 pipe, both measured slower.
constexpr double FIX_SCALE = 4294967296.0;  // 2^32: steps of 2.3e-10 K/A, |F| < 2^31 K/A


__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// the half-shell kernel's pair force factor f (force on i = f (r_i - r_j))
// with every rounding explicit; flj: the LJ part.  The same terms as
// spline_any and the group kernel: smoothed LJ (core below C1q, quadratic
// tail up to C2q) and the hyperbolic erfc spline d.x + d.y / (d.z + r^2)
__device__ __forceinline__ float pair_force_rn(const PairFS& P, float rr,
                                               const float4* __restrict__ erd, float sgrid,
                                               int ntab, float& flj) {
  const float x = __fmul_rn(P.Sq, rcp_approx(rr)), y = __fmul_rn(__fmul_rn(x, x), x);
  flj = rr < P.C1q ? __fmul_rn(__fmul_rn(P.E24, __fmaf_rn(__fmul_rn(2.f, y), y, -y)), x)
                   : (rr < P.C2q ? __fmul_rn(P.A4, __fadd_rn(rr, -P.C2q)) : 0.f);
  const int ix = min(__float_as_int(__fmaf_rn(rr, sgrid, 12582911.5f)) - 0x4B400000, ntab - 1);
  const float4 d = __ldg(erd + ix);
  return __fmaf_rn(__fmaf_rn(d.y, rcp_approx(__fadd_rn(d.z, rr)), d.x), P.qq, flj);
}

// the Drude terms of a pair in the half-shell kernel, every rounding
// explicit: (charge product) x (d.x + d.y / (d.z + r^2)) at the separation
// (ex, ey, ez); e: its energy when measuring
template <bool MEASURE>
__device__ __forceinline__ float drude_force_rn(const float4* __restrict__ erd,
                                                const float4* __restrict__ eru, float ex,
                                                float ey, float ez, float sgrid, int ntab,
                                                float q, float& e) {
  const float r2 = __fmaf_rn(ex, ex, __fmaf_rn(ey, ey, __fmul_rn(ez, ez)));
  const int ix = min(__float_as_int(__fmaf_rn(r2, sgrid, 12582911.5f)) - 0x4B400000, ntab - 1);
  const float4 d = __ldg(erd + ix);
  if (MEASURE) {
    float ee = 0.f;
    spline_any<true, true>(erd, eru, r2, sgrid, ntab, q, ee);
    e += ee;
  }
  return __fmul_rn(__fmaf_rn(d.y, rcp_approx(__fadd_rn(d.z, r2)), d.x), q);
}

// 7 CTAs per SM (72 registers, no spills): measured faster than 8 (64) and
// than no bound (95).  POLAR (Drude shells): four charge terms per pair,
// forces on both centres and both shells; the neighbour's six components
// (centre x y z, shell x y z) are reduce-scattered over the 8 home lanes
// in three levels (keeping 4, 2, 1 of 8 padded components), so lane i ends
// with component i and lanes 0..5 write them
template <bool MEASURE, bool POLAR, int NW>
__global__ void __launch_bounds__(NW * 32, MEASURE ? 1 : (POLAR ? 5 : 7))
    pair_half_mixed_kernel(PairArgs a, const int4* __restrict__ pj,
                           const PairF* __restrict__ ptab_g, const float4* __restrict__ erd,
                           const float4* __restrict__ eru, float sx, float sy, float sz, float cq,
                           float sgrid) {
  constexpr int NT = NW * 32;
  extern __shared__ float4 dyn_smem[];   // the nk x nk FP32 pair table
  __shared__ float4 sj[NW][32];
  __shared__ float4 sjd[POLAR ? NW : 1][32];
  __shared__ int sjt[NW][32];
  __shared__ double ered[NT];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int il = lane & 7, sl = lane >> 3;
  const int nk = a.nkind, ntab = a.ntab;
  PairFS* ptab = reinterpret_cast<PairFS*>(dyn_smem);
  for (int t = threadIdx.x; t < 3 * nk * nk; t += NT)
    dyn_smem[t] = reinterpret_cast<const float4*>(ptab_g + t / 3)[t % 3];
  __syncthreads();
  const int ncell = a.ncx * a.ncy * a.ncz;
  const int nitems = a.gstart[ncell];
  unsigned long long* facc = reinterpret_cast<unsigned long long*>(a.facc);
  const long dhalf = 3 * (long)a.ns;   // the shells' sums after the centres'
  // reduce-scatter roles: without shells lane i ends with component i >> 1
  // (0 x, 1 y, 2 z, 3 nothing) and lanes i = 0, 2, 4 write it; with shells
  // lane i ends with component i (0-2 centre, 3-5 shell, 6-7 nothing)
  const bool b2 = (il & 4) != 0, b1 = (il & 2) != 0, b0 = (il & 1) != 0;
  const int comp = POLAR ? il : il >> 1;
  const bool jw = POLAR ? il < 6 : (!b0 && comp < 3);
  const long joff = POLAR && il >= 3 ? dhalf - 3 : 0;   // shell components
  CSum es[9];

  for (int item = blockIdx.x * NW + warp; item < nitems; item += gridDim.x * NW) {
    const int c = a.gcell[item];
    const int cz = c % a.ncz, cy = (c / a.ncz) % a.ncy, cx = c / (a.ncy * a.ncz);
    const int hs = a.cell_start[c], he = a.cell_start[c + 1];
    const int i0 = hs + GROUP_SITES * (item - a.gstart[c]);
    const int ni = min(GROUP_SITES, he - i0);
    const unsigned refx = (unsigned)((((unsigned long long)(2 * cx + 1)) << 31) / a.ncx),
                   refy = (unsigned)((((unsigned long long)(2 * cy + 1)) << 31) / a.ncy),
                   refz = (unsigned)((((unsigned long long)(2 * cz + 1)) << 31) / a.ncz);
    const bool vi = il < ni;
    const int ti = i0 + il;
    const int4 me = vi ? pj[ti] : make_int4(0, 0, 0, 0);
    const float4 md = (POLAR && vi) ? a.pdj[ti] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int kind_i = me.w & 255, mol_i = me.w >> 8;
    const float xi = __fmul_rn((float)(int)((unsigned)me.x - refx), sx),
                yi = __fmul_rn((float)(int)((unsigned)me.y - refy), sy),
                zi = __fmul_rn((float)(int)((unsigned)me.z - refz), sz);
    float blx = vi ? xi : 3e38f, bly = vi ? yi : 3e38f, blz = vi ? zi : 3e38f;
    float bhx = vi ? xi : -3e38f, bhy = vi ? yi : -3e38f, bhz = vi ? zi : -3e38f;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      blx = fminf(blx, __shfl_xor_sync(0xffffffffu, blx, o));
      bly = fminf(bly, __shfl_xor_sync(0xffffffffu, bly, o));
      blz = fminf(blz, __shfl_xor_sync(0xffffffffu, blz, o));
      bhx = fmaxf(bhx, __shfl_xor_sync(0xffffffffu, bhx, o));
      bhy = fmaxf(bhy, __shfl_xor_sync(0xffffffffu, bhy, o));
      bhz = fmaxf(bhz, __shfl_xor_sync(0xffffffffu, bhz, o));
    }
    CSum fx, fy, fz, gx, gy, gz;
    for (int sp = 0; sp < a.nhspans; sp++) {
      const int4 o = a.hspans[sp];
      int x2 = cx + o.x, y2 = cy + o.y;
      x2 += (x2 < 0) ? a.ncx : (x2 >= a.ncx ? -a.ncx : 0);
      y2 += (y2 < 0) ? a.ncy : (y2 >= a.ncy ? -a.ncy : 0);
      const int col = (x2 * a.ncy + y2) * a.ncz;
      int za = cz + o.z, zb = cz + o.w;
      if (zb < 0) { za += a.ncz; zb += a.ncz; }
      if (za >= a.ncz) { za -= a.ncz; zb -= a.ncz; }
      int ra0, ra1, rb0 = 0, rb1 = -1;
      if (za < 0) { ra0 = za + a.ncz; ra1 = a.ncz - 1; rb0 = 0; rb1 = zb; }
      else if (zb >= a.ncz) { ra0 = za; ra1 = a.ncz - 1; rb0 = 0; rb1 = zb - a.ncz; }
      else { ra0 = za; ra1 = zb; }
      float ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0;
      float e_el = 0, e_lj = 0, e_vir = 0;
      PvF pv;
      pv.zero();
      for (int part = 0; part < 2; part++) {
        const int z0 = part ? rb0 : ra0, z1 = part ? rb1 : ra1;
        if (z1 < z0) continue;
        // home-cell sites before the group pair with it from their own group
        const int j0 = max(a.cell_start[col + z0], col + z0 == c ? i0 : 0),
                  j1 = a.cell_start[col + z1 + 1];
        for (int jb = j0; jb < j1; jb += 32) {
          const int j = jb + lane;
          bool keep = false;
          float4 f4 = make_float4(0.f, 0.f, 0.f, 0.f);
          if (j < j1) {
            const int4 q = pj[j];
            f4 = make_float4(__fmul_rn((float)(int)((unsigned)q.x - refx), sx),
                             __fmul_rn((float)(int)((unsigned)q.y - refy), sy),
                             __fmul_rn((float)(int)((unsigned)q.z - refz), sz),
                             __int_as_float(q.w));
            const float ddx = fmaxf(fmaxf(blx - f4.x, f4.x - bhx), 0.f),
                        ddy = fmaxf(fmaxf(bly - f4.y, f4.y - bhy), 0.f),
                        ddz = fmaxf(fmaxf(blz - f4.z, f4.z - bhz), 0.f);
            keep = fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz)) < cq;
          }
          const unsigned M = __ballot_sync(0xffffffffu, keep);
          if (keep) {
            const int slot = __popc(M & ((1u << lane) - 1u));
            sj[warp][slot] = f4;
            sjt[warp][slot] = j;
            if (POLAR) sjd[warp][slot] = a.pdj[j];
          }
          __syncwarp();
          const int n = __popc(M);
          // the whole warp iterates: the reduce-scatter needs every lane
          for (int t0 = 0; t0 < n; t0 += 4) {
            const int t = t0 + sl;
            const bool vt = t < n;
            const float4 q = sj[warp][vt ? t : 0];
            const int tj = sjt[warp][vt ? t : 0];
            const float dx = __fadd_rn(xi, -q.x), dy = __fadd_rn(yi, -q.y),
                        dz = __fadd_rn(zi, -q.z);
            const float rr = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
            const int qw = __float_as_int(q.w);
            const bool ok = vt && vi && rr < cq && (qw >> 8) != mol_i &&
                            (tj > ti || tj >= he || tj < hs);
            const PairFS P = ptab[kind_i * nk + (qw & 255)];
            float flj;
            float f = pair_force_rn(P, rr, erd, sgrid, ntab, flj);
            f = ok ? f : 0.f;
            ax = __fmaf_rn(f, dx, ax);
            ay = __fmaf_rn(f, dy, ay);
            az = __fmaf_rn(f, dz, az);
            float px = __fmul_rn(f, dx), py = __fmul_rn(f, dy), pz = __fmul_rn(f, dz);
            // the neighbour's shell (POLAR)
            float hx = 0.f, hy = 0.f, hz = 0.f;
            float e_p = 0.f;
            if (POLAR) {
              // shell(i) - centre(j), centre(i) - shell(j), shell(i) - shell(j)
              const float4 qd = sjd[warp][vt ? t : 0];
              const float ex = __fadd_rn(dx, md.x), ey = __fadd_rn(dy, md.y),
                          ez = __fadd_rn(dz, md.z);
              float fp = drude_force_rn<MEASURE>(erd, eru, ex, ey, ez, sgrid, ntab, P.qpc, e_p);
              const float cx2 = __fadd_rn(dx, -qd.x), cy2 = __fadd_rn(dy, -qd.y),
                          cz2 = __fadd_rn(dz, -qd.z);
              float fc = drude_force_rn<MEASURE>(erd, eru, cx2, cy2, cz2, sgrid, ntab, P.qcp,
                                                 e_p);
              const float ux = __fadd_rn(ex, -qd.x), uy = __fadd_rn(ey, -qd.y),
                          uz = __fadd_rn(ez, -qd.z);
              float fd = drude_force_rn<MEASURE>(erd, eru, ux, uy, uz, sgrid, ntab, P.qpp, e_p);
              fp = ok ? fp : 0.f;
              fc = ok ? fc : 0.f;
              fd = ok ? fd : 0.f;
              // home centre: + fc (cx2); home shell: + fp (e) + fd (u)
              ax = __fmaf_rn(fc, cx2, ax);
              ay = __fmaf_rn(fc, cy2, ay);
              az = __fmaf_rn(fc, cz2, az);
              bx = __fmaf_rn(fp, ex, __fmaf_rn(fd, ux, bx));
              by = __fmaf_rn(fp, ey, __fmaf_rn(fd, uy, by));
              bz = __fmaf_rn(fp, ez, __fmaf_rn(fd, uz, bz));
              // neighbour centre: -(f d + fp e); neighbour shell: -(fc cx2 + fd u)
              px = __fmaf_rn(fp, ex, px);
              py = __fmaf_rn(fp, ey, py);
              pz = __fmaf_rn(fp, ez, pz);
              hx = __fmaf_rn(fc, cx2, __fmul_rn(fd, ux));
              hy = __fmaf_rn(fc, cy2, __fmul_rn(fd, uy));
              hz = __fmaf_rn(fc, cz2, __fmul_rn(fd, uz));
              if (MEASURE && ok) {
                pv.add(ex, ey, ez, fp);
                pv.add(cx2, cy2, cz2, fc);
                pv.add(ux, uy, uz, fd);
              }
            }
            if (MEASURE && ok) {
              // energies and virial: no effect on the forces
              const float x = __fdividef(P.Sq, rr), y = x * x * x, xt = rr - P.C2q;
              e_lj += rr < P.C1q ? P.E4 * fmaf(y, y, -y) : (rr < P.C2q ? P.A * xt * xt : 0.f);
              e_vir += rr * flj;
              float e_el_p = 0.f;
              spline_any<true, true>(erd, eru, rr, sgrid, ntab, P.qq, e_el_p);
              e_el += e_el_p + e_p;
              pv.add(dx, dy, dz, f);
            }
            float k;
            if (POLAR) {
              // components 0-5 = (px, py, pz, hx, hy, hz), 6-7 zero; level 1
              // keeps 4 (xor 4), level 2 keeps 2 (xor 2), level 3 keeps 1
              const float v0 = b2 ? hy : px, v1 = b2 ? hz : py, v2 = b2 ? 0.f : pz,
                          v3 = b2 ? 0.f : hx;
              const float w0 = b2 ? px : hy, w1 = b2 ? py : hz, w2 = b2 ? pz : 0.f,
                          w3 = b2 ? hx : 0.f;
              const float k0 = __fadd_rn(v0, __shfl_xor_sync(0xffffffffu, w0, 4)),
                          k1 = __fadd_rn(v1, __shfl_xor_sync(0xffffffffu, w1, 4)),
                          k2 = __fadd_rn(v2, __shfl_xor_sync(0xffffffffu, w2, 4)),
                          k3 = __fadd_rn(v3, __shfl_xor_sync(0xffffffffu, w3, 4));
              const float m0 = __fadd_rn(b1 ? k2 : k0,
                                         __shfl_xor_sync(0xffffffffu, b1 ? k0 : k2, 2)),
                          m1 = __fadd_rn(b1 ? k3 : k1,
                                         __shfl_xor_sync(0xffffffffu, b1 ? k1 : k3, 2));
              k = __fadd_rn(b0 ? m1 : m0, __shfl_xor_sync(0xffffffffu, b0 ? m0 : m1, 1));
            } else {
              float k0 = b2 ? pz : px, k1 = b2 ? 0.f : py;
              const float s0 = b2 ? px : pz, s1 = b2 ? py : 0.f;
              k0 = __fadd_rn(k0, __shfl_xor_sync(0xffffffffu, s0, 4));
              k1 = __fadd_rn(k1, __shfl_xor_sync(0xffffffffu, s1, 4));
              k = b1 ? k1 : k0;
              k = __fadd_rn(k, __shfl_xor_sync(0xffffffffu, b1 ? k0 : k1, 2));
              k = __fadd_rn(k, __shfl_xor_sync(0xffffffffu, k, 1));
            }
            if (jw && vt)
              atomicAdd(facc + 3 * (long)tj + comp + joff,
                        (unsigned long long)__float2ll_rn(__fmul_rn(k, -(float)FIX_SCALE)));
          }
          __syncwarp();
        }
      }
      fx.add(ax); fy.add(ay); fz.add(az);
      if (POLAR) { gx.add(bx); gy.add(by); gz.add(bz); }
      if (MEASURE) {
        es[0].add(e_el); es[1].add(e_lj); es[2].add(e_vir);
        es[3].add(pv.p0); es[4].add(pv.p1); es[5].add(pv.p2);
        es[6].add(pv.p3); es[7].add(pv.p4); es[8].add(pv.p5);
      }
    }
    // the home sites' sums: the four s-lanes in a fixed order, then lane
    // s = 0, 1, 2 adds component x, y, z (of the centre and the shell)
    double g[6] = {fx.value(), fy.value(), fz.value(), 0, 0, 0};
    if (POLAR) {
      g[3] = gx.value();
      g[4] = gy.value();
      g[5] = gz.value();
    }
#pragma unroll
    for (int k = 0; k < (POLAR ? 6 : 3); k++) {
      g[k] += __shfl_xor_sync(0xffffffffu, g[k], 8);
      g[k] += __shfl_xor_sync(0xffffffffu, g[k], 16);
    }
    if (vi && sl < 3) {
      atomicAdd(facc + 3 * (long)ti + sl,
                (unsigned long long)__double2ll_rn((sl == 0 ? g[0] : (sl == 1 ? g[1] : g[2])) *
                                                   FIX_SCALE));
      if (POLAR)
        atomicAdd(facc + dhalf + 3 * (long)ti + sl,
                  (unsigned long long)__double2ll_rn(
                      (sl == 0 ? g[3] : (sl == 1 ? g[4] : g[5])) * FIX_SCALE));
    }
  }
  if (MEASURE) {
    // every unordered pair once; one row per CTA
    for (int k = 0; k < 9; k++) {
      ered[threadIdx.x] = es[k].value();
      __syncthreads();
      for (int w = NT / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) ered[threadIdx.x] += ered[threadIdx.x + w];
        __syncthreads();
      }
      if (threadIdx.x == 0) a.epart[blockIdx.x * NEN + k] = ered[0];
      __syncthreads();
    }
  }
}

// ------------------------------ group kernel, half shell, lanes on the
// neighbours (pair_variant 10, no Drude shells) --
//
// The work items, the half-shell z-runs, the candidate pruning against the
// cutoff sphere around the group's bounding box and the pair terms are
// those of pair_half_mixed_kernel; the roles of the lanes are transposed.
// The kept candidates are compacted into a ring of 64 per warp; whenever
// 32 are queued, each lane takes one and runs it against the group's (up
// to 8) home sites in turn, which every lane reads from shared memory
// (broadcast).  The neighbour's force stays in the lane's registers and goes
// into the fixed-point sums with three atomics after the 8 home sites: no
// per-pair shuffles, one float-to-integer conversion per component and
// neighbour.  The home sites' forces stay in 24 registers per lane and are
// reduce-scattered over the 32 lanes once per group (lane 3 i + d ends with
// component d of site i).  Home sites beyond the group's end are masked
// out of the pair test.  Every rounding is explicit, as in the lane-per-home
// kernel, so the measuring and the plain instantiation move the sites
// identically; the integer sums make the forces bit-reproducible.

// the z-ranges of half-shell span sp around cell (cx, cy, cz): column index
// col; run [ra0, ra1] and, where the run wraps through the box, [rb0, rb1]
__device__ __forceinline__ void half_span_runs(const PairArgs& a, int sp, int cx, int cy,
                                               int cz, int& col, int& ra0, int& ra1, int& rb0,
                                               int& rb1) {
  const int4 o = a.hspans[sp];
  int x2 = cx + o.x, y2 = cy + o.y;
  x2 += (x2 < 0) ? a.ncx : (x2 >= a.ncx ? -a.ncx : 0);
  y2 += (y2 < 0) ? a.ncy : (y2 >= a.ncy ? -a.ncy : 0);
  col = (x2 * a.ncy + y2) * a.ncz;
  int za = cz + o.z, zb = cz + o.w;
  if (zb < 0) { za += a.ncz; zb += a.ncz; }
  if (za >= a.ncz) { za -= a.ncz; zb -= a.ncz; }
  rb0 = 0;
  rb1 = -1;
  if (za < 0) { ra0 = za + a.ncz; ra1 = a.ncz - 1; rb1 = zb; }
  else if (zb >= a.ncz) { ra0 = za; ra1 = a.ncz - 1; rb1 = zb - a.ncz; }
  else { ra0 = za; ra1 = zb; }
}

constexpr int HT_RING = 64;   // compacted candidates per warp (a power of two >= 63)
// 5 CTAs per SM (96 registers): on 32768 waters with cells of half the
// cutoff 0.283 ms, against 0.294 ms with 6 (80 registers and a spill); the
// lane-per-home kernel takes 0.363 ms there.  One limit per lane for the
// pair test (instead of three tests per pair): 0.276 ms, the same forces
// bit for bit
#ifndef MG_HALF_T_MINB
#define MG_HALF_T_MINB 5      // CTAs per SM the register budget is set for
#endif

template <bool MEASURE, int NW>
__global__ void __launch_bounds__(NW * 32, MEASURE ? 1 : MG_HALF_T_MINB)
    pair_half_t_mixed_kernel(PairArgs a, const int4* __restrict__ pj,
                             const PairF* __restrict__ ptab_g, const float4* __restrict__ erd,
                             const float4* __restrict__ eru, float sx, float sy, float sz,
                             float cq, float sgrid) {
  constexpr int NT = NW * 32;
  extern __shared__ float4 dyn_smem[];   // the nk x nk FP32 pair table
  __shared__ float4 sq[NW][HT_RING];     // candidate positions (w: kind | mol << 8)
  __shared__ int sqt[NW][HT_RING];       // candidate sorted index
  __shared__ float4 sh[NW][GROUP_SITES]; // the group's home sites
  __shared__ double ered[MEASURE ? NT : 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int il = lane & 7;
  const int nk = a.nkind, ntab = a.ntab;
  PairFS* ptab = reinterpret_cast<PairFS*>(dyn_smem);
  for (int t = threadIdx.x; t < 3 * nk * nk; t += NT)
    dyn_smem[t] = reinterpret_cast<const float4*>(ptab_g + t / 3)[t % 3];
  __syncthreads();
  const int ncell = a.ncx * a.ncy * a.ncz;
  const int nitems = a.gstart[ncell];
  unsigned long long* facc = reinterpret_cast<unsigned long long*>(a.facc);
  CSum es[9];

  for (int item = blockIdx.x * NW + warp; item < nitems; item += gridDim.x * NW) {
    const int c = a.gcell[item];
    const int cz = c % a.ncz, cy = (c / a.ncz) % a.ncy, cx = c / (a.ncy * a.ncz);
    const int hs = a.cell_start[c], he = a.cell_start[c + 1];
    const int i0 = hs + GROUP_SITES * (item - a.gstart[c]);
    const int ni = min(GROUP_SITES, he - i0);
    const unsigned refx = (unsigned)((((unsigned long long)(2 * cx + 1)) << 31) / a.ncx),
                   refy = (unsigned)((((unsigned long long)(2 * cy + 1)) << 31) / a.ncy),
                   refz = (unsigned)((((unsigned long long)(2 * cz + 1)) << 31) / a.ncz);
    // the home sites (every 8-lane group holds all of them) and their box
    const bool vi = il < ni;
    const int4 me = vi ? pj[i0 + il] : make_int4(0, 0, 0, 0);
    const float xi = __fmul_rn((float)(int)((unsigned)me.x - refx), sx),
                yi = __fmul_rn((float)(int)((unsigned)me.y - refy), sy),
                zi = __fmul_rn((float)(int)((unsigned)me.z - refz), sz);
    float blx = vi ? xi : 3e38f, bly = vi ? yi : 3e38f, blz = vi ? zi : 3e38f;
    float bhx = vi ? xi : -3e38f, bhy = vi ? yi : -3e38f, bhz = vi ? zi : -3e38f;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      blx = fminf(blx, __shfl_xor_sync(0xffffffffu, blx, o));
      bly = fminf(bly, __shfl_xor_sync(0xffffffffu, bly, o));
      blz = fminf(blz, __shfl_xor_sync(0xffffffffu, blz, o));
      bhx = fmaxf(bhx, __shfl_xor_sync(0xffffffffu, bhx, o));
      bhy = fmaxf(bhy, __shfl_xor_sync(0xffffffffu, bhy, o));
      bhz = fmaxf(bhz, __shfl_xor_sync(0xffffffffu, bhz, o));
    }
    __syncwarp();   // the previous group's readers of sh are done
    if (lane < GROUP_SITES) sh[warp][lane] = make_float4(xi, yi, zi, __int_as_float(me.w));
    __syncwarp();
    float hx[GROUP_SITES], hy[GROUP_SITES], hz[GROUP_SITES];
#pragma unroll
    for (int i = 0; i < GROUP_SITES; i++) hx[i] = hy[i] = hz[i] = 0.f;

    // cnt queued candidates from ring slot h0: lane -> one candidate
    // against the home sites
    auto run = [&](int h0, int cnt) {
      const bool vt = lane < cnt;
      const int e = vt ? (h0 + lane) & (HT_RING - 1) : h0;   // a valid slot for idle lanes
      const float4 q = sq[warp][e];
      const int tj = sqt[warp][e];
      const int qw = __float_as_int(q.w);
      const int kj = qw & 255;
      // the home sites i < lim pair with this candidate: none for an idle
      // lane, those of the group, and of a candidate in the home cell only
      // the ones before it
      const bool inh = (unsigned)(tj - hs) < (unsigned)(he - hs);
      const int lim = !vt ? 0 : (inh ? min(ni, tj - i0) : ni);
      float px = 0.f, py = 0.f, pz = 0.f;
      float e_el = 0.f, e_lj = 0.f, e_vir = 0.f;
      PvF pv;
      pv.zero();
      // the home sites in turn, those beyond the group's end masked (sh
      // holds finite positions for them): without a branch per site the
      // compiler interleaves the sites' independent chains (0.283 ms on
      // 32768 waters against 0.304 ms with a warp-uniform branch per site)
#pragma unroll
      for (int i = 0; i < GROUP_SITES; i++) {
        {
          const float4 h = sh[warp][i];
          const float dx = __fadd_rn(h.x, -q.x), dy = __fadd_rn(h.y, -q.y),
                      dz = __fadd_rn(h.z, -q.z);
          const float rr = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
          const int hw = __float_as_int(h.w);
          const bool ok = i < lim && rr < cq && ((hw ^ qw) >> 8) != 0;
          const PairFS P = ptab[(hw & 255) * nk + kj];
          float flj;
          float f = pair_force_rn(P, rr, erd, sgrid, ntab, flj);
          f = ok ? f : 0.f;
          hx[i] = __fmaf_rn(f, dx, hx[i]);
          hy[i] = __fmaf_rn(f, dy, hy[i]);
          hz[i] = __fmaf_rn(f, dz, hz[i]);
          px = __fmaf_rn(f, dx, px);
          py = __fmaf_rn(f, dy, py);
          pz = __fmaf_rn(f, dz, pz);
          if (MEASURE && ok) {
            // energies and virial: no effect on the forces
            const float x = __fdividef(P.Sq, rr), y = x * x * x, xt = rr - P.C2q;
            e_lj += rr < P.C1q ? P.E4 * fmaf(y, y, -y) : (rr < P.C2q ? P.A * xt * xt : 0.f);
            e_vir += rr * flj;
            float e_el_p = 0.f;
            spline_any<true, true>(erd, eru, rr, sgrid, ntab, P.qq, e_el_p);
            e_el += e_el_p;
            pv.add(dx, dy, dz, f);
          }
        }
      }
      if (vt) {
        unsigned long long* fj = facc + 3 * (long)tj;
        atomicAdd(fj, (unsigned long long)__float2ll_rn(__fmul_rn(px, -(float)FIX_SCALE)));
        atomicAdd(fj + 1, (unsigned long long)__float2ll_rn(__fmul_rn(py, -(float)FIX_SCALE)));
        atomicAdd(fj + 2, (unsigned long long)__float2ll_rn(__fmul_rn(pz, -(float)FIX_SCALE)));
      }
      if (MEASURE) {
        es[0].add(e_el); es[1].add(e_lj); es[2].add(e_vir);
        es[3].add(pv.p0); es[4].add(pv.p1); es[5].add(pv.p2);
        es[6].add(pv.p3); es[7].add(pv.p4); es[8].add(pv.p5);
      }
      __syncwarp();   // the slots read here may be refilled next
    };

    int qh = 0, qn = 0;   // ring head and count (warp-uniform)
    for (int sp = 0; sp < a.nhspans; sp++) {
      int col, ra0, ra1, rb0, rb1;
      half_span_runs(a, sp, cx, cy, cz, col, ra0, ra1, rb0, rb1);
      for (int part = 0; part < 2; part++) {
        const int z0 = part ? rb0 : ra0, z1 = part ? rb1 : ra1;
        if (z1 < z0) continue;
        // home-cell sites before the group pair with it from their own group
        const int j0 = max(a.cell_start[col + z0], col + z0 == c ? i0 : 0),
                  j1 = a.cell_start[col + z1 + 1];
        for (int jb = j0; jb < j1; jb += 32) {
          const int j = jb + lane;
          bool keep = false;
          float4 f4 = make_float4(0.f, 0.f, 0.f, 0.f);
          if (j < j1) {
            const int4 q = pj[j];
            f4 = make_float4(__fmul_rn((float)(int)((unsigned)q.x - refx), sx),
                             __fmul_rn((float)(int)((unsigned)q.y - refy), sy),
                             __fmul_rn((float)(int)((unsigned)q.z - refz), sz),
                             __int_as_float(q.w));
            const float ddx = fmaxf(fmaxf(blx - f4.x, f4.x - bhx), 0.f),
                        ddy = fmaxf(fmaxf(bly - f4.y, f4.y - bhy), 0.f),
                        ddz = fmaxf(fmaxf(blz - f4.z, f4.z - bhz), 0.f);
            keep = fmaf(ddx, ddx, fmaf(ddy, ddy, ddz * ddz)) < cq;
          }
          const unsigned M = __ballot_sync(0xffffffffu, keep);
          if (keep) {
            // qn < 32 here, so the new slots never reach the queued ones
            const int slot = (qh + qn + __popc(M & ((1u << lane) - 1u))) & (HT_RING - 1);
            sq[warp][slot] = f4;
            sqt[warp][slot] = j;
          }
          qn += __popc(M);
          __syncwarp();
          if (qn >= 32) {
            run(qh, 32);
            qh = (qh + 32) & (HT_RING - 1);
            qn -= 32;
          }
        }
      }
    }
    if (qn > 0) run(qh, qn);

    // the home sites' sums: reduce-scatter of v[3 i + d] (24 values, 8
    // zero) over the lanes in a fixed order; lane k ends with v[k]
    float v[32];
#pragma unroll
    for (int i = 0; i < GROUP_SITES; i++) {
      v[3 * i] = hx[i];
      v[3 * i + 1] = hy[i];
      v[3 * i + 2] = hz[i];
    }
#pragma unroll
    for (int k = 3 * GROUP_SITES; k < 32; k++) v[k] = 0.f;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
      const bool up = (lane & w) != 0;
#pragma unroll
      for (int k = 0; k < w; k++) {
        const float keepv = up ? v[w + k] : v[k], sendv = up ? v[k] : v[w + k];
        v[k] = __fadd_rn(keepv, __shfl_xor_sync(0xffffffffu, sendv, w));
      }
    }
    if (lane < 3 * ni)
      atomicAdd(facc + 3 * (long)i0 + lane,
                (unsigned long long)__float2ll_rn(__fmul_rn(v[0], (float)FIX_SCALE)));
  }
  if (MEASURE) {
    // every unordered pair once; one row per CTA
    for (int k = 0; k < 9; k++) {
      ered[threadIdx.x] = es[k].value();
      __syncthreads();
      for (int w = NT / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) ered[threadIdx.x] += ered[threadIdx.x + w];
        __syncthreads();
      }
      if (threadIdx.x == 0) a.epart[blockIdx.x * NEN + k] = ered[0];
      __syncthreads();
    }
  }
}

// the fixed-point sums (sorted order) into the FP64 forces (site order),
// with shells the second half of each; the sums are cleared for the next
// evaluation
__global__ void finish_forces_kernel(int ns, int halves, const int* __restrict__ order,
                                     long long* __restrict__ facc, double* __restrict__ f) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ns) return;
  const int site = order[t];
  for (int h = 0; h < halves; h++) {
    const long o = 3 * (long)ns * h;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      f[o + 3 * (long)site + d] = (double)facc[o + 3 * (long)t + d] * (1.0 / FIX_SCALE);
      facc[o + 3 * (long)t + d] = 0;
    }
  }
}

cudaError_t k_pair_mixed(const Launch& L, const PairArgs& a, const int4* pj, const PairF* ptab,
                         const float4* erd, const float4* eru, bool measure, bool polar) {
  int ncell = a.ncx * a.ncy * a.ncz;
  float sx = (float)(a.Lx / 4294967296.0), sy = (float)(a.Ly / 4294967296.0),
        sz = (float)(a.Lz / 4294967296.0);
  const float cq = (float)a.cutoff_sq, sg = (float)a.sgrid, al = (float)a.alpha;
  const bool rel = !a.allpairs;
  if (a.group && a.newton && rel) {
    const size_t gsm = sizeof(PairFS) * (size_t)a.nkind * a.nkind;
    cudaError_t ge = cudaSuccess;
#define PAIR_HALF(M, P)                                                                         \
  do {                                                                                          \
    if (gsm > 48 * 1024)                                                                        \
      ge = cudaFuncSetAttribute(pair_half_mixed_kernel<M, P, GROUP_WARPS>,                     \
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsm);         \
    if (ge == cudaSuccess)                                                                      \
      pair_half_mixed_kernel<M, P, GROUP_WARPS><<<a.ngrid, GROUP_WARPS * 32, gsm, L.s>>>(      \
          a, pj, ptab, erd, eru, sx, sy, sz, cq, sg);                                           \
  } while (0)
#define PAIR_HALF_T(M)                                                                          \
  do {                                                                                          \
    if (gsm > 48 * 1024)                                                                        \
      ge = cudaFuncSetAttribute(pair_half_t_mixed_kernel<M, GROUP_WARPS>,                      \
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsm);         \
    if (ge == cudaSuccess)                                                                      \
      pair_half_t_mixed_kernel<M, GROUP_WARPS><<<a.ngrid, GROUP_WARPS * 32, gsm, L.s>>>(       \
          a, pj, ptab, erd, eru, sx, sy, sz, cq, sg);                                           \
  } while (0)
    // lanes on the neighbours (newton 2) without shells; with shells the
    // lane-per-home kernel
    if (polar) { if (measure) PAIR_HALF(true, true); else PAIR_HALF(false, true); }
    else if (a.newton == 2) { if (measure) PAIR_HALF_T(true); else PAIR_HALF_T(false); }
    else { if (measure) PAIR_HALF(true, false); else PAIR_HALF(false, false); }
#undef PAIR_HALF_T
#undef PAIR_HALF
    if (ge != cudaSuccess) return ge;
    LAUNCHED(L);
    finish_forces_kernel<<<cdiv(a.ns, 256), 256, 0, L.s>>>(a.ns, polar ? 2 : 1, a.order, a.facc,
                                                           a.f);
    LAUNCHED(L);
    return cudaGetLastError();
  }
  if (a.group && rel) {
    const size_t gsm = sizeof(PairFS) * (size_t)a.nkind * a.nkind;
    cudaError_t ge = cudaSuccess;
#define PAIR_GROUP(M, P)                                                                        \
  do {                                                                                          \
    if (gsm > 48 * 1024)                                                                        \
      ge = cudaFuncSetAttribute(pair_group_mixed_kernel<M, P, GROUP_WARPS>,                    \
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsm);         \
    if (ge == cudaSuccess)                                                                      \
      pair_group_mixed_kernel<M, P, GROUP_WARPS><<<a.ngrid, GROUP_WARPS * 32, gsm, L.s>>>(     \
          a, pj, ptab, erd, eru, sx, sy, sz, cq, sg);                                           \
  } while (0)
    if (polar) { if (measure) PAIR_GROUP(true, true); else PAIR_GROUP(false, true); }
    else { if (measure) PAIR_GROUP(true, false); else PAIR_GROUP(false, false); }
#undef PAIR_GROUP
    if (ge != cudaSuccess) return ge;
    LAUNCHED(L);
    return cudaGetLastError();
  }
  // the measuring kernel (energies, virial) always runs with 4 warps and the
  // spline through L1: with more registers per thread it keeps more CTAs
  // resident that way (1.0 ms on 32768 waters; 16 warps + shared-memory
  // spline, the fastest force-only choice there, 1.8 ms)
  const int nw = measure ? 4 : (a.pair_warps == 16 ? 16 : (a.pair_warps == 8 ? 8 : 4));
  const bool stab = a.spline_smem && !measure;
  const size_t dsm = sizeof(PairFS) * (size_t)a.nkind * a.nkind +
                     (stab ? sizeof(float4) * (size_t)a.ntab : 0);
  cudaError_t e = cudaSuccess;
#define PAIR_MIXED(M, P, R, W, S)                                                               \
  do {                                                                                          \
    if (dsm > 48 * 1024)                                                                        \
      e = cudaFuncSetAttribute(pair_mixed_kernel<M, P, R, W, S>,                                \
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm);          \
    if (e == cudaSuccess)                                                                       \
      pair_mixed_kernel<M, P, R, W, S><<<ncell, W * 32, dsm, L.s>>>(a, pj, ptab, erd, eru, sx,  \
                                                                     sy, sz, cq, sg, al);       \
  } while (0)
#define PAIR_MIXED_W(M, P, R)                              \
  do {                                                     \
    if (nw == 16) {                                        \
      if (stab) PAIR_MIXED(M, P, R, 16, true);             \
      else PAIR_MIXED(M, P, R, 16, false);                 \
    } else if (nw == 8) {                                  \
      if (stab) PAIR_MIXED(M, P, R, 8, true);              \
      else PAIR_MIXED(M, P, R, 8, false);                  \
    } else {                                               \
      if (stab) PAIR_MIXED(M, P, R, 4, true);              \
      else PAIR_MIXED(M, P, R, 4, false);                  \
    }                                                      \
  } while (0)
  if (polar) {
    if (measure) { if (rel) PAIR_MIXED_W(true, true, true); else PAIR_MIXED_W(true, true, false); }
    else { if (rel) PAIR_MIXED_W(false, true, true); else PAIR_MIXED_W(false, true, false); }
  } else {
    if (measure) { if (rel) PAIR_MIXED_W(true, false, true); else PAIR_MIXED_W(true, false, false); }
    else { if (rel) PAIR_MIXED_W(false, false, true); else PAIR_MIXED_W(false, false, false); }
  }
#undef PAIR_MIXED_W
#undef PAIR_MIXED
  if (e != cudaSuccess) return e;
  LAUNCHED(L);
  return cudaGetLastError();
}

template <bool MEASURE, bool POLAR>
__global__ void __launch_bounds__(PAIR_THREADS)
    pair_fp64_kernel(PairArgs a, const double4* __restrict__ pd, const PairD* __restrict__ ptab_g,
                     const double* __restrict__ ert) {
  __shared__ PairD ptab[MAX_KINDS * MAX_KINDS];
  __shared__ double4 sj[NWARP][32];
  __shared__ double4 sjd[POLAR ? NWARP : 1][32];
  __shared__ double red[NWARP][32][POLAR ? 6 : 3];
  __shared__ double ered[PAIR_THREADS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = a.nkind, ntab = a.ntab;
  for (int t = threadIdx.x; t < nk * nk; t += PAIR_THREADS) ptab[t] = ptab_g[t];
  __syncthreads();
  const int c = blockIdx.x;
  const int cz = c % a.ncz, cy = (c / a.ncz) % a.ncy, cx = c / (a.ncy * a.ncz);
  const int i0 = a.cell_start[c], ni = a.cell_start[c + 1] - i0;
  const double cq = a.cutoff_sq, sgrid = a.sgrid, alpha = a.alpha;
  double en[NEN];
#pragma unroll
  for (int k = 0; k < NEN; k++) en[k] = 0;
  for (int ib = 0; ib < ni; ib += 32) {
    const bool vi = ib + lane < ni;
    const int ti = i0 + ib + lane;
    const double4 me = vi ? pd[ti] : make_double4(0, 0, 0, 0);
    const double4 md = (POLAR && vi) ? a.pdd[ti] : make_double4(0, 0, 0, 0);
    const long long wi = __double_as_longlong(me.w);
    const int kind_i = (int)(wi & 255), mol_i = (int)(wi >> 8);
    double fx = 0, fy = 0, fz = 0, gx = 0, gy = 0, gz = 0;
    for (int s = warp; s < a.nstencil; s += NWARP) {
      const int4 o = a.stencil[s];
      int x2 = cx + o.x, y2 = cy + o.y, z2 = cz + o.z;
      double shx = 0, shy = 0, shz = 0;
      if (x2 < 0) { x2 += a.ncx; shx = -a.Lx; } else if (x2 >= a.ncx) { x2 -= a.ncx; shx = a.Lx; }
      if (y2 < 0) { y2 += a.ncy; shy = -a.Ly; } else if (y2 >= a.ncy) { y2 -= a.ncy; shy = a.Ly; }
      if (z2 < 0) { z2 += a.ncz; shz = -a.Lz; } else if (z2 >= a.ncz) { z2 -= a.ncz; shz = a.Lz; }
      const double xs = me.x - shx, ys = me.y - shy, zs = me.z - shz;
      const int c2 = (x2 * a.ncy + y2) * a.ncz + z2;
      const int j0 = a.cell_start[c2], nj = a.cell_start[c2 + 1] - j0;
      for (int jb = 0; jb < nj; jb += 32) {
        if (jb + lane < nj) {
          sj[warp][lane] = pd[j0 + jb + lane];
          if (POLAR) sjd[warp][lane] = a.pdd[j0 + jb + lane];
        }
        __syncwarp();
        const int cnt = min(32, nj - jb);
        for (int jj = 0; jj < cnt; jj++) {
          const double4 q = sj[warp][jj];
          double dx = xs - q.x, dy = ys - q.y, dz = zs - q.z;
          if (a.allpairs) {
            dx -= a.Lx * rint(dx / a.Lx);
            dy -= a.Ly * rint(dy / a.Ly);
            dz -= a.Lz * rint(dz / a.Lz);
          }
          const double rr = dx * dx + dy * dy + dz * dz;
          if (!vi || rr >= cq || j0 + jb + jj == ti) continue;
          const long long wj = __double_as_longlong(q.w);
          const PairD& P = ptab[kind_i * nk + (int)(wj & 255)];
          const bool excl = (int)(wj >> 8) == mol_i;
          if (!excl && rr < P.C2q) {
            double f, U;
            if (rr < P.C1q) {
              const double x = P.Sq / rr, y = x * x * x, z = y * y;
              f = P.E24 * (z + z - y) * x;
              U = P.E4 * (z - y);
            } else {
              const double x = rr - P.C2q;
              f = P.A4 * x;
              U = x * x * P.A;
            }
            fx += f * dx;
            fy += f * dy;
            fz += f * dz;
            if (MEASURE) {
              en[1] += U;
              en[2] += rr * f;
              en[3] += dx * f * dx;
              en[4] += dy * f * dy;
              en[5] += dz * f * dz;
              en[6] += dz * f * dy;
              en[7] += dx * f * dz;
              en[8] += dy * f * dx;
            }
          }
          if (P.qq != 0)
            term64<MEASURE>(dx, dy, dz, P.qq, excl, ert, sgrid, ntab, alpha, fx, fy, fz, en);
          if (POLAR) {
            const double4 qd = sjd[warp][jj];
            if (P.qpc != 0)
              term64<MEASURE>(dx + md.x, dy + md.y, dz + md.z, P.qpc, excl, ert, sgrid, ntab,
                              alpha, gx, gy, gz, en);
            if (P.qcp != 0)
              term64<MEASURE>(dx - qd.x, dy - qd.y, dz - qd.z, P.qcp, excl, ert, sgrid, ntab,
                              alpha, fx, fy, fz, en);
            if (P.qpp != 0)
              term64<MEASURE>(dx + md.x - qd.x, dy + md.y - qd.y, dz + md.z - qd.z, P.qpp, excl,
                              ert, sgrid, ntab, alpha, gx, gy, gz, en);
          }
        }
        __syncwarp();
      }
    }
    red[warp][lane][0] = fx;
    red[warp][lane][1] = fy;
    red[warp][lane][2] = fz;
    if (POLAR) {
      red[warp][lane][POLAR ? 3 : 0] = gx;
      red[warp][lane][POLAR ? 4 : 0] = gy;
      red[warp][lane][POLAR ? 5 : 0] = gz;
    }
    __syncthreads();
    if (warp == 0 && vi) {
      double g[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int w = 0; w < NWARP; w++)
#pragma unroll
        for (int k = 0; k < (POLAR ? 6 : 3); k++) g[k] += red[w][lane][k];
      const int site = a.order[ti];
      a.f[3 * site] = g[0];
      a.f[3 * site + 1] = g[1];
      a.f[3 * site + 2] = g[2];
      if (POLAR) {
        a.f[3 * (long)a.ns + 3 * site] = g[3];
        a.f[3 * (long)a.ns + 3 * site + 1] = g[4];
        a.f[3 * (long)a.ns + 3 * site + 2] = g[5];
      }
    }
    __syncthreads();
  }
  if (MEASURE) {
    for (int k = 0; k < 9; k++) {
      ered[threadIdx.x] = 0.5 * en[k];
      __syncthreads();
      for (int w = PAIR_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) ered[threadIdx.x] += ered[threadIdx.x + w];
        __syncthreads();
      }
      if (threadIdx.x == 0) a.epart[blockIdx.x * NEN + k] = ered[0];
      __syncthreads();
    }
  }
}

// ------------------------------------------------ Ewald exclusion terms --

// -erf(alpha r)/r of the intramolecular pairs (cook/ljqqnp.c:131-141, its
// Drude forms cook/ljqqpol.c) for the mixed cell path: each pair once, from
// the FP64 positions (nearest image), the term in FP32 as in the pair
// kernels, forces and energy summed in FP64.  Pairs beyond the cutoff are
// skipped, as the cell traversal never meets them.
// The force arithmetic rounds explicitly (`_rn`): the measuring
// instantiation also uses the products for the virial, and a product the
// compiler fuses into the force sum in one instantiation and not in the
// other would move the sites of a measured step differently.
__device__ __forceinline__ double excl_r2(double dx, double dy, double dz) {
  return __fma_rn(dx, dx, __fma_rn(dy, dy, __dmul_rn(dz, dz)));
}

template <bool MEASURE>
__device__ __forceinline__ void excl_pair(double dx, double dy, double dz, double qq, float alpha,
                                          double* fi, double* fj, double* en) {
  float fe;
  const float e = excl_term<float>((float)excl_r2(dx, dy, dz), alpha, &fe);
  const double fq = __dmul_rn((double)fe, qq);
  const double Fx = __dmul_rn(fq, dx), Fy = __dmul_rn(fq, dy), Fz = __dmul_rn(fq, dz);
  fi[0] = __dadd_rn(fi[0], Fx);
  fi[1] = __dadd_rn(fi[1], Fy);
  fi[2] = __dadd_rn(fi[2], Fz);
  fj[0] = __dadd_rn(fj[0], -Fx);
  fj[1] = __dadd_rn(fj[1], -Fy);
  fj[2] = __dadd_rn(fj[2], -Fz);
  if (MEASURE) {
    en[0] += (double)e * qq;
    en[1] += Fx * dx;
    en[2] += Fy * dy;
    en[3] += Fz * dz;
    en[4] += Fz * dy;
    en[5] += Fx * dz;
    en[6] += Fy * dx;
  }
}

__device__ __forceinline__ double near_img(double d, double L, double iL) {
  return d - L * rint(d * iL);
}

template <bool MEASURE, bool POLAR>
MG_BODY void excl_mixed_kernel_body(const ExclArgs& a,
    const int bx_,
    const int by_) {
  __shared__ double red[EXCL_THREADS];
  const int n = bx_ * EXCL_THREADS + threadIdx.x;
  double en[7] = {0, 0, 0, 0, 0, 0, 0};
  if (n < a.nmol) {
    const long ns3 = 3 * (long)a.ns;
    for (int p = a.xfirst[n]; p < a.xfirst[n + 1]; p++) {
      const int2 ij = a.xpair[p];
      const double4 q = a.xq[p];
      const double* ri = a.r + 3 * (long)ij.x;
      const double* rj = a.r + 3 * (long)ij.y;
      const double dx = near_img(ri[0] - rj[0], a.Lx, a.iLx),
                   dy = near_img(ri[1] - rj[1], a.Ly, a.iLy),
                   dz = near_img(ri[2] - rj[2], a.Lz, a.iLz);
      if (!(excl_r2(dx, dy, dz) < a.cutoff_sq)) continue;
      double* fi = a.f + 3 * (long)ij.x;
      double* fj = a.f + 3 * (long)ij.y;
      if (q.x != 0) excl_pair<MEASURE>(dx, dy, dz, q.x, a.alpha, fi, fj, en);
      if (POLAR) {
        const double* mi = ri + ns3;
        const double* mj = rj + ns3;
        double* gi = fi + ns3;
        double* gj = fj + ns3;
        if (q.y != 0)  // Drude(i) - centre(j)
          excl_pair<MEASURE>(dx + mi[0], dy + mi[1], dz + mi[2], q.y, a.alpha, gi, fj, en);
        if (q.z != 0)  // centre(i) - Drude(j)
          excl_pair<MEASURE>(dx - mj[0], dy - mj[1], dz - mj[2], q.z, a.alpha, fi, gj, en);
        if (q.w != 0)  // Drude(i) - Drude(j)
          excl_pair<MEASURE>(dx + mi[0] - mj[0], dy + mi[1] - mj[1], dz + mi[2] - mj[2], q.w,
                             a.alpha, gi, gj, en);
      }
    }
  }
  if (MEASURE) {
    // row layout of the pair kernels: el, lj, vir, Pvir[6], spare
    constexpr int slot[7] = {0, 3, 4, 5, 6, 7, 8};
    for (int k = 0; k < 10; k++) {
      double v = 0;
#pragma unroll
      for (int m = 0; m < 7; m++)
        if (slot[m] == k) v = en[m];
      red[threadIdx.x] = v;
      __syncthreads();
      for (int w = EXCL_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
      }
      if (threadIdx.x == 0) a.epart[bx_ * NEN + k] = red[0];
      __syncthreads();
    }
  }
}

template <bool MEASURE, bool POLAR>
__global__ void __launch_bounds__(EXCL_THREADS) excl_mixed_kernel(const __grid_constant__ ExclArgs a) {
  excl_mixed_kernel_body<MEASURE, POLAR>(a, blockIdx.x, 0);
}

cudaError_t k_excl_mixed(const Launch& L, const ExclArgs& a, bool measure, bool polar) {
  if (a.nmol <= 0) return cudaSuccess;
  const int nb = cdiv(a.nmol, EXCL_THREADS);
  if (measure) {
    if (polar) excl_mixed_kernel<true, true><<<nb, EXCL_THREADS, 0, L.s>>>(a);
    else excl_mixed_kernel<true, false><<<nb, EXCL_THREADS, 0, L.s>>>(a);
  } else {
    if (polar) excl_mixed_kernel<false, true><<<nb, EXCL_THREADS, 0, L.s>>>(a);
    else excl_mixed_kernel<false, false><<<nb, EXCL_THREADS, 0, L.s>>>(a);
  }
  LAUNCHED(L);
  return cudaGetLastError();
}

cudaError_t k_pair_fp64(const Launch& L, const PairArgs& a, const double4* pd, const PairD* ptab,
                        const double* ertab, bool measure, bool polar) {
  int ncell = a.ncx * a.ncy * a.ncz;
  if (polar) {
    if (measure)
      pair_fp64_kernel<true, true><<<ncell, PAIR_THREADS, 0, L.s>>>(a, pd, ptab, ertab);
    else
      pair_fp64_kernel<false, true><<<ncell, PAIR_THREADS, 0, L.s>>>(a, pd, ptab, ertab);
  } else {
    if (measure)
      pair_fp64_kernel<true, false><<<ncell, PAIR_THREADS, 0, L.s>>>(a, pd, ptab, ertab);
    else
      pair_fp64_kernel<false, false><<<ncell, PAIR_THREADS, 0, L.s>>>(a, pd, ptab, ertab);
  }
  LAUNCHED(L);
  return cudaGetLastError();
}

__global__ void gather_drude_kernel(int ns, const double* __restrict__ r,
                                    const int* __restrict__ order, float4* __restrict__ pdj,
                                    double4* __restrict__ pdd) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ns) return;
  const int i = order[t];
  const double* d = r + 3 * (long)ns + 3 * i;
  if (pdj) pdj[t] = make_float4((float)d[0], (float)d[1], (float)d[2], 0.f);
  if (pdd) pdd[t] = make_double4(d[0], d[1], d[2], 0.0);
}

cudaError_t k_gather_drude(const Launch& L, int ns, const double* r, const int* order,
                           float4* pdj, double4* pdd) {
  gather_drude_kernel<<<cdiv(ns, 256), 256, 0, L.s>>>(ns, r, order, pdj, pdd);
  LAUNCHED(L);
  return cudaGetLastError();
}

// --------------------------------------------------------------- k-space --

// Row of charge j: [q e^{2 pi i kx sx}, kx=0..Kx | e^{2 pi i ky sy}, ky=-Ky..Ky |
//                   e^{2 pi i kz sz}, kz=-Kz..Kz]
// f += fk (the k-space forces of the concurrent chain)
__global__ void add_forces_kernel(size_t n, const double* __restrict__ fk, double* __restrict__ f) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) f[i] += fk[i];
}

cudaError_t k_add_forces(const Launch& L, size_t n, const double* fk, double* f) {
  add_forces_kernel<<<(unsigned)((n + 255) / 256), 256, 0, L.s>>>(n, fk, f);
  LAUNCHED(L);
  return cudaGetLastError();
}

// fixed-point coordinates of every charge (Drude charges at r + rpol)
MG_BODY void charge_fixed_kernel_body(const KArgs& a,
    const double* __restrict__ r,
    uint4* __restrict__ qf,
    const int bx_,
    const int by_) {
  const int j = bx_ * blockDim.x + threadIdx.x;
  if (j >= a.nq) return;
  const int site = a.qsite[j];
  double x = r[3 * site], y = r[3 * site + 1], z = r[3 * site + 2];
  if (a.qdrude && a.qdrude[j]) {
    x += r[3 * (long)a.ns + 3 * site];
    y += r[3 * (long)a.ns + 3 * site + 1];
    z += r[3 * (long)a.ns + 3 * site + 2];
  }
  qf[j] = make_uint4((unsigned)fixed32(x, a.iLx), (unsigned)fixed32(y, a.iLy),
                     (unsigned)fixed32(z, a.iLz), 0u);
}

__global__ void charge_fixed_kernel(const __grid_constant__ KArgs a, const double* __restrict__ r, uint4* __restrict__ qf) {
  charge_fixed_kernel_body(a, r, qf, blockIdx.x, 0);
}

MG_BODY void phase_tables_mixed_kernel_body(const KArgs& a,
    const uint4* __restrict__ qf,
    float2* __restrict__ tab,
    const int bx_,
    const int by_) {
  long t = (long)bx_ * blockDim.x + threadIdx.x;
  if (t >= (long)a.nq * a.row) return;
  int j = (int)(t / a.row), e = (int)(t % a.row);
  int d, n;
  if (e <= a.Kx) { d = 0; n = e; }
  else if (e <= a.Kx + 2 * a.Ky + 1) { d = 1; n = e - (a.Kx + 1) - a.Ky; }
  else { d = 2; n = e - (a.Kx + 2 * a.Ky + 2); }   // Z(0..Kz) only
  const uint4 S4 = qf[j];
  const unsigned S = d == 0 ? S4.x : (d == 1 ? S4.y : S4.z);
  // exact integer phase n*s mod 1 in units of 2^-32
  int ph = (int)(S * (unsigned int)n);
  float tt = (float)ph * 2.3283064365386963e-10f;   // in [-0.5, 0.5)
  float sn, cs;
  sincospif(2.f * tt, &sn, &cs);
  if (d == 0) {
    float q = (float)a.qval[j];
    cs *= q;
    sn *= q;
  }
  tab[t] = make_float2(cs, sn);
}

__global__ void phase_tables_mixed_kernel(const __grid_constant__ KArgs a, const uint4* __restrict__ qf, float2* __restrict__ tab) {
  phase_tables_mixed_kernel_body(a, qf, tab, blockIdx.x, 0);
}

__global__ void phase_tables_fp64_kernel(KArgs a, const double* __restrict__ r,
                                         double2* __restrict__ tab) {
  long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)a.nq * a.row) return;
  int j = (int)(t / a.row), e = (int)(t % a.row);
  int site = a.qsite[j];
  int d, n;
  if (e <= a.Kx) { d = 0; n = e; }
  else if (e <= a.Kx + 2 * a.Ky + 1) { d = 1; n = e - (a.Kx + 1) - a.Ky; }
  else { d = 2; n = e - (a.Kx + 2 * a.Ky + 2) - a.Kz; }
  double Lb = d == 0 ? a.Lx : (d == 1 ? a.Ly : a.Lz);
  double xd = r[3 * site + d];
  if (a.qdrude && a.qdrude[j]) xd += r[3 * (long)a.ns + 3 * site + d];
  double s = xd / Lb;
  double ph = n * s;
  ph -= rint(ph);
  double sn, cs;
  sincospi(2.0 * ph, &sn, &cs);
  if (d == 0) {
    cs *= a.qval[j];
    sn *= a.qval[j];
  }
  tab[t] = make_double2(cs, sn);
}

cudaError_t k_phase_tables_mixed(const Launch& L, const KArgs& a, const double* r, float2* tab,
                                 uint4* qf) {
  charge_fixed_kernel<<<cdiv(a.nq, 256), 256, 0, L.s>>>(a, r, qf);
  LAUNCHED(L);
  long n = (long)a.nq * a.row;
  phase_tables_mixed_kernel<<<(int)((n + 255) / 256), 256, 0, L.s>>>(a, qf, tab);
  LAUNCHED(L);
  return cudaGetLastError();
}
cudaError_t k_phase_tables_fp64(const Launch& L, const KArgs& a, const double* r, double2* tab) {
  long n = (long)a.nq * a.row;
  phase_tables_fp64_kernel<<<(int)((n + 255) / 256), 256, 0, L.s>>>(a, r, tab);
  LAUNCHED(L);
  return cudaGetLastError();
}

template <typename T2>
struct CplxOps;
template <>
struct CplxOps<float2> {
  typedef float T;
  static __device__ __forceinline__ float2 mul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
  }
};
template <>
struct CplxOps<double2> {
  typedef double T;
  static __device__ __forceinline__ double2 mul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
  }
};

constexpr int SK_THREADS = 256;

// pass 1: each thread owns one task (<=KZT consecutive kz of a column) and
// sums q X Y Z over the charges of its chunk; charge rows are staged in
// shared memory STAGE at a time.
template <typename T2>
__global__ void __launch_bounds__(SK_THREADS)
    sk_kernel(KArgs a, const T2* __restrict__ tab, T2* __restrict__ part, int stage) {
  extern __shared__ unsigned char smem_raw[];
  T2* rows = reinterpret_cast<T2*>(smem_raw);
  const int ch = blockIdx.y;
  const int j0 = (int)((long)a.nq * ch / a.nchunk), j1 = (int)((long)a.nq * (ch + 1) / a.nchunk);
  const int tk = blockIdx.x * SK_THREADS + threadIdx.x;
  const bool valid = tk < a.ntask;
  KTask tsk = valid ? a.task[tk] : KTask{0, 0, 0, 0, 0, {0, 0, 0}};
  const int ix = tsk.kx, iy = a.Kx + 1 + a.Ky + tsk.ky,
            iz = a.Kx + 2 * a.Ky + 2 + a.Kz + tsk.kz0;
  T2 S[KZT];
#pragma unroll
  for (int m = 0; m < KZT; m++) S[m] = T2{0, 0};
  for (int js = j0; js < j1; js += stage) {
    const int nst = min(stage, j1 - js);
    __syncthreads();
    for (int t = threadIdx.x; t < nst * a.row; t += SK_THREADS)
      rows[t] = tab[(long)js * a.row + t];
    __syncthreads();
    if (valid) {
      for (int jj = 0; jj < nst; jj++) {
        const T2* R = rows + jj * a.row;
        const T2 U = CplxOps<T2>::mul(R[ix], R[iy]);
#pragma unroll
        for (int m = 0; m < KZT; m++) {
          if (m < tsk.n) {
            const T2 Z = R[iz + m];
            const T2 p = CplxOps<T2>::mul(U, Z);
            S[m].x += p.x;
            S[m].y += p.y;
          }
        }
      }
    }
  }
  if (valid) {
#pragma unroll
    for (int m = 0; m < KZT; m++)
      if (m < tsk.n) part[(long)ch * a.nk + tsk.k0 + m] = S[m];
  }
}

template <typename T2>
static cudaError_t launch_sk(const Launch& L, const KArgs& a, const T2* tab, T2* part) {
  int stage = (int)(40960 / (a.row * sizeof(T2)));
  if (stage < 1) stage = 1;
  if (stage > 64) stage = 64;
  size_t smem = (size_t)stage * a.row * sizeof(T2);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(sk_kernel<T2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  dim3 grid(cdiv(a.ntask, SK_THREADS), a.nchunk);
  sk_kernel<T2><<<grid, SK_THREADS, smem, L.s>>>(a, tab, part, stage);
  LAUNCHED(L);
  return cudaGetLastError();
}

cudaError_t k_sk_mixed(const Launch& L, const KArgs& a, const float2* tab, float2* part) {
  return launch_sk<float2>(L, a, tab, part);
}
cudaError_t k_sk_fp64(const Launch& L, const KArgs& a, const double2* tab, double2* part) {
  return launch_sk<double2>(L, a, tab, part);
}

// S(k) = sum over chunks (FP64, fixed order); energy and virial per k
// (sim/ewpass2m.c: E1 = |S|^2 ekk, ptf = 1/kk + (pi/alpha)^2) reduced per block
template <typename T2>
MG_BODY void sk_reduce_kernel_body(const KArgs& a,
    const T2* __restrict__ part,
    bool measure,
    double pi2_over_a2,
    const int bx_,
    const int by_) {
  __shared__ double red[256][7];
  const int k = bx_ * 256 + threadIdx.x;
  double e[7] = {0, 0, 0, 0, 0, 0, 0};
  if (k < a.nk) {
    double sr = 0, si = 0;
    for (int c = 0; c < a.nchunk; c++) {
      T2 v = part[(long)c * a.nk + k];
      sr += v.x;
      si += v.y;
    }
    a.S[2 * k] = sr;
    a.S[2 * k + 1] = si;
    const double ek = a.ekk[k];
    if (a.Wf) a.Wf[k] = make_float2((float)(ek * sr), (float)(-ek * si));
    if (a.Wd) a.Wd[k] = make_double2(ek * sr, -ek * si);
    if (measure) {
      const int4 kv = a.kvec[k];
      const double kx = kv.x / a.Lx, ky = kv.y / a.Ly, kz = kv.z / a.Lz;
      const double kk = kx * kx + ky * ky + kz * kz;
      const double E1 = (sr * sr + si * si) * a.ekk[k];
      const double ptf = 1 / kk + pi2_over_a2;
      e[0] = E1;
      e[1] = E1 * ptf * kx * kx;
      e[2] = E1 * ptf * ky * ky;
      e[3] = E1 * ptf * kz * kz;
      e[4] = E1 * ptf * ky * kz;
      e[5] = E1 * ptf * kx * kz;
      e[6] = E1 * ptf * kx * ky;
    }
  }
  if (!measure) return;
  for (int m = 0; m < 7; m++) red[threadIdx.x][m] = e[m];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int m = 0; m < 7; m++) red[threadIdx.x][m] += red[threadIdx.x + w][m];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int m = 0; m < 7; m++) a.ek_part[bx_ * 7 + m] = red[0][m];
}

template <typename T2>
__global__ void sk_reduce_kernel(const __grid_constant__ KArgs a, const T2* __restrict__ part, bool measure, double pi2_over_a2) {
  sk_reduce_kernel_body<T2>(a, part, measure, pi2_over_a2, blockIdx.x, 0);
}

cudaError_t k_sk_reduce_mixed(const Launch& L, const KArgs& a, const float2* part, bool measure) {
  const double pa = 9.869604401089358 / (a.alpha * a.alpha);
  sk_reduce_kernel<float2><<<cdiv(a.nk, 256), 256, 0, L.s>>>(a, part, measure, pa);
  LAUNCHED(L);
  return cudaGetLastError();
}
cudaError_t k_sk_reduce_fp64(const Launch& L, const KArgs& a, const double2* part, bool measure) {
  const double pa = 9.869604401089358 / (a.alpha * a.alpha);
  sk_reduce_kernel<double2><<<cdiv(a.nk, 256), 256, 0, L.s>>>(a, part, measure, pa);
  LAUNCHED(L);
  return cudaGetLastError();
}

// pass 2 (sim/ewpass2.c + sim/ewaldf.c): F_j += sum_k ekk (k/L) Im(conj(S_k) q_j e^{2 pi i k.r_j/L}).
// One thread per charge; the k list is walked column by column ((kx,ky) with
// consecutive kz): the phase at the first kz of a column comes from the
// per-charge rows (X Y Z products), later ones from the recurrence
// P <- P e^{2 pi i z/L}.  Column sums are FP32, folded into FP64 every
// KFOLD columns.
constexpr int KF_THREADS = 128;
constexpr int KFOLD = 16;

template <typename T2>
__global__ void __launch_bounds__(KF_THREADS)
    kforce_kernel(KArgs a, const T2* __restrict__ tab, const T2* __restrict__ W) {
  typedef typename CplxOps<T2>::T T;
  const int j = blockIdx.x * KF_THREADS + threadIdx.x;
  if (j >= a.nq) return;
  const T2* R = tab + (long)j * a.row;
  const int oy = a.Kx + 1 + a.Ky, oz = a.Kx + 2 * a.Ky + 2 + a.Kz;
  const T2 ez = a.Kz >= 1 ? R[oz + 1] : T2{1, 0};
  double Fx = 0, Fy = 0, Fz = 0;
  T gx = 0, gy = 0, gz = 0;
  int nf = 0;
  for (int c = 0; c < a.ncol; c++) {
    const KCol col = a.col[c];
    T2 P = CplxOps<T2>::mul(CplxOps<T2>::mul(R[col.kx], R[oy + col.ky]), R[oz + col.kz0]);
    T G = 0, Gz = 0;
    for (int m = 0; m < col.n; m++) {
      // W_k = ekk conj(S_k): g = ekk Im(conj(S) P)
      const T2 Wk = W[col.k0 + m];
      const T g = Wk.x * P.y + Wk.y * P.x;
      G += g;
      Gz += (T)(col.kz0 + m) * g;
      P = CplxOps<T2>::mul(P, ez);
    }
    gx += (T)col.kx * G;
    gy += (T)col.ky * G;
    gz += Gz;
    if (++nf == KFOLD) {
      nf = 0;
      Fx += gx; Fy += gy; Fz += gz;
      gx = gy = gz = 0;
    }
  }
  Fx += gx; Fy += gy; Fz += gz;
  const int site = a.qsite[j];
  a.f[3 * site] += Fx / a.Lx;
  a.f[3 * site + 1] += Fy / a.Ly;
  a.f[3 * site + 2] += Fz / a.Lz;
}

cudaError_t k_kforce_mixed(const Launch& L, const KArgs& a, const float2* tab) {
  kforce_kernel<float2><<<cdiv(a.nq, KF_THREADS), KF_THREADS, 0, L.s>>>(a, tab, a.Wf);
  LAUNCHED(L);
  return cudaGetLastError();
}
cudaError_t k_kforce_fp64(const Launch& L, const KArgs& a, const double2* tab) {
  kforce_kernel<double2><<<cdiv(a.nq, KF_THREADS), KF_THREADS, 0, L.s>>>(a, tab, a.Wd);
  LAUNCHED(L);
  return cudaGetLastError();
}

// out[k] = sum over rows of part[row*width+k], fixed order (one CTA)
MG_BODY void reduce_rows_kernel_body(const double* __restrict__ part,
    int nrows,
    int width,
    double* __restrict__ out,
    const int bx_,
    const int by_) {
  __shared__ double red[256];
  for (int k = 0; k < width; k++) {
    double s = 0;
    for (int r = threadIdx.x; r < nrows; r += 256) s += part[(long)r * width + k];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[k] = red[0];
    __syncthreads();
  }
}

__global__ void reduce_rows_kernel(const double* __restrict__ part, int nrows, int width, double* __restrict__ out) {
  reduce_rows_kernel_body(part, nrows, width, out, blockIdx.x, 0);
}

cudaError_t k_reduce_sum(const Launch& L, const double* part, int nrows, int width, double* out) {
  reduce_rows_kernel<<<1, 256, 0, L.s>>>(part, nrows, width, out);
  LAUNCHED(L);
  return cudaGetLastError();
}

// -------------------------------------------------------------- SHAKE --

// sim/constrd.c:767-839 + sim/verlet.c:101-104 + sim/shakev3.c (SHAKE=1,
// VERLET=3; Nose-Hoover's friction term of sim/verlet.c:22-37 when the
// thermostat state is given), one thread per molecule, FP64.  The new
// positions are then wrapped as cook's normalize(-1) does after the step
// (sim/norm.c:415-444): the molecule's lowest coordinate over its massive
// sites decides a shift of +L (below r0), -L (at or above r0 + L) or none.
constexpr int SH_THREADS = 128;

__device__ __forceinline__ double wrap_shift(double lo, double r0, double L) {
  return lo < r0 ? L : (lo >= r0 + L ? -L : 0.0);
}

// three-site, three-constraint molecules (rigid water) with the positions in
// registers: the same sweeps in the same order as the general path below
// (which works on the global array p), 15 FP64 operations per constraint
// and sweep: the per-constraint factors m^-1 omega/(m_i^-1 + m_j^-1)/d^2 and
// the tolerance eps d^2 are formed once per call (FP64 divisions and
// multiplications are slow on this GPU's narrow FP64 pipe).
__device__ __forceinline__ double3 sh_get(int k, const double3& a, const double3& b,
                                          const double3& c) {
  return k == 0 ? a : (k == 1 ? b : c);
}
__device__ __forceinline__ void sh_add(int k, double3& a, double3& b, double3& c, double s,
                                       double x, double y, double z) {
  if (k == 0) { a.x += s * x; a.y += s * y; a.z += s * z; }
  else if (k == 1) { b.x += s * x; b.y += s * y; b.z += s * z; }
  else { c.x += s * x; c.y += s * y; c.z += s * z; }
}

// Nose-Hoover with Verlet + SHAKE (cook's T_NOSE): the time-reversible
// velocity predictor of length k (sim/trvpscale.c:31-57; J. Chem. Theory
// Comput. 7, 3596 (2011)), b_0 = (2k+1)/(k+1), b_{j+1} = -b_j (k-j)/(k+j+2),
// predicts h v(t) = sum_j b_j r1(t - j h) for every degree of freedom and
// Vfactor = h dlogs/dt from the history of logs; the step then adds
// -Vfactor vpred to h^2 f/m (sim/verlet.c:22-37).  k grows by one per step
// up to the predictor length.
struct NoseStep {
  double b[MG_NOSE_MAXPRED + 1];
  double vf;
  int k, knew;
};

__device__ __forceinline__ NoseStep nose_begin(const ShakeArgs& a) {
  NoseStep q;
  q.k = (int)a.nh[NH_K];
  q.knew = min(a.nh_pred, q.k + 1);
  q.b[0] = (double)(2 * q.k + 1) / (q.k + 1);
  for (int j = 0; j < q.k; j++) q.b[j + 1] = -q.b[j] * (double)(q.k - j) / (q.k + j + 2);
  q.vf = 0;
  q.vf += q.b[0] * a.nh[NH_LOGSV];
  for (int j = 1; j <= q.k; j++) q.vf += q.b[j] * a.nh[NH_HIST + j - 1];
  return q;
}

// the friction displacement of degree of freedom t (r1 = its r1(t)); the
// history moves one slot back and takes r1
__device__ __forceinline__ double nose_dof(const ShakeArgs& a, const NoseStep& q, long long t,
                                           double r1) {
  double v = 0;
  v += q.b[0] * r1;
  for (int j = 1; j <= q.k; j++) v += q.b[j] * a.vhist[(j - 1) * a.nstride + t];
  for (int j = q.knew - 1; j >= 1; j--) a.vhist[j * a.nstride + t] = a.vhist[(j - 1) * a.nstride + t];
  if (q.knew > 0) a.vhist[t] = r1;
  return -q.vf * v;
}

// the measured quantities of a SHAKE step (MEAS): cook's En.virc and
// PTvirc (sim/virc.c, summed over the sweeps before the division by h^2 of
// sim/constrd.c:1038-1040) and the VERLET=3 kinetic tensor sum
// m (V1 V1 + V2 V2) of sim/shakev3.c:20-32 (before hscale), per molecule
struct ShakeMeas {
  double virc, pt[6], pk[6];
};
__device__ __forceinline__ void meas_zero(ShakeMeas& m) {
  m.virc = 0;
#pragma unroll
  for (int k = 0; k < 6; k++) m.pt[k] = m.pk[k] = 0;
}
// constraint virial of one constraint: virc += sq, PTvirc += (sq/bondq) rij rij
// (xx yy zz yz zx xy); sq = the sweep sum of (bondq - |pij|^2) omega/(mi+mj)
__device__ __forceinline__ void meas_cons(ShakeMeas& m, double sq, double sqb, double x, double y,
                                          double z) {
  m.virc += sq;
  m.pt[0] += sqb * (x * x);
  m.pt[1] += sqb * (y * y);
  m.pt[2] += sqb * (z * z);
  m.pt[3] += sqb * (y * z);
  m.pt[4] += sqb * (z * x);
  m.pt[5] += sqb * (x * y);
}
__device__ __forceinline__ void meas_kin(ShakeMeas& m, double mi, double v1x, double v1y,
                                         double v1z, double v2x, double v2y, double v2z) {
  m.pk[0] += (v1x * v1x + v2x * v2x) * mi;
  m.pk[1] += (v1y * v1y + v2y * v2y) * mi;
  m.pk[2] += (v1z * v1z + v2z * v2z) * mi;
  m.pk[3] += (v1y * v1z + v2y * v2z) * mi;
  m.pk[4] += (v1z * v1x + v2z * v2x) * mi;
  m.pk[5] += (v1x * v1y + v2x * v2y) * mi;
}

// ---- float-float SHAKE sweeps (mixed path, three-site molecules) ----
//
// The sweeps of the three-site path in float-float arithmetic: every site's
// position relative to the molecule's first site as hi + lo floats (about
// 48 bits), the bond vector and its squared length to about 1e-14 A^2, the
// deviation d then rounded to float (it only scales the displacements and
// meets the tolerance test).  The FP64 sweeps run on GB300's narrow FP64
// pipe; these run on the FP32 pipe.  Every rounding is explicit (`_rn`), so
// the measuring and the plain instantiation sweep identically.

__device__ __forceinline__ void ff_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fadd_rn(s, -a);
  e = __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -bb)), __fadd_rn(b, -bb));
}
__device__ __forceinline__ float ff_sel(int k, const float (&v)[3]) {
  return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]);
}
// (h, l) of site k += v: the hi sum's rounding error goes into lo exactly
__device__ __forceinline__ void ff_add(int k, float (&h)[3], float (&l)[3], float v) {
#pragma unroll
  for (int s = 0; s < 3; s++)
    if (s == k) {
      float t, e;
      ff_two_sum(h[s], v, t, e);
      h[s] = t;
      l[s] = __fadd_rn(l[s], e);
    }
}
// component of p_i - p_j: (hi, lo), not renormalised
__device__ __forceinline__ void ff_diff(int i, int j, const float (&h)[3], const float (&l)[3],
                                        float& dh, float& dl) {
  float e;
  ff_two_sum(ff_sel(i, h), -ff_sel(j, h), dh, e);
  dl = __fadd_rn(e, __fadd_rn(ff_sel(i, l), -ff_sel(j, l)));
}

// the SHAKE sweeps of cook (sim/constrd.c:821-839) on the three sites P
// (updated in place); returns true if the tolerance was not met in maxit
// sweeps; dsum: the deviations summed per constraint (measured steps)
template <bool MEAS>
__device__ __forceinline__ bool shake3_ff(double3 (&P)[3], const int (&ci)[3], const int (&cj)[3],
                                          const double (&bq)[3], const double (&tol)[3],
                                          const double (&awi)[3], const double (&awj)[3],
                                          const double (&rx)[3], const double (&ry)[3],
                                          const double (&rz)[3], int maxit,
                                          double (&dsum)[3]) {
  const double3 o = P[0];
  float hx[3], hy[3], hz[3], lx[3], ly[3], lz[3];
#pragma unroll
  for (int s = 0; s < 3; s++) {
    const double ux = P[s].x - o.x, uy = P[s].y - o.y, uz = P[s].z - o.z;
    hx[s] = __double2float_rn(ux);
    hy[s] = __double2float_rn(uy);
    hz[s] = __double2float_rn(uz);
    lx[s] = __double2float_rn(ux - (double)hx[s]);
    ly[s] = __double2float_rn(uy - (double)hy[s]);
    lz[s] = __double2float_rn(uz - (double)hz[s]);
  }
  float bqh[3], bql[3], tf[3], wi[3], wj[3], qx[3], qy[3], qz[3];
#pragma unroll
  for (int q = 0; q < 3; q++) {
    bqh[q] = __double2float_rn(bq[q]);
    bql[q] = __double2float_rn(bq[q] - (double)bqh[q]);
    tf[q] = __double2float_rn(tol[q]);
    wi[q] = __double2float_rn(awi[q]);
    wj[q] = __double2float_rn(awj[q]);
    qx[q] = __double2float_rn(rx[q]);
    qy[q] = __double2float_rn(ry[q]);
    qz[q] = __double2float_rn(rz[q]);
  }
  int it = 0;
  bool over;
  do {
    it++;
    over = false;
#pragma unroll
    for (int q = 0; q < 3; q++) {
      const int i = ci[q], j = cj[q];
      float xh, xl, yh, yl, zh, zl;
      ff_diff(i, j, hx, lx, xh, xl);
      ff_diff(i, j, hy, ly, yh, yl);
      ff_diff(i, j, hz, lz, zh, zl);
      // squares: hi^2 exactly as p + e, plus 2 hi lo
      const float px = __fmul_rn(xh, xh), py = __fmul_rn(yh, yh), pz = __fmul_rn(zh, zh);
      const float ex = __fmaf_rn(__fmul_rn(2.f, xh), xl, __fmaf_rn(xh, xh, -px)),
                  ey = __fmaf_rn(__fmul_rn(2.f, yh), yl, __fmaf_rn(yh, yh, -py)),
                  ez = __fmaf_rn(__fmul_rn(2.f, zh), zl, __fmaf_rn(zh, zh, -pz));
      float s1, e1, s2, e2;
      ff_two_sum(px, py, s1, e1);
      ff_two_sum(s1, pz, s2, e2);
      const float E = __fadd_rn(__fadd_rn(__fadd_rn(e1, e2), __fadd_rn(ex, ey)), ez);
      // d = bq - |p_i - p_j|^2
      float t, te;
      ff_two_sum(bqh[q], -s2, t, te);
      const float d = __fadd_rn(t, __fadd_rn(te, __fadd_rn(bql[q], -E)));
      over |= fabsf(d) > tf[q];
      if constexpr (MEAS) dsum[q] += (double)d;
      const float gi = __fmul_rn(d, wi[q]), gj = __fmul_rn(d, wj[q]);
      ff_add(i, hx, lx, __fmul_rn(gi, qx[q]));
      ff_add(i, hy, ly, __fmul_rn(gi, qy[q]));
      ff_add(i, hz, lz, __fmul_rn(gi, qz[q]));
      ff_add(j, hx, lx, __fmul_rn(gj, qx[q]));
      ff_add(j, hy, ly, __fmul_rn(gj, qy[q]));
      ff_add(j, hz, lz, __fmul_rn(gj, qz[q]));
    }
  } while (over && it < maxit);
#pragma unroll
  for (int s = 0; s < 3; s++)
    P[s] = make_double3(o.x + ((double)hx[s] + (double)lx[s]), o.y + ((double)hy[s] + (double)ly[s]),
                        o.z + ((double)hz[s] + (double)lz[s]));
  return over;
}

template <bool NOSE, bool MEAS, bool DF>
MG_BODY void shake_kernel_body(const ShakeArgs& a,
    const int bx_,
    const int by_) {
  __shared__ double red[SH_THREADS];
  const int n = bx_ * SH_THREADS + threadIdx.x;
  double kin = 0;
  [[maybe_unused]] ShakeMeas ms;
  if constexpr (MEAS) meas_zero(ms);
  [[maybe_unused]] NoseStep nose;
  if constexpr (NOSE) nose = nose_begin(a);
  if (n < a.nmol) {
    const int i0 = a.mol_first[n], i1 = a.mol_first[n + 1];
    const int c0 = a.mol_cfirst[n], c1 = a.mol_cfirst[n + 1];
    if (i1 - i0 == 3 && c1 - c0 == 3) {
      double3 P[3], R[3];
      double im[3];
#pragma unroll
      for (int s = 0; s < 3; s++) {
        const int i = i0 + s;
        R[s] = make_double3(a.r[3 * i], a.r[3 * i + 1], a.r[3 * i + 2]);
        im[s] = a.imass[i];
        if constexpr (NOSE) {
          const double dx = nose_dof(a, nose, 3 * i, a.r1[3 * i]);
          const double dy = nose_dof(a, nose, 3 * i + 1, a.r1[3 * i + 1]);
          const double dz = nose_dof(a, nose, 3 * i + 2, a.r1[3 * i + 2]);
          P[s] = make_double3(a.f[3 * i] * (a.hh * im[s]) + dx + R[s].x + a.r1[3 * i],
                              a.f[3 * i + 1] * (a.hh * im[s]) + dy + R[s].y + a.r1[3 * i + 1],
                              a.f[3 * i + 2] * (a.hh * im[s]) + dz + R[s].z + a.r1[3 * i + 2]);
        } else {
          P[s] = make_double3(a.f[3 * i] * (a.hh * im[s]) + R[s].x + a.r1[3 * i],
                              a.f[3 * i + 1] * (a.hh * im[s]) + R[s].y + a.r1[3 * i + 1],
                              a.f[3 * i + 2] * (a.hh * im[s]) + R[s].z + a.r1[3 * i + 2]);
        }
      }
      // per constraint: the tolerance as a bound on |d| (eps bq, so no
      // product per sweep) and the factors m_i^-1 wq, m_j^-1 wq that turn d
      // into the two displacements along r_ij
      int ci[3], cj[3];
      double bq[3], tol[3], awi[3], awj[3], rx[3], ry[3], rz[3];
      [[maybe_unused]] double dsum[3] = {0, 0, 0};
#pragma unroll
      for (int q = 0; q < 3; q++) {
        const int2 ij = a.cons[c0 + q];
        ci[q] = ij.x - i0;
        cj[q] = ij.y - i0;
        bq[q] = a.bondq[c0 + q];
        const double mi = a.imass[ij.x], mj = a.imass[ij.y];
        const double wq = a.omega / (mi + mj) * (1.0 / bq[q]);
        tol[q] = a.eps * bq[q];
        awi[q] = mi * wq;
        awj[q] = -(mj * wq);
        const double3 ri = sh_get(ci[q], R[0], R[1], R[2]), rj = sh_get(cj[q], R[0], R[1], R[2]);
        rx[q] = ri.x - rj.x;
        ry[q] = ri.y - rj.y;
        rz[q] = ri.z - rj.z;
      }
      int it = 0;
      bool over = false;
      if constexpr (DF) over = shake3_ff<MEAS>(P, ci, cj, bq, tol, awi, awj, rx, ry, rz, a.maxit, dsum);
      else do {
        it++;
        over = false;
#pragma unroll
        for (int q = 0; q < 3; q++) {
          const double3 pi = sh_get(ci[q], P[0], P[1], P[2]), pj = sh_get(cj[q], P[0], P[1], P[2]);
          const double px = pi.x - pj.x, py = pi.y - pj.y, pz = pi.z - pj.z;
          const double d = bq[q] - (px * px + py * py + pz * pz);
          over |= fabs(d) > tol[q];
          if constexpr (MEAS) dsum[q] += d;
          sh_add(ci[q], P[0], P[1], P[2], d * awi[q], rx[q], ry[q], rz[q]);
          sh_add(cj[q], P[0], P[1], P[2], d * awj[q], rx[q], ry[q], rz[q]);
        }
      } while (over && it < a.maxit);
      if (over) atomicOr(a.status, 1);
      if constexpr (MEAS) {
#pragma unroll
        for (int q = 0; q < 3; q++) {
          const int2 ij = a.cons[c0 + q];
          const double wb = a.omega / (a.imass[ij.x] + a.imass[ij.y]);
          meas_cons(ms, dsum[q] * wb, dsum[q] * wb / bq[q], rx[q], ry[q], rz[q]);
        }
      }
      double sx = 0, sy = 0, sz = 0;
      if (a.normalize) {
        double lx = 9e9, ly = 9e9, lz = 9e9;
#pragma unroll
        for (int s = 0; s < 3; s++)
          if (a.mass[i0 + s] != 0) {
            lx = fmin(lx, P[s].x);
            ly = fmin(ly, P[s].y);
            lz = fmin(lz, P[s].z);
          }
        sx = wrap_shift(lx, a.r0, a.Lb[0]);
        sy = wrap_shift(ly, a.r0, a.Lb[1]);
        sz = wrap_shift(lz, a.r0, a.Lb[2]);
      }
#pragma unroll
      for (int s = 0; s < 3; s++) {
        const int i = i0 + s;
        const double v1x = a.r1[3 * i], v1y = a.r1[3 * i + 1], v1z = a.r1[3 * i + 2];
        const double v2x = P[s].x - R[s].x, v2y = P[s].y - R[s].y, v2z = P[s].z - R[s].z;
        double v1s = 0, v2s = 0;
        v1s += v1x * v1x;
        v2s += v2x * v2x;
        v1s += v1y * v1y;
        v2s += v2y * v2y;
        v1s += v1z * v1z;
        v2s += v2z * v2z;
        kin += (v1s + v2s) * a.mass[i];
        if constexpr (MEAS) meas_kin(ms, a.mass[i], v1x, v1y, v1z, v2x, v2y, v2z);
        a.r1[3 * i] = v2x;
        a.r1[3 * i + 1] = v2y;
        a.r1[3 * i + 2] = v2z;
        a.r[3 * i] = P[s].x + sx;
        a.r[3 * i + 1] = P[s].y + sy;
        a.r[3 * i + 2] = P[s].z + sz;
      }
    } else {
    double* p = a.p;
    for (int i = i0; i < i1; i++)
      for (int k = 0; k < 3; k++)
        if constexpr (NOSE)
          p[3 * i + k] = a.f[3 * i + k] * (a.hh * a.imass[i]) +
                         nose_dof(a, nose, 3 * i + k, a.r1[3 * i + k]) + a.r[3 * i + k] +
                         a.r1[3 * i + k];
        else
          p[3 * i + k] = a.f[3 * i + k] * (a.hh * a.imass[i]) + a.r[3 * i + k] + a.r1[3 * i + k];
    if (c1 > c0) {
      int it = 0;
      double maxsq;
      do {
        it++;
        maxsq = 0;
        for (int al = c0; al < c1; al++) {
          const int2 ij = a.cons[al];
          const double bq = a.bondq[al];
          const double mi = a.imass[ij.x], mj = a.imass[ij.y];
          const double ibq = 1.0 / bq, wq = a.omega / (mi + mj) * ibq;
          double px = p[3 * ij.x] - p[3 * ij.y], py = p[3 * ij.x + 1] - p[3 * ij.y + 1],
                 pz = p[3 * ij.x + 2] - p[3 * ij.y + 2];
          const double d = bq - (px * px + py * py + pz * pz);
          maxsq = fmax(maxsq, fabs(d) * ibq);
          const double sq = d * wq;
          if constexpr (MEAS)
            meas_cons(ms, d * (a.omega / (mi + mj)), sq, a.r[3 * ij.x] - a.r[3 * ij.y],
                      a.r[3 * ij.x + 1] - a.r[3 * ij.y + 1], a.r[3 * ij.x + 2] - a.r[3 * ij.y + 2]);
          const double rx = (a.r[3 * ij.x] - a.r[3 * ij.y]) * sq,
                       ry = (a.r[3 * ij.x + 1] - a.r[3 * ij.y + 1]) * sq,
                       rz = (a.r[3 * ij.x + 2] - a.r[3 * ij.y + 2]) * sq;
          p[3 * ij.x] += mi * rx;
          p[3 * ij.x + 1] += mi * ry;
          p[3 * ij.x + 2] += mi * rz;
          p[3 * ij.y] -= mj * rx;
          p[3 * ij.y + 1] -= mj * ry;
          p[3 * ij.y + 2] -= mj * rz;
        }
      } while (maxsq > a.eps && it < a.maxit);
      if (maxsq > a.eps) atomicOr(a.status, 1);
    }
    double sh[3] = {0, 0, 0};
    if (a.normalize)
      for (int k = 0; k < 3; k++) {
        double lo = 9e9;
        for (int i = i0; i < i1; i++)
          if (a.mass[i] != 0) lo = fmin(lo, p[3 * i + k]);
        sh[k] = wrap_shift(lo, a.r0, a.Lb[k]);
      }
    for (int i = i0; i < i1; i++) {
      double v1s = 0, v2s = 0, v1[3], v2[3];
      for (int k = 0; k < 3; k++) {
        v1[k] = a.r1[3 * i + k];
        v2[k] = p[3 * i + k] - a.r[3 * i + k];
        v1s += v1[k] * v1[k];
        v2s += v2[k] * v2[k];
        a.r1[3 * i + k] = v2[k];
        a.r[3 * i + k] = p[3 * i + k] + sh[k];
      }
      kin += (v1s + v2s) * a.mass[i];
      if constexpr (MEAS) meas_kin(ms, a.mass[i], v1[0], v1[1], v1[2], v2[0], v2[1], v2[2]);
    }
    }
  }
  red[threadIdx.x] = kin;
  __syncthreads();
  for (int w = SH_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) a.kin_part[bx_] = red[0];
  if constexpr (MEAS) {
    // the 13 measured sums of the CTA in a fixed order: a shuffle tree per
    // warp, then the warps' sums in warp order (red[] is free again)
    __syncthreads();
    double v[13];
    v[0] = ms.virc;
#pragma unroll
    for (int k = 0; k < 6; k++) {
      v[1 + k] = ms.pt[k];
      v[7 + k] = ms.pk[k];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 13; k++) {
      double x = v[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) red[wid * 13 + k] = x;
    }
    __syncthreads();
    if (threadIdx.x < 13) {
      double x = 0;
      for (int w = 0; w < SH_THREADS / 32; w++) x += red[w * 13 + threadIdx.x];
      a.meas_part[(long)bx_ * 13 + threadIdx.x] = x;
    }
  }
}

template <bool NOSE, bool MEAS, bool DF>
__global__ void __launch_bounds__(SH_THREADS) shake_kernel(const __grid_constant__ ShakeArgs a) {
  shake_kernel_body<NOSE, MEAS, DF>(a, blockIdx.x, 0);
}

cudaError_t k_shake(const Launch& L, const ShakeArgs& a) {
  const int nb = cdiv(a.nmol, SH_THREADS);
#define SHAKE_LAUNCH(DF)                                                  \
  do {                                                                    \
    if (a.vhist) {                                                        \
      if (a.meas_part)                                                    \
        shake_kernel<true, true, DF><<<nb, SH_THREADS, 0, L.s>>>(a);      \
      else                                                                \
        shake_kernel<true, false, DF><<<nb, SH_THREADS, 0, L.s>>>(a);     \
    } else {                                                              \
      if (a.meas_part)                                                    \
        shake_kernel<false, true, DF><<<nb, SH_THREADS, 0, L.s>>>(a);     \
      else                                                                \
        shake_kernel<false, false, DF><<<nb, SH_THREADS, 0, L.s>>>(a);    \
    }                                                                     \
  } while (0)
  if (a.ffsweep) SHAKE_LAUNCH(true);
  else SHAKE_LAUNCH(false);
#undef SHAKE_LAUNCH
  LAUNCHED(L);
  return cudaGetLastError();
}

// ---------------------------------------------------------- FP32 probe --

// 8 independent FMA chains per thread: the FP32 issue rate of the device
__global__ void fma_probe_kernel(int iters, float* __restrict__ out) {
  float x[8];
  const float a = 0.999999f, b = 1e-7f;
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = (float)(threadIdx.x + k);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = fmaf(x[k], a, b);
  }
  float s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t k_fma_probe(cudaStream_t s, int blocks, int threads, int iters, float* out) {
  fma_probe_kernel<<<blocks, threads, 0, s>>>(iters, out);
  return cudaGetLastError();
}

}  // namespace mg

namespace mg {

// ------------------------------------------------------------ batches --
//
// The kernels of one MD step over every box of a batch, one launch each:
// blockIdx.y is the box, blockIdx.x the CTA of that box's own grid (the
// same CTAs, threads and arguments as the box's single launch, so every box
// gets its single-launch results bit for bit); CTAs beyond a box's grid
// return at once.

int cell_site_blocks(int ns) { return cdiv(ns, 256); }
int cell_order_blocks(int ncell) { return cdiv(ncell, ORDER_THREADS / 32); }

__global__ void batch_cell_count_kernel(const BoxStep* __restrict__ B) {
  const BoxStep& e = B[blockIdx.y];
  cell_count_kernel_body(e.ns, e.r, e.iL, e.ncx, e.ncy, e.ncz, e.kind, e.mol, e.pfix, e.key,
                         e.count, e.status, blockIdx.x);
}

__global__ void __launch_bounds__(SCAN_THREADS) batch_cell_scan_kernel(const BoxStep* __restrict__ B) {
  const BoxStep& e = B[blockIdx.y];
  cell_scan_kernel_body(e.ncx * e.ncy * e.ncz, e.count, e.start, e.cursor, e.gstart, 0, 0);
}

__global__ void batch_cell_scatter_kernel(const BoxStep* __restrict__ B) {
  const BoxStep& e = B[blockIdx.y];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= e.ns) return;
  e.slot_site[atomicAdd(e.cursor + e.key[i], 1)] = i;
}

__global__ void __launch_bounds__(ORDER_THREADS) batch_cell_order_kernel(const BoxStep* __restrict__ B) {
  const BoxStep& e = B[blockIdx.y];
  if ((int)blockIdx.x >= e.g_order) return;
  cell_order_kernel_body(e.ncx * e.ncy * e.ncz, e.start, e.slot_site, e.pfix, e.order, e.key_s,
                         e.pj, e.gstart, e.gcell, blockIdx.x, 0);
}

template <bool MEASURE>
__global__ void __launch_bounds__(4 * 32) batch_pair_kernel(const BoxStep* __restrict__ B) {
  const BoxStep& e = B[blockIdx.y];
  if ((int)blockIdx.x >= e.g_pair) return;
  pair_mixed_kernel_body<MEASURE, false, true, 4, false>(e.pa, e.pj, e.ptab, e.erd, e.eru, e.sx,
                                                         e.sy, e.sz, e.cq, e.sg, e.al,
                                                         blockIdx.x, 0);
}

template <bool MEASURE>
__global__ void __launch_bounds__(EXCL_THREADS) batch_excl_kernel(const BoxStep* __restrict__ B) {
  const BoxStep& e = B[blockIdx.y];
  if ((int)blockIdx.x >= e.g_excl) return;
  excl_mixed_kernel_body<MEASURE, false>(e.xa, blockIdx.x, 0);
}

__global__ void batch_charge_fixed_kernel(const BoxStep* __restrict__ B) {
  const BoxStep& e = B[blockIdx.y];
  if ((int)blockIdx.x >= e.g_charge) return;
  charge_fixed_kernel_body(e.ka, e.r, e.qf, blockIdx.x, 0);
}

__global__ void batch_phase_kernel(const BoxStep* __restrict__ B) {
  const BoxStep& e = B[blockIdx.y];
  if ((int)blockIdx.x >= e.g_phase) return;
  phase_tables_mixed_kernel_body(e.ka, e.qf, e.tab, blockIdx.x, 0);
}

__global__ void batch_sk_reduce_kernel(const BoxStep* __restrict__ B, bool measure) {
  const BoxStep& e = B[blockIdx.y];
  if ((int)blockIdx.x >= e.g_skr) return;
  const double pa = 9.869604401089358 / (e.ka.alpha * e.ka.alpha);
  sk_reduce_kernel_body<float2>(e.ka, e.part, measure, pa, blockIdx.x, 0);
}

template <bool MEAS>
__global__ void __launch_bounds__(SH_THREADS) batch_shake_kernel(const BoxStep* __restrict__ B) {
  const BoxStep& e = B[blockIdx.y];
  if ((int)blockIdx.x >= e.g_shake) return;
  if (e.sa.ffsweep) shake_kernel_body<false, MEAS, true>(e.sa, blockIdx.x, 0);
  else shake_kernel_body<false, MEAS, false>(e.sa, blockIdx.x, 0);
}

// sums k0..k1-1 of every box (one CTA each)
__global__ void batch_reduce_kernel(const BoxStep* __restrict__ B, int k0, int k1) {
  const BoxStep& e = B[blockIdx.y];
  for (int k = k0; k < k1; k++)
    reduce_rows_kernel_body(e.rpart[k], e.rrows[k], e.rwidth[k], e.rout[k], 0, 0);
}

__global__ void gather_status_kernel(const int* const* __restrict__ p, int n,
                                     int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = *p[i];
}

cudaError_t k_gather_status(cudaStream_t s, const int* const* p, int n, int* out) {
  gather_status_kernel<<<cdiv(n, 256), 256, 0, s>>>(p, n, out);
  return cudaGetLastError();
}

cudaError_t k_batch_cells(const Launch& L, const BoxStep* d, int nbox, const BatchGrid& g) {
  batch_cell_count_kernel<<<dim3(g.site, nbox), 256, 0, L.s>>>(d);
  batch_cell_scan_kernel<<<dim3(1, nbox), SCAN_THREADS, 0, L.s>>>(d);
  batch_cell_scatter_kernel<<<dim3(g.site, nbox), 256, 0, L.s>>>(d);
  batch_cell_order_kernel<<<dim3(g.order, nbox), ORDER_THREADS, 0, L.s>>>(d);
  *L.counter += 4;
  return cudaGetLastError();
}

cudaError_t k_batch_pairs(const Launch& L, const BoxStep* d, int nbox, const BatchGrid& g,
                          bool measure) {
  cudaError_t e = cudaSuccess;
  if (measure) {
    if (g.pair_smem > 48 * 1024)
      e = cudaFuncSetAttribute(batch_pair_kernel<true>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.pair_smem);
    if (e == cudaSuccess)
      batch_pair_kernel<true><<<dim3(g.pair, nbox), 128, g.pair_smem, L.s>>>(d);
    if (g.excl > 0) batch_excl_kernel<true><<<dim3(g.excl, nbox), EXCL_THREADS, 0, L.s>>>(d);
  } else {
    if (g.pair_smem > 48 * 1024)
      e = cudaFuncSetAttribute(batch_pair_kernel<false>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.pair_smem);
    if (e == cudaSuccess)
      batch_pair_kernel<false><<<dim3(g.pair, nbox), 128, g.pair_smem, L.s>>>(d);
    if (g.excl > 0) batch_excl_kernel<false><<<dim3(g.excl, nbox), EXCL_THREADS, 0, L.s>>>(d);
  }
  if (e != cudaSuccess) return e;
  *L.counter += 1 + (g.excl > 0 ? 1 : 0);
  // the FP32-core phase rows (none when every box is on the tensor cores)
  if (g.charge > 0) {
    batch_charge_fixed_kernel<<<dim3(g.charge, nbox), 256, 0, L.s>>>(d);
    ++*L.counter;
  }
  if (g.phase > 0) {
    batch_phase_kernel<<<dim3(g.phase, nbox), 256, 0, L.s>>>(d);
    ++*L.counter;
  }
  return cudaGetLastError();
}

cudaError_t k_batch_sk_reduce(const Launch& L, const BoxStep* d, int nbox, const BatchGrid& g,
                              bool measure) {
  batch_sk_reduce_kernel<<<dim3(g.skr, nbox), 256, 0, L.s>>>(d, measure);
  LAUNCHED(L);
  return cudaGetLastError();
}

cudaError_t k_batch_step(const Launch& L, const BoxStep* d, int nbox, const BatchGrid& g,
                         bool measure) {
  if (measure) {
    // the energies of the force evaluation (rows 0, 1), the step, its sums (2, 3)
    batch_reduce_kernel<<<dim3(1, nbox), 256, 0, L.s>>>(d, 0, 2);
    batch_shake_kernel<true><<<dim3(g.shake, nbox), SH_THREADS, 0, L.s>>>(d);
    batch_reduce_kernel<<<dim3(1, nbox), 256, 0, L.s>>>(d, 2, 4);
    *L.counter += 3;
  } else {
    batch_shake_kernel<false><<<dim3(g.shake, nbox), SH_THREADS, 0, L.s>>>(d);
    LAUNCHED(L);
  }
  return cudaGetLastError();
}

}  // namespace mg
