// Verlet neighbour lists for the r-space pair sum.
//
// cook re-bins its linked cells every step (cook/lc.c); here the cell list is
// used every few steps to build, per site, the list of sites within
// cutoff+skin, and the pair kernels walk those lists in between.  The set of
// pairs within the cutoff is the same as cook's as long as no site has moved
// more than skin/2 since the build; a kernel checks that every step and
// raises a status bit otherwise.
//
// Lists are stored row-major, entry k of sorted site t at nlist[t*cap + k],
// so that the warp that walks site t's list reads consecutive words.
// Entries are sorted-site indices; sites keep their sorted slot (and the
// fixed-point/FP64 gathers reuse the build's order) until the next build.
#include "mg_internal.h"
#include "mg_device.cuh"

namespace mg {

constexpr int NB_THREADS = 128;
constexpr int NB_WARPS = NB_THREADS / 32;

// One warp per sorted site: the lanes take 32 candidates of a stencil cell
// at a time (the cell's sites are contiguous in the sorted order), and the
// ones within cutoff+skin are compacted with a ballot and appended to the
// site's row in one coalesced store.  Entry order: stencil order, then
// sorted order within a cell (deterministic).
__global__ void __launch_bounds__(NB_THREADS)
    build_list_kernel(ListArgs a, int ns, const int* __restrict__ cell_of,
                      const int4* __restrict__ pj) {
  const int lane = threadIdx.x & 31;
  const int ti = blockIdx.x * NB_WARPS + (threadIdx.x >> 5);
  if (ti >= ns) return;
  const int c = cell_of[ti];
  const int cz = c % a.ncz, cy = (c / a.ncz) % a.ncy, cx = c / (a.ncy * a.ncz);
  const int4 me = pj[ti];
  int* row = a.nlist + (long)ti * a.cap;
  int cnt = 0;
  for (int s = 0; s < a.nstencil; s++) {
    const int4 o = a.stencil[s];
    int x2 = cx + o.x, y2 = cy + o.y, z2 = cz + o.z;
    x2 += (x2 < 0) ? a.ncx : (x2 >= a.ncx ? -a.ncx : 0);
    y2 += (y2 < 0) ? a.ncy : (y2 >= a.ncy ? -a.ncy : 0);
    z2 += (z2 < 0) ? a.ncz : (z2 >= a.ncz ? -a.ncz : 0);
    const int c2 = (x2 * a.ncy + y2) * a.ncz + z2;
    const int j0 = a.cell_start[c2], j1 = a.cell_start[c2 + 1];
    for (int jb = j0; jb < j1; jb += 32) {
      const int tj = jb + lane;
      bool in = false;
      if (tj < j1 && tj != ti) {
        const int4 q = pj[tj];
        const float dx = (float)(int)((unsigned)me.x - (unsigned)q.x) * a.sx;
        const float dy = (float)(int)((unsigned)me.y - (unsigned)q.y) * a.sy;
        const float dz = (float)(int)((unsigned)me.z - (unsigned)q.z) * a.sz;
        in = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < a.rlist2;
      }
      const unsigned m = __ballot_sync(0xffffffffu, in);
      const int pos = cnt + __popc(m & ((1u << lane) - 1u));
      if (in && pos < a.cap) row[pos] = tj;
      cnt += __popc(m);
    }
  }
  if (lane == 0) {
    a.ncount[ti] = min(cnt, a.cap);
    if (cnt > a.cap) atomicOr(a.status, 16);
  }
}

// One warp per home cell, lane = home site (grids of at least 2 cdiv + 1
// cells per edge): the neighbours of a stencil cell are staged once as float
// offsets of their nearest image from the home-cell centre (the pair
// kernel's scheme), and every lane appends its hits to a private buffer of 8
// entries in shared memory that goes to its row as two 16-byte stores.
// Entry order: stencil order, then sorted order (deterministic).
constexpr int NBC_BUF = 8;
__global__ void __launch_bounds__(32)
    build_list_cell_kernel(ListArgs a, const int4* __restrict__ pj) {
  __shared__ float4 sj[32];
  __shared__ int sidx[32];
  __shared__ __align__(16) int buf[32][NBC_BUF];
  const int lane = threadIdx.x;
  const int c = blockIdx.x;
  const int cz = c % a.ncz, cy = (c / a.ncz) % a.ncy, cx = c / (a.ncy * a.ncz);
  const unsigned refx = (unsigned)((((unsigned long long)(2 * cx + 1)) << 31) / a.ncx),
                 refy = (unsigned)((((unsigned long long)(2 * cy + 1)) << 31) / a.ncy),
                 refz = (unsigned)((((unsigned long long)(2 * cz + 1)) << 31) / a.ncz);
  const int i0 = a.cell_start[c], ni = a.cell_start[c + 1] - i0;
  for (int ib = 0; ib < ni; ib += 32) {
    const bool vi = ib + lane < ni;
    const int ti = i0 + ib + lane;
    const int4 me = vi ? pj[ti] : make_int4(0, 0, 0, 0);
    const float xi = (float)(int)((unsigned)me.x - refx) * a.sx,
                yi = (float)(int)((unsigned)me.y - refy) * a.sy,
                zi = (float)(int)((unsigned)me.z - refz) * a.sz;
    int* row = a.nlist + (long)ti * a.cap;
    int cnt = 0, nb = 0;
    for (int s = 0; s < a.nstencil; s++) {
      const int4 o = a.stencil[s];
      int x2 = cx + o.x, y2 = cy + o.y, z2 = cz + o.z;
      x2 += (x2 < 0) ? a.ncx : (x2 >= a.ncx ? -a.ncx : 0);
      y2 += (y2 < 0) ? a.ncy : (y2 >= a.ncy ? -a.ncy : 0);
      z2 += (z2 < 0) ? a.ncz : (z2 >= a.ncz ? -a.ncz : 0);
      const int c2 = (x2 * a.ncy + y2) * a.ncz + z2;
      const int j0 = a.cell_start[c2], nj = a.cell_start[c2 + 1] - j0;
      for (int jb = 0; jb < nj; jb += 32) {
        if (jb + lane < nj) {
          const int4 q = pj[j0 + jb + lane];
          sj[lane] = make_float4((float)(int)((unsigned)q.x - refx) * a.sx,
                                 (float)(int)((unsigned)q.y - refy) * a.sy,
                                 (float)(int)((unsigned)q.z - refz) * a.sz, 0.f);
          sidx[lane] = j0 + jb + lane;
        }
        __syncwarp();
        const int n = min(32, nj - jb);
        for (int jj = 0; jj < n; jj++) {
          const float4 q = sj[jj];
          const float dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
          const int tj = sidx[jj];
          if (vi && fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < a.rlist2 && tj != ti) {
            buf[lane][nb++] = tj;
            if (nb == NBC_BUF) {
              if (cnt + NBC_BUF <= a.cap) {
                int4* d = reinterpret_cast<int4*>(row + cnt);
                d[0] = *reinterpret_cast<const int4*>(&buf[lane][0]);
                d[1] = *reinterpret_cast<const int4*>(&buf[lane][4]);
              }
              cnt += NBC_BUF;
              nb = 0;
            }
          }
        }
        __syncwarp();
      }
    }
    if (vi) {
      for (int k = 0; k < nb; k++)
        if (cnt + k < a.cap) row[cnt + k] = buf[lane][k];
      cnt += nb;
      a.ncount[ti] = min(cnt, a.cap);
      if (cnt > a.cap) atomicOr(a.status, 16);
    }
  }
}

cudaError_t k_build_list_cells(const Launch& L, const ListArgs& a, const int4* pj) {
  build_list_cell_kernel<<<a.ncx * a.ncy * a.ncz, 32, 0, L.s>>>(a, pj);
  ++*L.counter;
  return cudaGetLastError();
}

cudaError_t k_build_list(const Launch& L, const ListArgs& a, int ns, const int* cell_of,
                         const int4* pj) {
  build_list_kernel<<<(ns + NB_WARPS - 1) / NB_WARPS, NB_THREADS, 0, L.s>>>(a, ns, cell_of, pj);
  ++*L.counter;
  return cudaGetLastError();
}

// positions at build time, and the largest displacement since then
__global__ void save_build_kernel(int ns, const double* __restrict__ r, double* __restrict__ rb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 3 * ns) rb[i] = r[i];
}

cudaError_t k_save_build(const Launch& L, int ns, const double* r, double* rb) {
  save_build_kernel<<<(3 * ns + 255) / 256, 256, 0, L.s>>>(ns, r, rb);
  ++*L.counter;
  return cudaGetLastError();
}

// largest squared displacement since the build (as the bits of a float,
// which order like the floats for non-negative values) into *dmax; a site
// beyond skin/2 sets bit 3 of *status (the lists may have missed a pair)
// displacement since the build taken to the nearest image: the per-step
// molecule wrapping moves sites by whole box lengths
__device__ __forceinline__ double near_image(double d, double L, double iL) {
  return d - L * rint(d * iL);
}

__global__ void check_skin_kernel(int ns, const double* __restrict__ r,
                                  const double* __restrict__ rb, double lim2, double3 Lb,
                                  double3 iL, int* __restrict__ status, int* __restrict__ dmax) {
  __shared__ float red[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float d2 = 0.f;
  if (i < ns) {
    const double dx = near_image(r[3 * i] - rb[3 * i], Lb.x, iL.x),
                 dy = near_image(r[3 * i + 1] - rb[3 * i + 1], Lb.y, iL.y),
                 dz = near_image(r[3 * i + 2] - rb[3 * i + 2], Lb.z, iL.z);
    const double dd = dx * dx + dy * dy + dz * dz;
    if (!(dd < lim2)) atomicOr(status, 8);
    d2 = (float)fmin(dd, 1e30);
  }
  red[threadIdx.x] = d2;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicMax(dmax, __float_as_int(red[0]));
}

cudaError_t k_check_skin(const Launch& L, int ns, const double* r, const double* rb, double lim2,
                         const double Lb[3], int* status, int* dmax) {
  check_skin_kernel<<<(ns + 255) / 256, 256, 0, L.s>>>(
      ns, r, rb, lim2, make_double3(Lb[0], Lb[1], Lb[2]),
      make_double3(1 / Lb[0], 1 / Lb[1], 1 / Lb[2]), status, dmax);
  ++*L.counter;
  return cudaGetLastError();
}

// --------------------------------------------------------- list kernels --

constexpr int NL_THREADS = 128;
constexpr int NL_WARPS = NL_THREADS / 32;

// Mixed precision pair sum over the lists: one warp per sorted site, the
// lanes walk its list 32 entries at a time (coalesced list reads, every lane
// busy); per-lane FP32 sums (FP64 for the excluded intramolecular terms),
// reduced over the warp in FP64.  Same pair arithmetic as pair_mixed_kernel
// (cook/ljqqnp.c, ljqqpol.c).
template <bool MEASURE, bool POLAR>
__global__ void __launch_bounds__(NL_THREADS)
    pair_list_mixed_kernel(PairArgs a, ListArgs l, const int4* __restrict__ pj,
                           const PairF* __restrict__ ptab_g, const float4* __restrict__ erd,
                           const float4* __restrict__ eru, float sx, float sy, float sz, float cq,
                           float sgrid, float alpha) {
  __shared__ PairF ptab[MAX_KINDS * MAX_KINDS];
  __shared__ double ered[NL_THREADS];
  const int nk = a.nkind, ntab = a.ntab;
  for (int t = threadIdx.x; t < nk * nk; t += NL_THREADS) ptab[t] = ptab_g[t];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int ti = blockIdx.x * NL_WARPS + (threadIdx.x >> 5);
  double en[NEN];
#pragma unroll
  for (int k = 0; k < NEN; k++) en[k] = 0;
  if (ti < a.ns) {
    const int4 me = pj[ti];
    const float4 md = POLAR ? a.pdj[ti] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int kind_i = me.w & 255, mol_i = me.w >> 8;
    const int cnt = l.ncount[ti];
    const int* row = l.nlist + (long)ti * l.cap;
    double fx = 0, fy = 0, fz = 0, gx = 0, gy = 0, gz = 0;
    float ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0;
    float e_el = 0, e_lj = 0, e_vir = 0;
    PvF pv;
    pv.zero();
    const PairF* prow = ptab + kind_i * nk;
    for (int k = lane; k < cnt; k += 32) {
      const int tj = row[k];
      const int4 q = pj[tj];
      const float dx = (float)(int)((unsigned)me.x - (unsigned)q.x) * sx;
      const float dy = (float)(int)((unsigned)me.y - (unsigned)q.y) * sy;
      const float dz = (float)(int)((unsigned)me.z - (unsigned)q.z) * sz;
      const float rr = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      if (rr >= cq) continue;
      const PairF P = prow[q.w & 255];
      float4 qd = make_float4(0.f, 0.f, 0.f, 0.f);
      if (POLAR) qd = a.pdj[tj];
      if ((q.w >> 8) == mol_i) {
        if (P.qq != 0.f) excl_acc<MEASURE>(dx, dy, dz, P.qqd, alpha, fx, fy, fz, en);
        if (POLAR) {
          if (P.qpc != 0.f)
            excl_acc<MEASURE>(dx + md.x, dy + md.y, dz + md.z, P.qpcd, alpha, gx, gy, gz, en);
          if (P.qcp != 0.f)
            excl_acc<MEASURE>(dx - qd.x, dy - qd.y, dz - qd.z, P.qcpd, alpha, fx, fy, fz, en);
          if (P.qpp != 0.f)
            excl_acc<MEASURE>(dx + md.x - qd.x, dy + md.y - qd.y, dz + md.z - qd.z, P.qppd,
                              alpha, gx, gy, gz, en);
        }
        continue;
      }
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
      if (P.qq != 0.f) f += spline_term<MEASURE>(erd, eru, rr, sgrid, ntab, P.qq, e_el);
      ax = fmaf(f, dx, ax);
      ay = fmaf(f, dy, ay);
      az = fmaf(f, dz, az);
      if (MEASURE) pv.add(dx, dy, dz, f);
      if (POLAR) {
        if (P.qpc != 0.f) {
          const float ex = dx + md.x, ey = dy + md.y, ez = dz + md.z;
          const float fp = spline_term<MEASURE>(erd, eru, fmaf(ex, ex, fmaf(ey, ey, ez * ez)),
                                                sgrid, ntab, P.qpc, e_el);
          bx = fmaf(fp, ex, bx);
          by = fmaf(fp, ey, by);
          bz = fmaf(fp, ez, bz);
          if (MEASURE) pv.add(ex, ey, ez, fp);
        }
        if (P.qcp != 0.f) {
          const float ex = dx - qd.x, ey = dy - qd.y, ez = dz - qd.z;
          const float fp = spline_term<MEASURE>(erd, eru, fmaf(ex, ex, fmaf(ey, ey, ez * ez)),
                                                sgrid, ntab, P.qcp, e_el);
          ax = fmaf(fp, ex, ax);
          ay = fmaf(fp, ey, ay);
          az = fmaf(fp, ez, az);
          if (MEASURE) pv.add(ex, ey, ez, fp);
        }
        if (P.qpp != 0.f) {
          const float ex = dx + md.x - qd.x, ey = dy + md.y - qd.y, ez = dz + md.z - qd.z;
          const float fp = spline_term<MEASURE>(erd, eru, fmaf(ex, ex, fmaf(ey, ey, ez * ez)),
                                                sgrid, ntab, P.qpp, e_el);
          bx = fmaf(fp, ex, bx);
          by = fmaf(fp, ey, by);
          bz = fmaf(fp, ez, bz);
          if (MEASURE) pv.add(ex, ey, ez, fp);
        }
      }
    }
    if (MEASURE) {
      en[0] += e_el; en[1] += e_lj; en[2] += e_vir;
      en[3] += pv.p0; en[4] += pv.p1; en[5] += pv.p2;
      en[6] += pv.p3; en[7] += pv.p4; en[8] += pv.p5;
    }
    // the site's force: lane sums (about cnt/32 terms each) reduced in FP64
    double v[6] = {fx + ax, fy + ay, fz + az, gx + bx, gy + by, gz + bz};
#pragma unroll
    for (int d = 0; d < (POLAR ? 6 : 3); d++)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[d] += __shfl_xor_sync(0xffffffffu, v[d], o);
    if (lane == 0) {
      const int site = a.order[ti];
      a.f[3 * site] = v[0];
      a.f[3 * site + 1] = v[1];
      a.f[3 * site + 2] = v[2];
      if (POLAR) {
        a.f[3 * (long)a.ns + 3 * site] = v[3];
        a.f[3 * (long)a.ns + 3 * site + 1] = v[4];
        a.f[3 * (long)a.ns + 3 * site + 2] = v[5];
      }
    }
  }
  if (MEASURE) {
    for (int k = 0; k < 9; k++) {
      ered[threadIdx.x] = 0.5 * en[k];
      __syncthreads();
      for (int w = NL_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) ered[threadIdx.x] += ered[threadIdx.x + w];
        __syncthreads();
      }
      if (threadIdx.x == 0) a.epart[blockIdx.x * NEN + k] = ered[0];
      __syncthreads();
    }
  }
}

cudaError_t k_pair_list_mixed(const Launch& L, const PairArgs& a, const ListArgs& l,
                              const int4* pj, const PairF* ptab, const float4* erd,
                              const float4* eru, bool measure, bool polar) {
  const int grid = list_blocks(a.ns, true);
  const float sx = (float)(a.Lx / 4294967296.0), sy = (float)(a.Ly / 4294967296.0),
              sz = (float)(a.Lz / 4294967296.0);
  const float cq = (float)a.cutoff_sq, sg = (float)a.sgrid, al = (float)a.alpha;
#define LAUNCH_PL(M, P) \
  pair_list_mixed_kernel<M, P><<<grid, NL_THREADS, 0, L.s>>>(a, l, pj, ptab, erd, eru, sx, sy, sz, cq, sg, al)
  if (polar) {
    if (measure) LAUNCH_PL(true, true);
    else LAUNCH_PL(false, true);
  } else {
    if (measure) LAUNCH_PL(true, false);
    else LAUNCH_PL(false, false);
  }
#undef LAUNCH_PL
  ++*L.counter;
  return cudaGetLastError();
}

// FP64 pair sum over the lists (nearest image taken per pair)
template <bool MEASURE, bool POLAR>
__global__ void __launch_bounds__(NL_THREADS)
    pair_list_fp64_kernel(PairArgs a, ListArgs l, const double4* __restrict__ pd,
                          const PairD* __restrict__ ptab_g, const double* __restrict__ ert) {
  __shared__ PairD ptab[MAX_KINDS * MAX_KINDS];
  __shared__ double ered[NL_THREADS];
  const int nk = a.nkind, ntab = a.ntab;
  for (int t = threadIdx.x; t < nk * nk; t += NL_THREADS) ptab[t] = ptab_g[t];
  __syncthreads();
  const int ti = blockIdx.x * NL_THREADS + threadIdx.x;
  const bool vi = ti < a.ns;
  const double cq = a.cutoff_sq, sgrid = a.sgrid, alpha = a.alpha;
  double en[NEN];
#pragma unroll
  for (int k = 0; k < NEN; k++) en[k] = 0;
  if (vi) {
    const double4 me = pd[ti];
    const double4 md = POLAR ? a.pdd[ti] : make_double4(0, 0, 0, 0);
    const long long wi = __double_as_longlong(me.w);
    const int kind_i = (int)(wi & 255), mol_i = (int)(wi >> 8);
    const int cnt = l.ncount[ti];
    double fx = 0, fy = 0, fz = 0, gx = 0, gy = 0, gz = 0;
    for (int k = 0; k < cnt; k++) {
      const int tj = l.nlist[(long)ti * l.cap + k];
      const double4 q = pd[tj];
      double dx = me.x - q.x, dy = me.y - q.y, dz = me.z - q.z;
      dx -= a.Lx * rint(dx / a.Lx);
      dy -= a.Ly * rint(dy / a.Ly);
      dz -= a.Lz * rint(dz / a.Lz);
      const double rr = dx * dx + dy * dy + dz * dz;
      if (rr >= cq) continue;
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
        const double4 qd = a.pdd[tj];
        if (P.qpc != 0)
          term64<MEASURE>(dx + md.x, dy + md.y, dz + md.z, P.qpc, excl, ert, sgrid, ntab, alpha,
                            gx, gy, gz, en);
        if (P.qcp != 0)
          term64<MEASURE>(dx - qd.x, dy - qd.y, dz - qd.z, P.qcp, excl, ert, sgrid, ntab, alpha,
                            fx, fy, fz, en);
        if (P.qpp != 0)
          term64<MEASURE>(dx + md.x - qd.x, dy + md.y - qd.y, dz + md.z - qd.z, P.qpp, excl,
                            ert, sgrid, ntab, alpha, gx, gy, gz, en);
      }
    }
    const int site = a.order[ti];
    a.f[3 * site] = fx;
    a.f[3 * site + 1] = fy;
    a.f[3 * site + 2] = fz;
    if (POLAR) {
      a.f[3 * (long)a.ns + 3 * site] = gx;
      a.f[3 * (long)a.ns + 3 * site + 1] = gy;
      a.f[3 * (long)a.ns + 3 * site + 2] = gz;
    }
  }
  if (MEASURE) {
    for (int k = 0; k < 9; k++) {
      ered[threadIdx.x] = 0.5 * en[k];
      __syncthreads();
      for (int w = NL_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) ered[threadIdx.x] += ered[threadIdx.x + w];
        __syncthreads();
      }
      if (threadIdx.x == 0) a.epart[blockIdx.x * NEN + k] = ered[0];
      __syncthreads();
    }
  }
}

cudaError_t k_pair_list_fp64(const Launch& L, const PairArgs& a, const ListArgs& l,
                             const double4* pd, const PairD* ptab, const double* ertab,
                             bool measure, bool polar) {
  const int grid = (a.ns + NL_THREADS - 1) / NL_THREADS;
#define LAUNCH_PL(M, P) \
  pair_list_fp64_kernel<M, P><<<grid, NL_THREADS, 0, L.s>>>(a, l, pd, ptab, ertab)
  if (polar) {
    if (measure) LAUNCH_PL(true, true);
    else LAUNCH_PL(false, true);
  } else {
    if (measure) LAUNCH_PL(true, false);
    else LAUNCH_PL(false, false);
  }
#undef LAUNCH_PL
  ++*L.counter;
  return cudaGetLastError();
}

int list_blocks(int ns, bool mixed) {
  return mixed ? (ns + NL_WARPS - 1) / NL_WARPS : (ns + NL_THREADS - 1) / NL_THREADS;
}

}  // namespace mg
