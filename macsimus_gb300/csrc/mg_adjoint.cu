// Adjoint of the force path (FP64): gradients of the energy E, the scalar
// virial W = sum r.f (LJ) + E_el and of a loss of the forces (through its
// weights g_i = dLoss/dF_i) with respect to the LJ (epsilon, sigma) of every
// pair of site kinds and to every site charge.  Pair terms are recomputed,
// nothing of the forward pass is stored but S(k) and the cell list.
//
//   LJ, below C1:  u = E4 (y^2 - y), y = (sigma/r)^6, f = 6 E4 (2y^2 - y)/r^2
//                  du/dsigma = E4 (12 y^2 - 6 y)/sigma,
//                  df/dsigma = 36 E4 y (4y - 1)/(sigma r^2)
//   smooth part:   u = A (r^2 - C2^2)^2, f = A4 (r^2 - C2^2), with
//                  dA/dsigma, dA4/dsigma from the host
//   both:          du/deps = u/eps, df/deps = f/eps  (u is linear in eps)
//   charges:       dE/dq_i = psi_i (r-space + k-space + self),
//                  dLoss/dq_i = sum_j (g_i - g_j).r_ij e_ij q_j + g_i.F^k_i/q_i
//                               + sum_k ekk Im(conj(Phi_i(k)) T(k)),
//                  T(k) = sum_j q_j (g_j.k/L) Phi_j(k)
#include "mg_internal.h"
#include "mg_device.cuh"

namespace mg {

constexpr int ADJ_THREADS = 128;
constexpr int ADJ_NW = ADJ_THREADS / 32;

// gradient weights in cell order: (g_x, g_y, g_z, q) of every sorted site
__global__ void adj_gather_kernel(int ns, const int* __restrict__ order,
                                  const double* __restrict__ g, const double* __restrict__ q,
                                  double4* __restrict__ gs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ns) return;
  const int i = order[t];
  gs[t] = g ? make_double4(g[3 * i], g[3 * i + 1], g[3 * i + 2], q[i])
            : make_double4(0, 0, 0, q[i]);
}

// CTA per home cell, warps split the stencil, lane = home site (the layout of
// the FP64 force kernel).  Per kind pair: 6 sums (dE/deps, dE/dsig, dW/deps,
// dW/dsig, dL/deps, dL/dsig) in shared memory, halved at the end (every
// pair is met from both ends); per site: dE/dq and dL/dq of the r-space sum.
__global__ void __launch_bounds__(ADJ_THREADS)
    adj_pair_kernel(PairArgs a, const double4* __restrict__ pd, const double4* __restrict__ gs,
                    const AdjPair* __restrict__ tab_g, const double* __restrict__ ert,
                    double* __restrict__ part, double* __restrict__ dEq, double* __restrict__ dLq) {
  __shared__ AdjPair tab[MAX_KINDS * MAX_KINDS];
  __shared__ double acc[MAX_KINDS * MAX_KINDS * 6];
  __shared__ double4 sj[ADJ_NW][32], sg[ADJ_NW][32];
  __shared__ double red[ADJ_NW][32][2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = a.nkind, nk2 = nk * nk;
  for (int t = threadIdx.x; t < nk2; t += ADJ_THREADS) tab[t] = tab_g[t];
  for (int t = threadIdx.x; t < nk2 * 6; t += ADJ_THREADS) acc[t] = 0;
  __syncthreads();
  const int c = blockIdx.x;
  const int cz = c % a.ncz, cy = (c / a.ncz) % a.ncy, cx = c / (a.ncy * a.ncz);
  const int i0 = a.cell_start[c], ni = a.cell_start[c + 1] - i0;
  const double cq = a.cutoff_sq;
  for (int ib = 0; ib < ni; ib += 32) {
    const bool vi = ib + lane < ni;
    const int ti = i0 + ib + lane;
    const double4 me = vi ? pd[ti] : make_double4(0, 0, 0, 0);
    const double4 gi = vi ? gs[ti] : make_double4(0, 0, 0, 0);
    const long long wi = __double_as_longlong(me.w);
    const int kind_i = (int)(wi & 255), mol_i = (int)(wi >> 8);
    double eq = 0, lq = 0;
    for (int s = warp; s < a.nstencil; s += ADJ_NW) {
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
          sg[warp][lane] = gs[j0 + jb + lane];
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
          const double4 gj = sg[warp][jj];
          const long long wj = __double_as_longlong(q.w);
          const int kj = (int)(wj & 255);
          const AdjPair& P = tab[kind_i * nk + kj];
          const double gd = (gi.x - gj.x) * dx + (gi.y - gj.y) * dy + (gi.z - gj.z) * dz;
          double phi = 0, e = 0;
          if ((int)(wj >> 8) == mol_i) {
            phi = excl_term<double>(rr, a.alpha, &e);
          } else {
            if (rr < P.C2q && P.E4 != 0) {
              double u, f, du, df;
              if (rr < P.C1q) {
                double y = P.Sq / rr;
                y = y * y * y;
                u = P.E4 * (y * y - y);
                f = 6 * P.E4 * (2 * y * y - y) / rr;
                du = P.E4 / P.sig * (12 * y * y - 6 * y);
                df = 36 * P.E4 * y * (4 * y - 1) / (P.sig * rr);
              } else {
                const double x = rr - P.C2q;
                u = P.A * x * x;
                f = P.A4 * x;
                du = P.dA * x * x;
                df = P.dA4 * x;
              }
              double* A = acc + 6 * (kind_i * nk + kj);
              atomicAdd(A + 0, u / P.eps);
              atomicAdd(A + 1, du);
              atomicAdd(A + 2, rr * f / P.eps);
              atomicAdd(A + 3, rr * df);
              atomicAdd(A + 4, gd * f / P.eps);
              atomicAdd(A + 5, gd * df);
            }
            if (gj.w != 0) {
              const double* p = ert + 6 * min((int)(rr * a.sgrid), a.ntab - 1);
              phi = p[1] / (p[2] + rr) + p[0];
              e = p[4] / (p[5] + rr) + p[3];
            }
          }
          eq += gj.w * phi;
          lq += gd * e * gj.w;
        }
        __syncwarp();
      }
    }
    red[warp][lane][0] = eq;
    red[warp][lane][1] = lq;
    __syncthreads();
    if (warp == 0 && vi) {
      double se = 0, sl = 0;
#pragma unroll
      for (int w = 0; w < ADJ_NW; w++) {
        se += red[w][lane][0];
        sl += red[w][lane][1];
      }
      const int site = a.order[ti];
      dEq[site] = se;
      dLq[site] = sl;
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < nk2 * 6; t += ADJ_THREADS)
    part[(long)blockIdx.x * nk2 * 6 + t] = 0.5 * acc[t];
}

// T_d(k) = sum_j g_jd (q_j Phi_j(k)) over a chunk of charges (grid.y)
__global__ void kadj_T_kernel(KArgs a, const double2* __restrict__ tab, const double* __restrict__ g,
                              double2* __restrict__ part) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.nk) return;
  const int4 kv = a.kvec[k];
  const int ch = blockIdx.y;
  const int j0 = (int)((long)a.nq * ch / gridDim.y), j1 = (int)((long)a.nq * (ch + 1) / gridDim.y);
  const int oy = a.Kx + 1 + a.Ky, oz = a.Kx + 2 * a.Ky + 2 + a.Kz;
  double2 T[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
  for (int j = j0; j < j1; j++) {
    const double2* R = tab + (long)j * a.row;
    const double2 X = R[kv.x], Y = R[oy + kv.y], Z = R[oz + kv.z];
    const double2 A = make_double2(X.x * Y.x - X.y * Y.y, X.x * Y.y + X.y * Y.x);
    const double2 P = make_double2(A.x * Z.x - A.y * Z.y, A.x * Z.y + A.y * Z.x);
    const int site = a.qsite[j];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double w = g[3 * site + d];
      T[d].x += w * P.x;
      T[d].y += w * P.y;
    }
  }
#pragma unroll
  for (int d = 0; d < 3; d++) part[((long)ch * a.nk + k) * 3 + d] = T[d];
}

// T(k) = sum_d (k_d/L_d) T_d(k), the chunks in a fixed order
__global__ void kadj_T_reduce_kernel(KArgs a, int nch, const double2* __restrict__ part,
                                     double2* __restrict__ T) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.nk) return;
  const int4 kv = a.kvec[k];
  const double w[3] = {kv.x / a.Lx, kv.y / a.Ly, kv.z / a.Lz};
  double tx = 0, ty = 0;
  for (int c = 0; c < nch; c++)
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double2 v = part[((long)c * a.nk + k) * 3 + d];
      tx += w[d] * v.x;
      ty += w[d] * v.y;
    }
  T[k] = make_double2(tx, ty);
}

// per charge: psi (k-space potential), F^k/q, sum_k ekk Im(conj(Phi) T)
__global__ void kadj_charge_kernel(KArgs a, const double2* __restrict__ tab,
                                   const double2* __restrict__ T, const double* __restrict__ g,
                                   double* __restrict__ dEq, double* __restrict__ dLq) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.nq) return;
  const int oy = a.Kx + 1 + a.Ky, oz = a.Kx + 2 * a.Ky + 2 + a.Kz;
  const double2* R = tab + (long)j * a.row;
  const double qj = a.qval[j], iq = 1.0 / qj;
  double psi = 0, fx = 0, fy = 0, fz = 0, kl = 0;
  for (int k = 0; k < a.nk; k++) {
    const int4 kv = a.kvec[k];
    const double2 X = R[kv.x], Y = R[oy + kv.y], Z = R[oz + kv.z];
    const double2 A = make_double2(X.x * Y.x - X.y * Y.y, X.x * Y.y + X.y * Y.x);
    const double px = (A.x * Z.x - A.y * Z.y) * iq, py = (A.x * Z.y + A.y * Z.x) * iq;
    const double sr = a.S[2 * k], si = a.S[2 * k + 1], ek = a.ekk[k];
    const double2 t = T[k];
    psi += ek * (sr * px + si * py);
    const double im = ek * (sr * py - si * px);
    fx += kv.x * im;
    fy += kv.y * im;
    fz += kv.z * im;
    kl += ek * (px * t.y - py * t.x);
  }
  const int site = a.qsite[j];
  dEq[site] += psi / (2 * 3.14159265358979323846) - 2 * a.alpha / 1.772453850905516 * qj;
  if (g)
    dLq[site] += g[3 * site] * fx / a.Lx + g[3 * site + 1] * fy / a.Ly +
                 g[3 * site + 2] * fz / a.Lz + kl;
}

static inline int cdiv_a(long a, long b) { return (int)((a + b - 1) / b); }

cudaError_t k_adjoint(const Launch& L, const PairArgs& pa, const KArgs& ka, const double4* pd,
                      const AdjPair* tab, const double* ert, const double2* ptab, const double* g,
                      const double* q, double4* gs, double* part, double* dEq, double* dLq,
                      double2* tpart, int ntch, double2* T) {
  const int ncell = pa.ncx * pa.ncy * pa.ncz;
  adj_gather_kernel<<<cdiv_a(pa.ns, 256), 256, 0, L.s>>>(pa.ns, pa.order, g, q, gs);
  adj_pair_kernel<<<ncell, ADJ_THREADS, 0, L.s>>>(pa, pd, gs, tab, ert, part, dEq, dLq);
  *L.counter += 2;
  if (ka.nq > 0 && ka.nk > 0) {
    if (g) {
      kadj_T_kernel<<<dim3(cdiv_a(ka.nk, 128), ntch), 128, 0, L.s>>>(ka, ptab, g, tpart);
      kadj_T_reduce_kernel<<<cdiv_a(ka.nk, 256), 256, 0, L.s>>>(ka, ntch, tpart, T);
      *L.counter += 2;
    } else {
      cudaMemsetAsync(T, 0, sizeof(double2) * ka.nk, L.s);
    }
    kadj_charge_kernel<<<cdiv_a(ka.nq, 128), 128, 0, L.s>>>(ka, ptab, T, g, dEq, dLq);
    *L.counter += 1;
  }
  return cudaGetLastError();
}

}  // namespace mg
