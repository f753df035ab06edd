// Per-site utilities of the MD state: playback frames and dependant sites.
//
// Dependant sites, cook's depend_t (sim/norm.c:1161-1360): massless sites
// placed from parent sites of their molecule -- linear ("Middle", DEP_M: a
// weighted sum, the charge site M of TIP4P water), "Rowlinson" (DEP_R: above
// parent D0 along the normal of the triangle D0 D1 D2) and "Lone" (DEP_L: an
// in-plane weighted sum plus wz along the normal of a frame built from the
// parents) -- and their forces redistributed onto the parents (depend_f).
// The tables list the dependants of a molecule consecutively, in cook's
// order; one thread walks the dependants of one molecule in table order, so
// the redistribution onto shared parents has no races and cook's summation
// order.  FP64, the reference's operation order.
#include "mg_internal.h"

namespace mg {

constexpr int DEP_THREADS = 128;

// the thread that owns dependant k: the first of its molecule in the table
__device__ __forceinline__ bool dep_owner(const DependArgs& a, int k) {
  return k == 0 || a.mol[a.site[k - 1]] != a.mol[a.site[k]];
}

__device__ __forceinline__ void vcross(const double* b, const double* c, double* a) {
  a[0] = b[1] * c[2] - b[2] * c[1];
  a[1] = b[2] * c[0] - b[0] * c[2];
  a[2] = b[0] * c[1] - b[1] * c[0];
}
__device__ __forceinline__ double vdot(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

__global__ void __launch_bounds__(DEP_THREADS)
    depend_r_kernel(DependArgs a, double* __restrict__ r) {
  const int k0 = blockIdx.x * DEP_THREADS + threadIdx.x;
  if (k0 >= a.ndep || !dep_owner(a, k0)) return;
  const int m = a.mol[a.site[k0]];
  for (int k = k0; k < a.ndep && a.mol[a.site[k]] == m; k++) {
    const int typ = a.type ? a.type[k] : 0;
    double* rd = r + 3 * (long)a.site[k];
    const int p0 = a.first[k];
    if (typ == 1) {
      // Rowlinson: D0 + wz l / |l|, l = (D1 - D0) x (D2 - D0) (sim/norm.c:1205-1214)
      const double* d0 = r + 3 * (long)a.parent[p0];
      const double* d1 = r + 3 * (long)a.parent[p0 + 1];
      const double* d2 = r + 3 * (long)a.parent[p0 + 2];
      const double h1[3] = {d1[0] - d0[0], d1[1] - d0[1], d1[2] - d0[2]};
      const double h2[3] = {d2[0] - d0[0], d2[1] - d0[1], d2[2] - d0[2]};
      double l[3];
      vcross(h1, h2, l);
      const double nrm = a.par[13 * (long)k] / sqrt(vdot(l, l));
      rd[0] = d0[0] + nrm * l[0];
      rd[1] = d0[1] + nrm * l[1];
      rd[2] = d0[2] + nrm * l[2];
    } else if (typ == 2) {
      // Lone: sum w D + wz z / |z|, z = (sum x D) x (sum y D) (sim/norm.c:1216-1231)
      const double* q = a.par + 13 * (long)k;
      double d[3] = {0, 0, 0}, xx[3] = {0, 0, 0}, yy[3] = {0, 0, 0}, zz[3];
      for (int c = 0; c < 3; c++) {
        const double* rp = r + 3 * (long)a.parent[p0 + c];
        const double w = a.w[p0 + c];
        for (int e = 0; e < 3; e++) {
          d[e] += w * rp[e];
          xx[e] += q[1 + c] * rp[e];
          yy[e] += q[4 + c] * rp[e];
        }
      }
      vcross(xx, yy, zz);
      const double rr = q[0] / sqrt(vdot(zz, zz));
      rd[0] = d[0] + rr * zz[0];
      rd[1] = d[1] + rr * zz[1];
      rd[2] = d[2] + rr * zz[2];
    } else {
      double x = 0, y = 0, z = 0;
      for (int p = p0; p < a.first[k + 1]; p++) {
        const double w = a.w[p];
        const double* rp = r + 3 * (long)a.parent[p];
        x += w * rp[0];
        y += w * rp[1];
        z += w * rp[2];
      }
      rd[0] = x;
      rd[1] = y;
      rd[2] = z;
    }
  }
}

// cook's virial tensor term of Q, F, G (sim/norm.c:1256-1262): Q (G_x F_x,
// G_y F_y, G_z F_z, G_y F_z, G_z F_x, G_x F_y) added to v[1..6]
__device__ __forceinline__ void ptens_add(double* v, double q, const double* F, const double* G) {
  v[1] += q * G[0] * F[0];
  v[2] += q * G[1] * F[1];
  v[3] += q * G[2] * F[2];
  v[4] += q * G[1] * F[2];
  v[5] += q * G[2] * F[0];
  v[6] += q * G[0] * F[1];
}

__global__ void __launch_bounds__(DEP_THREADS)
    depend_f_kernel(DependArgs a, const double* __restrict__ r, double* __restrict__ f) {
  const int k0 = blockIdx.x * DEP_THREADS + threadIdx.x;
  if (k0 >= a.ndep) return;
  double v[7] = {0, 0, 0, 0, 0, 0, 0};  // virial, tensor
  const int m = a.mol[a.site[k0]];
  const bool own = dep_owner(a, k0);
  for (int k = k0; own && k < a.ndep && a.mol[a.site[k]] == m; k++) {
    const int typ = a.type ? a.type[k] : 0;
    const double* fd = f + 3 * (long)a.site[k];
    const double F[3] = {fd[0], fd[1], fd[2]};
    const int p0 = a.first[k];
    if (typ == 1) {
      // Rowlinson (sim/norm.c:1304-1338): the torque of F about D0 through
      // forces along l on D1 and D2
      const int i0 = a.parent[p0], i1 = a.parent[p0 + 1], i2 = a.parent[p0 + 2];
      const double* d0 = r + 3 * (long)i0;
      const double* d1 = r + 3 * (long)i1;
      const double* d2 = r + 3 * (long)i2;
      const double* rl = r + 3 * (long)a.site[k];
      const double h1[3] = {d1[0] - d0[0], d1[1] - d0[1], d1[2] - d0[2]};
      const double h2[3] = {d2[0] - d0[0], d2[1] - d0[1], d2[2] - d0[2]};
      const double l[3] = {rl[0] - d0[0], rl[1] - d0[1], rl[2] - d0[2]};
      double M[3], Mp[3];
      vcross(l, F, M);
      vcross(l, M, Mp);
      const double h1h1 = vdot(h1, h1), h2h2 = vdot(h2, h2), h1h2 = vdot(h1, h2);
      const double det = (h1h1 * h2h2 - h1h2 * h1h2) * vdot(l, l);
      const double a1 = (vdot(Mp, h1) * h2h2 - vdot(Mp, h2) * h1h2) / det;
      const double a2 = (vdot(Mp, h2) * h1h1 - vdot(Mp, h1) * h1h2) / det;
      double* f0 = f + 3 * (long)i0;
      double* f1 = f + 3 * (long)i1;
      double* f2 = f + 3 * (long)i2;
      for (int e = 0; e < 3; e++) {
        f0[e] += F[e] - (a1 + a2) * l[e];
        f1[e] += a1 * l[e];
        f2[e] += a2 * l[e];
      }
      // the triangle's forces, and F moved from L to D0
      ptens_add(v, a1, l, h1);
      ptens_add(v, a2, l, h2);
      ptens_add(v, -1.0, l, F);
      v[0] -= vdot(l, F);
    } else if (typ == 2) {
      // Lone (sim/norm.c:1338-1368): w F on the parents plus forces along z
      // that carry the torque of F about the in-plane point
      const double* q = a.par + 13 * (long)k;
      const double* rd = r + 3 * (long)a.site[k];
      double xx[3] = {0, 0, 0}, yy[3] = {0, 0, 0}, zz[3];
      for (int c = 0; c < 3; c++) {
        const double* rp = r + 3 * (long)a.parent[p0 + c];
        for (int e = 0; e < 3; e++) {
          xx[e] += q[1 + c] * rp[e];
          yy[e] += q[4 + c] * rp[e];
        }
      }
      vcross(xx, yy, zz);
      const double rr = vdot(zz, zz);
      const double fx = vdot(xx, F) / sqrt(vdot(xx, xx) * rr);
      const double fy = vdot(yy, F) / sqrt(vdot(yy, yy) * rr);
      const double fz = vdot(zz, F) / rr;
      for (int c = 0; c < 3; c++) {
        const double alpha = fx * q[7 + c] + fy * q[10 + c];
        const double w = a.w[p0 + c];
        const double* rp = r + 3 * (long)a.parent[p0 + c];
        double* fp = f + 3 * (long)a.parent[p0 + c];
        for (int e = 0; e < 3; e++) fp[e] += w * F[e] + alpha * zz[e];
        const double dr[3] = {rp[0] - rd[0], rp[1] - rd[1], rp[2] - rd[2]};
        ptens_add(v, alpha, zz, dr);
      }
      const double wr = q[0] / sqrt(rr);
      v[0] -= wr * fz;
      ptens_add(v, -wr, F, zz);
    } else {
      for (int p = p0; p < a.first[k + 1]; p++) {
        const double w = a.w[p];
        double* fp = f + 3 * (long)a.parent[p];
        fp[0] += w * F[0];
        fp[1] += w * F[1];
        fp[2] += w * F[2];
      }
    }
  }
  if (a.vpart)
    for (int e = 0; e < 7; e++) a.vpart[7 * (long)k0 + e] = v[e];
}

// playback frame, sim/simils.c:1666-1686 in the same operation order:
// v = r1 * (1/h), or d = r (+ Drude offset) (- r1/2) (- L/2), then to float
__global__ void playback_frame_kernel(int ns, int what, int flags, const double* __restrict__ r,
                                      const double* __restrict__ r1, double ih, double3 Lh,
                                      float* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * ns) return;
  double v;
  if (what == 1) {
    v = ih * r1[t];
  } else {
    v = r[t];
    if (what == 2) v += r[3 * (long)ns + t];
    if (flags & 2) v -= 0.5 * r1[t];
    if (flags & 4) {
      const int k = t % 3;
      v -= k == 0 ? Lh.x : (k == 1 ? Lh.y : Lh.z);
    }
  }
  out[t] = (float)v;
}

cudaError_t k_playback_frame(const Launch& L, int ns, int what, int flags, const double* r,
                             const double* r1, double ih, const double Lb[3], float* out) {
  playback_frame_kernel<<<(3 * ns + 255) / 256, 256, 0, L.s>>>(
      ns, what, flags, r, r1, ih, make_double3(0.5 * Lb[0], 0.5 * Lb[1], 0.5 * Lb[2]), out);
  ++*L.counter;
  return cudaGetLastError();
}

cudaError_t k_depend_r(const Launch& L, const DependArgs& a, double* r) {
  if (a.ndep <= 0) return cudaSuccess;
  depend_r_kernel<<<(a.ndep + DEP_THREADS - 1) / DEP_THREADS, DEP_THREADS, 0, L.s>>>(a, r);
  ++*L.counter;
  return cudaGetLastError();
}

cudaError_t k_depend_f(const Launch& L, const DependArgs& a, const double* r, double* f) {
  if (a.ndep <= 0) return cudaSuccess;
  depend_f_kernel<<<(a.ndep + DEP_THREADS - 1) / DEP_THREADS, DEP_THREADS, 0, L.s>>>(a, r, f);
  ++*L.counter;
  return cudaGetLastError();
}

}  // namespace mg
