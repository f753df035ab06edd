// Per-site utilities of the MD state: playback frames and linear dependants.
//
// Linear ("Middle") dependant sites, cook's depend_t of type DEP_M: a massless
// site placed at a weighted sum of parent sites of its molecule (the charge
// site M of TIP4P water), sim/norm.c:1161-1195 (depend_r) and
// sim/norm.c:1276-1300 (depend_f).  The tables list the dependants of a
// molecule consecutively; one thread walks the dependants of one molecule in
// table order, so force redistribution onto shared parents has no races and
// the summation order is cook's.
#include "mg_internal.h"

namespace mg {

constexpr int DEP_THREADS = 128;

// the thread that owns dependant k: the first of its molecule in the table
__device__ __forceinline__ bool dep_owner(const DependArgs& a, int k) {
  return k == 0 || a.mol[a.site[k - 1]] != a.mol[a.site[k]];
}

__global__ void __launch_bounds__(DEP_THREADS)
    depend_r_kernel(DependArgs a, double* __restrict__ r) {
  const int k0 = blockIdx.x * DEP_THREADS + threadIdx.x;
  if (k0 >= a.ndep || !dep_owner(a, k0)) return;
  const int m = a.mol[a.site[k0]];
  for (int k = k0; k < a.ndep && a.mol[a.site[k]] == m; k++) {
    double x = 0, y = 0, z = 0;
    for (int p = a.first[k]; p < a.first[k + 1]; p++) {
      const double w = a.w[p];
      const double* rp = r + 3 * (long)a.parent[p];
      x += w * rp[0];
      y += w * rp[1];
      z += w * rp[2];
    }
    double* rd = r + 3 * (long)a.site[k];
    rd[0] = x;
    rd[1] = y;
    rd[2] = z;
  }
}

__global__ void __launch_bounds__(DEP_THREADS)
    depend_f_kernel(DependArgs a, double* __restrict__ f) {
  const int k0 = blockIdx.x * DEP_THREADS + threadIdx.x;
  if (k0 >= a.ndep || !dep_owner(a, k0)) return;
  const int m = a.mol[a.site[k0]];
  for (int k = k0; k < a.ndep && a.mol[a.site[k]] == m; k++) {
    const double* fd = f + 3 * (long)a.site[k];
    const double fx = fd[0], fy = fd[1], fz = fd[2];
    for (int p = a.first[k]; p < a.first[k + 1]; p++) {
      const double w = a.w[p];
      double* fp = f + 3 * (long)a.parent[p];
      fp[0] += w * fx;
      fp[1] += w * fy;
      fp[2] += w * fz;
    }
  }
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

cudaError_t k_depend_f(const Launch& L, const DependArgs& a, double* f) {
  if (a.ndep <= 0) return cudaSuccess;
  depend_f_kernel<<<(a.ndep + DEP_THREADS - 1) / DEP_THREADS, DEP_THREADS, 0, L.s>>>(a, f);
  ++*L.counter;
  return cudaGetLastError();
}

}  // namespace mg
