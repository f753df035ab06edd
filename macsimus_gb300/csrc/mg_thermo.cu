// Thermostats on the device (sim/thermo.c, applied after SHAKE as cook does
// in Shake(), sim/constrd.c:1033-1047): the half-step displacements
// r1 = h v are scaled by z, with 2 E_kin/f = En.T from the VERLET=3 kinetic
// energy of the step (the mean of the two half steps, sim/shakev3.c).
//
//   Berendsen  z = exp(-h/tau blogT(En.T, T))      (sim/thermo.c:157-163)
//              blogT(E, T) = ln(E/T)/2 kept in [-1, 1]  (sim/constrd.c:98-107)
//   Bussi      z = sqrt(e + c(1-e)(u1^2 + sum_{i<f} u_i^2) + 2 e sqrt(c(1-e)) u1),
//              e = exp(-h/tau), c = T/(f En.T)     (sim/thermo.c:165-179)
//
//   Nose-Hoover (kind 3; cook's T_NOSE with Verlet + SHAKE): the friction
//              term is in the SHAKE kernel; after the step
//              h dlogs/dt += h^2 (En.T/T - 1)/tau^2, logs += h dlogs/dt and
//              Eext = f T (logs_old + (tau/h)^2 (v_old^2 + v_new^2)/4)
//              (sim/thermo.c:180-212, VERLET=3); the old h dlogs/dt enters
//              the predictor history (sim/trvpscale.c)
//
// The Gaussian numbers of the Bussi thermostat come from a counter-based
// stream (SplitMix64 output function of seed + (step * 2^40 + i + 1) * gamma,
// Box-Muller on pairs), so that the draws of a step do not depend on the
// launch; the reference draws rndgauss().  The kinetic energy is the SHAKE
// kernel's per-block sums, added in a fixed order by every block.
#include "mg_internal.h"

namespace mg {

constexpr int TH_THREADS = 256;

__device__ __forceinline__ unsigned long long th_word(unsigned long long seed,
                                                      unsigned long long n) {
  unsigned long long z = seed + (n + 1) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Gaussian number i of a step: Box-Muller on words 2i and 2i+1 of the
// step's stream (uniforms in (0, 1])
__device__ __forceinline__ double th_gauss(unsigned long long seed, long long step, long long i) {
  const unsigned long long base = (unsigned long long)step << 40;
  const double s53 = 1.0 / 9007199254740992.0;
  const double u1 = ((double)(th_word(seed, base + 2 * i) >> 11) + 1.0) * s53;
  const double u2 = (double)(th_word(seed, base + 2 * i + 1) >> 11) * s53;
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

// Bussi: sum of squares of Gaussians 1..f-1 of the step, per block
__global__ void bussi_chi2_kernel(long long nf, unsigned long long seed,
                                  const long long* __restrict__ stepp, double* __restrict__ part) {
  __shared__ double red[TH_THREADS];
  const long long step = *stepp;
  double s = 0;
  for (long long i = 1 + blockIdx.x * (long long)TH_THREADS + threadIdx.x; i < nf;
       i += (long long)gridDim.x * TH_THREADS) {
    const double g = th_gauss(seed, step, i);
    s += g * g;
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = TH_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// the factor z (every block computes it from the same sums in the same
// order) and r1 *= z
__global__ void thermostat_scale_kernel(ThermoArgs a, const double* __restrict__ kin_part,
                                        const double* __restrict__ chi_part,
                                        double* __restrict__ r1) {
  __shared__ double zs;
  if (threadIdx.x == 0) {
    double k = 0;
    for (int b = 0; b < a.nkin; b++) k += kin_part[b];
    // cook's doubled kinetic energy sum m (V1^2 + V2^2) / (2 h^2) -> En.T
    const double ET = k / (2 * a.h * a.h) / a.nf;
    double z = 1;
    if (a.kind == 1) {
      double bl = ET > a.T * 7.38905609893065022723 ? 1
                  : (ET * 7.38905609893065022723 < a.T ? -1 : log(ET / a.T) / 2);
      z = exp(bl * -a.h / a.tau);
    } else if (a.kind == 2) {
      double uf = 0;
      for (int b = 0; b < a.nchi; b++) uf += chi_part[b];
      const double u1 = th_gauss(a.seed, *a.step, 0);
      const double e = exp(-a.h / a.tau), c = a.T / (a.nf * ET);
      z = sqrt(e + c * (1 - e) * (u1 * u1 + uf) + 2 * e * sqrt(c * (1 - e)) * u1);
    }
    zs = z;
    if (blockIdx.x == 0 && a.zout) *a.zout = z;
  }
  __syncthreads();
  const double z = zs;
  for (long long t = blockIdx.x * (long long)TH_THREADS + threadIdx.x; t < 3LL * a.ns;
       t += (long long)gridDim.x * TH_THREADS)
    r1[t] *= z;
}

// Nose-Hoover: one thread advances the thermostat state (NoseSlot) with the
// kinetic energy of the step, summed in the order of thermostat_scale_kernel
__global__ void nose_update_kernel(ThermoArgs a, const double* __restrict__ kin_part) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double k = 0;
  for (int b = 0; b < a.nkin; b++) k += kin_part[b];
  const double ET = k / (2 * a.h * a.h) / a.nf;
  double* s = a.nh;
  const int kk = (int)s[NH_K], knew = min(a.pred, kk + 1);
  const double lo = s[NH_LOGS], ld = s[NH_LOGSV];
  for (int j = knew - 1; j >= 1; j--) s[NH_HIST + j] = s[NH_HIST + j - 1];
  if (knew > 0) s[NH_HIST] = ld;
  const double lv = ld + a.h * a.h * (ET / a.T - 1) / (a.tau * a.tau);
  const double th = a.tau / a.h;
  s[NH_LOGSV] = lv;
  s[NH_LOGS] = lo + lv;
  s[NH_K] = knew;
  s[NH_EXT] = a.nf * a.T * (lo + th * th * (ld * ld + lv * lv) / 4);
  if (a.zout) *a.zout = 1;
}

// the step counter of the Bussi stream lives on the device (so that a
// captured step replays with fresh draws)
__global__ void step_increment_kernel(long long* step) { ++*step; }

cudaError_t k_thermostat(const Launch& L, const ThermoArgs& a, const double* kin_part,
                         double* chi_part, double* r1) {
  if (a.kind == 3) {
    nose_update_kernel<<<1, 32, 0, L.s>>>(a, kin_part);
    ++*L.counter;
    return cudaGetLastError();
  }
  if (a.kind == 2) {
    bussi_chi2_kernel<<<a.nchi, TH_THREADS, 0, L.s>>>((long long)a.nf, a.seed, a.step, chi_part);
    ++*L.counter;
  }
  const int grid = (int)std::min<long long>((3LL * a.ns + TH_THREADS - 1) / TH_THREADS, 4 * PARTITION_SMS);
  thermostat_scale_kernel<<<grid, TH_THREADS, 0, L.s>>>(a, kin_part, chi_part, r1);
  ++*L.counter;
  if (a.kind == 2) {
    step_increment_kernel<<<1, 1, 0, L.s>>>(a.step);
    ++*L.counter;
  }
  return cudaGetLastError();
}

// cook's bounddr (sim/norm.c:1513-1560), after the step and its thermostat:
// a site whose displacement in the step r1 is longer than drmax has r1
// scaled to that length; the number of such sites and the smallest factor
// are accumulated in rep[0] (count) and rep[1] (float bits of the factor,
// atomicMin on the bits of a positive float keeps the order)
__global__ void bounddr_kernel(int ns, double vvmax, double* __restrict__ r1,
                               unsigned int* __restrict__ rep) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns) return;
  double* p = r1 + 3 * (long)i;
  const double vv = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
  if (vv > vvmax) {
    const double q = sqrt(vvmax / vv);
    p[0] *= q;
    p[1] *= q;
    p[2] *= q;
    atomicAdd(rep, 1u);
    atomicMin(rep + 1, __float_as_uint((float)q));
  }
}

// cook's removedrifts for the momentum (sim/norm.c:677-705): the mass
// weighted sum of r1 (per CTA, then one fixed-order reduction), divided by
// the total mass of the free sites and subtracted from every site's r1
__global__ void __launch_bounds__(TH_THREADS)
momentum_part_kernel(int ns, const double* __restrict__ mass, const double* __restrict__ r1,
                     double* __restrict__ part) {
  __shared__ double red[3][TH_THREADS];
  const int i = blockIdx.x * TH_THREADS + threadIdx.x;
#pragma unroll
  for (int d = 0; d < 3; d++) red[d][threadIdx.x] = i < ns ? mass[i] * r1[3 * (long)i + d] : 0.0;
  __syncthreads();
  for (int w = TH_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int d = 0; d < 3; d++) red[d][threadIdx.x] += red[d][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 3) part[3 * (long)blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void momentum_remove_kernel(int ns, const double* __restrict__ P, double imass,
                                       double* __restrict__ r1, double* __restrict__ vout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double v0 = P[0] * imass, v1 = P[1] * imass, v2 = P[2] * imass;
  if (i == 0 && vout) {
    vout[0] = v0;
    vout[1] = v1;
    vout[2] = v2;
  }
  if (i >= ns) return;
  r1[3 * (long)i] -= v0;
  r1[3 * (long)i + 1] -= v1;
  r1[3 * (long)i + 2] -= v2;
}

int drift_blocks(int ns) { return (ns + TH_THREADS - 1) / TH_THREADS; }

cudaError_t k_remove_drift(const Launch& L, int ns, const double* mass, double total_mass,
                           double* r1, double* part, double* P, double* vout) {
  const int nb = drift_blocks(ns);
  momentum_part_kernel<<<nb, TH_THREADS, 0, L.s>>>(ns, mass, r1, part);
  ++*L.counter;
  cudaError_t e = k_reduce_sum(L, part, nb, 3, P);
  if (e != cudaSuccess) return e;
  momentum_remove_kernel<<<nb, TH_THREADS, 0, L.s>>>(ns, P, 1.0 / total_mass, r1, vout);
  ++*L.counter;
  return cudaGetLastError();
}

cudaError_t k_bounddr(const Launch& L, int ns, double drmax, double* r1, unsigned int* rep) {
  bounddr_kernel<<<(ns + TH_THREADS - 1) / TH_THREADS, TH_THREADS, 0, L.s>>>(ns, drmax * drmax,
                                                                              r1, rep);
  ++*L.counter;
  return cudaGetLastError();
}

}  // namespace mg
