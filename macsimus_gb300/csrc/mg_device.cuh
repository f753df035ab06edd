// Device helpers shared by the pair kernels (cell and neighbour-list forms).
#pragma once

#include "mg_internal.h"

namespace mg {

constexpr int NEN = 10;   // er, lj, vir, Pvir[6], (spare)

__device__ __forceinline__ double wrap01(double s) { return s - floor(s); }

// a coordinate as a 32-bit fixed-point fraction of the box edge (the
// difference of two such numbers, as 32-bit integers, is the nearest-image
// separation); iLb = 1 / box edge, formed once on the host (an FP64 division
// costs tens of operations on this GPU's narrow FP64 pipe)
__device__ __forceinline__ int fixed32(double x, double iLb) {
  double s = wrap01(x * iLb);
  long long v = llrint(s * 4294967296.0);
  return (int)(unsigned int)(v & 0xffffffffLL);
}
// the cell of a fixed-point coordinate among n cells along the edge
__device__ __forceinline__ int fixed_cell(int fx, int n) {
  return (int)(((unsigned long long)(unsigned)fx * (unsigned)n) >> 32);
}

// Ewald exclusion term -erf(alpha r)/r and its f/r (cook's exacterud_sqrt);
// with minus_const the constant 2 alpha/sqrt(pi) is taken off the energy
// (exacterud_sqrt_1, the centre-Drude pair of one site)
template <typename T>
__device__ __forceinline__ T excl_term(T rr, T alpha, T* erd, bool minus_const = false) {
  const T A = alpha * (T)(-1.1283791670955126);  // -2 alpha/sqrt(pi)
  T aq = alpha * alpha, err = aq * rr;
  if (err < (T)0.01) {
    // Taylor series of erf(x)/x in x^2, as the reference does for short pairs
    T su = 0, sd = 0, q = 1;
    for (int n = 1; n < 40; n++) {
      T rn = q / (T)(2 * n + 1);
      sd += rn * (T)n;
      su += rn;
      if (fabs(q) < (T)1e-17) break;
      q *= -err / (T)(n + 1);
    }
    *erd = A * aq * 2 * sd;
    return minus_const ? A * (-su * err) : A * (1 - su * err);
  }
  T r = sqrt(rr);
  T y = -erf(alpha * r) / r;
  *erd = (y - A * exp(-err)) / rr;
  return minus_const ? y - A : y;
}

// f/r of a spline term (erd), energy (eru) added to e when MEASURE
template <bool MEASURE>
__device__ __forceinline__ float spline_term(const float4* __restrict__ erd,
                                             const float4* __restrict__ eru, float r2, float sgrid,
                                             int ntab, float qq, float& e) {
  // floor(r2 sgrid) without a float-to-int conversion: r2 sgrid - 1/2 rounded
  // to an integer in the mantissa of 1.5 * 2^23 (0 <= r2 sgrid < 2^22; at an
  // exact knot either neighbouring interval gives the same value)
  const int ix = min(__float_as_int(fmaf(r2, sgrid, 12582911.5f)) - 0x4B400000, ntab - 1);
  const float4 d = __ldg(erd + ix);
  if (MEASURE) {
    const float4 u = __ldg(eru + ix);
    e += (__fdividef(u.y, u.z + r2) + u.x) * qq;
  }
  return (__fdividef(d.y, d.z + r2) + d.x) * qq;
}

// the same through any pointer (LDG: read-only path; else plain loads, e.g.
// from a copy of the table in shared memory)
template <bool MEASURE, bool LDG>
__device__ __forceinline__ float spline_any(const float4* erd, const float4* __restrict__ eru,
                                            float r2, float sgrid, int ntab, float qq, float& e) {
  const int ix = min(__float_as_int(fmaf(r2, sgrid, 12582911.5f)) - 0x4B400000, ntab - 1);
  const float4 d = LDG ? __ldg(erd + ix) : erd[ix];
  if (MEASURE) {
    const float4 u = __ldg(eru + ix);
    e += (__fdividef(u.y, u.z + r2) + u.x) * qq;
  }
  return (__fdividef(d.y, d.z + r2) + d.x) * qq;
}

// excluded intramolecular term: its Ewald correction is large and cancels
// the self term; evaluated in FP32 (an FP64 erf on a divergent lane would
// stall the warp on the slow FP64 pipe) and summed into FP64
template <bool MEASURE>
__device__ __forceinline__ void excl_acc(float dx, float dy, float dz, double qq, float alpha,
                                         double& fx, double& fy, double& fz, double* en) {
  float fe;
  const float e = excl_term<float>(fmaf(dx, dx, fmaf(dy, dy, dz * dz)), alpha, &fe);
  const double fq = (double)fe * qq;
  fx += fq * dx;
  fy += fq * dy;
  fz += fq * dz;
  if (MEASURE) {
    en[0] += (double)e * qq;
    en[3] += fq * dx * dx;
    en[4] += fq * dy * dy;
    en[5] += fq * dz * dz;
    en[6] += fq * dz * dy;
    en[7] += fq * dx * dz;
    en[8] += fq * dy * dx;
  }
}

// FP32 sum with a compensation term: s + c carries the sum of the added
// values to about FP64 accuracy for the few hundred terms of a site
// (Knuth's TwoSum, exact error of each addition into c)
struct CSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float t = s + x, bb = t - s;
    c += (s - (t - bb)) + (x - bb);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

struct PvF {
  float p0, p1, p2, p3, p4, p5;
  __device__ __forceinline__ void zero() { p0 = p1 = p2 = p3 = p4 = p5 = 0.f; }
  __device__ __forceinline__ void add(float dx, float dy, float dz, float f) {
    const float fdx = f * dx, fdy = f * dy, fdz = f * dz;
    p0 = fmaf(dx, fdx, p0);
    p1 = fmaf(dy, fdy, p1);
    p2 = fmaf(dz, fdz, p2);
    p3 = fmaf(dz, fdy, p3);
    p4 = fmaf(dx, fdz, p4);
    p5 = fmaf(dy, fdx, p5);
  }
};

// FP64 term at separation (dx,dy,dz): spline or exact exclusion; adds the
// force to (fx,fy,fz) and energy/virial to en
template <bool MEASURE>
__device__ __forceinline__ void term64(double dx, double dy, double dz, double qq, bool excl,
                                       const double* __restrict__ ert, double sgrid, int ntab,
                                       double alpha, double& fx, double& fy, double& fz,
                                       double* en) {
  const double r2 = dx * dx + dy * dy + dz * dz;
  double f, e;
  if (excl) {
    e = excl_term<double>(r2, alpha, &f);
  } else {
    const double* p = ert + 6 * min((int)(r2 * sgrid), ntab - 1);
    f = p[4] / (p[5] + r2) + p[3];
    e = p[1] / (p[2] + r2) + p[0];
  }
  f *= qq;
  const double fdx = f * dx, fdy = f * dy, fdz = f * dz;
  fx += fdx;
  fy += fdy;
  fz += fdz;
  if (MEASURE) {
    en[0] += e * qq;
    en[3] += dx * fdx;
    en[4] += dy * fdy;
    en[5] += dz * fdz;
    en[6] += dz * fdy;
    en[7] += dx * fdz;
    en[8] += dy * fdx;
  }
}


}  // namespace mg
