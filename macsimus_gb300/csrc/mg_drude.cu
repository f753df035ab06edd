// Drude (shell) polarizability on the device: the SCF relaxation step of
// sim/scf.c (selffield) and the ASPC predictor of sim/pred2.c, both in FP64.
//
// r and f hold 2*ns site vectors (cook's layout): centres, then the Drude
// displacements (r) / Drude forces (f).  Only sites with a Drude charge take
// part (dsite[] lists them).
#include "mg_internal.h"

namespace mg {

constexpr int DR_THREADS = 128;

// -erf(alpha r)/r + 2 alpha/sqrt(pi) and its f/r (exacterud_sqrt_1,
// sim/erexact.c:50-75): the Ewald correction of a site's own centre-Drude pair
__device__ __forceinline__ double self_pair_term(double rr, double alpha, double* erd) {
  const double A = alpha * -1.1283791670955126, aq = alpha * alpha, err = aq * rr;
  if (err < 0.01) {
    double su = 0, sd = 0, q = 1;
    for (int n = 1; n < 40; n++) {
      const double rn = q / (2 * n + 1);
      sd += rn * n;
      su += rn;
      if (fabs(q) < 1e-17) break;
      q *= -err / (n + 1);
    }
    *erd = A * aq * 2 * sd;
    return A * (-su * err);
  }
  const double r = sqrt(rr), y = -erf(alpha * r) / r;
  *erd = (y - A * exp(-err)) / rr;
  return y - A;
}

// One relaxation iteration: self-pair Ewald correction added to the Drude and
// centre forces, rpol <- (1-omega) rpol + omega alpha_qq fpol, the Drude force
// folded into the centre, spring energy (rpol.fpol, halved by the caller) and
// virial.  Partials per CTA: [el, self, Pvir0..5].
__global__ void __launch_bounds__(DR_THREADS)
    selffield_kernel(DrudeArgs a, double omega, double* __restrict__ r, double* __restrict__ f,
                     double* __restrict__ hist_out) {
  __shared__ double red[DR_THREADS][8];
  const int t = blockIdx.x * DR_THREADS + threadIdx.x;
  double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (t < a.nd) {
    const int i = a.dsite[t];
    double* rp = r + 3 * (long)a.ns + 3 * i;
    double* fp = f + 3 * (long)a.ns + 3 * i;
    double* fc = f + 3 * (long)i;
    const double d0 = rp[0], d1 = rp[1], d2 = rp[2];
    const double rr = d0 * d0 + d1 * d1 + d2 * d2;
    const double fq = a.qc[t] * a.qp[t];
    double byerd;
    const double e = self_pair_term(rr, a.alpha, &byerd);
    const double ff = fq * byerd;
    double p0 = fp[0] + ff * d0, p1 = fp[1] + ff * d1, p2 = fp[2] + ff * d2;
    double c0 = fc[0] - ff * d0, c1 = fc[1] - ff * d1, c2 = fc[2] - ff * d2;
    acc[0] = fq * e;
    acc[2] = d0 * ff * d0;
    acc[3] = d1 * ff * d1;
    acc[4] = d2 * ff * d2;
    acc[5] = d2 * ff * d1;
    acc[6] = d0 * ff * d2;
    acc[7] = d1 * ff * d0;
    const double w = omega * a.aqq[t];
    const double n0 = (1 - omega) * d0 + w * p0, n1 = (1 - omega) * d1 + w * p1,
                 n2 = (1 - omega) * d2 + w * p2;
    acc[1] = n0 * p0 + n1 * p1 + n2 * p2;
    acc[2] -= n0 * p0;
    acc[3] -= n1 * p1;
    acc[4] -= n2 * p2;
    acc[5] -= n1 * p2;
    acc[6] -= n2 * p0;
    acc[7] -= n0 * p1;
    // cook stops when a shell, before or after the iteration, is outside
    // the sphere of radius el.minqq around its site (sim/scf.c:137 and
    // :255): flag it, the host reports MG_ERR_SCF
    if (!(rr < a.minqq2) || !(n0 * n0 + n1 * n1 + n2 * n2 < a.minqq2)) atomicOr(a.status, 4);
    rp[0] = n0;
    rp[1] = n1;
    rp[2] = n2;
    fp[0] = p0;
    fp[1] = p1;
    fp[2] = p2;
    fc[0] = c0 + p0;
    fc[1] = c1 + p1;
    fc[2] = c2 + p2;
    if (hist_out) {
      hist_out[3 * t] = n0;
      hist_out[3 * t + 1] = n1;
      hist_out[3 * t + 2] = n2;
    }
  }
  for (int k = 0; k < 8; k++) red[threadIdx.x][k] = acc[k];
  __syncthreads();
  for (int s = DR_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int k = 0; k < 8; k++) red[threadIdx.x][k] += red[threadIdx.x + s][k];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 8; k++) a.part[blockIdx.x * 8 + k] = red[0][k];
}

cudaError_t k_selffield(const Launch& L, const DrudeArgs& a, double omega, double* r, double* f,
                        double* hist_out) {
  selffield_kernel<<<(a.nd + DR_THREADS - 1) / DR_THREADS, DR_THREADS, 0, L.s>>>(a, omega, r, f,
                                                                                hist_out);
  ++*L.counter;
  return cudaGetLastError();
}

// ASPC predictor: rpol(t+h) = sum_i B_i rpol_corrected(t - i h), history in a
// ring of K2 slots of 3*nd doubles, slot h the latest
__global__ void aspc_predict_kernel(DrudeArgs a, const double* __restrict__ hist, int K2, int h,
                                    AspcCoef B, double* __restrict__ r) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * a.nd) return;
  double p = 0;
  for (int i = 0; i < B.n; i++) p += B.b[i] * hist[(long)((h - i + K2) % K2) * 3 * a.nd + t];
  r[3 * (long)a.ns + 3 * a.dsite[t / 3] + t % 3] = p;
}

cudaError_t k_aspc_predict(const Launch& L, const DrudeArgs& a, const double* hist, int K2, int h,
                           const AspcCoef& B, double* r) {
  aspc_predict_kernel<<<(3 * a.nd + 255) / 256, 256, 0, L.s>>>(a, hist, K2, h, B, r);
  ++*L.counter;
  return cudaGetLastError();
}

// history slots from a state: rpol of the Drude sites of r (second half)
__global__ void drude_take_kernel(DrudeArgs a, const double* __restrict__ r,
                                  double* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * a.nd) return;
  out[t] = r[3 * (long)a.ns + 3 * a.dsite[t / 3] + t % 3];
}

cudaError_t k_drude_take(const Launch& L, const DrudeArgs& a, const double* r, double* out) {
  drude_take_kernel<<<(3 * a.nd + 255) / 256, 256, 0, L.s>>>(a, r, out);
  ++*L.counter;
  return cudaGetLastError();
}

// the inverse: shell displacements of the Drude sites into r's second half
__global__ void drude_put_kernel(DrudeArgs a, const double* __restrict__ in,
                                 double* __restrict__ r) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * a.nd) return;
  r[3 * (long)a.ns + 3 * a.dsite[t / 3] + t % 3] = in[t];
}

cudaError_t k_drude_put(const Launch& L, const DrudeArgs& a, const double* in, double* r) {
  drude_put_kernel<<<(3 * a.nd + 255) / 256, 256, 0, L.s>>>(a, in, r);
  ++*L.counter;
  return cudaGetLastError();
}

}  // namespace mg
