// Ewald pass 2 (k-space forces, sim/ewpass2.c + sim/ewaldf.c) on the tensor
// cores.  For a (kx,ky) row of the k set and a charge j the pass needs
//   H  = W(row,0) + sum_{kz>0} (P.x c - M.y s,  M.x s + P.y c)
//   Hz =            sum_{kz>0} kz (M.x c - P.y s,  P.x s + M.y c)
// with W+- = W(row, +-kz) = ekk conj(S), P = W+ + W-, M = W+ - W-, and
// Z(kz) = (c, s) = e^{2 pi i kz z_j / Lz}; then A = q_j X(kx) Y(ky) and
//   F_x += kx Im(A H),  F_y += ky Im(A H),  F_z += Im(A Hz).
// (H.x, H.y, Hz.x, Hz.y) are linear in the vector
//   z_j = [c(0), c(1..Kz), s(1..Kz)]  (length 2 Kz + 1, padded to KP),
// so for a tile of 128 charges and 32 rows they are one product
//   D[128 x 128] = Z[128 x KP] V[128 x KP]^T,
// V holding four coefficient columns per row (built from W by
// kf_tc_vb_kernel).  The product runs on the tcgen05 tensor cores in TF32
// with each operand split as hi + lo (hi TF32-rounded, lo the FP32 rest) and
// three products hi*hi + hi*lo + lo*hi accumulated in FP32 in TMEM: the
// result carries FP32 accuracy.  The epilogue (four warps, one TMEM lane per
// charge) forms A from the phase rows and accumulates the force.
//
// One CTA per 128 charges: warp 4 streams the V tiles into shared memory
// with bulk copies (two stages) and issues the MMAs into two TMEM buffers
// of 128 columns; warps 0-3 drain the other buffer meanwhile.  Every wait is
// bounded; a wait that gives up sets bit 16 of the status word.
#include "mg_device.cuh"
#include "mg_internal.h"
#include "mg_tc.cuh"

namespace mg {

constexpr int TC_M = 128;             // charges per tile
constexpr int TC_N = 128;             // D columns per tile
constexpr int TC_ROWS = TC_N / 4;     // k rows per tile
constexpr long TC_WAIT = 1L << 24;    // polls before a wait gives up

// A operand: z_j of every charge, tile by tile (hi then lo, K-major layout)
__global__ void kf_tc_za_kernel(int nq, int ntm, int row, int oz, int Kz, int KP,
                                const float2* __restrict__ tab, float* __restrict__ za) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)ntm * TC_M * KP) return;
  const int j = (int)(t / KP), kk = (int)(t % KP);
  float v = 0.f;
  if (j < nq) {
    const float2* zr = tab + (long)j * row + oz;   // Z(0..Kz)
    if (kk <= Kz) v = zr[kk].x;
    else if (kk <= 2 * Kz) v = zr[kk - Kz].y;
  }
  float hi, lo;
  tc::tf32_split(v, hi, lo);
  float* base = za + (size_t)(j / TC_M) * 2 * TC_M * KP;
  const uint32_t o = tc::kmajor_offset(j % TC_M, kk, KP) >> 2;
  base[o] = hi;
  base[(size_t)TC_M * KP + o] = lo;
}

// B operand: per row r the columns 4r .. 4r+3 = coefficients of H.x, H.y,
// Hz.x, Hz.y over z_j (hi then lo per tile of 32 rows)
__global__ void kf_tc_vb_kernel(int nrows, int ntn, int Kz, int KP, const KRow* __restrict__ krows,
                                const float2* __restrict__ W, float* __restrict__ vb) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)ntn * TC_N * KP) return;
  const int n = (int)(t / KP), kk = (int)(t % KP);
  const int r = n / 4, comp = n % 4;
  float v = 0.f;
  if (r < nrows && kk <= 2 * Kz) {
    const KRow rw = krows[r];
    auto Wat = [&](int kz) {
      return (kz >= rw.kzlo && kz <= rw.kzhi) ? W[rw.kstart + kz - rw.kzlo] : make_float2(0.f, 0.f);
    };
    if (kk == 0) {
      const float2 w0 = Wat(0);
      v = comp == 0 ? w0.x : (comp == 1 ? w0.y : 0.f);
    } else {
      const int z = kk <= Kz ? kk : kk - Kz;
      const float2 wp = Wat(z), wm = Wat(-z);
      const float Px = wp.x + wm.x, Py = wp.y + wm.y, Mx = wp.x - wm.x, My = wp.y - wm.y;
      const float zf = (float)z;
      if (kk <= Kz)   // coefficients of c(z)
        v = comp == 0 ? Px : (comp == 1 ? Py : (comp == 2 ? zf * Mx : zf * My));
      else            // coefficients of s(z)
        v = comp == 0 ? -My : (comp == 1 ? Mx : (comp == 2 ? -(zf * Py) : zf * Px));
    }
  }
  float hi, lo;
  tc::tf32_split(v, hi, lo);
  float* base = vb + (size_t)(n / TC_N) * 2 * TC_N * KP;
  const uint32_t o = tc::kmajor_offset(n % TC_N, kk, KP) >> 2;
  base[o] = hi;
  base[(size_t)TC_N * KP + o] = lo;
}

struct KfTc {
  int nq, ns, KP, ntm, ntn, nrows, nxy, oyl, row;
  const float* za;
  const float* vb;
  const float2* tab;
  const KRow* krows;
  const int* qsite;
  const int* qdrude;
  double Lx, Ly, Lz;
  double* f;
  int* status;
};

// per k row: (kx, ky) as floats and the offsets of X(kx), Y(ky) in the
// shared phase block
struct TcRow {
  float kx, ky;
  int ox, oy;
};

size_t kf_tc_smem(int KP, int nxy, int nrows) {
  const size_t ab = (size_t)2 * TC_M * KP * 4;   // one operand tile, hi + lo
  return 3 * ab + (size_t)nxy * TC_M * sizeof(float2) + (size_t)nrows * sizeof(TcRow) + 128;
}

__global__ void __launch_bounds__(160, 1) kf_tc_kernel(KfTc a) {
  extern __shared__ __align__(1024) unsigned char smem_tc[];
  const uint32_t ab = (uint32_t)(2 * TC_M * a.KP * 4);
  unsigned char* As = smem_tc;                 // Z tile (hi | lo)
  unsigned char* Bs = smem_tc + ab;            // two V stages
  float2* XY = reinterpret_cast<float2*>(smem_tc + 3 * (size_t)ab);   // [nxy][128]
  TcRow* rk = reinterpret_cast<TcRow*>(XY + (size_t)a.nxy * TC_M);
  uint64_t* bars = reinterpret_cast<uint64_t*>(rk + a.nrows);
  uint64_t* bar_a = bars;
  uint64_t* full = bars + 1;    // [2] V stage loaded
  uint64_t* bfree = bars + 3;   // [2] V stage consumed
  uint64_t* tfull = bars + 5;   // [2] TMEM buffer written
  uint64_t* tfree = bars + 7;   // [2] TMEM buffer drained
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 9);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = blockIdx.x;

  if (warp < 4) {
    for (int t = tid; t < a.nxy * TC_M; t += 128) {
      const int e = t / TC_M, m = t % TC_M, j = mt * TC_M + m;
      XY[t] = j < a.nq ? a.tab[(long)j * a.row + e] : make_float2(0.f, 0.f);
    }
    for (int r = tid; r < a.nrows; r += 128) {
      const KRow rw = a.krows[r];
      rk[r] = TcRow{(float)rw.kx, (float)rw.ky, rw.kx * TC_M, (a.oyl + rw.ky) * TC_M};
    }
  }
  if (tid == 0) {
    tc::mbar_init(bar_a, 1);
    for (int s = 0; s < 2; s++) {
      tc::mbar_init(full + s, 1);
      tc::mbar_init(bfree + s, 1);
      tc::mbar_init(tfull + s, 1);
      tc::mbar_init(tfree + s, 4);
    }
  }
  if (warp == 4) tc::tmem_alloc(tslot, 2 * TC_N);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;

  if (warp == 4) {
    if (lane == 0) {
      const uint32_t half = (uint32_t)(TC_M * a.KP * 4), sbo = (uint32_t)(a.KP / 4) * 128;
      const uint32_t idesc = tc::idesc_tf32(TC_M, TC_N);
      const size_t tile_f = (size_t)2 * TC_M * a.KP;   // floats per operand tile
      tc::mbar_expect_tx(bar_a, ab);
      tc::bulk_g2s(As, a.za + (size_t)mt * tile_f, ab, bar_a);
      for (int t = 0; t < 2 && t < a.ntn; t++) {
        tc::mbar_expect_tx(full + t, ab);
        tc::bulk_g2s(Bs + (size_t)t * ab, a.vb + (size_t)t * tile_f, ab, full + t);
      }
      bool ok = tc::mbar_wait(bar_a, 0, TC_WAIT);
      const uint32_t a_hi = tc::smem_u32(As), a_lo = a_hi + half;
      for (int t = 0; ok && t < a.ntn; t++) {
        const int s = t & 1;
        ok = tc::mbar_wait(full + s, (t >> 1) & 1, TC_WAIT);
        if (ok && t >= 2) ok = tc::mbar_wait(tfree + s, ((t - 2) >> 1) & 1, TC_WAIT);
        if (!ok) break;
        tc::fence_after_sync();
        const uint32_t d = tbase + (uint32_t)(s * TC_N);
        const uint32_t b_hi = tc::smem_u32(Bs + (size_t)s * ab), b_lo = b_hi + half;
        for (int ks = 0; ks < a.KP / 8; ks++) {
          const uint32_t o = 256u * ks;
          tc::mma_tf32(d, tc::smem_desc(a_hi + o, 128, sbo), tc::smem_desc(b_hi + o, 128, sbo),
                       idesc, ks > 0 ? 1u : 0u);
          tc::mma_tf32(d, tc::smem_desc(a_hi + o, 128, sbo), tc::smem_desc(b_lo + o, 128, sbo),
                       idesc, 1u);
          tc::mma_tf32(d, tc::smem_desc(a_lo + o, 128, sbo), tc::smem_desc(b_hi + o, 128, sbo),
                       idesc, 1u);
        }
        tc::mma_commit(tfull + s);
        tc::mma_commit(bfree + s);
        // refill the stage of tile t-1 with tile t+1 once its products are done
        if (t >= 1 && t + 1 < a.ntn) {
          const int s1 = (t + 1) & 1;
          ok = tc::mbar_wait(bfree + s1, ((t - 1) >> 1) & 1, TC_WAIT);
          if (!ok) break;
          tc::mbar_expect_tx(full + s1, ab);
          tc::bulk_g2s(Bs + (size_t)s1 * ab, a.vb + (size_t)(t + 1) * tile_f, ab, full + s1);
        }
      }
      if (!ok) atomicOr(a.status, 16);
    }
    __syncwarp();
  } else {
    const int m = 32 * warp + lane;
    CSum Fx, Fy, Fz;
    bool ok = true;
    for (int t = 0; t < a.ntn; t++) {
      const int s = t & 1;
      ok = tc::mbar_wait(tfull + s, (t >> 1) & 1, TC_WAIT);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) break;
      tc::fence_after_sync();
      float gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll 1
      for (int c = 0; c < TC_N / 16; c++) {
        float v[16];
        tc::tmem_ld16(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)(s * TC_N + 16 * c), v);
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int r = t * TC_ROWS + 4 * c + q;
          if (r < a.nrows) {
            const TcRow kr = rk[r];
            const float2 X = XY[kr.ox + m], Y = XY[kr.oy + m];
            const float Ax = X.x * Y.x - X.y * Y.y, Ay = X.x * Y.y + X.y * Y.x;
            const float g = Ax * v[4 * q + 1] + Ay * v[4 * q];
            gx = fmaf(kr.kx, g, gx);
            gy = fmaf(kr.ky, g, gy);
            gz += Ax * v[4 * q + 3] + Ay * v[4 * q + 2];
          }
        }
      }
      Fx.add(gx);
      Fy.add(gy);
      Fz.add(gz);
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(tfree + s);
    }
    if (!ok && lane == 0) atomicOr(a.status, 16);
    const int j = mt * TC_M + m;
    if (ok && j < a.nq) {
      const int site = a.qsite[j];
      double* fo = a.f + 3 * (long)site + (a.qdrude && a.qdrude[j] ? 3 * (long)a.ns : 0);
      fo[0] += __dmul_rn(Fx.value(), 1.0 / a.Lx);
      fo[1] += __dmul_rn(Fy.value(), 1.0 / a.Ly);
      fo[2] += __dmul_rn(Fz.value(), 1.0 / a.Lz);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 4) tc::tmem_dealloc(tbase, 2 * TC_N);
}

bool kf_tc_fits(const KArgs& a, int nrows) {
  const int KP = ((2 * a.Kz + 1) + 7) / 8 * 8;
  return kf_tc_smem(KP, (a.Kx + 1) + (2 * a.Ky + 1), nrows) <= 227 * 1024;
}

int kf_tc_kp(const KArgs& a) { return ((2 * a.Kz + 1) + 7) / 8 * 8; }

cudaError_t k_kf_tc_za(const Launch& L, const KArgs& a, const float2* tab, float* za) {
  const int KP = kf_tc_kp(a), ntm = (a.nq + TC_M - 1) / TC_M;
  const long n = (long)ntm * TC_M * KP;
  kf_tc_za_kernel<<<(int)((n + 255) / 256), 256, 0, L.s>>>(a.nq, ntm, a.row,
                                                          a.Kx + 2 * a.Ky + 2, a.Kz, KP, tab, za);
  ++*L.counter;
  return cudaGetLastError();
}

cudaError_t k_kf_tc(const Launch& L, const KArgs& a, int nrows, const float2* tab,
                    const float* za, float* vb) {
  const int KP = kf_tc_kp(a), ntm = (a.nq + TC_M - 1) / TC_M;
  const int ntn = (4 * nrows + TC_N - 1) / TC_N;
  const long nv = (long)ntn * TC_N * KP;
  kf_tc_vb_kernel<<<(int)((nv + 255) / 256), 256, 0, L.s>>>(nrows, ntn, a.Kz, KP, a.krows, a.Wf,
                                                           vb);
  ++*L.counter;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  KfTc k;
  k.nq = a.nq;
  k.ns = a.ns;
  k.KP = KP;
  k.ntm = ntm;
  k.ntn = ntn;
  k.nrows = nrows;
  k.nxy = (a.Kx + 1) + (2 * a.Ky + 1);
  k.oyl = a.Kx + 1 + a.Ky;
  k.row = a.row;
  k.za = za;
  k.vb = vb;
  k.tab = tab;
  k.krows = a.krows;
  k.qsite = a.qsite;
  k.qdrude = a.qdrude;
  k.Lx = a.Lx;
  k.Ly = a.Ly;
  k.Lz = a.Lz;
  k.f = a.f;
  k.status = a.status;
  const size_t smem = kf_tc_smem(KP, k.nxy, nrows);
  e = cudaFuncSetAttribute(kf_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kf_tc_kernel<<<ntm, 160, smem, L.s>>>(k);
  ++*L.counter;
  return cudaGetLastError();
}

}  // namespace mg
