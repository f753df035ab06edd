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
// result carries FP32 accuracy.  The epilogue forms A from the phase rows
// and accumulates the force.
//
// One CTA per 128 charges, 17 warps.  Warp 16 bulk-copies the charges' tile
// (Z and their phase rows) and streams the V tiles into shared memory (two
// stages), and one of its threads issues the MMAs into two TMEM buffers of
// 128 columns.  Warps 0-15 drain the other buffer meanwhile: four warps per
// TMEM lane quarter (32 charges), each taking 8 of the tile's 32 rows.  The
// rows run in (kx, ky) order, so X(kx) changes rarely along a warp's rows.
// Every wait is bounded; a wait that gives up sets bit 16 of the status word.
#include "mg_device.cuh"
#include "mg_internal.h"
#include "mg_tc.cuh"

#include <algorithm>

namespace mg {

constexpr int TC_M = 128;             // charges per tile
#ifndef MG_KF_N
#define MG_KF_N 128
#endif
#ifndef MG_KF_NS
#define MG_KF_NS 2
#endif
// Pass-2 tile shape.  Measured on 32768 waters: 128 columns (32 k rows) in
// two stages 0.219 ms, 64 columns in four stages (the same shared memory
// and TMEM) 0.310 ms: the fixed cost of a tile's barrier round trips
// outweighs the deeper pipeline.
constexpr int TC_N = MG_KF_N;         // D columns per tile (64 or 128)
constexpr int TC_ROWS = TC_N / 4;     // k rows per tile
constexpr int TC_NS = MG_KF_NS;       // V stages in shared memory = TMEM buffers of TC_N columns
static_assert(TC_N == 64 || TC_N == 128, "pass-2 tile: 64 or 128 columns");
// tcgen05.alloc takes a power of two of at least 32 columns
static_assert(TC_NS * TC_N <= 256 && (TC_NS * TC_N & (TC_NS * TC_N - 1)) == 0,
              "pass-2 TMEM: a power of two of at most 256 columns");
constexpr long TC_WAIT = 1L << 24;    // polls before a wait gives up
constexpr int TC_EPI_WARPS = 16;      // four per TMEM lane quarter
constexpr int TC_EPI_ROWS = TC_ROWS / (TC_EPI_WARPS / 4);   // rows per warp and tile
constexpr int TC_EPI_LD = TC_EPI_ROWS / 4;                   // 16-column TMEM loads per warp and tile
constexpr int TC_THREADS = 32 * (TC_EPI_WARPS + 1);
constexpr int SK_G = 32;              // pass 1: charges per pipeline stage
constexpr int SK_PW = 16;             // pass 1: producer warps
constexpr int SK_THREADS = 32 * (SK_PW + 1);
constexpr int SK_R = 64;              // pass 1: k rows per tile (re and im: 128 lanes)
constexpr int SK_NS = 3;              // pass 1: pipeline stages
// pass 1: the producer warps drain group i - SK_LAG after forming group i's
// A tile, from SK_TB = SK_LAG + 1 TMEM buffers of 64 columns: the drain
// reads a group whose products finished long ago, and the products of a
// group reuse a buffer drained the iteration before, so neither side waits
#ifndef SK_LAG
#define SK_LAG 2
#endif
constexpr int SK_TB = SK_LAG + 1;
constexpr uint32_t SK_TCOLS = SK_TB <= 2 ? 128u : 256u;   // allocated TMEM columns
static_assert(SK_PW == 16, "pass-1 drain: four warps per TMEM lane quarter");
constexpr int SK_FOLD = 8;            // pass 1: group sums per compensated add
constexpr int SK_CPT = SK_G * SK_R / (32 * SK_PW);   // pass 1: charges per producer thread
static_assert(SK_CPT % 4 == 0, "pass-1 producers store whole 16-byte chunks");

// A tiles, one per 128 charges: z_j (hi, then lo, K-major layout), then the
// charges' phase values X(0..Kx) | Y(-Ky..Ky) transposed ([e][128] float2)
// for the epilogue; tile stride 256 (KP + nxy) floats.  With zb, also the
// pass-1 Z^T tiles (per 32 charges, rows kk of z_j, K = the charges).  One
// CTA per group of 32 charges: the group's phase rows are read once,
// coalesced, into shared memory; every warp store then writes a whole
// 128-byte core matrix (8 rows x 4 values) or 256 contiguous bytes of the
// phase block.  Charges at or beyond nq and rows beyond 2 Kz are zero.
__global__ void __launch_bounds__(256) kf_tc_prep_kernel(int nq, int row, int oz, int Kz, int KP,
                                                         int nxy, int KN,
                                                         const float2* __restrict__ tab,
                                                         float* __restrict__ za,
                                                         float* __restrict__ zb) {
  extern __shared__ float2 st_prep[];   // [32][row]
  const int g = blockIdx.x, j0 = g * SK_G;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nvalid = min(SK_G, max(0, nq - j0));
  for (int t = tid; t < SK_G * row; t += 256)
    st_prep[t] = t / row < nvalid ? tab[(long)j0 * row + t] : make_float2(0.f, 0.f);
  __syncthreads();
  // component kk of z_j = [c(0..Kz), s(1..Kz)] of charge c of the group
  auto zval = [&](int c, int kk) -> float {
    const float2* zr = st_prep + c * row + oz;
    return kk <= Kz ? zr[kk].x : (kk <= 2 * Kz ? zr[kk - Kz].y : 0.f);
  };
  const int r = lane & 7, cc = lane >> 3;   // row and 4-byte column inside a core matrix
  const int m0 = SK_G * (g % (TC_M / SK_G));  // first row of the group in its 128-charge tile
  const size_t tile_f = (size_t)2 * TC_M * (KP + nxy);
  float* base = za + (size_t)(g / (TC_M / SK_G)) * tile_f;
  for (int q = warp; q < (SK_G / 8) * (KP / 4); q += 8) {
    const int c = 8 * (q / (KP / 4)) + r, kk = 4 * (q % (KP / 4)) + cc;
    float hi, lo;
    tc::tf32_split(zval(c, kk), hi, lo);
    const uint32_t o = tc::kmajor_offset(m0 + c, kk, KP) >> 2;
    base[o] = hi;
    base[(size_t)TC_M * KP + o] = lo;
  }
  if (zb) {
    float* zt = zb + (size_t)g * 2 * SK_G * KN;
    for (int q = warp; q < (KN / 8) * (SK_G / 4); q += 8) {
      const int kk = 8 * (q / (SK_G / 4)) + r, c = 4 * (q % (SK_G / 4)) + cc;
      float hi, lo;
      tc::tf32_split(zval(c, kk), hi, lo);
      const uint32_t o = tc::kmajor_offset(kk, c, SK_G) >> 2;
      zt[o] = hi;
      zt[(size_t)SK_G * KN + o] = lo;
    }
  }
  float2* xy = reinterpret_cast<float2*>(base + (size_t)2 * TC_M * KP);
  for (int t = tid; t < nxy * SK_G; t += 256) {
    const int e = t / SK_G, c = t % SK_G;
    xy[(size_t)e * TC_M + m0 + c] = st_prep[c * row + e];
  }
}

// The same tiles computed straight from the positions (tensor-core path):
// per group of 32 charges the fixed-point coordinates and the phase rows
// (the arithmetic of charge_fixed_kernel and phase_tables_mixed_kernel, so
// the values are the same bit for bit), written to the phase table for
// pass 1 and, through shared memory, to the operand tiles.
__device__ __forceinline__ void kf_tc_phase_body(const KArgs& a_in, const double* __restrict__ r, int KP, int nxy,
                              int KN, float2* __restrict__ tab, float* __restrict__ za,
                              float* __restrict__ zb, const int bx_) {
  const KArgs a = a_in;   // a local copy (see kf_tc_body)
  extern __shared__ float2 st_ph[];   // [32][row]
  __shared__ uint4 sfix[SK_G];
  __shared__ float sq[SK_G];
  const int g = bx_, j0 = g * SK_G, row = a.row, Kz = a.Kz;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nvalid = min(SK_G, max(0, a.nq - j0));
  if (tid < SK_G) {
    uint4 f = make_uint4(0u, 0u, 0u, 0u);
    float q = 0.f;
    if (tid < nvalid) {
      const int j = j0 + tid, site = a.qsite[j];
      double x = r[3 * site], y = r[3 * site + 1], z = r[3 * site + 2];
      if (a.qdrude && a.qdrude[j]) {
        x += r[3 * (long)a.ns + 3 * site];
        y += r[3 * (long)a.ns + 3 * site + 1];
        z += r[3 * (long)a.ns + 3 * site + 2];
      }
      f = make_uint4((unsigned)fixed32(x, a.iLx), (unsigned)fixed32(y, a.iLy),
                     (unsigned)fixed32(z, a.iLz), 0u);
      q = (float)a.qval[j];
    }
    sfix[tid] = f;
    sq[tid] = q;
  }
  __syncthreads();
  for (int t = tid; t < SK_G * row; t += 256) {
    const int c = t / row, e = t % row;
    float2 v = make_float2(0.f, 0.f);
    if (c < nvalid) {
      int d, n;
      if (e <= a.Kx) { d = 0; n = e; }
      else if (e <= a.Kx + 2 * a.Ky + 1) { d = 1; n = e - (a.Kx + 1) - a.Ky; }
      else { d = 2; n = e - (a.Kx + 2 * a.Ky + 2); }
      const uint4 S4 = sfix[c];
      const unsigned S = d == 0 ? S4.x : (d == 1 ? S4.y : S4.z);
      const int ph = (int)(S * (unsigned int)n);
      const float tt = (float)ph * 2.3283064365386963e-10f;
      float sn, cs;
      sincospif(2.f * tt, &sn, &cs);
      if (d == 0) {
        cs *= sq[c];
        sn *= sq[c];
      }
      v = make_float2(cs, sn);
      tab[(long)j0 * row + t] = v;
    }
    st_ph[t] = v;
  }
  __syncthreads();
  auto zval = [&](int c, int kk) -> float {
    const float2* zr = st_ph + c * row + (a.Kx + 2 * a.Ky + 2);
    return kk <= Kz ? zr[kk].x : (kk <= 2 * Kz ? zr[kk - Kz].y : 0.f);
  };
  const int rr = lane & 7, cc = lane >> 3;
  const int m0 = SK_G * (g % (TC_M / SK_G));
  const size_t tile_f = (size_t)2 * TC_M * (KP + nxy);
  float* base = za + (size_t)(g / (TC_M / SK_G)) * tile_f;
  for (int q = warp; q < (SK_G / 8) * (KP / 4); q += 8) {
    const int c = 8 * (q / (KP / 4)) + rr, kk = 4 * (q % (KP / 4)) + cc;
    float hi, lo;
    tc::tf32_split(zval(c, kk), hi, lo);
    const uint32_t o = tc::kmajor_offset(m0 + c, kk, KP) >> 2;
    base[o] = hi;
    base[(size_t)TC_M * KP + o] = lo;
  }
  if (zb) {
    float* zt = zb + (size_t)g * 2 * SK_G * KN;
    for (int q = warp; q < (KN / 8) * (SK_G / 4); q += 8) {
      const int kk = 8 * (q / (SK_G / 4)) + rr, c = 4 * (q % (SK_G / 4)) + cc;
      float hi, lo;
      tc::tf32_split(zval(c, kk), hi, lo);
      const uint32_t o = tc::kmajor_offset(kk, c, SK_G) >> 2;
      zt[o] = hi;
      zt[(size_t)SK_G * KN + o] = lo;
    }
  }
  float2* xy = reinterpret_cast<float2*>(base + (size_t)2 * TC_M * KP);
  for (int t = tid; t < nxy * SK_G; t += 256) {
    const int e = t / SK_G, c = t % SK_G;
    xy[(size_t)e * TC_M + m0 + c] = st_ph[c * row + e];
  }
}

// B operand: per row r the columns 4r .. 4r+3 = coefficients of H.x, H.y,
// Hz.x, Hz.y over z_j (hi then lo per tile of 32 rows)
__device__ __forceinline__ void kf_tc_vb_body(int nrows, int ntn, int Kz, int KP, const KRow* __restrict__ krows,
                           const float2* __restrict__ W, float* __restrict__ vb, const int bx_) {
  const long t = (long)bx_ * blockDim.x + threadIdx.x;
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

// A tile (Z hi | lo, phase block), two V stages, barriers (nrows: kept for
// the callers; the row table is read from global memory)
size_t kf_tc_smem(int KP, int nxy, int nrows) {
  (void)nrows;
  return (size_t)1024 * (KP + nxy) + (size_t)TC_NS * 8 * TC_N * KP + 256;
}

__device__ __forceinline__ void kf_tc_body(const KfTc& a_in, const int bx_) {
  // a local copy: the stores below cannot alias it, so its fields stay in
  // registers instead of being reloaded through the reference
  const KfTc a = a_in;
  extern __shared__ __align__(1024) unsigned char smem_tc[];
  const uint32_t zb = 1024u * a.KP;              // Z tile bytes (hi | lo)
  const uint32_t vbytes = 8u * TC_N * a.KP;      // V tile bytes (hi | lo)
  const uint32_t ab = zb + 1024u * a.nxy;        // A tile with the phase block
  unsigned char* As = smem_tc;
  const float2* XY = reinterpret_cast<const float2*>(smem_tc + zb);   // [nxy][128]
  unsigned char* Bs = smem_tc + ab;              // TC_NS V stages of vbytes
  // the row table is read through L1 (every lane of a warp reads the same
  // row), which keeps nrows x 16 bytes out of shared memory: boxes up to
  // |n| <= 23 fit
  uint64_t* bars = reinterpret_cast<uint64_t*>(Bs + (size_t)TC_NS * vbytes);
  uint64_t* bar_a = bars;
  uint64_t* full = bars + 1;               // [NS] V stage loaded
  uint64_t* bfree = full + TC_NS;          // [NS] V stage consumed
  uint64_t* tfull = bfree + TC_NS;         // [NS] TMEM buffer written
  uint64_t* tfree = tfull + TC_NS;         // [NS] TMEM buffer drained
  uint32_t* tslot = reinterpret_cast<uint32_t*>(tfree + TC_NS);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mt = bx_;
  constexpr int PW = TC_EPI_WARPS;               // producer warp

  if (tid == 0) {
    tc::mbar_init(bar_a, 1);
    for (int s = 0; s < TC_NS; s++) {
      tc::mbar_init(full + s, 1);
      tc::mbar_init(bfree + s, 1);
      tc::mbar_init(tfull + s, 1);
      tc::mbar_init(tfree + s, TC_EPI_WARPS);
    }
  }
  if (warp == PW) tc::tmem_alloc(tslot, TC_NS * TC_N);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;

  if (warp == PW) {
    if (lane == 0) {
      const uint32_t half = zb / 2, sbo = (uint32_t)(a.KP / 4) * 128;
      const uint32_t idesc = tc::idesc_tf32(TC_M, TC_N);
      const size_t atile_f = (size_t)2 * TC_M * (a.KP + a.nxy), vtile_f = (size_t)2 * TC_N * a.KP;
      tc::mbar_expect_tx(bar_a, ab);
      tc::bulk_g2s(As, a.za + (size_t)mt * atile_f, ab, bar_a);
      for (int t = 0; t < TC_NS && t < a.ntn; t++) {
        tc::mbar_expect_tx(full + t, vbytes);
        tc::bulk_g2s(Bs + (size_t)t * vbytes, a.vb + (size_t)t * vtile_f, vbytes, full + t);
      }
      bool ok = tc::mbar_wait(bar_a, 0, TC_WAIT);
      const uint32_t a_hi = tc::smem_u32(As), a_lo = a_hi + half;
      // tile t: V stage and TMEM buffer s = t % NS, the (t / NS)-th use of each
      for (int t = 0; ok && t < a.ntn; t++) {
        const int s = t % TC_NS, use = t / TC_NS;
        ok = tc::mbar_wait(full + s, use & 1, TC_WAIT);
        if (ok && use > 0) ok = tc::mbar_wait(tfree + s, (use - 1) & 1, TC_WAIT);
        if (!ok) break;
        tc::fence_after_sync();
        const uint32_t d = tbase + (uint32_t)(s * TC_N);
        const uint32_t b_hi = tc::smem_u32(Bs + (size_t)s * vbytes), b_lo = b_hi + vbytes / 2;
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
        // refill the stage of tile t-1 with tile t-1+NS once its products are done
        if (t >= 1 && t - 1 + TC_NS < a.ntn) {
          const int s1 = (t - 1) % TC_NS;
          ok = tc::mbar_wait(bfree + s1, ((t - 1) / TC_NS) & 1, TC_WAIT);
          if (!ok) break;
          tc::mbar_expect_tx(full + s1, vbytes);
          tc::bulk_g2s(Bs + (size_t)s1 * vbytes, a.vb + (size_t)(t - 1 + TC_NS) * vtile_f, vbytes,
                       full + s1);
        }
      }
      if (!ok) atomicOr(a.status, 16);
    }
    __syncwarp();
  } else {
    // warp w: TMEM lanes 32 (w % 4) .. (its charges), columns 32 (w / 4) ..
    // (rows 8 (w / 4) .. 8 (w / 4) + 7 of each tile)
    const int qd = warp & 3, hf = warp >> 2;
    const int m = 32 * qd + lane;
    bool ok = tc::mbar_wait(bar_a, 0, TC_WAIT);
    ok = __all_sync(0xffffffffu, ok);
    CSum Fx, Fy, Fz;
    int cur_ox = -1;
    float2 X = make_float2(0.f, 0.f);
    // the TMEM loads of tile t+1 are issued before tile t is worked on, so
    // their latency hides behind the arithmetic (two register sets; the loop
    // is unrolled by two so that both stay in registers)
    auto wait_full = [&](int t) {
      bool w = tc::mbar_wait(tfull + t % TC_NS, (t / TC_NS) & 1, TC_WAIT);
      w = __all_sync(0xffffffffu, w);
      if (w) tc::fence_after_sync();
      return w;
    };
    auto issue = [&](int t, uint32_t (&v)[TC_EPI_LD][16]) {
      const uint32_t ta = tbase + ((uint32_t)(32 * qd) << 16) +
                          (uint32_t)((t % TC_NS) * TC_N + 4 * TC_EPI_ROWS * hf);
#pragma unroll
      for (int l = 0; l < TC_EPI_LD; l++) tc::tmem_ld16_async(ta + 16 * l, v[l]);
    };
    auto finish = [&](int t, uint32_t (&v)[TC_EPI_LD][16]) {
      tc::tmem_wait(v[0]);
#pragma unroll
      for (int l = 1; l < TC_EPI_LD; l++) tc::tmem_regs_after_wait(v[l]);
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(tfree + t % TC_NS);   // the buffer may take tile t+NS
    };
    auto work = [&](int t, const uint32_t (&v)[TC_EPI_LD][16]) {
      float gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
      for (int i = 0; i < TC_EPI_ROWS; i++) {
        const int r = t * TC_ROWS + TC_EPI_ROWS * hf + i;
        if (r < a.nrows) {
          const uint32_t* w = &v[i >> 2][4 * (i & 3)];
          const float hx = __uint_as_float(w[0]), hy = __uint_as_float(w[1]),
                      zx = __uint_as_float(w[2]), zy = __uint_as_float(w[3]);
          const int4 kq = __ldg(reinterpret_cast<const int4*>(a.rows) + r);
          const TcRow kr{__int_as_float(kq.x), __int_as_float(kq.y), kq.z, kq.w};
          if (kr.ox != cur_ox) {
            cur_ox = kr.ox;
            X = XY[kr.ox + m];
          }
          const float2 Y = XY[kr.oy + m];
          const float Ax = X.x * Y.x - X.y * Y.y, Ay = X.x * Y.y + X.y * Y.x;
          const float g = Ax * hy + Ay * hx;
          gx = fmaf(kr.kx, g, gx);
          gy = fmaf(kr.ky, g, gy);
          gz += Ax * zy + Ay * zx;
        }
      }
      Fx.add(gx);
      Fy.add(gy);
      Fz.add(gz);
    };
    uint32_t va[TC_EPI_LD][16], vb[TC_EPI_LD][16];
    if (ok && a.ntn > 0) {
      ok = wait_full(0);
      if (ok) {
        issue(0, va);
        finish(0, va);
      }
    }
    for (int t = 0; ok && t < a.ntn; t += 2) {
      // va holds tile t
      const bool n1 = t + 1 < a.ntn, n2 = t + 2 < a.ntn;
      if (n1) {
        ok = wait_full(t + 1);
        if (!ok) break;
        issue(t + 1, vb);
      }
      work(t, va);
      if (!n1) break;
      finish(t + 1, vb);
      if (n2) {
        ok = wait_full(t + 2);
        if (!ok) break;
        issue(t + 2, va);
      }
      work(t + 1, vb);
      if (n2) finish(t + 2, va);
    }
    if (!ok && lane == 0) atomicOr(a.status, 16);
    // the four warps of a lane quarter: the others hand their sums to the
    // first through the first V stage (the last products read it long before
    // the epilogue drained their TMEM buffer)
    float* part = reinterpret_cast<float*>(Bs);
    tc::named_sync(1, 32 * TC_EPI_WARPS);
    if (hf > 0) {
      float* p = part + (size_t)(hf - 1) * 6 * TC_M;
      p[0 * TC_M + m] = Fx.s;
      p[1 * TC_M + m] = Fx.c;
      p[2 * TC_M + m] = Fy.s;
      p[3 * TC_M + m] = Fy.c;
      p[4 * TC_M + m] = Fz.s;
      p[5 * TC_M + m] = Fz.c;
    }
    tc::named_sync(1, 32 * TC_EPI_WARPS);
    const int j = mt * TC_M + m;
    if (hf == 0 && ok && j < a.nq) {
      double sx = Fx.value(), sy = Fy.value(), sz = Fz.value();
      for (int h = 0; h < TC_EPI_WARPS / 4 - 1; h++) {
        const float* p = part + (size_t)h * 6 * TC_M;
        sx += (double)p[0 * TC_M + m] + (double)p[1 * TC_M + m];
        sy += (double)p[2 * TC_M + m] + (double)p[3 * TC_M + m];
        sz += (double)p[4 * TC_M + m] + (double)p[5 * TC_M + m];
      }
      const int site = a.qsite[j];
      double* fo = a.f + 3 * (long)site + (a.qdrude && a.qdrude[j] ? 3 * (long)a.ns : 0);
      fo[0] += __dmul_rn(sx, 1.0 / a.Lx);
      fo[1] += __dmul_rn(sy, 1.0 / a.Ly);
      fo[2] += __dmul_rn(sz, 1.0 / a.Lz);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == PW) tc::tmem_dealloc(tbase, TC_NS * TC_N);
}

// ------------------------------------------------------------- pass 1 --
//
// S(row, +-kz) = sum_j a_j(row) Z_kz(j) with a_j(row) = q_j X_j(kx) Y_j(ky):
// for 64 rows at a time, D[128 x KN] = A[128 x 32] Z^T[KN x 32]^T summed
// over groups of 32 charges, A's lanes r and 64 + r holding Re and Im of
// a_j(row r) and Z^T's rows [c(0..Kz), s(1..Kz)].  Per row
//   P = (sum Re a c, sum Re a s),  Q = (sum Im a s, sum Im a c),
//   S(+kz) = (P.x - Q.x, P.y + Q.y),  S(-kz) = (P.x + Q.x, Q.y - P.y),
// the +-kz symmetry of the FP32-core kernel.  A is formed in shared memory
// by sixteen warps from the charges' phase rows (bulk-copied per group with the
// Z^T tile), split hi + lo like the operands of pass 2, and multiplied in
// TF32 as three products.  CTA (row tile, charge chunk); the chunk's partial
// S go to part[chunk][k], summed in FP64 by the reduce kernel.


__host__ __device__ size_t sk_tc_stage(int KN, int row) {
  const size_t b = (size_t)2 * 128 * SK_G * 4 + (size_t)256 * KN + (size_t)256 * row;
  return (b + 1023) / 1024 * 1024;
}
size_t sk_tc_smem(int KN, int row) {
  return SK_NS * sk_tc_stage(KN, row) + SK_R * sizeof(KRow) + 128;
}

__device__ __forceinline__ void sk_tc_body(const SkTc& a_in, const int bx_) {
  const SkTc a = a_in;   // a local copy (see kf_tc_body)
  extern __shared__ __align__(1024) unsigned char smem_sk[];
  const size_t stb = sk_tc_stage(a.KN, a.row);
  const uint32_t abytes = 2 * 128 * SK_G * 4;             // A tile, hi | lo
  const uint32_t zbytes = 256u * a.KN, tbytes = 256u * a.row;
  KRow* rows = reinterpret_cast<KRow*>(smem_sk + SK_NS * stb);
  uint64_t* bars = reinterpret_cast<uint64_t*>(rows + SK_R);
  uint64_t* load = bars;                 // [NS] Z^T + phase rows of a group loaded
  uint64_t* afull = bars + SK_NS;        // [NS] A tile written
  uint64_t* freeb = bars + 2 * SK_NS;    // [NS] stage consumed by the products
  uint64_t* tfull = bars + 3 * SK_NS;    // [SK_TB] a group's sums in TMEM buffer b
  uint64_t* tfree = tfull + SK_TB;       // [SK_TB] TMEM buffer b drained
  uint32_t* tslot = reinterpret_cast<uint32_t*>(tfree + SK_TB);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int rt = bx_ % a.nrt, ch = bx_ / a.nrt;
  const int g0 = ch * a.gpc, ng = min(a.gpc, a.ngroups - g0), r0 = rt * SK_R;
  auto stage = [&](int s) { return smem_sk + (size_t)s * stb; };

  if (tid < SK_R)
    rows[tid] = r0 + tid < a.nrows ? a.krows[r0 + tid] : KRow{0, 0, 1, 0, 0, {0, 0, 0}};
  if (tid == 0) {
    for (int s = 0; s < SK_NS; s++) {
      tc::mbar_init(load + s, 1);
      tc::mbar_init(afull + s, SK_PW);
      tc::mbar_init(freeb + s, 1);
    }
    for (int b = 0; b < SK_TB; b++) {
      tc::mbar_init(tfull + b, 1);
      tc::mbar_init(tfree + b, SK_PW);
    }
  }
  if (warp == SK_PW) tc::tmem_alloc(tslot, SK_TCOLS);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;

  if (warp == SK_PW) {
    if (lane == 0) {
      auto issue_load = [&](int i) {
        const int s = i % SK_NS, g = g0 + i;
        unsigned char* st = stage(s);
        tc::mbar_expect_tx(load + s, zbytes + tbytes);
        tc::bulk_g2s(st + abytes, a.zb + (size_t)g * 2 * SK_G * a.KN, zbytes, load + s);
        tc::bulk_g2s(st + abytes + zbytes, a.tab + (size_t)g * SK_G * a.row, tbytes, load + s);
      };
      for (int i = 0; i < SK_NS && i < ng; i++) issue_load(i);
      const uint32_t idesc = tc::idesc_tf32(128, a.KN);
      bool ok = true;
      for (int i = 0; i < ng; i++) {
        const int s = i % SK_NS, b = i % SK_TB;
        ok = tc::mbar_wait(afull + s, (i / SK_NS) & 1, TC_WAIT);
        // buffer b last held group i - SK_TB, drained SK_LAG groups later
        if (ok && i >= SK_TB) ok = tc::mbar_wait(tfree + b, (i / SK_TB - 1) & 1, TC_WAIT);
        if (!ok) break;
        tc::fence_after_sync();
        const uint32_t d = tbase + 64u * b;
        const uint32_t a_hi = tc::smem_u32(stage(s)), a_lo = a_hi + abytes / 2;
        const uint32_t b_hi = a_hi + abytes, b_lo = b_hi + zbytes / 2;
#pragma unroll
        for (int ks = 0; ks < SK_G / 8; ks++) {
          const uint32_t o = 256u * ks;
          // every group starts a fresh accumulator: the tensor core's FP32
          // sums round toward zero, long sums would drift
          tc::mma_tf32(d, tc::smem_desc(a_hi + o, 128, 1024), tc::smem_desc(b_hi + o, 128, 1024),
                       idesc, ks > 0 ? 1u : 0u);
          tc::mma_tf32(d, tc::smem_desc(a_hi + o, 128, 1024), tc::smem_desc(b_lo + o, 128, 1024),
                       idesc, 1u);
          tc::mma_tf32(d, tc::smem_desc(a_lo + o, 128, 1024), tc::smem_desc(b_hi + o, 128, 1024),
                       idesc, 1u);
        }
        tc::mma_commit(freeb + s);
        tc::mma_commit(tfull + b);
        // refill the stage of group i-1 with group i-1+NS once its products
        // are done (the producers saw that stage's copy complete, so they
        // are done reading it too)
        if (i >= 1 && i - 1 + SK_NS < ng) {
          const int s1 = (i - 1) % SK_NS;
          ok = tc::mbar_wait(freeb + s1, ((i - 1) / SK_NS) & 1, TC_WAIT);
          if (!ok) break;
          issue_load(i - 1 + SK_NS);
        }
      }
      if (!ok) atomicOr(a.status, 16);
    }
    __syncwarp();
  } else {
    // producers: thread = (row r, 4 charges of the group), writing four
    // charges per 16-byte store; a warp's 32 rows fall on 8 different
    // 16-byte columns of the 8-row core matrices, so each store takes the
    // minimum of four shared-memory wavefronts.  The same warps drain the
    // group sums from TMEM one group behind: warp w reads lanes 32 (w % 4)
    // .. and the 8-column chunks w / 4 and w / 4 + 4 of the KN columns
    const int r = tid & (SK_R - 1), c0 = (tid >> 6) * SK_CPT;
    const KRow rw = rows[r];
    const bool valid = r0 + r < a.nrows;
    const int ox = rw.kx, oy = a.oyl + rw.ky;
    const uint32_t oR = tc::kmajor_offset(r, 0, SK_G), oI = tc::kmajor_offset(SK_R + r, 0, SK_G);
    const int qd = warp & 3, hf = warp >> 2;
    const bool ch1 = 8 * (hf + 4) < a.KN;   // second chunk present (KN > 32)
    // group sums: plain FP32 over SK_FOLD groups (rounded to nearest, so
    // unbiased), then into compensated sums
    CSum acc[16];
    float pend[16];
#pragma unroll
    for (int c = 0; c < 16; c++) pend[c] = 0.f;
    bool ok = true;
    auto drain = [&](int i) {
      const int b = i % SK_TB;
      bool w = tc::mbar_wait(tfull + b, (i / SK_TB) & 1, TC_WAIT);
      w = __all_sync(0xffffffffu, w);
      if (!w) return false;
      tc::fence_after_sync();
      uint32_t v[2][8];
      const uint32_t ta = tbase + ((uint32_t)(32 * qd) << 16) + 64u * b + (uint32_t)(8 * hf);
      tc::tmem_ld8_async(ta, v[0]);
      if (ch1) tc::tmem_ld8_async(ta + 32, v[1]);
      tc::tmem_wait8(v[0]);
      tc::tmem_regs_after_wait8(v[1]);
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(tfree + b);
#pragma unroll
      for (int c = 0; c < 8; c++) pend[c] += __uint_as_float(v[0][c]);
      if (ch1)
#pragma unroll
        for (int c = 0; c < 8; c++) pend[8 + c] += __uint_as_float(v[1][c]);
      if ((i & (SK_FOLD - 1)) == SK_FOLD - 1 || i == ng - 1) {
#pragma unroll
        for (int c = 0; c < 16; c++) {
          acc[c].add(pend[c]);
          pend[c] = 0.f;
        }
      }
      return true;
    };
    for (int i = 0; ok && i < ng; i++) {
      const int s = i % SK_NS;
      // the copy into stage s was issued after the products of group i-NS
      // (the last readers of its A tile) completed
      ok = tc::mbar_wait(load + s, (i / SK_NS) & 1, TC_WAIT);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) break;
      unsigned char* st = stage(s);
      const float2* tb = reinterpret_cast<const float2*>(st + abytes + zbytes);
#pragma unroll
      for (int h = 0; h < SK_CPT / 4; h++) {
        float rh[4], rl[4], ih[4], il[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const int jj = c0 + 4 * h + c;
          float re = 0.f, im = 0.f;
          if (valid) {
            const float2 X = tb[jj * a.row + ox], Y = tb[jj * a.row + oy];
            re = X.x * Y.x - X.y * Y.y;
            im = X.x * Y.y + X.y * Y.x;
          }
          tc::tf32_split(re, rh[c], rl[c]);
          tc::tf32_split(im, ih[c], il[c]);
        }
        // columns c0+4h .. c0+4h+3 of the K-major tile: one 16-byte chunk
        const uint32_t ko = (uint32_t)((c0 + 4 * h) >> 2) << 7;
        *reinterpret_cast<float4*>(st + oR + ko) = make_float4(rh[0], rh[1], rh[2], rh[3]);
        *reinterpret_cast<float4*>(st + abytes / 2 + oR + ko) =
            make_float4(rl[0], rl[1], rl[2], rl[3]);
        *reinterpret_cast<float4*>(st + oI + ko) = make_float4(ih[0], ih[1], ih[2], ih[3]);
        *reinterpret_cast<float4*>(st + abytes / 2 + oI + ko) =
            make_float4(il[0], il[1], il[2], il[3]);
      }
      tc::fence_async_smem();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(afull + s);
      if (i >= SK_LAG) ok = drain(i - SK_LAG);
    }
    for (int i = max(0, ng - SK_LAG); ok && i < ng; i++) ok = drain(i);
    if (!ok && lane == 0) atomicOr(a.status, 16);
    // the row sums, in FP64, through the first stage (no product or copy is
    // pending any more): D row m = r (Re) or 64 + r (Im)
    double* Dsm = reinterpret_cast<double*>(stage(0));
    const int m = 32 * qd + lane;
    tc::named_sync(1, 32 * SK_PW);
#pragma unroll
    for (int c = 0; c < 8; c++) {
      Dsm[m * 64 + 8 * hf + c] = acc[c].value();
      if (ch1) Dsm[m * 64 + 8 * (hf + 4) + c] = acc[8 + c].value();
    }
    tc::named_sync(1, 32 * SK_PW);
    if (warp < 2 && ok && ng > 0) {
      const KRow w = rows[m];
      const double* re = Dsm + m * 64;
      const double* im = Dsm + (m + SK_R) * 64;
      float2* out = a.part + (size_t)ch * a.nk;
      for (int kz = 0; kz <= a.Kz; kz++) {
        const double Px = re[kz], Qy = im[kz];
        const double Py = kz ? re[a.Kz + kz] : 0.0, Qx = kz ? im[a.Kz + kz] : 0.0;
        if (kz >= w.kzlo && kz <= w.kzhi)
          out[w.kstart + kz - w.kzlo] = make_float2((float)(Px - Qx), (float)(Py + Qy));
        if (kz > 0 && -kz >= w.kzlo && -kz <= w.kzhi)
          out[w.kstart - kz - w.kzlo] = make_float2((float)(Px + Qx), (float)(Qy - Py));
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == SK_PW) tc::tmem_dealloc(tbase, SK_TCOLS);
}

int sk_tc_kn(const KArgs& a) { return ((2 * a.Kz + 1) + 15) / 16 * 16; }

bool sk_tc_fits(const KArgs& a) {
  return sk_tc_kn(a) <= 64 && sk_tc_smem(sk_tc_kn(a), a.row) <= 227 * 1024;
}

size_t sk_tc_zb_floats(const KArgs& a) {
  const int ntm = (a.nq + TC_M - 1) / TC_M;
  return (size_t)ntm * (TC_M / SK_G) * 2 * SK_G * sk_tc_kn(a);
}

int kf_tc_kp(const KArgs& a) { return ((2 * a.Kz + 1) + 7) / 8 * 8; }

bool kf_tc_fits(const KArgs& a, int nrows) {
  return kf_tc_smem(kf_tc_kp(a), (a.Kx + 1) + (2 * a.Ky + 1), nrows) <= 227 * 1024;
}

size_t kf_tc_za_floats(const KArgs& a) {
  const int ntm = (a.nq + TC_M - 1) / TC_M;
  return (size_t)ntm * 2 * TC_M * (kf_tc_kp(a) + (a.Kx + 1) + (2 * a.Ky + 1));
}

size_t kf_tc_vb_floats(const KArgs& a, int nrows) {
  const int ntn = (4 * nrows + TC_N - 1) / TC_N;
  return (size_t)ntn * 2 * TC_N * kf_tc_kp(a);
}

void kf_tc_rows(const KArgs& a, const std::vector<KRow>& krows, std::vector<TcRow>* out) {
  const int oyl = a.Kx + 1 + a.Ky;
  out->clear();
  for (const KRow& r : krows)
    out->push_back(TcRow{(float)r.kx, (float)r.ky, r.kx * TC_M, (oyl + r.ky) * TC_M});
}

cudaError_t k_kf_tc_za(const Launch& L, const KArgs& a, const float2* tab, float* za, float* zb) {
  const int KP = kf_tc_kp(a), ntm = (a.nq + TC_M - 1) / TC_M;
  const int nxy = (a.Kx + 1) + (2 * a.Ky + 1);
  const size_t smem = sizeof(float2) * SK_G * (size_t)a.row;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kf_tc_prep_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  kf_tc_prep_kernel<<<ntm * (TC_M / SK_G), 256, smem, L.s>>>(
      a.nq, a.row, a.Kx + 2 * a.Ky + 2, a.Kz, KP, nxy, sk_tc_kn(a), tab, za, zb);
  ++*L.counter;
  return cudaGetLastError();
}

void sk_tc_split(const KArgs& a, int nrows, int* nch, int* gpc) {
  const int nrt = (nrows + SK_R - 1) / SK_R, ngroups = (a.nq + SK_G - 1) / SK_G;
  const int c = std::max(1, std::min(ngroups / 64, PARTITION_SMS / nrt));
  *gpc = (ngroups + c - 1) / c;
  *nch = (ngroups + *gpc - 1) / *gpc;
}

void tc_box(const KArgs& a, int nrows, int nch, int gpc, const KRow* tckrows, const TcRow* rows,
            const double* r, float2* tab, float* za, float* zb, float* vb, float2* part,
            TcBox* out) {
  TcBox& b = *out;
  b = TcBox{};
  b.ka = a;
  b.r = r;
  b.tab = tab;
  b.za = za;
  b.zb = zb;
  b.KP = kf_tc_kp(a);
  b.nxy = (a.Kx + 1) + (2 * a.Ky + 1);
  b.KN = sk_tc_kn(a);
  const int ntm = (a.nq + TC_M - 1) / TC_M;
  b.g_phase = ntm * (TC_M / SK_G);
  b.smem_phase = sizeof(float2) * SK_G * (size_t)a.row;
  if (zb) {
    SkTc& k = b.sk;
    k.KP = b.KP;
    k.KN = b.KN;
    k.Kz = a.Kz;
    k.nrows = nrows;
    k.nrt = (nrows + SK_R - 1) / SK_R;
    k.ngroups = (a.nq + SK_G - 1) / SK_G;
    k.gpc = gpc;
    k.row = a.row;
    k.oyl = a.Kx + 1 + a.Ky;
    k.nk = a.nk;
    k.tab = tab;
    k.zb = zb;
    k.krows = a.krows;
    k.part = part;
    k.status = a.status;
    b.g_sk = k.nrt * nch;
    b.smem_sk = sk_tc_smem(k.KN, a.row);
  }
  KfTc& k = b.kf;
  k.nq = a.nq;
  k.ns = a.ns;
  k.KP = b.KP;
  k.ntm = ntm;
  k.ntn = (4 * nrows + TC_N - 1) / TC_N;
  k.nrows = nrows;
  k.nxy = b.nxy;
  k.za = za;
  k.vb = vb;
  k.rows = rows;
  k.qsite = a.qsite;
  k.qdrude = a.qdrude;
  k.Lx = a.Lx;
  k.Ly = a.Ly;
  k.Lz = a.Lz;
  k.f = a.f;
  k.status = a.status;
  b.tckrows = tckrows;
  b.vb = vb;
  b.g_vb = (int)(((long)k.ntn * TC_N * b.KP + 255) / 256);
  b.g_kf = ntm;
  b.smem_kf = kf_tc_smem(b.KP, b.nxy, nrows);
}

// ---------------------------------------------------------------- launches --
//
// The tensor-core passes of a list of boxes, one launch each (blockIdx.y =
// box; CTAs beyond a box's own grid return before they touch TMEM or a
// barrier).  A single box is a list of one: a box of a batch runs the same
// kernel with the same arguments as the box alone, so it gets the same
// results bit for bit.

__global__ void __launch_bounds__(256) batch_tc_phase_kernel(const TcBox* __restrict__ B) {
  const TcBox& b = B[blockIdx.y];
  if ((int)blockIdx.x >= b.g_phase) return;
  kf_tc_phase_body(b.ka, b.r, b.KP, b.nxy, b.KN, b.tab, b.za, b.zb, blockIdx.x);
}

__global__ void __launch_bounds__(SK_THREADS, 1) batch_sk_tc_kernel(const TcBox* __restrict__ B) {
  const TcBox& b = B[blockIdx.y];
  if ((int)blockIdx.x >= b.g_sk) return;
  sk_tc_body(b.sk, blockIdx.x);
}

__global__ void batch_tc_vb_kernel(const TcBox* __restrict__ B) {
  const TcBox& b = B[blockIdx.y];
  if ((int)blockIdx.x >= b.g_vb) return;
  kf_tc_vb_body(b.kf.nrows, b.kf.ntn, b.ka.Kz, b.KP, b.tckrows, b.ka.Wf, b.vb, blockIdx.x);
}

__global__ void __launch_bounds__(TC_THREADS, 1) batch_kf_tc_kernel(const TcBox* __restrict__ B) {
  const TcBox& b = B[blockIdx.y];
  if ((int)blockIdx.x >= b.g_kf) return;
  kf_tc_body(b.kf, blockIdx.x);
}

cudaError_t k_batch_tc_phase(const Launch& L, const TcBox* d, int nbox, int grid, size_t smem) {
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(batch_tc_phase_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  batch_tc_phase_kernel<<<dim3(grid, nbox), 256, smem, L.s>>>(d);
  ++*L.counter;
  return cudaGetLastError();
}

cudaError_t k_batch_sk_tc(const Launch& L, const TcBox* d, int nbox, int grid, size_t smem) {
  cudaError_t e = cudaFuncSetAttribute(batch_sk_tc_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  batch_sk_tc_kernel<<<dim3(grid, nbox), SK_THREADS, smem, L.s>>>(d);
  ++*L.counter;
  return cudaGetLastError();
}

cudaError_t k_batch_kf_tc(const Launch& L, const TcBox* d, int nbox, int gvb, int gkf,
                          size_t smem) {
  batch_tc_vb_kernel<<<dim3(gvb, nbox), 256, 0, L.s>>>(d);
  ++*L.counter;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(batch_kf_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem);
  if (e != cudaSuccess) return e;
  batch_kf_tc_kernel<<<dim3(gkf, nbox), TC_THREADS, smem, L.s>>>(d);
  ++*L.counter;
  return cudaGetLastError();
}

}  // namespace mg
