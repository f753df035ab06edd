// Tensor-core self-test: one M = 128 TF32 product D = A B^T through TMEM,
// the same descriptors, MMA issue, mbarrier completion and TMEM loads as the
// tensor-core Ewald kernels, checked against a host product by the tests.
#include <cuda_runtime.h>

#include "../../include/macgpu.h"
#include "mg_internal.h"
#include "mg_tc.cuh"

namespace mg {

__global__ void __launch_bounds__(128)
    tc_selftest_kernel(const float* __restrict__ A, const float* __restrict__ B,
                       float* __restrict__ C, int N, int K, uint32_t ncols, int* status) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  unsigned char* As = tc_smem;
  unsigned char* Bs = As + 128 * K * 4;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(Bs + N * K * 4);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int t = tid; t < 128 * K; t += 128)
    *reinterpret_cast<float*>(As + tc::kmajor_offset(t / K, t % K, K)) = A[t];
  for (int t = tid; t < N * K; t += 128)
    *reinterpret_cast<float*>(Bs + tc::kmajor_offset(t / K, t % K, K)) = B[t];
  tc::fence_async_smem();
  if (tid == 0) tc::mbar_init(mbar, 1);
  if (warp == 0) tc::tmem_alloc(tslot, ncols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *tslot;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_tf32(128, N);
    const uint32_t sbo = (uint32_t)(K / 4) * 128;
    for (int s = 0; s < K / 8; s++) {
      const uint64_t ad = tc::smem_desc(tc::smem_u32(As) + 256 * s, 128, sbo);
      const uint64_t bd = tc::smem_desc(tc::smem_u32(Bs) + 256 * s, 128, sbo);
      tc::mma_tf32(tbase, ad, bd, idesc, s > 0 ? 1u : 0u);
    }
    tc::mma_commit(mbar);
  }
  bool ok = tc::mbar_wait(mbar, 0, 1L << 22);
  ok = __all_sync(0xffffffffu, ok);
  tc::fence_after_sync();
  if (ok) {
    for (int c = 0; c < N; c += 16) {
      float v[16];
      tc::tmem_ld16(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
#pragma unroll
      for (int i = 0; i < 16; i++) C[(size_t)(32 * warp + lane) * N + c + i] = v[i];
    }
  } else {
    if (lane == 0) atomicOr(status, 1);
    // the products may still be in flight: wait once more before the TMEM
    // is released
    tc::mbar_wait(mbar, 0, 1L << 22);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tbase, ncols);
}

}  // namespace mg

using namespace mg;

extern "C" int mg_tc_selftest(const float* A, const float* B, float* C, int n, int k) {
  if (!A || !B || !C || n < 16 || n > 256 || n % 16 || k < 8 || k > 64 || k % 8)
    return MG_ERR_ARG;
  uint32_t ncols = 32;
  while ((int)ncols < n) ncols *= 2;
  float *dA = nullptr, *dB = nullptr, *dC = nullptr;
  int* dst = nullptr;
  int rc = MG_OK, st = 0;
  const size_t smem = (size_t)(128 + n) * k * 4 + 16;
  cudaError_t e = cudaMalloc(&dA, sizeof(float) * 128 * k);
  if (e == cudaSuccess) e = cudaMalloc(&dB, sizeof(float) * n * k);
  if (e == cudaSuccess) e = cudaMalloc(&dC, sizeof(float) * 128 * n);
  if (e == cudaSuccess) e = cudaMalloc(&dst, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(dst, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(dA, A, sizeof(float) * 128 * k, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB, B, sizeof(float) * n * k, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
  if (e == cudaSuccess) {
    tc_selftest_kernel<<<1, 128, smem>>>(dA, dB, dC, n, k, ncols, dst);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&st, dst, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(C, dC, sizeof(float) * 128 * n, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) rc = MG_ERR_CUDA;
  else if (st) rc = MG_ERR_CUDA;
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(dst);
  return rc;
}
