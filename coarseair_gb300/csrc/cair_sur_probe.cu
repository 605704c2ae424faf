// Self-test of the tensor-core operand conventions (cair_tc.cuh): one 128 x N x 16 BF16 MMA with
// FP32 accumulation in TMEM, its operands staged by the CTA's threads in the canonical no-swizzle
// layouts, B either K-major or MN-major.  The descriptor's two byte offsets are arguments, so a
// test can check which of the two assignments (K stride, M/N stride) the hardware reads.  Offsets
// are at most 2048 B and each operand region is 40 KB: 16 core matrices at any such offset plus one
// more stay inside the region, so no assignment reads outside the CTA's shared memory.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/cair_gpu.h"
#include "cair_tc.cuh"

namespace {

using namespace cair;

constexpr int kRegion = 40960;

__global__ void __launch_bounds__(128) k_tc_probe(const __nv_bfloat16* __restrict__ A,
                                                  const __nv_bfloat16* __restrict__ B, int N, int b_mn,
                                                  uint32_t a_lbo, uint32_t a_sbo, uint32_t b_lbo, uint32_t b_sbo,
                                                  float* __restrict__ D, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sa = sm;
  unsigned char* sb = sm + kRegion;
  uint64_t* bar = (uint64_t*)(sm + 2 * kRegion);
  uint32_t* tslot = (uint32_t*)(sm + 2 * kRegion + 16);
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < 2 * kRegion / 16; i += 128) ((uint4*)sm)[i] = make_uint4(0, 0, 0, 0);
  __syncthreads();
  // A[128][16] K-major: core (r/8, k/8) at (k/8)*2048 + (r/8)*128
  for (int r = tid; r < 128; r += 128)
    for (int k = 0; k < 16; ++k) *(__nv_bfloat16*)(sa + tc::kmaj_off(r, k, 128)) = A[r * 16 + k];
  // B[N][16]: K-major core (n/8, k/8) at (k/8)*N*16 + (n/8)*128, rows of 8 k;
  //           MN-major core (n/8, k/8) at (n/8)*256 + (k/8)*128, rows of 8 n (one row per k)
  for (int n = tid; n < N; n += 128)
    for (int k = 0; k < 16; ++k) {
      const uint32_t off = b_mn ? (uint32_t)((n >> 3) * 256 + (k >> 3) * 128 + (k & 7) * 16 + (n & 7) * 2)
                                : tc::kmaj_off(n, k, N);
      *(__nv_bfloat16*)(sb + off) = B[n * 16 + k];
    }
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::mbar_fence_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, 128);
    tc::tmem_relinquish();
  }
  tc::fence_smem_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  if (tid == 0) {
    const uint64_t ad = tc::sdesc(tc::smem_u32(sa), a_lbo, a_sbo);
    const uint64_t bd = tc::sdesc(tc::smem_u32(sb), b_lbo, b_sbo);
    tc::mma_bf16(tmem, ad, bd, tc::idesc_bf16(128, N, b_mn != 0), 0u);
    tc::mma_commit(bar);
  }
  const bool ok = tc::mbar_wait(bar, 0);
  tc::fence_after_sync();
  if (!ok) atomicExch(err, 1);
  if (__syncthreads_or(!ok) == 0) {
    for (int c = 0; c < N; c += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[tid * N + c + i] = v[i];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

// Throughput of back-to-back MMAs: one CTA issues `nmma` 128 x 128 x 16 BF16 MMAs into one
// accumulator, A and B no-swizzle K-major operands of K = 128 (K-steps cycling over the 8 steps),
// issue and completion timed with clock64 by the issuing thread.  Operand contents do not matter.
__global__ void __launch_bounds__(128) k_tc_rate(int nmma, int nsplit, long long* cycles, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* sa = sm;                 // 3 parts x 32 KB
  unsigned char* sb = sm + 3 * 32768;     // 32 KB
  uint64_t* bar = (uint64_t*)(sm + 4 * 32768);
  uint32_t* tslot = (uint32_t*)(sm + 4 * 32768 + 16);
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < 4 * 32768 / 16; i += 128) ((uint4*)sm)[i] = make_uint4(0x3f803f80u, 0, 0, 0);
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::mbar_fence_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, 128);
    tc::tmem_relinquish();
  }
  tc::fence_smem_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  long long t0 = 0, t1 = 0, t2 = 0;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, 128, false);
    t0 = clock64();
    for (int m = 0; m < nmma; ++m) {
      const int ks = m & 7, s = (m >> 3) % nsplit;
      const uint64_t ad = tc::sdesc(tc::smem_u32(sa) + s * 32768 + ks * 4096, 2048, 128);
      const uint64_t bd = tc::sdesc(tc::smem_u32(sb) + ks * 4096, 2048, 128);
      tc::mma_bf16(tmem, ad, bd, idesc, m > 0 ? 1u : 0u);
    }
    tc::mma_commit(bar);
    t1 = clock64();
  }
  const bool ok = tc::mbar_wait(bar, 0);
  if (tid == 0) {
    t2 = clock64();
    cycles[0] = t1 - t0;
    cycles[1] = t2 - t0;
  }
  if (!ok) atomicExch(err, 1);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

}  // namespace

// Internal (not in include/cair_gpu.h): cycles to issue and to complete `nmma` back-to-back
// 128 x 128 x 16 BF16 MMAs (k_tc_rate) on one SM.
extern "C" int cair_internal_tc_rate(int nmma, int nsplit, long long* issue_cycles, long long* total_cycles) {
  if (nmma < 1 || nmma > 100000 || nsplit < 1 || nsplit > 3 || !issue_cycles || !total_cycles) return CAIR_EINVAL;
  long long* d = nullptr;
  int* dErr = nullptr;
  int rc = CAIR_OK;
  const size_t smem = 4 * 32768 + 64;
  if (cudaMalloc(&d, 16) != cudaSuccess || cudaMalloc(&dErr, 4) != cudaSuccess) {
    rc = CAIR_ECUDA;
  } else {
    cudaMemset(dErr, 0, 4);
    cudaFuncSetAttribute(k_tc_rate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_tc_rate<<<1, 128, smem>>>(nmma, nsplit, d, dErr);
    long long h[2] = {0, 0};
    int e = 0;
    if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = CAIR_ECUDA;
    else {
      cudaMemcpy(&e, dErr, 4, cudaMemcpyDeviceToHost);
      cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost);
      if (e) rc = CAIR_ETIMEOUT;
      *issue_cycles = h[0];
      *total_cycles = h[1];
    }
  }
  cudaFree(d);
  cudaFree(dErr);
  return rc;
}

// Internal (not in include/cair_gpu.h): D[128][N] = A[128][16] x B[N][16]^T through one tcgen05.mma,
// with the given descriptor offsets.  N is 16 or 128.  Returns 0, CAIR_EINVAL, CAIR_ECUDA, or
// CAIR_ETIMEOUT if the completion wait ran out.
extern "C" int cair_internal_tc_probe(const void* A, const void* B, int N, int b_mn, uint32_t a_lbo, uint32_t a_sbo,
                                      uint32_t b_lbo, uint32_t b_sbo, float* D) {
  if (!A || !B || !D || (N != 16 && N != 128) || a_lbo > 2048 || a_sbo > 2048 || b_lbo > 2048 || b_sbo > 2048)
    return CAIR_EINVAL;
  __nv_bfloat16 *dA = nullptr, *dB = nullptr;
  float* dD = nullptr;
  int* dErr = nullptr;
  int rc = CAIR_OK;
  const size_t smem = 2 * kRegion + 64;
  if (cudaMalloc(&dA, 128 * 16 * 2) != cudaSuccess || cudaMalloc(&dB, (size_t)N * 16 * 2) != cudaSuccess ||
      cudaMalloc(&dD, (size_t)128 * N * 4) != cudaSuccess || cudaMalloc(&dErr, 4) != cudaSuccess) {
    rc = CAIR_ECUDA;
  } else {
    cudaMemcpy(dA, A, 128 * 16 * 2, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B, (size_t)N * 16 * 2, cudaMemcpyHostToDevice);
    cudaMemset(dErr, 0, 4);
    cudaFuncSetAttribute(k_tc_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_tc_probe<<<1, 128, smem>>>(dA, dB, N, b_mn, a_lbo, a_sbo, b_lbo, b_sbo, dD, dErr);
    int e = 0;
    if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = CAIR_ECUDA;
    else {
      cudaMemcpy(&e, dErr, 4, cudaMemcpyDeviceToHost);
      if (e) rc = CAIR_ETIMEOUT;
      else cudaMemcpy(D, dD, (size_t)128 * N * 4, cudaMemcpyDeviceToHost);
    }
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(dErr);
  return rc;
}

// ------------------------------------------------------------------------------------------
// FP64 timing probes for the warp integrator's design: one warp alone on the GPU runs a chain of
// n dependent operations on `active` of its lanes and records clock64 around it.
//   mode 0: x = fma(x, a, b)                                   (dependent DFMA latency)
//   mode 1: four independent DFMA chains per lane              (issue rate of one warp)
//   mode 2: a level of the programs: load from shared memory, DFMA, store, __syncwarp
// ------------------------------------------------------------------------------------------
__global__ void k_fp64_probe(int n, int active, int mode, long long* out, double* sink) {
  __shared__ double s[64];
  const int lane = threadIdx.x & 31;
  s[lane] = 1.0 + lane * 1e-3;
  s[lane + 32] = 1.0 - lane * 1e-3;
  __syncwarp();
  double x = 1.0 + lane * 1e-3, x1 = x + 0.5, x2 = x + 0.25, x3 = x + 0.125;
  const double a = 0.9999999, b = 1e-7;
  const long long t0 = clock64();
  if (lane < active) {
    if (mode == 0) {
      for (int i = 0; i < n; ++i) x = fma(x, a, b);
    } else if (mode == 1) {
      for (int i = 0; i < n; ++i) {
        x = fma(x, a, b);
        x1 = fma(x1, a, b);
        x2 = fma(x2, a, b);
        x3 = fma(x3, a, b);
      }
      x = x + x1 + x2 + x3;
    }
  }
  if (mode == 2) {
    for (int i = 0; i < n; ++i) {
      if (lane < active) {
        const double v = s[(i * 7 + lane) & 63];
        s[(i * 5 + lane + 11) & 63] = fma(v, a, b);
      }
      __syncwarp();
    }
    x = s[lane];
  }
  __syncwarp();
  const long long t1 = clock64();
  if (lane == 0) out[0] = t1 - t0;
  sink[lane] = x;
}

// Internal (not in include/cair_gpu.h): clock64 cycles of k_fp64_probe on one warp.
extern "C" int cair_internal_fp64_probe(int n, int active, int mode, long long* cycles) {
  if (n < 1 || n > (1 << 20) || active < 1 || active > 32 || mode < 0 || mode > 2 || !cycles) return CAIR_EINVAL;
  long long* d = nullptr;
  double* sink = nullptr;
  int rc = CAIR_OK;
  if (cudaMalloc(&d, 8) != cudaSuccess || cudaMalloc(&sink, 32 * sizeof(double)) != cudaSuccess) {
    rc = CAIR_ECUDA;
  } else {
    k_fp64_probe<<<1, 32>>>(n, active, mode, d, sink);
    if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) rc = CAIR_ECUDA;
    else cudaMemcpy(cycles, d, 8, cudaMemcpyDeviceToHost);
  }
  cudaFree(d);
  cudaFree(sink);
  return rc;
}
