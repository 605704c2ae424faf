// Kernels of the learned N3 surrogate (cair_sur.cuh): the weight images, batched evaluation, the
// training step (energy + force loss, its parameter gradient by hand-written forward, input-
// gradient, tangent and reverse passes on the tensor cores), Adam, the training targets from the
// FP64 surface, and the persistent integrator that runs Bulirsch-Stoer attempts on the surrogate
// with a per-attempt gate back to the FP64 surface.
#define CAIR_MODEL_TU  // model-independent kernels are built in the API translation unit
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "cair_kernels.cuh"
#include "cair_sur.cuh"
#include "cair_sur_launch.h"

namespace cair {
namespace sur {

constexpr int kNtot = 13;  // right-hand-side evaluations of one NSteps = 3 attempt
constexpr float kDSkip = 1e-9f;

// ------------------------------------------------------------------------------------------
// Parameters -> shared-memory image
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void image_put(const float* __restrict__ P, unsigned char* __restrict__ img, int p) {
  if (p < P_W2) {
    const int j = (p - P_W1) / NF, i = (p - P_W1) % NF;
    *(__nv_bfloat16*)(img + I_W1 + tc::kmaj_off(j, i, 128)) = __float2bfloat16_rn(P[p]);
  } else if (p < P_W3) {
    const int j = (p - P_W2) / NH, i = (p - P_W2) % NH;
    *(__nv_bfloat16*)(img + I_W2 + tc::kmaj_off(j, i, 128)) = __float2bfloat16_rn(P[p]);
  } else if (p < P_B2) {
    const int j = (p - P_W3) / NH, i = (p - P_W3) % NH;
    *(__nv_bfloat16*)(img + I_W3 + tc::kmaj_off(j, i, 128)) = __float2bfloat16_rn(P[p]);
  } else if (p < P_B3) {
    ((float*)(img + I_B2))[p - P_B2] = P[p];
  } else if (p < P_W4) {
    ((float*)(img + I_B3))[p - P_B3] = P[p];
  } else if (p < P_B4) {
    ((float*)(img + I_W4))[p - P_W4] = P[p];
  } else if (p == P_B4) {
    ((float*)(img + I_B4))[0] = P[p];
  }
}

__global__ void k_sur_image(const float* __restrict__ P, unsigned char* __restrict__ img) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < NPARAM; p += gridDim.x * blockDim.x) image_put(P, img, p);
}

// Adam (Kingma & Ba 2015) on the FP32 parameters, then the BF16 image; clears the gradient.
__global__ void k_sur_adam(float* __restrict__ P, float* __restrict__ G, float* __restrict__ M, float* __restrict__ V,
                           unsigned char* __restrict__ img, float lr, float b1, float b2, float eps, float c1,
                           float c2) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < NPARAM; p += gridDim.x * blockDim.x) {
    const float g = G[p];
    const float m = b1 * M[p] + (1.0f - b1) * g;
    const float v = b2 * V[p] + (1.0f - b2) * g * g;
    M[p] = m;
    V[p] = v;
    P[p] -= lr * (m * c1) / (sqrtf(v * c2) + eps);
    G[p] = 0.0f;
    image_put(P, img, p);
  }
}

// ------------------------------------------------------------------------------------------
// Engine passes.  NHALF = 2 stages a 128-wide operand in two 64-wide halves (the integrator keeps
// two networks resident and has room for half an operand); NHALF = 1 stages it whole.  TMEM
// columns: blocks of 128 at 0, 128, 256, 384.
// ------------------------------------------------------------------------------------------
template <int NHALF>
struct Stage {
  static constexpr int KC = 128 / NHALF;
  static constexpr uint32_t SPLIT = 128u * KC * 2u;  // bytes of one BF16 part of the operand
};

// 16 consecutive FP32 values of a vector in shared memory (16-byte aligned), zeros for nullptr.
__device__ __forceinline__ void ld_vec16(const float* p, float (&b)[16]) {
  if (!p) {
#pragma unroll
    for (int i = 0; i < 16; ++i) b[i] = 0.0f;
    return;
  }
#pragma unroll
  for (int i = 0; i < 16; i += 4) {
    const float4 q = *reinterpret_cast<const float4*>(p + i);
    b[i] = q.x; b[i + 1] = q.y; b[i + 2] = q.z; b[i + 3] = q.w;
  }
}

// z_out = tanh(z_in + bias) x W^T over the 128 inputs.
template <int NHALF>
__device__ __forceinline__ void hidden(Cta& c, int* err, const unsigned char* img, int w_off, const float* bias,
                                       unsigned char* buf, uint32_t zin, uint32_t zout) {
  using St = Stage<NHALF>;
#pragma unroll 1
  for (int hf = 0; hf < NHALF; ++hf) {
    if (!c.dead) {
#pragma unroll 1
      for (int cc = c.part * (St::KC / c.parts); cc < (c.part + 1) * (St::KC / c.parts); cc += 16) {
        float v[16], b[16];
        ld16(c, zin + hf * St::KC + cc, v);
        ld_vec16(bias ? bias + hf * St::KC + cc : nullptr, b);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          float t, s;
          tanh_s(v[i] + b[i], t, s);
          v[i] = t;
        }
        put16<3>(buf, St::SPLIT, c.row, cc, v);
      }
    }
    phase(c, err, [&] {
      issue_block<3>(c.tmem + zout, buf, St::SPLIT, 0, St::KC / 16, img + w_off, hf * St::KC, 128, false, hf > 0);
    });
  }
}

// y = w4 . tanh(z3 + b3) + b4; with BACK also u2 = (w4 * s3) x W3 into column block u2.
template <int NHALF, bool BACK>
__device__ __forceinline__ float output(Cta& c, int* err, const unsigned char* img, unsigned char* buf, uint32_t z3,
                                        uint32_t u2) {
  using St = Stage<NHALF>;
  const float* b3 = (const float*)(img + I_B3);
  const float* w4 = (const float*)(img + I_W4);
  float y = 0.0f;
#pragma unroll 1
  for (int hf = 0; hf < NHALF; ++hf) {
    if (!c.dead) {
#pragma unroll 1
      for (int cc = c.part * (St::KC / c.parts); cc < (c.part + 1) * (St::KC / c.parts); cc += 16) {
        float v[16], bb[16], ww[16];
        ld16(c, z3 + hf * St::KC + cc, v);
        ld_vec16(b3 + hf * St::KC + cc, bb);
        ld_vec16(w4 + hf * St::KC + cc, ww);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          float t, s;
          tanh_s(v[i] + bb[i], t, s);
          y = fmaf(ww[i], t, y);
          v[i] = ww[i] * s;
        }
        if (BACK) put16<3>(buf, St::SPLIT, c.row, cc, v);
      }
    }
    if (BACK)
      phase(c, err, [&] {
        issue_block<3>(c.tmem + u2, buf, St::SPLIT, 0, St::KC / 16, img + I_W3, hf * St::KC, 128, true, hf > 0);
      });
  }
  if (c.parts == 2) {  // the row's two partial sums
    if (c.part == 1) c.yshare[c.row] = y;
    __syncthreads();
    if (c.part == 0) y += c.yshare[c.row];
  }
  return y + ((const float*)(img + I_B4))[0];
}

// dcol = (s(z + bias) * u) x W over W's outputs (the transposed use of the weight image), N its inputs.
template <int NHALF>
__device__ __forceinline__ void backward(Cta& c, int* err, const unsigned char* img, int w_off, int N,
                                         const float* bias, unsigned char* buf, uint32_t ucol, uint32_t zcol,
                                         uint32_t dcol) {
  using St = Stage<NHALF>;
#pragma unroll 1
  for (int hf = 0; hf < NHALF; ++hf) {
    if (!c.dead) {
#pragma unroll 1
      for (int cc = c.part * (St::KC / c.parts); cc < (c.part + 1) * (St::KC / c.parts); cc += 16) {
        float u[16], z[16], b[16];
        ld16(c, ucol + hf * St::KC + cc, u);
        ld16(c, zcol + hf * St::KC + cc, z);
        ld_vec16(bias ? bias + hf * St::KC + cc : nullptr, b);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          float t, s;
          tanh_s(z[i] + b[i], t, s);
          u[i] *= s;
        }
        put16<3>(buf, St::SPLIT, c.row, cc, u);
      }
    }
    phase(c, err, [&] {
      issue_block<3>(c.tmem + dcol, buf, St::SPLIT, 0, St::KC / 16, img + w_off, hf * St::KC, N, true, hf > 0);
    });
  }
}

// One member's value and input gradient g = dy/df; the features must already be in buf.
template <int NHALF>
__device__ __forceinline__ float member_eval(Cta& c, int* err, const unsigned char* img, unsigned char* buf,
                                             float (&g)[16]) {
  using St = Stage<NHALF>;
  phase(c, err, [&] { issue_block<3>(c.tmem + 0, buf, St::SPLIT, 0, 1, img + I_W1, 0, 128, false, false); });
  hidden<NHALF>(c, err, img, I_W2, nullptr, buf, 0, 128);
  hidden<NHALF>(c, err, img, I_W3, (const float*)(img + I_B2), buf, 128, 256);
  const float y = output<NHALF, true>(c, err, img, buf, 256, 384);
  backward<NHALF>(c, err, img, I_W2, 128, (const float*)(img + I_B2), buf, 384, 128, 256);
  backward<NHALF>(c, err, img, I_W1, 16, nullptr, buf, 256, 0, 384);
  if (!c.dead) ld16(c, 384, g);
  else
#pragma unroll
    for (int i = 0; i < 16; ++i) g[i] = 0.0f;
  return y;
}

// One member's value only (TMEM blocks 256 and 384); the features must already be in buf.
template <int NHALF>
__device__ __forceinline__ float member_value(Cta& c, int* err, const unsigned char* img, unsigned char* buf) {
  using St = Stage<NHALF>;
  phase(c, err, [&] { issue_block<3>(c.tmem + 256, buf, St::SPLIT, 0, 1, img + I_W1, 0, 128, false, false); });
  hidden<NHALF>(c, err, img, I_W2, nullptr, buf, 256, 384);
  hidden<NHALF>(c, err, img, I_W3, (const float*)(img + I_B2), buf, 384, 256);
  return output<NHALF, false>(c, err, img, buf, 256, 0);
}

// The integrator calls the network passes out of line: its Bulirsch-Stoer state (about 240
// registers) is saved once around each call instead of being kept live through the epilogues, which
// then have the register file for their 16-wide chunks.
__device__ __noinline__ float member_eval_call(Cta& c, int* err, const unsigned char* img, unsigned char* buf,
                                               float* g) {
  float gg[16];
  const float y = member_eval<2>(c, err, img, buf, gg);
#pragma unroll
  for (int i = 0; i < 16; ++i) g[i] = gg[i];
  return y;
}
__device__ __noinline__ float member_value_call(Cta& c, int* err, const unsigned char* img, unsigned char* buf) {
  return member_value<2>(c, err, img, buf);
}

// V3 [Eh] and dV3/dR [Eh/bohr] from y [eV] and g, with the features recomputed at R.
__device__ __forceinline__ void v3_of(const SurConst& C, const double (&R)[3], float y, const float (&g)[16],
                                      double& v3, double (&dv3)[3]) {
  Feat F;
  features(C, R, F);
  v3 = (double)(F.D * y) / kEvPerEh;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float a = F.dD[k] * y, b = 0.0f;
#pragma unroll
    for (int i = 0; i < NINV; ++i) b = fmaf(g[i], F.J[i][k], b);
    dv3[k] = (double)(a + F.D * b) / kEvPerEh;
  }
}

// ------------------------------------------------------------------------------------------
// CTA set-up and tear-down
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void copy_image(unsigned char* dst, const unsigned char* __restrict__ src) {
  for (int i = threadIdx.x; i < IMAGE / 16; i += blockDim.x) ((uint4*)dst)[i] = ((const uint4*)src)[i];
}

__device__ __forceinline__ void cta_open(Cta& c, uint64_t* bar, uint32_t* tslot, float* yshare = nullptr) {
  c.tid = threadIdx.x;
  c.row = threadIdx.x & 127;
  c.parts = blockDim.x / 128;
  c.part = threadIdx.x >> 7;
  c.yshare = yshare;
  c.lane_off = (uint32_t)(((threadIdx.x >> 5) & 3) * 32) << 16;
  c.bar = bar;
  c.phase = 0;
  c.dead = false;
  if (threadIdx.x == 0) {
    tc::mbar_init(bar, 1);
    tc::mbar_fence_init();
  }
  if (threadIdx.x < 32) {
    tc::tmem_alloc(tslot, 512);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  c.tmem = *tslot;
}

__device__ __forceinline__ void cta_close(Cta& c) {
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc::fence_after_sync();
    tc::tmem_dealloc(c.tmem, 512);
  }
}

// Shared memory of the two-network kernels (evaluation, integrator)
constexpr int SM_IMG_A = 0;
constexpr int SM_IMG_B = ((IMAGE + 1023) / 1024) * 1024;
constexpr int SM_BUF2 = 2 * SM_IMG_B;
constexpr int SM_BAR2 = SM_BUF2 + 3 * (int)Stage<2>::SPLIT;
constexpr int SM_Y2 = SM_BAR2 + 64;
constexpr int SMEM2 = SM_Y2 + 128 * 4;
constexpr int NT2 = 256;  // threads of the two-network kernels: two per tile row

// ------------------------------------------------------------------------------------------
// Batched evaluation: both members' values, member A's input gradient and the surrogate's
// V3 and dV3/dR at n geometries (pair distances R[n][3]).  The same passes as the integrator.
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NT2, 1) k_sur_eval(SurConst C, const unsigned char* __restrict__ gimgA,
                                                     const unsigned char* __restrict__ gimgB, int64_t n,
                                                     const double* __restrict__ Rin, float* __restrict__ ya,
                                                     float* __restrict__ yb, float* __restrict__ g,
                                                     double* __restrict__ v3, double* __restrict__ dv3, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* imgA = sm + SM_IMG_A;
  unsigned char* imgB = sm + SM_IMG_B;
  unsigned char* buf = sm + SM_BUF2;
  copy_image(imgA, gimgA);
  copy_image(imgB, gimgB);
  Cta c;
  cta_open(c, (uint64_t*)(sm + SM_BAR2), (uint32_t*)(sm + SM_BAR2 + 16), (float*)(sm + SM_Y2));
  const int64_t ntile = (n + 127) / 128;
#pragma unroll 1
  for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    if (__syncthreads_or(c.dead)) break;
    const int64_t row = tile * 128 + c.row;
    const bool valid = row < n && c.part == 0;   // the row's owner reads its input and writes its outputs
    double R[3] = {2.1, 4.0, 6.0};
    if (valid)
#pragma unroll
      for (int k = 0; k < 3; ++k) R[k] = Rin[3 * row + k];
    Feat F;
    features(C, R, F);
    if (c.part == 0) put16<3>(buf, Stage<2>::SPLIT, c.row, 0, F.f);
    const float vb = member_value<2>(c, err, imgB, buf);
    if (c.part == 0) put16<3>(buf, Stage<2>::SPLIT, c.row, 0, F.f);
    float gg[16];
    const float va = member_eval<2>(c, err, imgA, buf, gg);
    if (valid && !c.dead) {
      ya[row] = va;
      yb[row] = vb;
#pragma unroll
      for (int i = 0; i < 16; ++i) g[16 * row + i] = gg[i];
      double v, d[3];
      v3_of(C, R, va, gg, v, d);
      v3[row] = v;
#pragma unroll
      for (int k = 0; k < 3; ++k) dv3[3 * row + k] = d[k];
    }
  }
  cta_close(c);
}

// ------------------------------------------------------------------------------------------
// Training step
// ------------------------------------------------------------------------------------------
constexpr int SM_IMG_T = 0;
constexpr int SM_BUF_T = SM_IMG_B;                         // after one image
constexpr int SM_SUM_T = SM_BUF_T + 3 * (int)Stage<1>::SPLIT;
constexpr int NSUM = 3 * NH + 4;                           // b2, b3, w4 gradients, b4, loss_e, loss_f, rows
constexpr int SM_BAR_T = SM_SUM_T + NSUM * 4;
constexpr int SMEM_T = SM_BAR_T + 64;
constexpr int NVEC = 7;                                    // per-row vectors kept in global scratch
enum { V_H1, V_H2, V_H3, V_U2, V_U1, V_Z1D, V_Z2D };

struct TrainArgs {
  SurConst C;
  const unsigned char* img;      // the member's image
  const cair_sur_sample* samples;
  const int64_t* idx;            // the batch: sample indices
  int64_t nbatch;
  float wE, wF;                  // loss weights, already divided by the batch size
  float* grad;                   // [NPARAM], accumulated
  double* loss;                  // [2] energy and force parts, accumulated
  float* scratch;                // [gridDim.x][NVEC][128][128]
  int* err;
};

__device__ __forceinline__ float* vec_row(const TrainArgs& A, int v) {
  return A.scratch + (((size_t)blockIdx.x * NVEC + v) * 128 + threadIdx.x) * 128;
}
__device__ __forceinline__ void save16(float* row, int k0, const float (&v)[16]) {
#pragma unroll
  for (int i = 0; i < 16; i += 4) *(float4*)(row + k0 + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
}
__device__ __forceinline__ void load16(const float* row, int k0, float (&v)[16]) {
#pragma unroll
  for (int i = 0; i < 16; i += 4) {
    const float4 q = *(const float4*)(row + k0 + i);
    v[i] = q.x; v[i + 1] = q.y; v[i + 2] = q.z; v[i + 3] = q.w;
  }
}
// column r of a K-major [rows][128] operand (K = the tile's rows): element (j, r) for j < rows
__device__ __forceinline__ void put_col(unsigned char* buf, int rows, int r, int j0, const float (&v)[16]) {
#pragma unroll
  for (int i = 0; i < 16; ++i)
    *(__nv_bfloat16*)(buf + tc::kmaj_off(j0 + i, r, rows)) = __float2bfloat16_rn(v[i]);
}

// TMEM block of an M = 128 gradient (row j = this thread, ncol columns) added to grad[base + j * ncol + i]
__device__ __forceinline__ void flush_grad(const Cta& c, uint32_t col, int ncol, float* grad) {
  for (int cc = 0; cc < ncol; cc += 16) {
    float v[16];
    ld16(c, col + cc, v);
#pragma unroll
    for (int i = 0; i < 16; ++i) atomicAdd(grad + (size_t)c.tid * ncol + cc + i, v[i]);
  }
}

__global__ void __launch_bounds__(128, 1) k_sur_grad(TrainArgs A) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* img = sm + SM_IMG_T;
  unsigned char* buf = sm + SM_BUF_T;
  float* sums = (float*)(sm + SM_SUM_T);
  constexpr uint32_t SP = Stage<1>::SPLIT;  // 32 KB: one 128 x 128 BF16 operand
  copy_image(img, A.img);
  for (int i = threadIdx.x; i < NSUM; i += 128) sums[i] = 0.0f;
  Cta c;
  cta_open(c, (uint64_t*)(sm + SM_BAR_T), (uint32_t*)(sm + SM_BAR_T + 16));
  const float* b2 = (const float*)(img + I_B2);
  const float* b3 = (const float*)(img + I_B3);
  const float* w4 = (const float*)(img + I_W4);
  const int r = threadIdx.x;
  float* H1 = vec_row(A, V_H1); float* H2 = vec_row(A, V_H2); float* H3 = vec_row(A, V_H3);
  float* U2 = vec_row(A, V_U2); float* U1 = vec_row(A, V_U1);
  float* Z1d = vec_row(A, V_Z1D); float* Z2d = vec_row(A, V_Z2D);
  const int64_t ntile = (A.nbatch + 127) / 128;
#pragma unroll 1
  for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    if (__syncthreads_or(c.dead)) break;
    const int64_t row = tile * 128 + r;
    const bool valid = row < A.nbatch;
    double R[3] = {2.1, 4.0, 6.0};
    float Et = 0.0f, Gt[3] = {0.0f, 0.0f, 0.0f};
    if (valid) {
      const cair_sur_sample& S = A.samples[A.idx[row]];
      R[0] = S.R[0]; R[1] = S.R[1]; R[2] = S.R[2];
      Et = S.e;
      Gt[0] = S.g[0]; Gt[1] = S.g[1]; Gt[2] = S.g[2];
    }
    const float wE = valid ? A.wE : 0.0f, wF = valid ? A.wF : 0.0f;
    Feat F;
    features(A.C, R, F);
    // ---- forward (three-part operands) ----
    put16<3>(buf, SP, r, 0, F.f);
    phase(c, A.err, [&] { issue_block<3>(c.tmem + 0, buf, SP, 0, 1, img + I_W1, 0, 128, false, false); });
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float v[16];
        ld16(c, 0 + cc, v);
        for (int i = 0; i < 16; ++i) { float t, s; tanh_s(v[i], t, s); v[i] = t; }
        save16(H1, cc, v);
        put16<3>(buf, SP, r, cc, v);
      }
    phase(c, A.err, [&] { issue_block<3>(c.tmem + 128, buf, SP, 0, 8, img + I_W2, 0, 128, false, false); });
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float v[16];
        ld16(c, 128 + cc, v);
        for (int i = 0; i < 16; ++i) { float t, s; tanh_s(v[i] + b2[cc + i], t, s); v[i] = t; }
        save16(H2, cc, v);
        put16<3>(buf, SP, r, cc, v);
      }
    phase(c, A.err, [&] { issue_block<3>(c.tmem + 256, buf, SP, 0, 8, img + I_W3, 0, 128, false, false); });
    float y = ((const float*)(img + I_B4))[0];
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float v[16], hv[16];
        ld16(c, 256 + cc, v);
        for (int i = 0; i < 16; ++i) {
          float t, s;
          tanh_s(v[i] + b3[cc + i], t, s);
          hv[i] = t;
          y = fmaf(w4[cc + i], t, y);
          v[i] = w4[cc + i] * s;  // delta3
        }
        save16(H3, cc, hv);
        put16<3>(buf, SP, r, cc, v);
      }
    // ---- input gradient ----
    phase(c, A.err, [&] { issue_block<3>(c.tmem + 384, buf, SP, 0, 8, img + I_W3, 0, 128, true, false); });
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float u[16], h[16];
        ld16(c, 384 + cc, u);
        save16(U2, cc, u);
        load16(H2, cc, h);
        for (int i = 0; i < 16; ++i) u[i] *= (1.0f - h[i]) * (1.0f + h[i]);
        put16<3>(buf, SP, r, cc, u);
      }
    phase(c, A.err, [&] { issue_block<3>(c.tmem + 0, buf, SP, 0, 8, img + I_W2, 0, 128, true, false); });
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float u[16], h[16];
        ld16(c, 0 + cc, u);
        save16(U1, cc, u);
        load16(H1, cc, h);
        for (int i = 0; i < 16; ++i) u[i] *= (1.0f - h[i]) * (1.0f + h[i]);
        put16<3>(buf, SP, r, cc, u);
      }
    phase(c, A.err, [&] { issue_block<3>(c.tmem + 128, buf, SP, 0, 8, img + I_W1, 0, 16, true, false); });
    // ---- loss: E = D y, dE/dR_k = dD_k y + D sum_i g_i J_ik ----
    float g[16], cvec[16], ry = 0.0f;
    for (int i = 0; i < 16; ++i) g[i] = cvec[i] = 0.0f;
    if (!c.dead) {
      ld16(c, 128, g);
      const float e = F.D * y - Et;
      float rg[3];
      for (int k = 0; k < 3; ++k) {
        float b = 0.0f;
        for (int i = 0; i < NINV; ++i) b = fmaf(g[i], F.J[i][k], b);
        rg[k] = F.dD[k] * y + F.D * b - Gt[k];
      }
      atomicAdd(&sums[3 * NH + 1], wE * e * e);
      atomicAdd(&sums[3 * NH + 2], wF * (rg[0] * rg[0] + rg[1] * rg[1] + rg[2] * rg[2]));
      ry = 2.0f * wE * e * F.D;
      for (int k = 0; k < 3; ++k) ry = fmaf(2.0f * wF * rg[k], F.dD[k], ry);
      for (int i = 0; i < NINV; ++i) {
        float a = 0.0f;
        for (int k = 0; k < 3; ++k) a = fmaf(2.0f * wF * rg[k] * F.D, F.J[i][k], a);
        cvec[i] = a;
      }
      atomicAdd(&sums[3 * NH + 0], ry);  // b4
      put16<1>(buf, SP, r, 0, cvec);
    }
    // ---- tangent forward along c (one-part operands) ----
    phase(c, A.err, [&] { issue_block<1>(c.tmem + 256, buf, SP, 0, 1, img + I_W1, 0, 128, false, false); });
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float z[16], h[16];
        ld16(c, 256 + cc, z);
        save16(Z1d, cc, z);
        load16(H1, cc, h);
        for (int i = 0; i < 16; ++i) z[i] *= (1.0f - h[i]) * (1.0f + h[i]);
        put16<1>(buf, SP, r, cc, z);
      }
    phase(c, A.err, [&] { issue_block<1>(c.tmem + 384, buf, SP, 0, 8, img + I_W2, 0, 128, false, false); });
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float z[16], h[16];
        ld16(c, 384 + cc, z);
        save16(Z2d, cc, z);
        load16(H2, cc, h);
        for (int i = 0; i < 16; ++i) z[i] *= (1.0f - h[i]) * (1.0f + h[i]);
        put16<1>(buf, SP, r, cc, z);
      }
    phase(c, A.err, [&] { issue_block<1>(c.tmem + 0, buf, SP, 0, 8, img + I_W3, 0, 128, false, false); });
    // ---- reverse, layer 3: hbar3 = ry w4 - 2 h3 zd3 w4, zbar3 = s3 hbar3 ----
    unsigned char* slot0 = buf;
    unsigned char* slot1 = buf + SP;
    unsigned char* slot2 = buf + 2 * SP;
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float zd[16], h3[16], h2[16], z2d[16], zb[16], d3[16], hd2[16];
        ld16(c, 0 + cc, zd);
        load16(H3, cc, h3);
        load16(H2, cc, h2);
        load16(Z2d, cc, z2d);
        for (int i = 0; i < 16; ++i) {
          const int j = cc + i;
          const float s3 = (1.0f - h3[i]) * (1.0f + h3[i]);
          const float hb = w4[j] * (ry - 2.0f * h3[i] * zd[i]);
          zb[i] = s3 * hb;
          d3[i] = w4[j] * s3;
          hd2[i] = (1.0f - h2[i]) * (1.0f + h2[i]) * z2d[i];
          atomicAdd(&sums[2 * NH + j], ry * h3[i] + s3 * zd[i]);  // w4
          atomicAdd(&sums[NH + j], zb[i]);                         // b3
        }
        put16<1>(slot0, SP, r, cc, zb);
        put_col(slot1, 128, r, cc, d3);
        put_col(slot2, 128, r, cc, hd2);
      }
    phase(c, A.err, [&] {
      issue_block<1>(c.tmem + 128, slot0, SP, 0, 8, img + I_W3, 0, 128, true, false);   // hbar2
      issue_block<1>(c.tmem + 256, slot1, SP, 0, 8, slot2, 0, 128, false, false);       // W3 grad, part 1
    });
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float zd[16], h3[16], h2[16], zb[16];
        ld16(c, 0 + cc, zd);
        load16(H3, cc, h3);
        load16(H2, cc, h2);
        for (int i = 0; i < 16; ++i) {
          const float s3 = (1.0f - h3[i]) * (1.0f + h3[i]);
          zb[i] = s3 * w4[cc + i] * (ry - 2.0f * h3[i] * zd[i]);
        }
        put_col(slot1, 128, r, cc, zb);
        put_col(slot2, 128, r, cc, h2);
      }
    phase(c, A.err, [&] { issue_block<1>(c.tmem + 256, slot1, SP, 0, 8, slot2, 0, 128, false, true); });
    if (!c.dead) flush_grad(c, 256, 128, A.grad + P_W3);
    // ---- reverse, layer 2: hbar2 += -2 h2 zd2 u2, zbar2 = s2 hbar2 ----
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float hb[16], h2[16], z2d[16], u2[16], h1[16], z1d[16], zb[16], d2[16], hd1[16];
        ld16(c, 128 + cc, hb);
        load16(H2, cc, h2); load16(Z2d, cc, z2d); load16(U2, cc, u2);
        load16(H1, cc, h1); load16(Z1d, cc, z1d);
        for (int i = 0; i < 16; ++i) {
          const float s2 = (1.0f - h2[i]) * (1.0f + h2[i]);
          zb[i] = s2 * (hb[i] - 2.0f * h2[i] * z2d[i] * u2[i]);
          d2[i] = s2 * u2[i];
          hd1[i] = (1.0f - h1[i]) * (1.0f + h1[i]) * z1d[i];
          atomicAdd(&sums[cc + i], zb[i]);  // b2
        }
        put16<1>(slot0, SP, r, cc, zb);
        put_col(slot1, 128, r, cc, d2);
        put_col(slot2, 128, r, cc, hd1);
      }
    phase(c, A.err, [&] {
      issue_block<1>(c.tmem + 384, slot0, SP, 0, 8, img + I_W2, 0, 128, true, false);   // hbar1
      issue_block<1>(c.tmem + 0, slot1, SP, 0, 8, slot2, 0, 128, false, false);         // W2 grad, part 1
    });
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float hb[16], h2[16], z2d[16], u2[16], h1[16], zb[16];
        ld16(c, 128 + cc, hb);
        load16(H2, cc, h2); load16(Z2d, cc, z2d); load16(U2, cc, u2); load16(H1, cc, h1);
        for (int i = 0; i < 16; ++i) {
          const float s2 = (1.0f - h2[i]) * (1.0f + h2[i]);
          zb[i] = s2 * (hb[i] - 2.0f * h2[i] * z2d[i] * u2[i]);
        }
        put_col(slot1, 128, r, cc, zb);
        put_col(slot2, 128, r, cc, h1);
      }
    phase(c, A.err, [&] { issue_block<1>(c.tmem + 0, slot1, SP, 0, 8, slot2, 0, 128, false, true); });
    if (!c.dead) flush_grad(c, 0, 128, A.grad + P_W2);
    // ---- reverse, layer 1: hbar1 += -2 h1 zd1 u1, zbar1 = s1 hbar1; W1 grad = d1^T c + zbar1^T f ----
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float h1[16], u1[16], d1[16];
        load16(H1, cc, h1); load16(U1, cc, u1);
        for (int i = 0; i < 16; ++i) d1[i] = (1.0f - h1[i]) * (1.0f + h1[i]) * u1[i];
        put_col(slot1, 128, r, cc, d1);
      }
    if (!c.dead) put_col(slot2, 16, r, 0, cvec);
    phase(c, A.err, [&] { issue_block<1>(c.tmem + 128, slot1, SP, 0, 8, slot2, 0, 16, false, false); });
    if (!c.dead)
      for (int cc = 0; cc < 128; cc += 16) {
        float hb[16], h1[16], z1d[16], u1[16], zb[16];
        ld16(c, 384 + cc, hb);
        load16(H1, cc, h1); load16(Z1d, cc, z1d); load16(U1, cc, u1);
        for (int i = 0; i < 16; ++i) {
          const float s1 = (1.0f - h1[i]) * (1.0f + h1[i]);
          zb[i] = s1 * (hb[i] - 2.0f * h1[i] * z1d[i] * u1[i]);
        }
        put_col(slot1, 128, r, cc, zb);
      }
    if (!c.dead) put_col(slot2, 16, r, 0, F.f);
    phase(c, A.err, [&] { issue_block<1>(c.tmem + 128, slot1, SP, 0, 8, slot2, 0, 16, false, true); });
    if (!c.dead) flush_grad(c, 128, 16, A.grad + P_W1);
    if (!c.dead && valid) atomicAdd(&sums[3 * NH + 3], 1.0f);
  }
  __syncthreads();
  if (!c.dead) {
    for (int j = threadIdx.x; j < NH; j += 128) {
      atomicAdd(A.grad + P_B2 + j, sums[j]);
      atomicAdd(A.grad + P_B3 + j, sums[NH + j]);
      atomicAdd(A.grad + P_W4 + j, sums[2 * NH + j]);
    }
    if (threadIdx.x == 0) {
      atomicAdd(A.grad + P_B4, sums[3 * NH]);
      atomicAdd(A.loss + 0, (double)sums[3 * NH + 1]);
      atomicAdd(A.loss + 1, (double)sums[3 * NH + 2]);
    }
  }
  cta_close(c);
}

// ------------------------------------------------------------------------------------------
// Training targets from the FP64 N3 surface: V3 = (the polynomial part - 457.4) kcal/mol and its
// gradient, in eV and eV/bohr (pes_n3's MEG variables and adjoint sweep).
// ------------------------------------------------------------------------------------------
__global__ void k_sur_targets(DevSys S, int64_t n, const double* __restrict__ R, cair_sur_sample* __restrict__ out) {
  const DevPes& P = S.pes[0];
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    double x[6], dx[6], vp, g[3];
    const double inv_ab = 1.0 / 1.5;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double d = R[3 * k + i] * CAIR_B_TO_ANG - 1.098;
      const double e = fexp(-d - (d * d) * inv_ab);
      const int j = i == 2 ? 3 : i;
      x[j] = e;
      dx[j] = (-((2.0 * d) * inv_ab) - 1.0) * e;
    }
    x[2] = x[4] = x[5] = 0.0;
    dx[2] = dx[4] = dx[5] = 0.0;
    CAIR_PIP_N3(x, dx, P.coef, 457.4, vp, g);
    cair_sur_sample s;
    for (int i = 0; i < 3; ++i) s.R[i] = R[3 * k + i];
    s.e = (float)((vp - 457.4) * CAIR_KCM_TO_HARTREE * kEvPerEh);
    for (int i = 0; i < 3; ++i) s.g[i] = (float)(g[i] * CAIR_KCM_TO_HARTREE * CAIR_B_TO_ANG * kEvPerEh);
    out[k] = s;
  }
}

// ------------------------------------------------------------------------------------------
// Persistent integrator on the surrogate (N3 UMN, NSteps = 3).  One CTA of 128 threads, one
// trajectory per thread, CTA-lockstep: every thread runs the same attempts (a thread without a
// trajectory runs them on a copy of a valid state and discards the result), so each right-hand
// side is one 128-row tile of the network.  At the first evaluation of every attempt the gate
// evaluates member B too: an attempt whose start lies outside the training range (where D matters)
// or where |D (yA - yB)| exceeds gate_ev runs all its evaluations on the FP64 surface.  The end
// check and the energy that judges conservation use the FP64 surface.
// ------------------------------------------------------------------------------------------
struct SurLane {
  Cta* c;
  int* err;
  const unsigned char* imgA;
  const unsigned char* imgB;
  unsigned char* buf;
  const SurConst* C;
  int ev;
  bool fb, active;
  unsigned long long n_fb, n_sur, n_rng, n_ens;
};

struct RhsSur {
  const DevSys& S;
  const DevPes& P;
  SurLane& z;
  __device__ RhsSur(const DevSys& s, const DevPes& p, SurLane& l) : S(s), P(p), z(l) {}
  __device__ __forceinline__ void operator()(const double (&y)[12], double (&yp)[12]) const {
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const int i0 = j % 3;
      double acc = 0.0 + S.Tpq[j + 9 * i0] * y[i0];
      acc = acc + S.Tpq[j + 9 * (i0 + 3)] * y[i0 + 3];
      yp[6 + j] = acc;
    }
    double Q[9], R[3], Ri[3];
#pragma unroll
    for (int i = 0; i < 6; ++i) Q[i] = y[6 + i];
    rp3(S, Q, R, Ri);
    const bool first = (z.ev % kNtot) == 0;
    bool gate_rng = false;
    float Dv = 0.0f;
    {
      Feat F;
      features(*z.C, R, F);
      gate_rng = !F.in_range;
      Dv = F.D;
      put16<3>(z.buf, Stage<2>::SPLIT, z.c->row, 0, F.f);
    }
    // a tile none of whose trajectories is in the three-body region (D below kDSkip, where V3_s is
    // below 1e-9 of the network's output) skips the network: V3_s = 0 there to that accuracy
    const bool net = __syncthreads_or(z.active && Dv > kDSkip) != 0;
    float yb = 0.0f, ya = 0.0f, g[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) g[i] = 0.0f;
    if (net) {
      if (first) {
        yb = member_value_call(*z.c, z.err, z.imgB, z.buf);
        Feat F;
        features(*z.C, R, F);
        put16<3>(z.buf, Stage<2>::SPLIT, z.c->row, 0, F.f);
      }
      ya = member_eval_call(*z.c, z.err, z.imgA, z.buf, g);
    }
    if (first) {
      // the gate, with hysteresis: a trajectory sent to the FP64 surface stays there until it leaves
      // the three-body region (D <= gate_dmin), so it meets the surrogate's fit error once
      const bool rng = gate_rng && Dv > z.C->gate_dmin;
      const bool ens = fabsf(Dv * (ya - yb)) > z.C->gate_ev;
      z.fb = z.active && ((z.fb && Dv > z.C->gate_dmin) || rng || ens || z.c->dead);
      if (z.active) {
        if (z.fb) ++z.n_fb; else ++z.n_sur;
        if (rng) ++z.n_rng;
        if (ens) ++z.n_ens;
      }
    }
    // the two-body part stays FP64 (in FP32 its force near the bond minimum would carry ~1e-6
    // relative rounding, which multiplies the attempts of an eps = 1e-8 integrator)
    double dvd[3], dVdR[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      double v;
      n2_umn<true>(R[i], v, dvd[i]);
    }
    if (z.fb) {
      double x[6], dx[6], vp, gp[3];
      const double inv_ab = 1.0 / 1.5;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const double d = R[i] * CAIR_B_TO_ANG - 1.098;
        const double e = fexp(-d - (d * d) * inv_ab);
        const int j = i == 2 ? 3 : i;
        x[j] = e;
        dx[j] = (-((2.0 * d) * inv_ab) - 1.0) * e;
      }
      x[2] = x[4] = x[5] = 0.0;
      dx[2] = dx[4] = dx[5] = 0.0;
      CAIR_PIP_N3(x, dx, P.coef, 457.4, vp, gp);
#pragma unroll
      for (int i = 0; i < 3; ++i) dVdR[i] = dvd[i] + gp[i] * CAIR_KCM_TO_HARTREE * CAIR_B_TO_ANG;
    } else {
      double v3, d3[3];
      v3_of(*z.C, R, ya, g, v3, d3);
#pragma unroll
      for (int i = 0; i < 3; ++i) dVdR[i] = dvd[i] + d3[i];
    }
    double m[6];
    trans_to_cart_3(S, Ri, Q, dVdR, m);
#pragma unroll
    for (int i = 0; i < 6; ++i) yp[i] = -m[i];
    ++z.ev;
  }
};

struct SurRunArgs {
  SurConst C;
  const unsigned char* imgA;
  const unsigned char* imgB;
  unsigned long long* counters;  // fallback attempts, surrogate attempts, range-gated, ensemble-gated
  int* err;
};

__global__ void __launch_bounds__(NT2, 1) k_integrate_sur(DevSys S, IntegrateArgs A, SurRunArgs Z) {
  constexpr int NE = 12, NP = 3;
  extern __shared__ __align__(1024) unsigned char sm[];
  copy_image(sm + SM_IMG_A, Z.imgA);
  copy_image(sm + SM_IMG_B, Z.imgB);
  Cta c;
  cta_open(c, (uint64_t*)(sm + SM_BAR2), (uint32_t*)(sm + SM_BAR2 + 16), (float*)(sm + SM_Y2));
  if (c.part == 1) {
    // The second thread of each row holds no trajectory: it meets the owners' barriers one for one
    // (the loop test, then per right-hand side the tile's network test and, when the network runs,
    // member B at an attempt's first evaluation and member A), doing its half of each epilogue.
    float g[16];
    int ev = 0;
#pragma unroll 1
    for (;;) {
      if (__syncthreads_or(c.dead) || !__syncthreads_or(0)) break;
#pragma unroll 1
      for (int e = 0; e < S.ncall * kNtot; ++e, ++ev) {
        const bool first = (ev % kNtot) == 0;
        if (__syncthreads_or(0)) {
          if (first) member_value_call(c, Z.err, sm + SM_IMG_B, sm + SM_BUF2);
          member_eval_call(c, Z.err, sm + SM_IMG_A, sm + SM_BUF2, g);
        }
      }
    }
    cta_close(c);
    return;
  }
  const DevPes& P = S.pes[0];
  SurLane z{&c, Z.err, sm + SM_IMG_A, sm + SM_IMG_B, sm + SM_BUF2, &Z.C, 0, false, false, 0, 0, 0, 0};
  RhsSur f(S, P, z);
  unsigned long long c_att = 0, c_acc = 0, c_rej = 0;
  const bool incstp = S.incstp != 0;
  const int ncall = S.ncall;
  unsigned long long k = 0;
  bool active = false;
  int irej = 0, iste = 0, irej0 = 0, iste0 = 0;
  int64_t att = 0;
  double y[NE], x = 0.0, h = 1.0, smax = 0.0, smin = 0.0, H = 0.0;
#pragma unroll
  for (int i = 0; i < NE; ++i) y[i] = A.paq[i];  // a valid state for a thread that never has a trajectory
  auto take = [&]() {
    const unsigned long long q = atomicAdd(A.queue, 1ull);
    active = q < (unsigned long long)A.n;
    if (!active) return;
    k = A.order ? (unsigned long long)A.order[q] : q;
#pragma unroll
    for (int i = 0; i < NE; ++i) y[i] = A.paq[NE * k + i];
    x = A.t[k]; h = A.dt[k]; smax = A.smax[k]; smin = A.smin[k]; H = 0.0;
    irej = irej0 = A.irej[k];
    iste = iste0 = A.iste[k];
    att = 0;
    z.fb = false;
  };
  take();
#pragma unroll 1
  for (;;) {
    if (__syncthreads_or(c.dead) || !__syncthreads_or(active)) break;
    z.active = active;
    int bad = 0;
#pragma unroll 1
    for (int a = 0; a < ncall; ++a)
      bad |= bs_attempt<NE, 3>(f, y, x, h, A.erra + NE * k, S.relax, incstp, smax, smin, irej, iste);
    if (active && !c.dead) {
      att += ncall;
      double rpi[NP];
      H = hamiltonian<CAIR_PES_N3_UMN>(S, P, y, rpi);
      bool conv = x > S.tmax;
#pragma unroll
      for (int p = 0; p < NP; ++p) conv = conv || (rpi[p] < S.rpimax);
      if (bad || conv || att >= A.max_attempts) {
#pragma unroll
        for (int i = 0; i < NE; ++i) A.paq[NE * k + i] = y[i];
        A.t[k] = x;
        A.dt[k] = h;
        A.H[k] = H;
        A.smax[k] = smax;
        A.smin[k] = smin;
        A.irej[k] = irej;
        A.iste[k] = iste;
        A.status[k] = bad ? CAIR_TRAJ_NONFINITE : (conv ? CAIR_TRAJ_DONE : CAIR_TRAJ_ATTEMPT_CAP);
        c_att += att;
        c_acc += iste - iste0;
        c_rej += irej - irej0;
        take();
      }
    }
  }
  if (c_att) {
    atomicAdd(A.counters + 0, c_att);
    atomicAdd(A.counters + 1, c_acc);
    atomicAdd(A.counters + 2, c_rej);
    atomicAdd(A.counters + 3, c_att * (unsigned long long)kNtot);
    atomicAdd(A.counters + 4, c_att / (unsigned long long)(ncall > 0 ? ncall : 1));
  }
  if (z.n_fb) atomicAdd(Z.counters + 0, z.n_fb);
  if (z.n_sur) atomicAdd(Z.counters + 1, z.n_sur);
  if (z.n_rng) atomicAdd(Z.counters + 2, z.n_rng);
  if (z.n_ens) atomicAdd(Z.counters + 3, z.n_ens);
  cta_close(c);
}

}  // namespace sur
}  // namespace cair

// ==========================================================================================
// Host side
// ==========================================================================================
using namespace cair;
using namespace cair::sur;

struct cair_surrogate {
  int device = 0;
  int nsm = 0;
  SurConst C{};
  float* d_param[2] = {nullptr, nullptr};  // FP32 parameters of each member
  float* d_grad[2] = {nullptr, nullptr};
  float* d_m[2] = {nullptr, nullptr};
  float* d_v[2] = {nullptr, nullptr};
  unsigned char* d_img[2] = {nullptr, nullptr};
  int adam_t[2] = {0, 0};
  double* d_loss = nullptr;         // [2]
  float* d_scratch = nullptr;       // training per-row vectors
  size_t scratch_bytes = 0;
  unsigned long long* d_ctr = nullptr;  // [4] gate counters
  int* d_err = nullptr;
  std::string err;
};

namespace {

int sfail(cair_surrogate* s, int code, const std::string& m) {
  if (s) s->err = m;
  return code;
}

#define SUR_TRY(s, call)                                                                   \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return sfail(s, CAIR_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int check_err_flag(cair_surrogate* s, cudaStream_t st) {
  int e = 0;
  SUR_TRY(s, cudaMemcpyAsync(&e, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  SUR_TRY(s, cudaStreamSynchronize(st));
  if (e) {
    cudaMemsetAsync(s->d_err, 0, sizeof(int), st);
    return sfail(s, CAIR_ETIMEOUT, "a tensor-core completion wait ran out (the kernel stopped and freed its TMEM)");
  }
  return 0;
}

std::once_flag g_attr_once;
void set_attrs() {
  cudaFuncSetAttribute(k_sur_eval, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM2);
  cudaFuncSetAttribute(k_integrate_sur, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM2);
  cudaFuncSetAttribute(k_sur_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_T);
}

}  // namespace

namespace cair {

int sur_integrate_launch(cair_surrogate* s, int nsm, cudaStream_t st, const DevSys& S, const IntegrateArgs& A) {
  std::call_once(g_attr_once, set_attrs);
  int64_t g = std::min<int64_t>(nsm, (A.n + 127) / 128);
  if (g < 1) g = 1;
  SurRunArgs Z{s->C, s->d_img[0], s->d_img[1], s->d_ctr, s->d_err};
  k_integrate_sur<<<(int)g, NT2, SMEM2, st>>>(S, A, Z);
  return cudaGetLastError() == cudaSuccess ? 0 : CAIR_ECUDA;
}

int sur_targets_launch(const DevSys& S, int nsm, cudaStream_t st, int64_t n, const double* R, cair_sur_sample* out) {
  int64_t g = std::min<int64_t>((int64_t)nsm * 8, (n + 127) / 128);
  if (g < 1) g = 1;
  k_sur_targets<<<(int)g, 128, 0, st>>>(S, n, R, out);
  return cudaGetLastError() == cudaSuccess ? 0 : CAIR_ECUDA;
}

const char* sur_last_error(const cair_surrogate* s) { return s ? s->err.c_str() : ""; }

}  // namespace cair

extern "C" {

int cair_sur_create(cair_surrogate** out, int device) {
  if (!out) return CAIR_EINVAL;
  *out = nullptr;
  auto* s = new cair_surrogate();
  s->device = device;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete s;
    return CAIR_ECUDA;
  }
  cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, device);
  int cc_major = 0, cc_minor = 0;
  cudaDeviceGetAttribute(&cc_major, cudaDevAttrComputeCapabilityMajor, device);
  cudaDeviceGetAttribute(&cc_minor, cudaDevAttrComputeCapabilityMinor, device);
  bool ok = cc_major == 10 && cc_minor == 3;
  for (int m = 0; ok && m < 2; ++m) {
    ok = cudaMalloc(&s->d_param[m], NPARAM * 4) == cudaSuccess && cudaMalloc(&s->d_grad[m], NPARAM * 4) == cudaSuccess &&
         cudaMalloc(&s->d_m[m], NPARAM * 4) == cudaSuccess && cudaMalloc(&s->d_v[m], NPARAM * 4) == cudaSuccess &&
         cudaMalloc(&s->d_img[m], IMAGE) == cudaSuccess;
    if (ok) {
      cudaMemset(s->d_param[m], 0, NPARAM * 4);
      cudaMemset(s->d_grad[m], 0, NPARAM * 4);
      cudaMemset(s->d_m[m], 0, NPARAM * 4);
      cudaMemset(s->d_v[m], 0, NPARAM * 4);
      cudaMemset(s->d_img[m], 0, IMAGE);
    }
  }
  ok = ok && cudaMalloc(&s->d_loss, 16) == cudaSuccess && cudaMalloc(&s->d_ctr, 32) == cudaSuccess &&
       cudaMalloc(&s->d_err, 4) == cudaSuccess;
  if (ok) {
    cudaMemset(s->d_ctr, 0, 32);
    cudaMemset(s->d_err, 0, 4);
    ok = cudaDeviceSynchronize() == cudaSuccess;
  }
  if (!ok) {
    cair_sur_destroy(s);
    return cc_major == 10 ? CAIR_ECUDA : CAIR_EUNSUPPORTED;
  }
  s->C.sigma_d = 2e-3f;
  s->C.gate_ev = 1e-3f;
  s->C.gate_dmin = 1e-3f;
  for (int i = 0; i < NINV; ++i) {
    s->C.mu[i] = 0.0f;
    s->C.isd[i] = 1.0f;
    s->C.fmin[i] = -1e30f;
    s->C.fmax[i] = 1e30f;
  }
  *out = s;
  return 0;
}

void cair_sur_destroy(cair_surrogate* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  for (int m = 0; m < 2; ++m) {
    cudaFree(s->d_param[m]);
    cudaFree(s->d_grad[m]);
    cudaFree(s->d_m[m]);
    cudaFree(s->d_v[m]);
    cudaFree(s->d_img[m]);
  }
  cudaFree(s->d_loss);
  cudaFree(s->d_scratch);
  cudaFree(s->d_ctr);
  cudaFree(s->d_err);
  delete s;
}

const char* cair_sur_last_error(const cair_surrogate* s) { return s ? s->err.c_str() : "null surrogate"; }

int cair_sur_set_consts(cair_surrogate* s, const cair_sur_consts* c) {
  if (!s || !c) return CAIR_EINVAL;
  if (!(c->sigma_d > 0.0f) || !(c->gate_ev > 0.0f)) return sfail(s, CAIR_EINVAL, "cair_sur_set_consts: bad constants");
  for (int i = 0; i < NINV; ++i) {
    s->C.mu[i] = c->mu[i];
    s->C.isd[i] = c->isd[i];
    s->C.fmin[i] = c->fmin[i];
    s->C.fmax[i] = c->fmax[i];
  }
  s->C.sigma_d = c->sigma_d;
  s->C.gate_ev = c->gate_ev;
  s->C.gate_dmin = c->gate_dmin;
  return 0;
}

int cair_sur_get_consts(const cair_surrogate* s, cair_sur_consts* c) {
  if (!s || !c) return CAIR_EINVAL;
  for (int i = 0; i < NINV; ++i) {
    c->mu[i] = s->C.mu[i];
    c->isd[i] = s->C.isd[i];
    c->fmin[i] = s->C.fmin[i];
    c->fmax[i] = s->C.fmax[i];
  }
  c->sigma_d = s->C.sigma_d;
  c->gate_ev = s->C.gate_ev;
  c->gate_dmin = s->C.gate_dmin;
  return 0;
}

int cair_sur_set_params(cair_surrogate* s, int member, const float* params) {
  if (!s || member < 0 || member > 1 || !params) return CAIR_EINVAL;
  SUR_TRY(s, cudaSetDevice(s->device));
  SUR_TRY(s, cudaMemcpy(s->d_param[member], params, NPARAM * 4, cudaMemcpyHostToDevice));
  SUR_TRY(s, cudaMemset(s->d_m[member], 0, NPARAM * 4));
  SUR_TRY(s, cudaMemset(s->d_v[member], 0, NPARAM * 4));
  SUR_TRY(s, cudaMemset(s->d_grad[member], 0, NPARAM * 4));
  s->adam_t[member] = 0;
  k_sur_image<<<(NPARAM + 255) / 256, 256>>>(s->d_param[member], s->d_img[member]);
  SUR_TRY(s, cudaGetLastError());
  SUR_TRY(s, cudaDeviceSynchronize());
  return 0;
}

int cair_sur_get_params(cair_surrogate* s, int member, float* params) {
  if (!s || member < 0 || member > 1 || !params) return CAIR_EINVAL;
  SUR_TRY(s, cudaSetDevice(s->device));
  SUR_TRY(s, cudaMemcpy(params, s->d_param[member], NPARAM * 4, cudaMemcpyDeviceToHost));
  return 0;
}

int cair_sur_nparam(void) { return NPARAM; }

int cair_sur_eval_dev(cair_surrogate* s, int64_t n, const double* R, float* ya, float* yb, float* g, double* v3,
                      double* dv3, void* stream) {
  if (!s || n < 0 || (n > 0 && (!R || !ya || !yb || !g || !v3 || !dv3))) return CAIR_EINVAL;
  if (n == 0) return 0;
  std::call_once(g_attr_once, set_attrs);
  cudaStream_t st = (cudaStream_t)stream;
  int64_t grid = std::min<int64_t>(s->nsm, (n + 127) / 128);
  k_sur_eval<<<(int)grid, NT2, SMEM2, st>>>(s->C, s->d_img[0], s->d_img[1], n, R, ya, yb, g, v3, dv3, s->d_err);
  SUR_TRY(s, cudaGetLastError());
  return check_err_flag(s, st);
}

int cair_sur_grad_dev(cair_surrogate* s, int member, int64_t nbatch, const cair_sur_sample* samples,
                      const int64_t* idx, float w_e, float w_f, void* stream) {
  if (!s || member < 0 || member > 1 || nbatch < 1 || !samples || !idx) return CAIR_EINVAL;
  std::call_once(g_attr_once, set_attrs);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t grid = std::min<int64_t>(s->nsm, (nbatch + 127) / 128);
  const size_t need = (size_t)grid * NVEC * 128 * 128 * 4;
  if (need > s->scratch_bytes) {
    cudaFree(s->d_scratch);
    s->d_scratch = nullptr;
    s->scratch_bytes = 0;
    SUR_TRY(s, cudaMalloc(&s->d_scratch, need));
    s->scratch_bytes = need;
  }
  TrainArgs A{s->C, s->d_img[member], samples, idx, nbatch, w_e / (float)nbatch, w_f / (float)nbatch,
              s->d_grad[member], s->d_loss, s->d_scratch, s->d_err};
  k_sur_grad<<<(int)grid, 128, SMEM_T, st>>>(A);
  SUR_TRY(s, cudaGetLastError());
  return 0;
}

int cair_sur_get_grad(cair_surrogate* s, int member, float* grad) {
  if (!s || member < 0 || member > 1 || !grad) return CAIR_EINVAL;
  SUR_TRY(s, cudaDeviceSynchronize());
  if (int e = check_err_flag(s, 0)) return e;
  SUR_TRY(s, cudaMemcpy(grad, s->d_grad[member], NPARAM * 4, cudaMemcpyDeviceToHost));
  return 0;
}

int cair_sur_adam_dev(cair_surrogate* s, int member, float lr, void* stream) {
  if (!s || member < 0 || member > 1 || !(lr > 0.0f)) return CAIR_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  const int t = ++s->adam_t[member];
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f / (1.0f - powf(b1, (float)t)), c2 = 1.0f / (1.0f - powf(b2, (float)t));
  k_sur_adam<<<(NPARAM + 255) / 256, 256, 0, st>>>(s->d_param[member], s->d_grad[member], s->d_m[member],
                                                   s->d_v[member], s->d_img[member], lr, b1, b2, 1e-8f, c1, c2);
  SUR_TRY(s, cudaGetLastError());
  return 0;
}

int cair_sur_take_loss(cair_surrogate* s, double* loss, void* stream) {
  if (!s || !loss) return CAIR_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  SUR_TRY(s, cudaMemcpyAsync(loss, s->d_loss, 16, cudaMemcpyDeviceToHost, st));
  SUR_TRY(s, cudaMemsetAsync(s->d_loss, 0, 16, st));
  if (int e = check_err_flag(s, st)) return e;
  return 0;
}

int cair_sur_counters(cair_surrogate* s, int64_t* out, int reset) {
  if (!s || !out) return CAIR_EINVAL;
  unsigned long long c[4];
  SUR_TRY(s, cudaDeviceSynchronize());
  SUR_TRY(s, cudaMemcpy(c, s->d_ctr, 32, cudaMemcpyDeviceToHost));
  for (int i = 0; i < 4; ++i) out[i] = (int64_t)c[i];
  if (reset) SUR_TRY(s, cudaMemset(s->d_ctr, 0, 32));
  return 0;
}

}  // extern "C"
