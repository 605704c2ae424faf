// Learned surrogate of the N3 UMN three-body term on the tensor cores.
//
// The N3 UMN surface (N3_UMN_PES_Class.F90:332-382) is V = sum_i V_N2(R_i) + (457.4 + sum_k C_k B_k(x))
// kcal/mol, x_i = exp(-d_i - d_i^2 / 1.5) the MEG variables of the three pair distances (d_i in
// angstrom from 1.098).  The polynomial part minus its constant is the three-body term V3: it has
// no one-variable terms, so it vanishes whenever two of the x_i do, i.e. in every asymptotic
// channel.  The surrogate keeps the FP64 diatomics and replaces V3 by
//
//     V3_s(R) = D(x) * y(f(x)),   D = 1 - exp(-(x1 x2 + x1 x3 + x2 x3) / sigma_D),
//
// y a 16 -> 128 -> 128 -> 128 -> 1 tanh network on f: the ten S3-orbit sums of the x_i of degree
// 1..4, normalised, five zeros and a constant 1 (the first layer's bias).  D makes V3_s exactly 0
// where V3 is, so the surrogate's energy is the FP64 surface's at the start and the end of a
// collision.
//
// Precision.  Hidden-layer weights are BF16; each activation row entering an MMA is split exactly
// into three BF16 parts (cair_tc.cuh split3), so the three MMAs per layer give W x a to FP32
// accumulation; tanh, the output layer (FP32 weights) and everything per row run in FP32.  A
// Bulirsch-Stoer attempt at eps = 1e-8 tolerates relative force noise of about 1e-7; plain BF16
// activations (1e-3) or a two-part split (1e-5) would shrink its steps many times over.
//
// One CTA of 128 threads evaluates 128 rows: thread r owns row r, which is TMEM lane r of every
// M = 128 accumulator, so its epilogue (bias, tanh, the next operand's split, the output dot
// product and the backward products) never leaves the thread.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

#include "cair_tc.cuh"

namespace cair {
namespace sur {

constexpr int NF = 16;      // network inputs: 10 invariants, 5 zeros, 1 constant
constexpr int NINV = 10;    // S3-orbit sums of degree 1..4
constexpr int NH = 128;     // hidden width
constexpr double kEvPerEh = 27.211386245988;
constexpr double kKcalToEh = 0.159360144e-2;   // the reference's kcm_To_Hartree

// FP32 parameter vector (Adam's variable): W1[128][16] (column 15 = first-layer bias), W2, W3
// [128][128] (out, in), b2, b3, w4 [128], b4.
constexpr int P_W1 = 0;
constexpr int P_W2 = P_W1 + NH * NF;
constexpr int P_W3 = P_W2 + NH * NH;
constexpr int P_B2 = P_W3 + NH * NH;
constexpr int P_B3 = P_B2 + NH;
constexpr int P_W4 = P_B3 + NH;
constexpr int P_B4 = P_W4 + NH;
constexpr int NPARAM = P_B4 + 1;

// Shared-memory image of one network (built from the parameters by k_sur_image): BF16 W1, W2, W3
// in the K-major operand layout (rows = outputs, K = inputs), then FP32 b2, b3, w4, b4.
constexpr int I_W1 = 0;
constexpr int I_W2 = I_W1 + NH * NF * 2;
constexpr int I_W3 = I_W2 + NH * NH * 2;
constexpr int I_B2 = I_W3 + NH * NH * 2;
constexpr int I_B3 = I_B2 + NH * 4;
constexpr int I_W4 = I_B3 + NH * 4;
constexpr int I_B4 = I_W4 + NH * 4;
constexpr int IMAGE = I_B4 + 16;

// Descriptor byte offsets of the operand layouts (cair_tc.cuh kmaj_off with rows = 128).  In the
// no-swizzle mode the leading-dimension offset is the step between core matrices along K and the
// stride-dimension offset the step along M/N, for K-major and MN-major operands alike (checked on
// the GPU by cair_sur_probe.cu): K-major operands step 2048 B along K and 128 B along M/N; a weight
// image read as the MN-major operand of the backward products steps 128 B along K (its outputs)
// and 2048 B along N (its inputs).
constexpr uint32_t KM_LBO = 2048, KM_SBO = 128;
constexpr uint32_t MN_LBO = 128, MN_SBO = 2048;

// Surrogate constants shared by the ensemble (set at training time, read by every kernel).
struct SurConst {
  float mu[NINV], isd[NINV];    // feature normalisation f = (raw - mu) * isd
  float fmin[NINV], fmax[NINV]; // normalised feature range of the training set (the range gate)
  float sigma_d;                // damping scale of D
  float gate_ev;                // ensemble disagreement |D (yA - yB)| that sends an attempt to FP64 [eV]
  float gate_dmin;              // the range gate applies where D exceeds this
  float pad;
};

// ------------------------------------------------------------------------------------------
// Features
// ------------------------------------------------------------------------------------------
struct Feat {
  float f[NF];          // network input
  float J[NINV][3];     // d f_i / d R_k (normalised), k over the three pair distances
  float D, dD[3];       // damping and dD / dR_k
  bool in_range;        // every feature inside the training range
};

__device__ __forceinline__ void features(const SurConst& C, const double (&R)[3], Feat& F) {
  float x[3], dx[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float d = (float)(R[i] * 0.52917721092 - 1.098);
    x[i] = __expf(-d - d * d * (1.0f / 1.5f));
    dx[i] = (-1.0f - d * (2.0f / 1.5f)) * x[i] * 0.52917721092f;
  }
  const float s1 = x[0] + x[1] + x[2];
  const float x2[3] = {x[0] * x[0], x[1] * x[1], x[2] * x[2]};
  const float x3[3] = {x2[0] * x[0], x2[1] * x[1], x2[2] * x[2]};
  const float s2 = x2[0] + x2[1] + x2[2];
  const float s3 = x3[0] + x3[1] + x3[2];
  const float p11 = x[0] * x[1] + x[0] * x[2] + x[1] * x[2];
  const float p111 = x[0] * x[1] * x[2];
  float raw[NINV];
  raw[0] = s1;
  raw[1] = s2;
  raw[2] = p11;
  raw[3] = s3;
  raw[4] = s2 * s1 - s3;                                   // sum_{i != j} x_i^2 x_j
  raw[5] = p111;
  raw[6] = x2[0] * x2[0] + x2[1] * x2[1] + x2[2] * x2[2];  // sum x_i^4
  raw[7] = s3 * s1 - raw[6];                               // sum_{i != j} x_i^3 x_j
  raw[8] = x2[0] * x2[1] + x2[0] * x2[2] + x2[1] * x2[2];  // sum_{i < j} x_i^2 x_j^2
  raw[9] = p111 * s1;
  // d raw / d x_k
  float dr[NINV][3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float o = s1 - x[k];                      // sum of the other two
    const float po = x[(k + 1) % 3] * x[(k + 2) % 3];  // product of the other two
    dr[0][k] = 1.0f;
    dr[1][k] = 2.0f * x[k];
    dr[2][k] = o;
    dr[3][k] = 3.0f * x2[k];
    dr[4][k] = 2.0f * x[k] * o + (s2 - x2[k]);
    dr[5][k] = po;
    dr[6][k] = 4.0f * x3[k];
    dr[7][k] = 3.0f * x2[k] * o + (s3 - x3[k]);
    dr[8][k] = 2.0f * x[k] * (s2 - x2[k]);
    dr[9][k] = po * s1 + p111;
  }
  bool ok = true;
#pragma unroll
  for (int i = 0; i < NINV; ++i) {
    const float v = (raw[i] - C.mu[i]) * C.isd[i];
    F.f[i] = v;
    ok = ok && v >= C.fmin[i] && v <= C.fmax[i];
#pragma unroll
    for (int k = 0; k < 3; ++k) F.J[i][k] = dr[i][k] * C.isd[i] * dx[k];
  }
#pragma unroll
  for (int i = NINV; i < NF - 1; ++i) F.f[i] = 0.0f;
  F.f[NF - 1] = 1.0f;
  F.in_range = ok;
  const float e = __expf(-p11 / C.sigma_d);
  F.D = 1.0f - e;
#pragma unroll
  for (int k = 0; k < 3; ++k) F.dD[k] = e / C.sigma_d * dr[2][k] * dx[k];
}

// tanh(x) = 1 - q, q = 2 / (exp(2x) + 1), and s = 1 - tanh(x)^2 = q (2 - q): exp and the division
// on the special-function unit, each within 2 ulp, so h and s carry FP32-level rounding (absolute
// for s where the unit saturates); exp(2x) beyond 2^126 gives q = 0, h = 1, s = 0.
__device__ __forceinline__ void tanh_s(float x, float& h, float& s) {
  const float q = __fdividef(2.0f, __expf(2.0f * x) + 1.0f);
  h = 1.0f - q;
  s = q * (2.0f - q);
}

// ------------------------------------------------------------------------------------------
// CTA engine: 128 threads, one TMEM allocation of 512 columns, one mbarrier.
// ------------------------------------------------------------------------------------------
// A CTA of 128 or 256 threads works on one 128-row tile.  Thread t serves row t % 128 (TMEM lane
// t % 128, which warps w and w + 4 can both read); with 256 threads the two threads of a row split
// each epilogue's columns, part 0 (t < 128, the row's owner) taking the first half.
struct Cta {
  uint32_t tmem;       // TMEM base address
  uint64_t* bar;       // MMA completion barrier
  uint32_t phase;      // parity of the next completion
  int tid;
  int row;             // tile row of this thread
  int part, parts;     // this thread's share of a row's columns, of `parts`
  float* yshare;       // shared memory [128]: the second part's output partial sums
  uint32_t lane_off;   // this warp's TMEM lane quarter, as an address offset
  bool dead;           // a completion wait ran out: the CTA stops issuing work
};

// Operand rows: thread r writes 16 consecutive K values of its row r into a K-major operand of 128
// rows (core matrices of 8 rows x 8 K), as NS exact BF16 parts stored split_bytes apart.
// A pair of FP32 values as a packed BF16x2 (round to nearest even, low half = a) and its value back.
__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  const __nv_bfloat162 p = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&p);
}
__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

template <int NS>
__device__ __forceinline__ void put16(unsigned char* buf, uint32_t split_bytes, int r, int k0, const float (&v)[16]) {
  uint32_t w[NS][8];
#pragma unroll
  for (int i = 0; i < 16; i += 2) {
    // the exact three-part split of cair_tc.cuh split3, two values per conversion
    float a = v[i], b = v[i + 1];
    const uint32_t p0 = pack_bf16x2(a, b);
    w[0][i / 2] = p0;
    if (NS == 3) {
      a -= bf16_lo(p0);
      b -= bf16_hi(p0);
      const uint32_t p1 = pack_bf16x2(a, b);
      a -= bf16_lo(p1);
      b -= bf16_hi(p1);
      w[1 % NS][i / 2] = p1;
      w[2 % NS][i / 2] = pack_bf16x2(a, b);
    }
  }
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    unsigned char* b = buf + s * split_bytes;
    *(uint4*)(b + tc::kmaj_off(r, k0, 128)) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
    *(uint4*)(b + tc::kmaj_off(r, k0 + 8, 128)) = make_uint4(w[s][4], w[s][5], w[s][6], w[s][7]);
  }
}

// One MMA phase: every thread publishes its shared-memory writes, thread 0 issues, everyone waits
// for completion.  A wait that runs out marks the thread's warp dead at once (so the warp's
// .sync.aligned TMEM loads stay converged), the whole CTA at the barrier of the next phase, and
// sets *err; a dead CTA issues nothing more.
template <class Issue>
__device__ __forceinline__ void phase(Cta& c, int* err, Issue issue) {
  tc::fence_smem_async();
  tc::fence_before_sync();
  c.dead = __syncthreads_or(c.dead) != 0;
  if (c.dead) return;
  if (c.tid == 0) {
    tc::fence_after_sync();
    issue();
    tc::mma_commit(c.bar);
  }
  const bool ok = tc::mbar_wait(c.bar, c.phase);
  c.dead = __any_sync(0xffffffffu, !ok) != 0;
  if (!ok) atomicExch(err, 1);
  c.phase ^= 1u;
  tc::fence_after_sync();
}

// MMAs of one operand block: D[cols] (+)= sum over NS parts and ksteps of A x B.  A: K-major split
// buffer (parts split_bytes apart), K-steps of 16 from a_k0; B: a weight image, K-major (forward)
// or MN-major (backward, transposed use), its K offset b_k0.
template <int NS>
__device__ __forceinline__ void issue_block(uint32_t d_tmem, const unsigned char* abuf, uint32_t split_bytes, int a_k0,
                                            int nk, const unsigned char* wimg, int b_k0, int N, bool b_mn,
                                            bool accumulate) {
  const uint32_t idesc = tc::idesc_bf16(128, N, b_mn);
  const uint32_t a0 = tc::smem_u32(abuf), w0 = tc::smem_u32(wimg);
#pragma unroll 1
  for (int s = 0; s < NS; ++s)
#pragma unroll 1
    for (int ks = 0; ks < nk; ++ks) {
      const uint64_t ad = tc::sdesc(a0 + s * split_bytes + (uint32_t)((a_k0 / 8 + 2 * ks) * 2048), KM_LBO, KM_SBO);
      const int kb = b_k0 / 8 + 2 * ks;  // first K core-matrix group of this step in the weight image
      const uint64_t bd = b_mn ? tc::sdesc(w0 + (uint32_t)(kb * 128), MN_LBO, MN_SBO)
                               : tc::sdesc(w0 + (uint32_t)(kb * N * 16), KM_LBO == 2048 ? (uint32_t)(N * 16) : 128u,
                                           KM_LBO == 2048 ? 128u : (uint32_t)(N * 16));
      tc::mma_bf16(d_tmem, ad, bd, idesc, (accumulate || s > 0 || ks > 0) ? 1u : 0u);
    }
}

__device__ __forceinline__ void ld16(const Cta& c, uint32_t col, float (&v)[16]) {
  tc::tmem_ld16(c.tmem + c.lane_off + col, v);
}

}  // namespace sur
}  // namespace cair
