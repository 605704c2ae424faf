// Lane-parallel right-hand sides for the warp integrator (cair_warp.cu): the interpreter of the
// generated level programs of generated/warp_prog.h (written by gen/gen_warp.py from the same
// formulas as the surfaces of cair_device.cuh) and the constant loading.  Used by the kernel, where
// the 16 lanes of a half-warp execute the instructions of a level, and by the host test harness,
// which runs the same programs one instruction after the other.
#pragma once
#include "cair_device.cuh"
#include "generated/warp_prog.h"

namespace cair {

enum { WK_SOP = 0, WK_EXP = 1, WK_RSQRT = 2, WK_RECIP = 3, WK_TANH = 4 };
enum { WS_LIT = 0, WS_TPQ = 1, WS_MMIMN = 2, WS_O2AB = 3, WS_COEF = 4, WS_PES = 5 };

// One program: nlev levels of W records of 8 words (lane l of level L executes record W L + l, W the
// model's group width): w0 = active << 31 | kind << 28 | nterm << 24 | signed << 23 | term signs << 20
// (nterm and `signed` uniform over the level), w1 = result byte offset, w2..w7 = byte offsets of the
// factors a0, b0, a1, b1, a2, b2.
struct WProg {
  const unsigned* rec;
  int nlev;
};

// A surface model's programs over one slot layout: constants [0, nconst) (surface / system values,
// literals and the hoisted values the const program computes), the NE inputs, then the values.
struct WModel {
  int nslot, nconst;
  const unsigned char* csrc;
  const unsigned short* cidx;
  const double* clit;
  WProg cprog, grad, energy;
  const unsigned short *gin, *gout, *ein, *eout;  // grad: y -> dy/dt; energy: y -> (H, 1/R_p)
};

#define CAIR_WPROG(key, KEY, name, NAME) \
  WProg { wp_##key##_##name##_rec, WP_##KEY##_##NAME##_NLEV }
#define CAIR_WMODEL(key, KEY)                                                                                  \
  WModel {                                                                                                     \
    WP_##KEY##_NSLOT, WP_##KEY##_NCONST, wp_##key##_csrc, wp_##key##_cidx, wp_##key##_clit,                   \
        CAIR_WPROG(key, KEY, cprog, CPROG), CAIR_WPROG(key, KEY, grad, GRAD), CAIR_WPROG(key, KEY, energy, ENERGY), \
        wp_##key##_grad_in, wp_##key##_grad_out, wp_##key##_energy_in, wp_##key##_energy_out                   \
  }

// Surface models that have programs (the UMN surfaces, O3 NN and the O3 BNN samples), and the diatomic
// their programs evaluate.
__host__ __device__ constexpr bool warp_model_built(int model) {
  return model == CAIR_PES_O3_UMN || model == CAIR_PES_N3_UMN || model == CAIR_PES_O4_UMN ||
         model == CAIR_PES_N4_UMN || model == CAIR_PES_O3_NN || model == CAIR_PES_O3_BNN;
}
__host__ __device__ constexpr int warp_model_diat(int model) {
  return (model == CAIR_PES_N3_UMN || model == CAIR_PES_N4_UMN) ? CAIR_DIAT_N2_UMN_FORN4 : CAIR_DIAT_O2_UMN;
}

// Per model: lanes of the group that evaluates one right-hand side (16: a half-warp, so the two
// halves of a warp run different midpoint sequences; 32: the whole warp, NE = 18 equations),
// slots of a group, and the levels of the grad and energy programs.
#define CAIR_WPICK(MODEL, FIELD)                                                                      \
  (MODEL == CAIR_PES_O3_UMN ? WP_O3_UMN_##FIELD : MODEL == CAIR_PES_N3_UMN ? WP_N3_UMN_##FIELD           \
   : MODEL == CAIR_PES_O4_UMN ? WP_O4_UMN_##FIELD : MODEL == CAIR_PES_N4_UMN ? WP_N4_UMN_##FIELD         \
   : MODEL == CAIR_PES_O3_NN ? WP_O3_NN_##FIELD : WP_O3_BNN_##FIELD)
template <int MODEL>
struct WCfg {
  static constexpr int W = CAIR_WPICK(MODEL, LANES);
  static constexpr int NSLOT = CAIR_WPICK(MODEL, NSLOT);
  static constexpr int NLEV = CAIR_WPICK(MODEL, GRAD_NLEV) + CAIR_WPICK(MODEL, ENERGY_NLEV);
  static constexpr int NG = 32 / W;  // groups per warp
};

template <int MODEL>
__device__ __forceinline__ WModel wmodel() {
  if (MODEL == CAIR_PES_O3_UMN) return CAIR_WMODEL(o3_umn, O3_UMN);
  if (MODEL == CAIR_PES_N3_UMN) return CAIR_WMODEL(n3_umn, N3_UMN);
  if (MODEL == CAIR_PES_O4_UMN) return CAIR_WMODEL(o4_umn, O4_UMN);
  if (MODEL == CAIR_PES_N4_UMN) return CAIR_WMODEL(n4_umn, N4_UMN);
  if (MODEL == CAIR_PES_O3_NN) return CAIR_WMODEL(o3_nn, O3_NN);
  return CAIR_WMODEL(o3_bnn, O3_BNN);
}

// Value of constant slot i for surface P.  Hoisted slots (source 255) are the const program's.
__device__ __forceinline__ double wp_const(const WModel& m, const DevSys& S, const DevPes& P, int i) {
  const int idx = m.cidx[i];
  switch (m.csrc[i]) {
    case WS_LIT: return m.clit[i];
    case WS_TPQ: return S.Tpq[idx];
    case WS_MMIMN: return S.mMiMn[idx];
    case WS_O2AB: return S.o2_ab[idx];
    case WS_COEF: return P.coef[idx];
    case WS_PES:
      return idx == 0 ? P.a : idx == 1 ? P.ab : idx == 2 ? P.ra : idx == 3 ? P.rb : idx == 4 ? P.inv_a : P.inv_ab;
    default: return 0.0;
  }
}

// One record: a sum of up to three products (a multiply, then fused multiply-adds in term order; a
// term's sign, where the generator could not fold it into a constant factor, goes on the first
// factor's sign bit with an integer XOR, off the FP64 pipe), the table-driven exponential, a
// reciprocal square root, a reciprocal or tanh.  The term count and whether signs are present are the same
// for every lane of a level, so its branches are uniform.
__device__ __forceinline__ double wp_ld(const char* sb, unsigned off) {
  return *reinterpret_cast<const double*>(sb + off);
}
__device__ __forceinline__ double wp_flip(double a, unsigned meta, int j) {
  return __hiloint2double(__double2hiint(a) ^ (int)((meta << (11 - j)) & 0x80000000u), __double2loint(a));
}

__device__ __forceinline__ double wp_eval(uint4 c0, uint4 c1, const char* sb) {
  const unsigned meta = c0.x, kind = (meta >> 28) & 7u;
  if (kind == WK_SOP) {
    const unsigned nt = (meta >> 24) & 3u;
    const bool sg = (meta >> 23) & 1u;
    double a0 = wp_ld(sb, c0.z);
    const double b0 = wp_ld(sb, c0.w);
    if (sg) a0 = wp_flip(a0, meta, 0);
    double r = a0 * b0;
    if (nt > 1) {
      double a1 = wp_ld(sb, c1.x);
      const double b1 = wp_ld(sb, c1.y);
      if (sg) a1 = wp_flip(a1, meta, 1);
      r = fma(a1, b1, r);
    }
    if (nt > 2) {
      double a2 = wp_ld(sb, c1.z);
      const double b2 = wp_ld(sb, c1.w);
      if (sg) a2 = wp_flip(a2, meta, 2);
      r = fma(a2, b2, r);
    }
    return r;
  }
  const double x = wp_ld(sb, c0.z);
  if (kind == WK_EXP) return fexp(x);
  if (kind == WK_RSQRT) return rsqrt(x);
  if (kind == WK_TANH) return ftanh(x);
  return 1.0 / x;
}

// A whole program by one thread (the host harness), record after record.
__device__ __forceinline__ void wp_run_serial(const WProg& p, int width, double* s) {
  char* sb = reinterpret_cast<char*>(s);
  for (int r = 0; r < width * p.nlev; ++r) {
    const unsigned* w = p.rec + 8 * r;
    if (w[0] >> 31) {
      const uint4 c0 = {w[0], w[1], w[2], w[3]}, c1 = {w[4], w[5], w[6], w[7]};
      *reinterpret_cast<double*>(sb + w[1]) = wp_eval(c0, c1, sb);
    }
  }
}

}  // namespace cair
