// Lane-parallel right-hand sides for the warp integrator (cair_warp.cu): the interpreter of the
// generated level programs of generated/warp_prog.h (written by gen/gen_warp.py from the same
// formulas as the surfaces of cair_device.cuh) and the constant loading.  Used by the kernel, where
// the 16 lanes of a half-warp execute the instructions of a level, and by the host test harness,
// which runs the same programs one instruction after the other.
#pragma once
#include "cair_device.cuh"
#include "generated/warp_prog.h"

namespace cair {

enum { WK_SOP = 0, WK_EXP = 1, WK_RSQRT = 2, WK_RECIP = 3 };
enum { WS_LIT = 0, WS_TPQ = 1, WS_MMIMN = 2, WS_O2AB = 3, WS_COEF = 4, WS_PES = 5 };

// One program: nlev levels of 16 records of 4 words (lane l of level L executes record 16 L + l):
// w0 = active << 31 | kind << 28 | nterm << 24 | out slot; w1..w3 = terms a | sign << 15 | b << 16.
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

// Surface models that have programs (3-atom UMN surfaces).
__host__ __device__ constexpr bool warp_model_built(int model) {
  return model == CAIR_PES_O3_UMN || model == CAIR_PES_N3_UMN;
}

template <int MODEL>
__device__ __forceinline__ WModel wmodel() {
  if (MODEL == CAIR_PES_O3_UMN) return CAIR_WMODEL(o3_umn, O3_UMN);
  return CAIR_WMODEL(n3_umn, N3_UMN);
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

// One record: a sum of up to three signed products (a multiply, then fused multiply-adds in term
// order), the table-driven exponential, a reciprocal square root or a reciprocal.  The operands of
// every term are loaded before the arithmetic starts.
// The term's sign goes on the first factor's sign bit with an integer XOR: a per-lane select of -a
// would cost an FP64 instruction (a negation on the FP64 pipe) per term.
__device__ __forceinline__ double wp_signed(double a, unsigned w) {
  return __hiloint2double(__double2hiint(a) ^ (int)((w & 0x8000u) << 16), __double2loint(a));
}

__device__ __forceinline__ double wp_eval(unsigned w0, unsigned w1, unsigned w2, unsigned w3, const double* s) {
  const unsigned kind = (w0 >> 28) & 3u;
  if (kind == WK_SOP) {
    const unsigned nt = (w0 >> 24) & 3u;
    const double a0 = wp_signed(s[w1 & 0x7fffu], w1), b0 = s[w1 >> 16];
    const double a1 = wp_signed(s[w2 & 0x7fffu], w2), b1 = s[w2 >> 16];
    const double a2 = wp_signed(s[w3 & 0x7fffu], w3), b2 = s[w3 >> 16];
    double r = a0 * b0;
    if (nt > 1) r = fma(a1, b1, r);
    if (nt > 2) r = fma(a2, b2, r);
    return r;
  }
  const double x = s[w1 & 0x7fffu];
  if (kind == WK_EXP) return fexp(x);
  if (kind == WK_RSQRT) return rsqrt(x);
  return 1.0 / x;
}

// A whole program by one thread (the host harness), record after record.
__device__ __forceinline__ void wp_run_serial(const WProg& p, double* s) {
  for (int r = 0; r < 16 * p.nlev; ++r) {
    const unsigned* w = p.rec + 4 * r;
    if (w[0] >> 31) s[w[0] & 0xffffu] = wp_eval(w[0], w[1], w[2], w[3], s);
  }
}

}  // namespace cair
