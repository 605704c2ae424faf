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

// One program: nlev levels (kind | count << 8, first node), nodes (out | nterm << 16, first term or
// operand slot), terms (a | sign << 15 | b << 16).
struct WProg {
  const unsigned* lev;
  const unsigned* node;
  const unsigned* term;
  int nlev, nnode, nterm;  // nnode, nterm: array lengths in words
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

#define CAIR_WPROG(key, name)                                                                                  \
  WProg {                                                                                                      \
    wp_##key##_##name##_lev, wp_##key##_##name##_node, wp_##key##_##name##_term,                              \
        (int)(sizeof(wp_##key##_##name##_lev) / sizeof(unsigned) / 2),                                        \
        (int)(sizeof(wp_##key##_##name##_node) / sizeof(unsigned)),                                           \
        (int)(sizeof(wp_##key##_##name##_term) / sizeof(unsigned))                                            \
  }
#define CAIR_WMODEL(key, KEY)                                                                                  \
  WModel {                                                                                                     \
    WP_##KEY##_NSLOT, WP_##KEY##_NCONST, wp_##key##_csrc, wp_##key##_cidx, wp_##key##_clit,                   \
        CAIR_WPROG(key, cprog), CAIR_WPROG(key, grad), CAIR_WPROG(key, energy), wp_##key##_grad_in,           \
        wp_##key##_grad_out, wp_##key##_energy_in, wp_##key##_energy_out                                       \
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

// One instruction: a sum of signed products (a multiply, then fused multiply-adds in term order),
// the table-driven exponential, a reciprocal square root or a reciprocal.
__device__ __forceinline__ double wp_eval(unsigned kind, unsigned nx, unsigned ny, const unsigned* __restrict__ term,
                                          const double* s) {
  if (kind == WK_SOP) {
    const unsigned nt = nx >> 16;
    const unsigned* t = term + ny;
    unsigned tm = t[0];
    double a = s[tm & 0x7fffu];
    double r = ((tm & 0x8000u) ? -a : a) * s[tm >> 16];
    for (unsigned j = 1; j < nt; ++j) {
      tm = t[j];
      a = s[tm & 0x7fffu];
      r = fma((tm & 0x8000u) ? -a : a, s[tm >> 16], r);
    }
    return r;
  }
  const double x = s[ny];
  if (kind == WK_EXP) return fexp(x);
  if (kind == WK_RSQRT) return rsqrt(x);
  return 1.0 / x;
}

// The instructions of level L that lane gl of `width` lanes executes (gl, gl + width, ...).
__device__ __forceinline__ void wp_level(const WProg& p, int L, double* s, int gl, int width) {
  const unsigned lv = p.lev[2 * L], base = p.lev[2 * L + 1];
  const unsigned kind = lv & 0xffu, cnt = lv >> 8;
  for (unsigned i = (unsigned)gl; i < cnt; i += (unsigned)width) {
    const unsigned nx = p.node[2 * (base + i)], ny = p.node[2 * (base + i) + 1];
    s[nx & 0xffffu] = wp_eval(kind, nx, ny, p.term, s);
  }
}

// A whole program by one thread (the host harness).
__device__ __forceinline__ void wp_run_serial(const WProg& p, double* s) {
  for (int L = 0; L < p.nlev; ++L) wp_level(p, L, s, 0, 1);
}

}  // namespace cair
