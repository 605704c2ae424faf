// Device-side building blocks of the GB300 trajectory path: diatomic potentials, MEG
// variables, the UMN surfaces with analytic gradients, pair distances, Hamilton's
// equations and the Bulirsch-Stoer attempt.  FP64 throughout; one thread owns one
// trajectory and keeps its phase-space state in registers.
#pragma once
#include <cstdint>
#include "../../include/cair_gpu.h"

#define CAIR_B_TO_ANG 0.52917721092
#define CAIR_KCM_TO_HARTREE 0.159360144e-2
#define CAIR_KCMANG_TO_HARTB 0.843297564e-3

namespace cair {

struct DevPes {
  int32_t model;
  int32_t ncoef;
  const double* coef;   // device copy of C(1:ncoef)
  double a, ab, ra, rb; // MEG parameters
  double inv_a;         // One/This%a, evaluated once on the host
  double inv_ab;
};

struct DevSys {
  int32_t natoms, nv, ne, npairs, npes, nsteps, ncall, incstp, diat;
  double mass[4];
  double mMiMn[3];
  double Tpq[81];       // column-major (i,j) -> [i + 9 j]
  double Tqp[81];
  double eps;           // "Error control parameter" (SetErrorFactor)
  double dt0;
  double relax, rmax, tmax, rpimax;
  double o2_ab[8];      // alpha * beta**k          (O2_UMN Ev2gm2 exponent factors)
  double o2_cd[8];      // 2 * a(k) * alpha * beta**k (O2_UMN Ev2gm2_Grad factors)
  DevPes pes[CAIR_MAX_PES];
};

// ------------------------------------------------------------------------------------------
// Exponential on the FP64 pipe with 10 operations: Tang's table-driven method (ACM TOMS
// 15(2), 144-157, 1989) with 64 subintervals.  x = (64 k + j) ln2/64 + r, |r| <= ln2/128;
// exp(x) = 2^k 2^(j/64) (1 + p(r)), p the degree-5 Taylor polynomial of exp(r) - 1
// (truncation r^6/720 < 3.6e-17, 0.16 ulp).  The result is within about one ulp; |x| >= 707
// (not met on this path's surfaces) goes to the CUDA library.
// ------------------------------------------------------------------------------------------
}  // namespace cair
#include "generated/exp_table.h"
namespace cair {
__device__ static const double kExpTab[64] = {
#define X(i) kCairExp2Table[i]
    X(0),  X(1),  X(2),  X(3),  X(4),  X(5),  X(6),  X(7),  X(8),  X(9),  X(10), X(11), X(12),
    X(13), X(14), X(15), X(16), X(17), X(18), X(19), X(20), X(21), X(22), X(23), X(24), X(25),
    X(26), X(27), X(28), X(29), X(30), X(31), X(32), X(33), X(34), X(35), X(36), X(37), X(38),
    X(39), X(40), X(41), X(42), X(43), X(44), X(45), X(46), X(47), X(48), X(49), X(50), X(51),
    X(52), X(53), X(54), X(55), X(56), X(57), X(58), X(59), X(60), X(61), X(62), X(63)
#undef X
};

__device__ __forceinline__ double fexp(double x) {
#ifdef CAIR_PARITY_MATH
  return exp(x);  // the parity build (cair_parity.cu): CUDA's correctly rounded-to-within-1-ulp exp
#endif
  // |x| < 707 (and not NaN) read off the high word with an integer compare: an FP64 comparison
  // would take a slot of the FP64 pipe
  if ((__double2hiint(x) & 0x7fffffff) >= 0x40861800) return exp(x);
  const double shifter = 6755399441055744.0;  // 1.5 * 2^52: the sum rounds to an integer
  const double t = fma(x, CAIR_EXP_INV_L, shifter);
  const double N = t - shifter;
  const int n = __double2loint(t);
  double r = fma(-N, CAIR_EXP_L1, x);
  r = fma(-N, CAIR_EXP_L2, r);
  double p = fma(r, 1.0 / 120.0, 1.0 / 24.0);
  p = fma(p, r, 1.0 / 6.0);
  p = fma(p, r, 0.5);
  p = fma(p, r, 1.0);
  p = p * r;
  const double T = __ldg(kExpTab + (n & 63));
  const double y = fma(T, p, T);
  return __hiloint2double(__double2hiint(y) + ((n >> 6) << 20), __double2loint(y));
}

// ------------------------------------------------------------------------------------------
// Diatomic potentials
// ------------------------------------------------------------------------------------------
__device__ __constant__ static const double kO2A[8] = {
    -1.488979427684798e3, 1.881435846488955e4, -1.053475425838226e5, 2.755135591229064e5,
    -4.277588997761775e5, 4.404104009614092e5, -2.946204062950765e5, 1.176861219078620e5};

// O2 UMN dispersion (O2_UMN_DiatomicPotential_Class.F90 edisp / edisp_Grad)
template <bool GRAD>
__device__ __forceinline__ void o2_disp(double rb, double& vd, double& dvd) {
  const double r2r4 = 2.59361680, rs6 = 0.5299, rs8 = 2.20, c6 = 12.8;
  const double c8step = 3.0 * c6 * (r2r4 * r2r4);
  double tmp = sqrt(c8step / c6);
  double ss = rs6 * tmp + rs8;
  double s2 = ss * ss, s3 = s2 * ss, s6 = s3 * s3, s4 = s2 * s2, s8 = s4 * s4;
  double r2 = rb * rb, r3 = r2 * rb, r4 = r2 * r2, r6 = r3 * r3, r8 = r4 * r4;
  double d6 = r6 + s6, d8 = r8 + s8;
  // one division for both denominators: 1/d6 = d8/(d6 d8), 1/d8 = d6/(d6 d8)
  double q = 1.0 / (d6 * d8);
  double i6 = d8 * q, i8 = d6 * q;
  double e6 = c6 * i6, e8 = c8step * i8;
  vd = -e6 - 2.0 * e8;
  if (GRAD) {
    double r5 = r4 * rb, r7 = r4 * r3;
    double e6dr = c6 * (-6.0 * r5) * (i6 * i6);
    double e8dr = c8step * (-8.0 * r7) * (i8 * i8);
    dvd = (-e6dr - 2.0 * e8dr) * (1.0 / CAIR_B_TO_ANG);
  }
}

// O2 UMN (Ev2gm2 / Ev2gm2_Grad): V [Eh] and dV/dR [Eh/bohr] for R in bohr
template <bool GRAD>
__device__ __forceinline__ void o2_umn(const DevSys& S, double r, double& v, double& dv) {
  double rang = r * CAIR_B_TO_ANG;
  double r2 = rang * rang;
  double vv = 0.0, dd = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    double e = fexp(-(S.o2_ab[k] * r2));
    vv = vv + kO2A[k] * e;
    if (GRAD) dd = dd - S.o2_cd[k] * rang * e;
  }
  vv = vv * 1.e-3;
  double vd, dvd = 0.0;
  o2_disp<GRAD>(r, vd, dvd);
  v = vv + vd;
  if (GRAD) dv = (dd * 1.e-3 + dvd) * CAIR_B_TO_ANG;
}

// N2 UMN_ForN4 (Ev2gm2 / Ev2gm2_Grad): V [Eh], dV/dR [Eh/bohr]
template <bool GRAD>
__device__ __forceinline__ void n2_umn(double r, double& v, double& dv) {
  const double cs0 = 2.70963254293, cs1 = 1.32620177271e-1, cs2 = 2.96757048793e-1,
               cs3 = 1.97112432229e-1, cs4 = -5.02002309588e-1, cs5 = 3.80734244606e-1,
               cs6 = 1.21001628750;
  const double de = 228.7, red = 1.098, red4 = 1.4534810048;
  double rang = r * CAIR_B_TO_ANG;
  double r3 = (rang * rang) * rang;
  double r4 = r3 * rang;
  double ts = r4 + red4;
  double its = 1.0 / ts;
  double y = (r4 - red4) * its;
  double y2 = y * y, y3 = y2 * y, y4 = y2 * y2, y5 = y3 * y2, y6 = y3 * y3;
  double fy = cs0 + cs1 * y + cs2 * y2 + cs3 * y3 + cs4 * y4 + cs5 * y5 + cs6 * y6;
  double u = fexp(-(fy * (rang - red)));
  double minu = 1.0 - u;
  v = (de * (minu * minu) - de) * CAIR_KCM_TO_HARTREE + 0.0;
  if (GRAD) {
    double dfdy = cs1 + 2.0 * cs2 * y + 3.0 * cs3 * y2 + 4.0 * cs4 * y3 + 5.0 * cs5 * y4 + 6.0 * cs6 * y5;
    double dydr = 8.0 * r3 * red4 * (its * its);
    double dfdr = dfdy * dydr;
    double dvk = 2.0 * de * minu * u * (dfdr * (rang - red) + fy);
    dv = dvk * CAIR_KCM_TO_HARTREE * CAIR_B_TO_ANG;
  }
}

// The pair term of the N4 UMN PIPNN surface and the N2 UMN_PIPNN_ForN4 diatomic: Ev2gm2 (and
// Ev2gm2_Grad) with the D3(BJ) dispersion of an N-N pair (iz = 7, r2r4 = 2.71175247, C6 = 19.7,
// rs6 = 0.5299, rs8 = 2.20), N4_UMN_PIPNN_PES_Class.F90:1471-1748 and
// N2_UMN_PIPNN_ForN4_DiatomicPotential_Class.F90:116-365.  r [Ang] -> kcal/mol, kcal/mol/Ang.
template <bool GRAD>
__device__ __forceinline__ void n2p_ev2gm2(double r, double& v, double& dv) {
  const double as0 = 2.7475450369759, as1 = 0.218868498415108, as2 = 0.248885765371433,
               as3 = -0.229295466336412, as4 = -0.653389048592838, as5 = 1.03611964035396,
               as6 = 1.71287482791961;
  const double de = 225.213, re = 1.098, re4 = (re * re) * (re * re);
  const double r2 = r * r, r3 = r2 * r, r4 = r2 * r2;
  const double y = (r4 - re4) / (r4 + re4);
  const double y2 = y * y, y3 = y * y2, y4 = y2 * y2, y5 = y2 * y3, y6 = y3 * y3;
  const double fy = as0 + as1 * y + as2 * y2 + as3 * y3 + as4 * y4 + as5 * y5 + as6 * y6;
  const double u = fexp(-(fy * (r - re)));
  // edisp on the distance in bohr
  const double c6 = 19.7, c8 = ((3.0 * c6) * 2.71175247) * 2.71175247;
  const double sd = 0.5299 * sqrt(c8 / c6) + 2.20;
  const double s2 = sd * sd, s3 = s2 * sd, s4 = s2 * s2, s6 = s3 * s3, s8 = s4 * s4;
  const double rb = r / CAIR_B_TO_ANG;
  const double b2 = rb * rb, b3 = b2 * rb, b4 = b2 * b2, b6 = b3 * b3, b8 = b4 * b4;
  const double d6 = b6 + s6, d8 = b8 + s8;
  const double e6 = c6 / d6, e8 = c8 / d8;
  const double h2k = 1.0 / CAIR_KCM_TO_HARTREE;
  v = ((de * (1.0 - u)) * (1.0 - u) - de) + (0.0 + (-e6 - 2.0 * e8) * h2k);
  if (GRAD) {
    const double dfdy = as1 + 2.0 * as2 * y + 3.0 * as3 * y2 + 4.0 * as4 * y3 + 5.0 * as5 * y4 + 6.0 * as6 * y5;
    const double rr = r4 + re4;
    const double dfdr = dfdy * (((8.0 * r3) * re4) / (rr * rr));
    const double e6dr = c6 * (-(6.0 * (b3 * b2))) / (d6 * d6);
    const double e8dr = c8 * (-(8.0 * (b4 * b3))) / (d8 * d8);
    dv = (((2.0 * de) * (1.0 - u)) * u) * (dfdr * (r - re) + fy) + ((-e6dr - 2.0 * e8dr) * h2k) / CAIR_B_TO_ANG;
  }
}

// N2 UMN_PIPNN_ForN4 (DiatomicPotential_N2 / Compute_Vd_dVd_N2): V [Eh], dV/dR [Eh/bohr]
template <bool GRAD>
__device__ __forceinline__ void n2_pipnn(double r, double& v, double& dv) {
  double vk, dk = 0.0;
  n2p_ev2gm2<GRAD>(r * CAIR_B_TO_ANG, vk, dk);
  v = vk * CAIR_KCM_TO_HARTREE + 0.0;
  if (GRAD) dv = dk * CAIR_KCM_TO_HARTREE * CAIR_B_TO_ANG;
}

// The diatomic of the surfaces' own pair terms (O2 UMN, N2 UMN_ForN4)
template <bool GRAD>
__device__ __forceinline__ void diat(const DevSys& S, double r, double& v, double& dv) {
  if (S.diat == CAIR_DIAT_O2_UMN) o2_umn<GRAD>(S, r, v, dv);
  else n2_umn<GRAD>(r, v, dv);
}

// The system's diatomic for initial conditions and final states: any of the three.  The UMN_PIPNN_ForN4
// one comes with the N4 UMN PIPNN surface only, whose pair term is its own, so the surfaces' kernels
// keep the two-way choice above.
template <bool GRAD>
__device__ __forceinline__ void diat_any(const DevSys& S, double r, double& v, double& dv) {
  if (S.diat == CAIR_DIAT_N2_UMN_PIPNN_FORN4) n2_pipnn<GRAD>(r, v, dv);
  else diat<GRAD>(S, r, v, dv);
}

}  // namespace cair

#include "generated/pip_n3.cuh"
#include "generated/pip_o3.cuh"
#include "generated/pip_o4.cuh"
#include "generated/pip_n4.cuh"
#include "generated/pip_n4nn.cuh"
// gradient of the PIP part: reverse mode (adjoint sweep) unless CAIR_PIP_FORWARD selects the
// forward mode, whose operation order is the reference's
#ifdef CAIR_PIP_FORWARD
#define CAIR_PIP_O3 pip_o3_eval
#define CAIR_PIP_N3 pip_n3_eval
#else
#define CAIR_PIP_O3 pip_o3_eval_rev
#define CAIR_PIP_N3 pip_n3_eval_rev
#endif

namespace cair {

// ------------------------------------------------------------------------------------------
// TransToCart (PES_Class.F90:252-360, implementation 2)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void trans_to_cart_3(const DevSys& S, const double* Ri, const double* Q,
                                                const double* dVdR, double* m) {
  double d0 = dVdR[0] * Ri[0], d1 = dVdR[1] * Ri[1], d2 = dVdR[2] * Ri[2];
  double m1 = S.mMiMn[0], m2 = S.mMiMn[1];
  double a1 = (1.0 - m1) * d1, b1 = m1 * d2, a2 = m2 * d1, b2 = (1.0 - m2) * d2;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double X0 = Q[c] - Q[3 + c], X1 = Q[c] - Q[6 + c], X2 = Q[3 + c] - Q[6 + c];
    m[c] = d0 * X0 + a1 * X1 - b1 * X2;
    m[3 + c] = -(d0 * X0) - a2 * X1 + b2 * X2;
  }
}

__device__ __forceinline__ void trans_to_cart_4(const DevSys& S, const double* Ri, const double* Q,
                                                const double* dVdR, double* m) {
  double d[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) d[i] = dVdR[i] * Ri[i];
  double m1 = S.mMiMn[0], m2 = S.mMiMn[1], m3 = S.mMiMn[2];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double X0 = Q[c] - Q[3 + c], X1 = Q[c] - Q[6 + c], X2 = Q[c] - Q[9 + c];
    double X3 = Q[3 + c] - Q[6 + c], X4 = Q[3 + c] - Q[9 + c], X5 = Q[6 + c] - Q[9 + c];
    m[c] = d[0] * X0 + d[1] * X1 + (1.0 - m1) * d[2] * X2 - m1 * d[4] * X4 - m1 * d[5] * X5;
    m[3 + c] = -(d[0] * X0) - m2 * d[2] * X2 + d[3] * X3 + (1.0 - m2) * d[4] * X4 - m2 * d[5] * X5;
    m[6 + c] = -(d[1] * X1) - m3 * d[2] * X2 - d[3] * X3 - m3 * d[4] * X4 + (1.0 - m3) * d[5] * X5;
  }
}

// ------------------------------------------------------------------------------------------
// Surfaces.  GRAD = false gives PES%Potential (energy only).
// ------------------------------------------------------------------------------------------
// O3 UMN (Compute_O3_UMN_PES_1d, O3_UMN_PES_Class.F90:259-326)
template <bool GRAD>
__device__ __forceinline__ void pes_o3(const DevSys& S, const DevPes& P, const double* R, const double* Ri,
                                       const double* Q, double& V, double* dVdR, double* dVdQ) {
  double x[3], dx[3], vd[3], dvd[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double rang = R[i] * CAIR_B_TO_ANG;
    double d1 = rang - P.ra, d2 = rang - P.rb;
    double e = fexp(-(d1 * P.inv_a) - (d2 * d2) * P.inv_ab);
    x[i] = e;
    if (GRAD) dx[i] = (-((2.0 * d2) * P.inv_ab) - P.inv_a) * e;
    diat<GRAD>(S, R[i], vd[i], dvd[i]);
  }
  double vdiat = (vd[0] + vd[1]) + vd[2];
  double vp;
  const double* __restrict__ C = P.coef;
  if (GRAD) {
    double g[3];
    CAIR_PIP_O3(x, dx, C, 0.0, vp, g);
    V = (vp * CAIR_KCM_TO_HARTREE) + vdiat;
#pragma unroll
    for (int i = 0; i < 3; ++i) dVdR[i] = g[i] * CAIR_KCMANG_TO_HARTB + dvd[i];
    trans_to_cart_3(S, Ri, Q, dVdR, dVdQ);
  } else {
    pip_o3_value(x, C, 0.0, vp);
    V = (vp * CAIR_KCM_TO_HARTREE) + vdiat;
  }
}

// N3 UMN (Compute_N3_UMN_PES_1d, N3_UMN_PES_Class.F90:332-382, on the N4 PIP with the
// three pinned 10^3-bohr pairs contributing exact zeros)
template <bool GRAD>
__device__ __forceinline__ void pes_n3(const DevSys& S, const DevPes& P, const double* R, const double* Ri,
                                       const double* Q, double& V, double* dVdR, double* dVdQ) {
  double x[6], dx[6], vd[3], dvd[3];
  const double inv_ab = 1.0 / 1.5;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    double d = R[i] * CAIR_B_TO_ANG - 1.098;
    double e = fexp(-d - (d * d) * inv_ab);
    int j = i == 2 ? 3 : i;  // RTemp(1), RTemp(2), RTemp(4)
    x[j] = e;
    if (GRAD) dx[j] = (-((2.0 * d) * inv_ab) - 1.0) * e;
    diat<GRAD>(S, R[i], vd[i], dvd[i]);
  }
  x[2] = x[4] = x[5] = 0.0;
  dx[2] = dx[4] = dx[5] = 0.0;
  double vdiat = ((0.0 + vd[0]) + vd[1]) + vd[2];
  double vp;
  const double* __restrict__ C = P.coef;
  if (GRAD) {
    double g[3];
    CAIR_PIP_N3(x, dx, C, 457.4, vp, g);
    V = vdiat + (vp + 0.0) * CAIR_KCM_TO_HARTREE;
#pragma unroll
    for (int i = 0; i < 3; ++i) dVdR[i] = dvd[i] + g[i] * CAIR_KCM_TO_HARTREE * CAIR_B_TO_ANG;
    trans_to_cart_3(S, Ri, Q, dVdR, dVdQ);
  } else {
    pip_n3_value(x, C, 457.4, vp);
    V = vdiat + (vp + 0.0) * CAIR_KCM_TO_HARTREE;
  }
}

// tanh from the table-driven exponential: tanh|x| = 1 - 2 / (exp(2|x|) + 1), sign restored.
// Absolute error within a few ulp of 1 (the relative error grows as |x| -> 0, where the network
// only needs the absolute value); |x| > 20 returns +-1 (1 - tanh(20) < 2^-113).  Inline, so the
// network keeps its activations in registers instead of spilling them around library calls.
__device__ __forceinline__ double ftanh(double x) {
  const double a = fabs(x);
  const double t = a > 20.0 ? 1.0 : 1.0 - 2.0 / (fexp(2.0 * a) + 1.0);
  return copysign(t, x);
}

// O3 NN (O3_NN_PES_Class.F90).  Device layout of the coefficients, repacked from the reference's
// arrays at cair_create with the hidden layers zero-padded to 20 and 10 neurons (a padded neuron has
// z = 0, tanh(z) = 0 and zero outgoing weights, so it adds exact zeros):
#define CAIR_NN_H1 20
#define CAIR_NN_H2 10
#define CAIR_NN_LAM 0      // Lambda
#define CAIR_NN_RE 1       // re
#define CAIR_NN_MEAN 2     // Scaling_MEAN(3)
#define CAIR_NN_SD 5       // Scaling_SD(3)
#define CAIR_NN_YSC 8      // y_Scaling
#define CAIR_NN_B3 9       // b3
#define CAIR_NN_W1 10      // W1(6, 20): [i + 6 j]
#define CAIR_NN_W1P 130    // W1 storage read as 3 x NHL1 (Potential's dgemm): [l + 3 j]
#define CAIR_NN_B1 190     // b1(20)
#define CAIR_NN_W2 210     // W2(20, 10): [j + 20 k]
#define CAIR_NN_B2 410     // b2(10)
#define CAIR_NN_W3 420     // W3(10)
#define CAIR_NN_NCOEF 430
#define CAIR_BNN_NOISE 430 // BNN: the sample's Noise
#define CAIR_BNN_NCOEF 431
#define CAIR_EV_TO_HARTREE (1.0 / 27.2113839712790)

// GRAD: Compute_O3_NN_PES_1d (357-477): six features G of p = exp(-Lambda (R - re)), network
// 6 -> tanh(20) -> tanh(10) -> 1, gradient by one adjoint sweep (dV/dG) contracted with dG/dR
// (the reference builds dG/dR first and carries the three directions forward).
// !GRAD: O3_NN_Potential_From_R (250-297): three scaled features on W1's storage read as 3 x NHL1.
// BNN (BNN_PES_Class.F90: Compute_BNN_PES_1d 565-640, BNN_Potential_From_R 395-442): the same two
// networks with the output v taken through VExp = exp(v + Noise): V = (VExp - y_Scaling) eV + the
// diatomics, dV/dR = VExp dv/dR eV + the diatomics'.
template <bool GRAD, bool BNN = false>
__device__ __forceinline__ void pes_o3nn(const DevSys& S, const DevPes& P, const double* R, const double* Ri,
                                         const double* Q, double& V, double* dVdR, double* dVdQ) {
  const double* __restrict__ c = P.coef;
  const double lam = c[CAIR_NN_LAM], re = c[CAIR_NN_RE];
  double p[3], vd[3], dvd[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    p[i] = fexp(-(lam * (R[i] - re)));
    diat<true>(S, R[i], vd[i], dvd[i]);  // Compute_Vd_dVd in both routines
  }
  const double vdiat = (vd[0] + vd[1]) + vd[2];
  const double gvp[3] = {p[0] * p[1], p[1] * p[2], p[2] * p[0]};
  if (GRAD) {
    const double gvs[3] = {p[1] + p[2], p[2] + p[0], p[0] + p[1]};
    const double gprod = gvp[0] * p[2];
    double G[6];
    G[0] = (gvp[0] + gvp[1]) + gvp[2];
    G[1] = gprod;
    const double gc0 = gvp[0] * p[0], gc1 = gvp[0] * p[1], gc2 = gvp[1] * p[1], gc3 = gvp[1] * p[2],
                 gc4 = gvp[2] * p[0], gc5 = gvp[2] * p[2];
    G[2] = ((((gc0 + gc1) + gc2) + gc3) + gc4) + gc5;
    G[3] = ((((gc0 * p[0] + gc1 * p[1]) + gc2 * p[1]) + gc3 * p[2]) + gc4 * p[0]) + gc5 * p[2];
    G[4] = (gc0 * p[2] + gc2 * p[0]) + gc5 * p[1];
    G[5] = (gc0 * p[1] + gc2 * p[2]) + gc4 * p[2];
    // forward
    double y1[CAIR_NN_H1];
#pragma unroll
    for (int j = 0; j < CAIR_NN_H1; ++j) {
      double z = 0.0;
#pragma unroll
      for (int i = 0; i < 6; ++i) z += G[i] * c[CAIR_NN_W1 + i + 6 * j];
      y1[j] = ftanh(z + c[CAIR_NN_B1 + j]);
    }
    double v = 0.0, d2[CAIR_NN_H2];
#pragma unroll
    for (int k = 0; k < CAIR_NN_H2; ++k) {
      double z = 0.0;
#pragma unroll
      for (int j = 0; j < CAIR_NN_H1; ++j) z += y1[j] * c[CAIR_NN_W2 + j + CAIR_NN_H1 * k];
      const double y2 = ftanh(z + c[CAIR_NN_B2 + k]);
      const double w3 = c[CAIR_NN_W3 + k];
      v += y2 * w3;
      d2[k] = w3 * (1.0 - y2 * y2);
    }
    v += c[CAIR_NN_B3];
    const double vout = BNN ? fexp(v + c[CAIR_BNN_NOISE]) : v;
    V = (vout - c[CAIR_NN_YSC]) * CAIR_EV_TO_HARTREE + vdiat;
    const double dscale = BNN ? vout * CAIR_EV_TO_HARTREE : CAIR_EV_TO_HARTREE;
    // adjoint sweep: dV/dG
    double gG[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int j = 0; j < CAIR_NN_H1; ++j) {
      double s = 0.0;
#pragma unroll
      for (int k = 0; k < CAIR_NN_H2; ++k) s += c[CAIR_NN_W2 + j + CAIR_NN_H1 * k] * d2[k];
      s *= 1.0 - y1[j] * y1[j];
#pragma unroll
      for (int i = 0; i < 6; ++i) gG[i] += c[CAIR_NN_W1 + i + 6 * j] * s;
    }
    // dG/dR (Compute_O3_NN_PES_1d dG(:,1:6)) contracted with dV/dG
    const double inv_lam = 1.0 / lam;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const double psq = lam * (p[r] * p[r]), pcu = lam * ((p[r] * p[r]) * p[r]);
      const int a = (r + 1) % 3, b = (r + 2) % 3;
      const double psqs = lam * (p[a] * p[a]) + lam * (p[b] * p[b]);
      const double pcus = lam * ((p[a] * p[a]) * p[a]) + lam * ((p[b] * p[b]) * p[b]);
      const double gvps = -(lam * (gvp[r] + gvp[(r + 2) % 3]));
      double t = gvps * gG[0];
      t += -(lam * gprod) * gG[1];
      t += -((2.0 * gvs[r]) * psq + p[r] * psqs) * gG[2];
      t += -((3.0 * gvs[r]) * pcu + p[r] * pcus) * gG[3];
      t += -((lam * gprod) * (2.0 * p[r] + gvs[r])) * gG[4];
      t += -(((2.0 * psq) * psqs) * inv_lam) * gG[5];
      dVdR[r] = t * dscale + dvd[r];
    }
    trans_to_cart_3(S, Ri, Q, dVdR, dVdQ);
  } else {
    const double gvs[3] = {p[0] + p[1], p[1] + p[2], p[2] + p[0]};
    double G[3];
    G[0] = (gvp[0] + gvp[1]) + gvp[2];
    G[1] = gvp[0] * p[2];
    G[2] = (gvp[0] * gvs[0] + gvp[1] * gvs[1]) + gvp[2] * gvs[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) G[i] = (G[i] - c[CAIR_NN_MEAN + i]) / c[CAIR_NN_SD + i];
    double y1[CAIR_NN_H1];
#pragma unroll
    for (int j = 0; j < CAIR_NN_H1; ++j) {
      double z = c[CAIR_NN_B1 + j];
#pragma unroll
      for (int l = 0; l < 3; ++l) z += c[CAIR_NN_W1P + l + 3 * j] * G[l];
      y1[j] = ftanh(z);
    }
    double v = 0.0;
#pragma unroll
    for (int k = 0; k < CAIR_NN_H2; ++k) {
      double z = c[CAIR_NN_B2 + k];
#pragma unroll
      for (int j = 0; j < CAIR_NN_H1; ++j) z += c[CAIR_NN_W2 + j + CAIR_NN_H1 * k] * y1[j];
      v += ftanh(z) * c[CAIR_NN_W3 + k];
    }
    v += c[CAIR_NN_B3];
    const double vout = BNN ? fexp(v + c[CAIR_BNN_NOISE]) : v;
    V = (vout - c[CAIR_NN_YSC]) * CAIR_EV_TO_HARTREE + vdiat;
  }
}

// O4 UMN (Compute_O4_UMN_PES_1d, O4_UMN_PES_Class.F90:269-298 -> O4pes 310-370): MEG variables
// of the six pairs, O4 PIP (430 terms, gradient by the generated adjoint sweep), six O2 diatomics.
template <bool GRAD>
__device__ __forceinline__ void pes_o4(const DevSys& S, const DevPes& P, const double* R, const double* Ri,
                                       const double* Q, double& V, double* dVdR, double* dVdQ) {
  double x[6], dx[6], vd[6], dvd[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double rang = R[i] * CAIR_B_TO_ANG;
    double d1 = rang - P.ra, d2 = rang - P.rb;
    double e = fexp(-(d1 * P.inv_a) - (d2 * d2) * P.inv_ab);
    x[i] = e;
    if (GRAD) dx[i] = (-((2.0 * d2) * P.inv_ab) - P.inv_a) * e;
    diat<GRAD>(S, R[i], vd[i], dvd[i]);
  }
  double vdiat = 0.0;
#pragma unroll
  for (int i = 0; i < 6; ++i) vdiat = vdiat + vd[i];
  double vp;
  const double* __restrict__ C = P.coef;
  if (GRAD) {
    double g[6];
    pip_o4_eval_rev(x, dx, C, 0.0, vp, g);
    V = vp * CAIR_KCM_TO_HARTREE + vdiat;
#pragma unroll
    for (int i = 0; i < 6; ++i) dVdR[i] = g[i] * CAIR_KCM_TO_HARTREE * CAIR_B_TO_ANG + dvd[i];
    trans_to_cart_4(S, Ri, Q, dVdR, dVdQ);
  } else {
    pip_o4_value(x, C, 0.0, vp);
    V = vp * CAIR_KCM_TO_HARTREE + vdiat;
  }
}

// N4 UMN (Compute_N4_UMN_PES_1d, N4_UMN_PES_Class.F90:329-361 -> n4pes 373-417): the N4 PIP on all
// six MEG variables (the N3 surface is the same fit with three pairs pinned), six N2 diatomics.
template <bool GRAD>
__device__ __forceinline__ void pes_n4(const DevSys& S, const DevPes& P, const double* R, const double* Ri,
                                       const double* Q, double& V, double* dVdR, double* dVdQ) {
  double x[6], dx[6], vd[6], dvd[6];
  const double inv_ab = 1.0 / 1.5;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double d = R[i] * CAIR_B_TO_ANG - 1.098;
    double e = fexp(-d - (d * d) * inv_ab);
    x[i] = e;
    if (GRAD) dx[i] = (-((2.0 * d) * inv_ab) - 1.0) * e;
    diat<GRAD>(S, R[i], vd[i], dvd[i]);
  }
  double vdiat = 0.0;
#pragma unroll
  for (int i = 0; i < 6; ++i) vdiat = vdiat + vd[i];
  double vp;
  const double* __restrict__ C = P.coef;
  if (GRAD) {
    double g[6];
    pip_n4_eval_rev(x, dx, C, 457.4, vp, g);
    V = (vp * CAIR_KCM_TO_HARTREE + 0.0) + vdiat;
#pragma unroll
    for (int i = 0; i < 6; ++i) dVdR[i] = g[i] * CAIR_KCM_TO_HARTREE * CAIR_B_TO_ANG + dvd[i];
    trans_to_cart_4(S, Ri, Q, dVdR, dVdQ);
  } else {
    pip_n4_value(x, C, 457.4, vp);
    V = (vp * CAIR_KCM_TO_HARTREE + 0.0) + vdiat;
  }
}

// N4 UMN PIPNN (N4_UMN_PIPNN_PES_Class.F90).  Coefficients as packed at cair_create:
// UseSurface(3), iFunc, NInput = 276, NHid1 = 5, NHid2 = 90, NOutput = 1, then per network
// pdel(277), pavg(277), W1(276, 5), b1(5), W2(5, 90), b2(90), W3(90), b3.
#define CAIR_PIPNN_HDR 8
#define CAIR_PIPNN_NIN 276
#define CAIR_PIPNN_H1 5
#define CAIR_PIPNN_H2 90
#define CAIR_PIPNN_NET (2 * (CAIR_PIPNN_NIN + 1) + CAIR_PIPNN_NIN * CAIR_PIPNN_H1 + CAIR_PIPNN_H1 + \
                        CAIR_PIPNN_H1 * CAIR_PIPNN_H2 + 2 * CAIR_PIPNN_H2 + 1)

// tranfun (962-984): 1 tansig, 2 logsig, 3 purelin
__device__ __forceinline__ double pipnn_tranfun(double x, int ifunc) {
  if (ifunc == 1) return ftanh(x);
  if (ifunc == 2) return 1.0 / (1.0 + fexp(-x));
  return x;
}

// getpot (743-799): the inputs normalised, two hidden layers, the linear output de-normalised.  Each
// neuron's sum runs from its bias over its inputs in ascending order, as the reference's loops do;
// the second hidden layer feeds the output sum neuron by neuron.
__device__ __forceinline__ double pipnn_net(const double* __restrict__ c, int ifunc, const double* b) {
  const double* __restrict__ pdel = c;
  const double* __restrict__ pavg = pdel + CAIR_PIPNN_NIN + 1;
  const double* __restrict__ W1 = pavg + CAIR_PIPNN_NIN + 1;
  const double* __restrict__ b1 = W1 + CAIR_PIPNN_NIN * CAIR_PIPNN_H1;
  const double* __restrict__ W2 = b1 + CAIR_PIPNN_H1;
  const double* __restrict__ b2 = W2 + CAIR_PIPNN_H1 * CAIR_PIPNN_H2;
  const double* __restrict__ W3 = b2 + CAIR_PIPNN_H2;
  const double* __restrict__ b3 = W3 + CAIR_PIPNN_H2;
  double a[CAIR_PIPNN_H1];
#pragma unroll
  for (int j = 0; j < CAIR_PIPNN_H1; ++j) a[j] = b1[j];
#pragma unroll 4
  for (int i = 0; i < CAIR_PIPNN_NIN; ++i) {
    const double y = (b[i] - pavg[i]) / pdel[i];
#pragma unroll
    for (int j = 0; j < CAIR_PIPNN_H1; ++j) a[j] = a[j] + y * W1[i + CAIR_PIPNN_NIN * j];
  }
#pragma unroll
  for (int j = 0; j < CAIR_PIPNN_H1; ++j) a[j] = pipnn_tranfun(a[j], ifunc);
  double o = b3[0];
#pragma unroll 2
  for (int k = 0; k < CAIR_PIPNN_H2; ++k) {
    double h = b2[k];
#pragma unroll
    for (int j = 0; j < CAIR_PIPNN_H1; ++j) h = h + a[j] * W2[j + CAIR_PIPNN_H1 * k];
    o = o + pipnn_tranfun(h, ifunc) * W3[k];
  }
  return o * pdel[CAIR_PIPNN_NIN] + pavg[CAIR_PIPNN_NIN];
}

// n4pipNN (450-657) in kcal/mol at the bond lengths rb [Ang]: the six N2 pair terms, the N4 PIP basis
// of exp(-rb / alpha) (alpha = 1), the mean of the selected networks (eV) times 23.0605, minus VInf
// (the mean of the selected networks' values at infinite separation, line 96).
__device__ __forceinline__ double pipnn_kcal(const double* __restrict__ c, const double* rb) {
  double vn2 = 0.0, x[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double v, d;
    n2p_ev2gm2<false>(rb[i], v, d);
    vn2 = vn2 + v;
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) x[i] = fexp(-rb[i]);
  double b[CAIR_PIPNN_NIN];
  pip_n4_basis(x, b);
  const int ifunc = (int)c[3];
  const double vinf_s[3] = {-0.021346263746904, -0.196886061330806, -0.030606048118131};
  double vs[3] = {0.0, 0.0, 0.0}, vinf = 0.0;
  int nuse = 0;
#pragma unroll 1
  for (int k = 0; k < 3; ++k)
    if (c[k] == 1.0) {
      vs[k] = pipnn_net(c + CAIR_PIPNN_HDR + k * CAIR_PIPNN_NET, ifunc, b);
      vinf = vinf + vinf_s[k];
      nuse += 1;
    }
  vinf = vinf / (double)nuse;
  const double v = ((vs[0] + vs[1]) + vs[2]) / (double)nuse;
  return (v * 23.0605 + vn2) - vinf;
}

// Compute_N4_UMN_PIPNN_PES_1d (410-439): V, dVdR by n4pipNN's central differences (dr = 1e-5 Ang; the
// bond lengthened by dr, then shortened by 2 dr, then restored, one bond after the other) and
// dVdQ = 0, which the reference returns, so the surface exerts no force on the trajectories (Hamilton's
// equations for this model skip it).  One evaluation site in a loop keeps the kernels to one copy of
// the 276-function basis.
template <bool GRAD>
__device__ __forceinline__ void pes_n4pipnn(const DevSys& S, const DevPes& P, const double* R, double& V,
                                            double* dVdR, double* dVdQ) {
  const double* __restrict__ c = P.coef;
  const double dr = 1.0e-5;
  double rb[6], vp = 0.0;
#pragma unroll
  for (int i = 0; i < 6; ++i) rb[i] = R[i] * CAIR_B_TO_ANG;
#pragma unroll 1
  for (int e = 0; e < (GRAD ? 13 : 1); ++e) {
    const int i = (e - 1) >> 1;
    if (e > 0) rb[i] = (e & 1) ? rb[i] + dr : rb[i] - 2.0 * dr;
    const double v = pipnn_kcal(c, rb);
    if (e == 0) {
      V = v * CAIR_KCM_TO_HARTREE;
    } else if (e & 1) {
      vp = v;
    } else {
      dVdR[i] = ((vp - v) / (2.0 * dr)) * CAIR_KCMANG_TO_HARTB;
      rb[i] = rb[i] + dr;
    }
  }
  if (GRAD) {
#pragma unroll
    for (int i = 0; i < 9; ++i) dVdQ[i] = 0.0;
  }
}

// Sizes of a surface model's system: atoms, NEqtVar, NEqtTot, pairs
template <int MODEL>
struct Traits {
  static constexpr int NA =
      (MODEL == CAIR_PES_O4_UMN || MODEL == CAIR_PES_N4_UMN || MODEL == CAIR_PES_N4_PIPNN) ? 4 : 3;
  static constexpr int NV = 3 * (NA - 1);
  static constexpr int NE = 2 * NV;
  static constexpr int NP = NA * (NA - 1) / 2;
};

template <int MODEL, bool GRAD>
__device__ __forceinline__ void pes(const DevSys& S, const DevPes& P, const double* R, const double* Ri,
                                    const double* Q, double& V, double* dVdR, double* dVdQ) {
  if (MODEL == CAIR_PES_O3_UMN) pes_o3<GRAD>(S, P, R, Ri, Q, V, dVdR, dVdQ);
  else if (MODEL == CAIR_PES_O3_NN) pes_o3nn<GRAD>(S, P, R, Ri, Q, V, dVdR, dVdQ);
  else if (MODEL == CAIR_PES_O3_BNN) pes_o3nn<GRAD, true>(S, P, R, Ri, Q, V, dVdR, dVdQ);
  else if (MODEL == CAIR_PES_O4_UMN) pes_o4<GRAD>(S, P, R, Ri, Q, V, dVdR, dVdQ);
  else if (MODEL == CAIR_PES_N4_UMN) pes_n4<GRAD>(S, P, R, Ri, Q, V, dVdR, dVdQ);
  else if (MODEL == CAIR_PES_N4_PIPNN) pes_n4pipnn<GRAD>(S, P, R, V, dVdR, dVdQ);
  else pes_n3<GRAD>(S, P, R, Ri, Q, V, dVdR, dVdQ);
}

// ------------------------------------------------------------------------------------------
// Pair distances (Compute_Rp_CartCoord_3Atoms, Collision_Class.F90:2244-2275); Q has room
// for the last atom, which is written to Q[NV..NV+2].
// ------------------------------------------------------------------------------------------
// Distances from one reciprocal square root each: 1/R = rsqrt(R^2), R = R^2 (1/R).  The parity
// build takes the reference's order instead: R = sqrt(R^2), then 1/R by division.
__device__ __forceinline__ void dist_pair(double s2, double& R, double& Ri) {
#ifdef CAIR_PARITY_MATH
  R = sqrt(s2);
  Ri = 1.0 / R;
#else
  Ri = rsqrt(s2);
  R = s2 * Ri;
#endif
}

__device__ __forceinline__ void rp3(const DevSys& S, double* Q, double* Rp, double* Ri) {
  const double m1 = S.mMiMn[0], m2 = S.mMiMn[1];
#pragma unroll
  for (int c = 0; c < 3; ++c) Q[6 + c] = m1 * Q[c] + m2 * Q[3 + c];
  double a, b, c, s2;
  a = Q[0] - Q[3]; b = Q[1] - Q[4]; c = Q[2] - Q[5];
  s2 = a * a + b * b + c * c; dist_pair(s2, Rp[0], Ri[0]);
  a = Q[0] - Q[6]; b = Q[1] - Q[7]; c = Q[2] - Q[8];
  s2 = a * a + b * b + c * c; dist_pair(s2, Rp[1], Ri[1]);
  a = Q[3] - Q[6]; b = Q[4] - Q[7]; c = Q[5] - Q[8];
  s2 = a * a + b * b + c * c; dist_pair(s2, Rp[2], Ri[2]);
}

// Compute_Rp_CartCoord_4Atoms (Collision_Class.F90:2279-2316): pairs 1-2, 1-3, 1-4, 2-3, 2-4, 3-4;
// the fourth atom is written to Q[9..11].
__device__ __forceinline__ void rp4(const DevSys& S, double* Q, double* Rp, double* Ri) {
  const double m1 = S.mMiMn[0], m2 = S.mMiMn[1], m3 = S.mMiMn[2];
#pragma unroll
  for (int c = 0; c < 3; ++c) Q[9 + c] = m1 * Q[c] + m2 * Q[3 + c] + m3 * Q[6 + c];
  constexpr int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const double a = Q[3 * pa[k]] - Q[3 * pb[k]], b = Q[3 * pa[k] + 1] - Q[3 * pb[k] + 1],
                 c = Q[3 * pa[k] + 2] - Q[3 * pb[k] + 2];
    const double s2 = a * a + b * b + c * c;
    dist_pair(s2, Rp[k], Ri[k]);
  }
}

template <int NA>
__device__ __forceinline__ void rp(const DevSys& S, double* Q, double* Rp, double* Ri) {
  if (NA == 3) rp3(S, Q, Rp, Ri);
  else rp4(S, Q, Rp, Ri);
}

// ------------------------------------------------------------------------------------------
// Hamilton's equations (ODE_System.F90:45-96): y = [p(NV), q(NV)]
// ------------------------------------------------------------------------------------------
template <int MODEL>
struct Rhs {
  using T = Traits<MODEL>;
  const DevSys& S;
  const DevPes& P;
  __device__ Rhs(const DevSys& s, const DevPes& p) : S(s), P(p) {}
  __device__ __forceinline__ void operator()(const double (&y)[T::NE], double (&yp)[T::NE]) const {
    // dq_j/dt = sum_{i = j mod 3, ascending} Tpq(j,i) p_i
#pragma unroll
    for (int j = 0; j < T::NV; ++j) {
      const int i0 = j % 3;
      double acc = 0.0 + S.Tpq[j + 9 * i0] * y[i0];
#pragma unroll
      for (int i = i0 + 3; i < T::NV; i += 3) acc = acc + S.Tpq[j + 9 * i] * y[i];
      yp[T::NV + j] = acc;
    }
    if (MODEL == CAIR_PES_N4_PIPNN) {
      // the surface's dVdQ is zero (Compute_N4_UMN_PIPNN_PES_1d), so dp/dt = -0
#pragma unroll
      for (int i = 0; i < T::NV; ++i) yp[i] = -0.0;
      return;
    }
    double Q[3 * T::NA], R[T::NP], Ri[T::NP], V, dVdR[T::NP], dVdQ[T::NV];
#pragma unroll
    for (int i = 0; i < T::NV; ++i) Q[i] = y[T::NV + i];
    rp<T::NA>(S, Q, R, Ri);
    pes<MODEL, true>(S, P, R, Ri, Q, V, dVdR, dVdQ);
#pragma unroll
    for (int i = 0; i < T::NV; ++i) yp[i] = -dVdQ[i];
  }
};

// Hamiltonian_1d (Collision_Class.F90:2046-2111); returns H, fills Rpi
template <int MODEL>
__device__ __forceinline__ double hamiltonian(const DevSys& S, const DevPes& P, const double (&y)[Traits<MODEL>::NE],
                                              double (&Rpi)[Traits<MODEL>::NP]) {
  using T = Traits<MODEL>;
  double h = 0.0;
#pragma unroll
  for (int i = 0; i < T::NV; ++i) {
    const int j0 = i % 3;
    double eki = 0.0 + S.Tpq[j0 + 9 * i] * y[j0];
#pragma unroll
    for (int j = j0 + 3; j < T::NV; j += 3) eki = eki + S.Tpq[j + 9 * i] * y[j];
    h = h + y[i] * eki;
  }
  double Q[3 * T::NA], R[T::NP], V;
#pragma unroll
  for (int i = 0; i < T::NV; ++i) Q[i] = y[T::NV + i];
  rp<T::NA>(S, Q, R, Rpi);
  pes<MODEL, false>(S, P, R, Rpi, Q, V, nullptr, nullptr);
  return h * 0.5 + V;
}

// ------------------------------------------------------------------------------------------
// Bulirsch-Stoer attempt (Integrate_ODE_1d, ODE_Solver.F90:225-358; mmidv 363-462;
// RatPolExtrap 467-541), one trajectory, NS extrapolation steps.
// ------------------------------------------------------------------------------------------
__host__ __device__ constexpr int nseq_of(int i) {
  return i == 0 ? 2 : i == 1 ? 4 : i == 2 ? 6 : i == 3 ? 8 : i == 4 ? 12 : i == 5 ? 16 : i == 6 ? 24 : 32;
}

// |a - b| / s < 1 exactly as IEEE division then comparison would decide, without the division
// and off the FP64 pipe in the common case.  The magnitudes' bit patterns order like the values
// (s finite, d finite or NaN): |d| more than 64 ulps below |s| gives |d|/s <= 1 - 2^-47, which
// rounds below 1; |d| >= |s| (or d NaN) gives fl(|d|/s) >= 1 (or NaN); the 64 ulps between
// take the division.
__device__ __forceinline__ long long mag_bits(double x) { return __double_as_longlong(x) & 0x7fffffffffffffffll; }

__device__ __forceinline__ bool err_below_one(double d, double s) {
  const long long ad = mag_bits(d), as = mag_bits(s);
  if (ad + 64 < as) return true;
  if (ad >= as) return false;
  return fabs(d / s) < 1.0;
}

// d is NaN, from its bit pattern (an FP64 comparison would take a slot of the FP64 pipe)
__device__ __forceinline__ bool is_nan_bits(double d) { return mag_bits(d) > 0x7ff0000000000000ll; }

// Extrapolation step `S1` (1-based) of RatPolExtrap for one system of NE equations.
// d holds the columns 1..NS-1 of the reference's d table (column NS is only ever read
// as zero); yt receives ytry(:, S1) for S1 < NS, ylast receives ytry(:, NS).
template <int S1, int NE, int NS>
__device__ __forceinline__ void extrap_stage(const double (&yest)[NE], const double (&xs)[NS],
                                             double (&d)[NS - 1][NE], double (&yt)[NS - 1][NE],
                                             double (&ylast)[NE]) {
  const double xest = xs[S1 - 1];
  if (S1 == 1) {
#pragma unroll
    for (int j = 0; j < NE; ++j) {
      if (NS > 1) { yt[0][j] = yest[j]; d[0][j] = yest[j]; }
      else ylast[j] = yest[j];
    }
    return;
  }
  constexpr int m1 = S1 < NS ? S1 : NS;
  double fx[NS + 1];
#pragma unroll
  for (int k = 1; k <= m1 - 1; ++k) fx[k + 1] = xs[S1 - k - 1] / xest;
#pragma unroll
  for (int j = 0; j < NE; ++j) {
    double yy = yest[j], v = d[0][j], c = yy;
    d[0][j] = yy;
#pragma unroll
    for (int k = 2; k <= m1; ++k) {
      double b1 = fx[k] * v;
      double b = (c - v) / ((b1 - c) + 1.0E-40);
      double ddy = c * b;
      c = b1 * b;
      // column k was written at an earlier stage unless k == S1 (then it is still zero)
      v = (k < S1 && k - 1 < NS - 1) ? d[k - 1][j] : 0.0;
      if (k - 1 < NS - 1) d[k - 1][j] = ddy;
      yy = yy + ddy;
    }
    if (S1 < NS) yt[S1 - 1][j] = yy;
    else ylast[j] = yy;
  }
}

template <int NE, int NS>
__device__ __forceinline__ void extrap_dispatch(int stage, const double (&yest)[NE], const double (&xs)[NS],
                                                double (&d)[NS - 1][NE], double (&yt)[NS - 1][NE],
                                                double (&ylast)[NE]) {
  switch (stage) {
    case 1: extrap_stage<1, NE, NS>(yest, xs, d, yt, ylast); break;
    case 2: if (NS >= 2) extrap_stage<(NS >= 2 ? 2 : 1), NE, NS>(yest, xs, d, yt, ylast); break;
    case 3: if (NS >= 3) extrap_stage<(NS >= 3 ? 3 : 1), NE, NS>(yest, xs, d, yt, ylast); break;
    case 4: if (NS >= 4) extrap_stage<(NS >= 4 ? 4 : 1), NE, NS>(yest, xs, d, yt, ylast); break;
    default: break;
  }
}

__host__ __device__ constexpr int nseq_total(int ns) { return ns == 0 ? 1 : nseq_of(ns - 1) + nseq_total(ns - 1); }

__device__ __forceinline__ double htemp_of(int stage) {
  // One / dfloat(nseq(iSteps)), folded at compile time (same value as the division)
  return stage == 1 ? 1.0 / 2.0 : stage == 2 ? 1.0 / 4.0 : stage == 3 ? 1.0 / 6.0 : 1.0 / 8.0;
}

// One Bulirsch-Stoer attempt.  The 1 + sum(nseq) right-hand-side evaluations of the
// attempt run through a single call site of f, so the surface is inlined once and every
// thread of a warp evaluates its right-hand side in lockstep.
template <int NE, int NS, class F>
__device__ __forceinline__ int bs_attempt(const F& f, double (&y)[NE], double& x, double& h,
                                          const double* __restrict__ yscal, double relax, bool incstp,
                                          double& smax, double& smin, int& irej, int& iste) {
  static_assert(NS >= 2 && NS <= 4, "NSteps 2..4 are built");
  constexpr int NTOT = nseq_total(NS);
  double dydx[NE], ym[NE], yn[NE], fo[NE], ylast[NE];
  double d[NS - 1][NE], yt[NS - 1][NE], xs[NS];
#pragma unroll
  for (int i = 0; i < NE; ++i) yn[i] = y[i];
  int stage = 0, sub = 0, nst = 1;
  double hs = 0.0, h2 = 0.0;
#pragma unroll 1
  for (int e = 0; e < NTOT; ++e) {
    f(yn, fo);
    if (stage == 0 || sub == nst) {
      if (stage == 0) {
#pragma unroll
        for (int i = 0; i < NE; ++i) dydx[i] = fo[i];
      } else {
        // end of mmidv: yout = Half*(ym + yn + h*yout), then the extrapolation
#pragma unroll
        for (int i = 0; i < NE; ++i) fo[i] = 0.5 * (ym[i] + yn[i] + hs * fo[i]);
        const double hh = h * htemp_of(stage);
        xs[stage - 1] = hh * hh;
        extrap_dispatch<NE, NS>(stage, fo, xs, d, yt, ylast);
      }
      ++stage;
      if (stage <= NS) {
        nst = nseq_of(stage - 1);
        hs = h * htemp_of(stage);
        h2 = 2.0 * hs;
        sub = 1;
#pragma unroll
        for (int i = 0; i < NE; ++i) { ym[i] = y[i]; yn[i] = y[i] + hs * dydx[i]; }
      }
    } else {
#pragma unroll
      for (int i = 0; i < NE; ++i) {
        double ys = ym[i] + h2 * fo[i];
        ym[i] = yn[i];
        yn[i] = ys;
      }
      ++sub;
    }
  }
  // errmax(k) < 1 for k = 1..NS-1
  bool below[NS - 1];
  int nan = 0;
#pragma unroll
  for (int k = 0; k < NS - 1; ++k) {
    bool ok = true;
#pragma unroll
    for (int i = 0; i < NE; ++i) {
      double dd = yt[k][i] - ylast[i];
      if (is_nan_bits(dd)) nan = 1;
      ok = err_below_one(dd, yscal[i]) && ok;
    }
    below[k] = ok;
  }
  int iconv = 0;
#pragma unroll
  for (int is = 2; is <= NS; ++is) {
    int j = NS + 1 - is;
    if (!below[j - 1]) break;
    iconv = j;
  }
  if (below[NS - 2]) {
    x = x + h;
#pragma unroll
    for (int i = 0; i < NE; ++i) y[i] = ylast[i];
    smin = (smin < h) ? smin : h;
    smax = (smax > h) ? smax : h;
    iste += 1;
    if (iconv < NS - 1 && incstp) {
      double ratio = 0.0;
#pragma unroll
      for (int k = 1; k < NS - 1; ++k)
        if (iconv == k) ratio = (double)nseq_of(NS - 1) / (double)nseq_of(k);
      h = h * (ratio + relax) / (1.0 + relax);
    }
  } else {
    constexpr int kk = (NS / 2) < 1 ? 1 : NS / 2;
    h = h / (double)nseq_of(kk - 1);
    irej += 1;
  }
  return nan;
}

}  // namespace cair
