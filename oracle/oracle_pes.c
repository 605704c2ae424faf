/*
 * Oracle (test infrastructure): diatomic potentials, PIP evaluation and the three UMN
 * surfaces of the hot path, restated from the CoarseAIR Fortran.  Build with
 * -ffp-contract=off so that no multiply-add is fused (the reference's x86 gfortran
 * build has no FMA).
 */
#include <math.h>
#include <string.h>
#include "oracle.h"
#include "pip_tables.h"

/* src/Parameters/Parameters_Module.F90:82-87 */
#define B_TO_ANG        0.52917721092
#define KCM_TO_HARTREE  0.159360144e-2
#define KCMANG_TO_HARTB 0.843297564e-3

/* libgfortran pow_r8_i4 (binary powering), used where the reference raises to a
 * variable integer power (O2_UMN_DiatomicPotential_Class.F90 beta**k). */
static double powi_gf(double a, int b) {
  double p = 1.0, x = a;
  unsigned u;
  if (b == 0) return 1.0;
  if (b < 0) { u = (unsigned)(-b); x = 1.0 / x; } else u = (unsigned)b;
  for (;;) {
    if (u & 1u) p *= x;
    u >>= 1;
    if (u) x *= x; else break;
  }
  return p;
}

/* ------------------------------------------------------------------------------------------ */
/* O2 UMN diatomic: src/DiatomicPotentials/O2_UMN_DiatomicPotential_Class.F90                 */
/* ------------------------------------------------------------------------------------------ */
static const double O2_A[8] = {-1.488979427684798e3, 1.881435846488955e4, -1.053475425838226e5,
                               2.755135591229064e5, -4.277588997761775e5, 4.404104009614092e5,
                               -2.946204062950765e5, 1.176861219078620e5};
static const double O2_ALPHA = 9.439784362354936e-1;
static const double O2_BETA = 1.262242998506810;

/* edisp / edisp_Grad (lines 323-381) */
static void o2_edisp(double rb, double* e6, double* e8, double* e6dr, double* e8dr) {
  const double r2r4 = 2.59361680, rs6 = 0.5299, rs8 = 2.20, c6 = 12.8;
  double c8step = 3.0 * c6 * (r2r4 * r2r4);
  double tmp = sqrt(c8step / c6);
  double s = rs6 * tmp + rs8;
  double s2 = s * s, s3 = s2 * s, s6 = s3 * s3, s4 = s2 * s2, s8 = s4 * s4;
  double r2 = rb * rb, r3 = r2 * rb, r4 = r2 * r2, r5 = r4 * rb, r6 = r3 * r3, r7 = r4 * r3, r8 = r4 * r4;
  double d6 = r6 + s6, d8 = r8 + s8;
  *e6 = c6 / d6;
  *e8 = c8step / d8;
  if (e6dr) {
    *e6dr = c6 * (-6.0 * r5) / (d6 * d6);
    *e8dr = c8step * (-8.0 * r7) / (d8 * d8);
  }
}

/* Ev2gm2 (lines 214-247) + d3disp (283-300): energy in hartree from R in Angstrom */
static double o2_ev2gm2(double rang) {
  double v = 0.0;
  for (int k = 0; k <= 7; ++k) v = v + O2_A[k] * exp(-(O2_ALPHA * powi_gf(O2_BETA, k) * (rang * rang)));
  v = v * 1.e-3;
  double rb = rang / B_TO_ANG, e6, e8;
  o2_edisp(rb, &e6, &e8, 0, 0);
  return v + (-e6 - 2.0 * e8);
}

/* Ev2gm2_Grad (lines 250-280) + d3disp_Grad (303-320): V [Eh], dV [Eh/Ang] */
static void o2_ev2gm2_grad(double rang, double* v, double* dv) {
  double vv = 0.0, dd = 0.0;
  for (int k = 0; k <= 7; ++k) vv = vv + O2_A[k] * exp(-(O2_ALPHA * powi_gf(O2_BETA, k) * (rang * rang)));
  vv = vv * 1.e-3;
  for (int k = 0; k <= 7; ++k)
    dd = dd - 2.0 * O2_A[k] * O2_ALPHA * powi_gf(O2_BETA, k) * rang *
                  exp(-(O2_ALPHA * powi_gf(O2_BETA, k) * (rang * rang)));
  dd = dd * 1.e-3;
  double rb = rang / B_TO_ANG, e6, e8, e6dr, e8dr;
  o2_edisp(rb, &e6, &e8, &e6dr, &e8dr);
  *v = vv + (-e6 - 2.0 * e8);
  *dv = dd + (-e6dr - 2.0 * e8dr) / B_TO_ANG;
}

/* ------------------------------------------------------------------------------------------ */
/* N2 UMN_ForN4 diatomic: src/DiatomicPotentials/N2_UMN_ForN4_DiatomicPotential_Class.F90     */
/* ------------------------------------------------------------------------------------------ */
static const double N2_CS[7] = {2.70963254293, 1.32620177271e-1, 2.96757048793e-1, 1.97112432229e-1,
                                -5.02002309588e-1, 3.80734244606e-1, 1.21001628750};
static const double N2_DE = 228.7, N2_RED = 1.098, N2_RED4 = 1.4534810048;

/* Ev2gm2 / Ev2gm2_Grad (lines 139-207): kcal/mol, kcal/mol/Ang */
static void n2_ev2gm2(double rang, double* v, double* dv) {
  double r3 = (rang * rang) * rang;
  double r4 = r3 * rang;
  double ts = r4 + N2_RED4;
  double y = (r4 - N2_RED4) / ts;
  double y2 = y * y, y3 = y2 * y, y4 = y2 * y2, y5 = y3 * y2, y6 = y3 * y3;
  double fy = N2_CS[0] + N2_CS[1] * y + N2_CS[2] * y2 + N2_CS[3] * y3 + N2_CS[4] * y4 + N2_CS[5] * y5 +
              N2_CS[6] * y6;
  double u = exp(-(fy * (rang - N2_RED)));
  double minu = 1.0 - u;
  *v = N2_DE * (minu * minu) - N2_DE;
  if (dv) {
    double dfdy = N2_CS[1] + 2.0 * N2_CS[2] * y + 3.0 * N2_CS[3] * y2 + 4.0 * N2_CS[4] * y3 +
                  5.0 * N2_CS[5] * y4 + 6.0 * N2_CS[6] * y5;
    double dydr = 8.0 * r3 * N2_RED4 / (ts * ts);
    double dfdr = dfdy * dydr;
    *dv = 2.0 * N2_DE * minu * u * (dfdr * (rang - N2_RED) + fy);
  }
}

/* ------------------------------------------------------------------------------------------ */
/* N2 UMN_PIPNN_ForN4: src/DiatomicPotentials/N2_UMN_PIPNN_ForN4_DiatomicPotential_Class.F90;  */
/* the same Ev2gm2 + D3(BJ) dispersion is the pair term of the N4 UMN PIPNN surface           */
/* (N4_UMN_PIPNN_PES_Class.F90:1471-1748).  Powers as gfortran expands them (x^5 = x^3 x^2,   */
/* x^6 = x^3 x^3, x^8 = x^4 x^4).                                                              */
/* ------------------------------------------------------------------------------------------ */
static const double N2P_AS[7] = {2.7475450369759, 0.218868498415108, 0.248885765371433, -0.229295466336412,
                                 -0.653389048592838, 1.03611964035396, 1.71287482791961};
static const double N2P_DE = 225.213, N2P_RE = 1.098;
#define HARTREE_TO_KCM (1.0 / KCM_TO_HARTREE)

/* edisp for one N-N pair (iz = 7: r2r4 = 2.71175247; C6 = 19.7, rs6 = 0.5299, rs8 = 2.20), r [bohr] */
static void n2p_edisp(double r, double* e6, double* e8, double* e6dr, double* e8dr) {
  const double c6 = 19.7, r2r4 = 2.71175247, a1 = 0.5299, a2 = 2.20;
  const double c8 = ((3.0 * c6) * r2r4) * r2r4;
  const double tmp = sqrt(c8 / c6), s = a1 * tmp + a2;
  const double s2 = s * s, s3 = s2 * s, s4 = s2 * s2, s6 = s3 * s3, s8 = s4 * s4;
  const double r2 = r * r, r3 = r2 * r, r4 = r2 * r2, r6 = r3 * r3, r8 = r4 * r4;
  const double d6 = r6 + s6, d8 = r8 + s8;
  *e6 = c6 / d6;
  *e8 = c8 / d8;
  if (e6dr) {
    const double r5 = r3 * r2, r7 = r4 * r3;
    *e6dr = c6 * (-(6.0 * r5)) / (d6 * d6);
    *e8dr = c8 * (-(8.0 * r7)) / (d8 * d8);
  }
}

/* Ev2gm2 / Ev2gm2_Grad (diatomic class 116-225; surface 1471-1551): kcal/mol, kcal/mol/Ang */
static void n2p_ev2gm2(double rang, double* v, double* dv) {
  const double r2 = rang * rang, r3 = r2 * rang, r4 = r2 * r2, re2 = N2P_RE * N2P_RE, re4 = re2 * re2;
  const double y = (r4 - re4) / (r4 + re4);
  const double y2 = y * y, y3 = y * y2, y4 = y2 * y2, y5 = y2 * y3, y6 = y3 * y3;
  const double fy = N2P_AS[0] + N2P_AS[1] * y + N2P_AS[2] * y2 + N2P_AS[3] * y3 + N2P_AS[4] * y4 +
                    N2P_AS[5] * y5 + N2P_AS[6] * y6;
  const double u = exp(-(fy * (rang - N2P_RE)));
  double e6, e8, e6dr, e8dr;
  n2p_edisp(rang / B_TO_ANG, &e6, &e8, dv ? &e6dr : 0, dv ? &e8dr : 0);
  *v = ((N2P_DE * (1.0 - u)) * (1.0 - u) - N2P_DE) + (0.0 + (-e6 - 2.0 * e8) * HARTREE_TO_KCM);
  if (dv) {
    const double dfdy = N2P_AS[1] + 2.0 * N2P_AS[2] * y + 3.0 * N2P_AS[3] * y2 + 4.0 * N2P_AS[4] * y3 +
                        5.0 * N2P_AS[5] * y4 + 6.0 * N2P_AS[6] * y5;
    const double rr = r4 + re4;
    const double dydr = ((8.0 * r3) * re4) / (rr * rr);
    const double dfdr = dfdy * dydr;
    *dv = (((2.0 * N2P_DE) * (1.0 - u)) * u) * (dfdr * (rang - N2P_RE) + fy) +
          ((-e6dr - 2.0 * e8dr) * HARTREE_TO_KCM) / B_TO_ANG;
  }
}

double orc_diat_V(int model, double r) {
  double rang = r * B_TO_ANG;
  if (model == ORC_DIAT_O2_UMN) return o2_ev2gm2(rang);          /* DiatomicPotential_O2_UMN 95-106 */
  double v;
  if (model == ORC_DIAT_N2_UMN_PIPNN_FORN4) {                     /* DiatomicPotential_N2 91-101 */
    n2p_ev2gm2(rang, &v, 0);
    return v * KCM_TO_HARTREE + 0.0;
  }
  n2_ev2gm2(rang, &v, 0);
  return v * KCM_TO_HARTREE + 0.0;                                /* DiatomicPotential_N2 99-110 */
}

void orc_diat_VdV(int model, double r, double* v, double* dv) {
  double rang = r * B_TO_ANG, vd, dvd;
  if (model == ORC_DIAT_O2_UMN) {                                 /* Compute_Vd_dVd_O2_UMN 109-124 */
    o2_ev2gm2_grad(rang, &vd, &dvd);
    *v = vd;
    *dv = dvd * B_TO_ANG;
  } else if (model == ORC_DIAT_N2_UMN_PIPNN_FORN4) {              /* Compute_Vd_dVd_N2 105-115 */
    n2p_ev2gm2(rang, &vd, &dvd);
    *v = vd * KCM_TO_HARTREE + 0.0;
    *dv = dvd * KCM_TO_HARTREE * B_TO_ANG;
  } else {                                                        /* Compute_Vd_dVd_N2 114-130 */
    n2_ev2gm2(rang, &vd, &dvd);
    *v = vd * KCM_TO_HARTREE + 0.0;
    *dv = dvd * KCM_TO_HARTREE * B_TO_ANG;
  }
}

/* Rounding-level scales of a diatomic evaluation at r [bohr]: the same sums on absolute values
 * (O2 UMN: the eight Gaussian terms cancel to ~1e-3 of their sum; N2: De (1-u)^2 - De cancels at
 * large r), for V [Eh] and dV/dr [Eh/bohr]. */
static void n2p_scale(double rang, double* sv, double* sdv) {
  const double r3 = (rang * rang) * rang, r4 = r3 * rang, re4 = (N2P_RE * N2P_RE) * (N2P_RE * N2P_RE), ts = r4 + re4;
  const double y = (r4 - re4) / ts;
  double fa = 0.0, fy = 0.0, yi = 1.0, dfa = 0.0, yj = 1.0;
  for (int i = 0; i < 7; ++i) { fa += fabs(N2P_AS[i]) * fabs(yi); fy += N2P_AS[i] * yi; yi *= y; }
  for (int i = 1; i < 7; ++i) { dfa += i * fabs(N2P_AS[i]) * fabs(yj); yj *= y; }
  const double dydr = 8.0 * r3 * re4 / (ts * ts);
  const double u = exp(-(fy * (rang - N2P_RE))), minu = 1.0 - u, dr = fabs(rang - N2P_RE);
  const double arg = fa * dr * (1.0 + fabs(fy * (rang - N2P_RE)));
  double e6, e8, e6dr, e8dr;
  n2p_edisp(rang / B_TO_ANG, &e6, &e8, &e6dr, &e8dr);
  *sv = N2P_DE * (minu * minu) + N2P_DE + 2.0 * N2P_DE * fabs(minu) * u * arg + (e6 + 2.0 * e8) * HARTREE_TO_KCM;
  *sdv = 2.0 * N2P_DE * (fabs(minu) + u) * u * (dfa * dydr * dr + fa) * (1.0 + arg) +
         (fabs(e6dr) + 2.0 * fabs(e8dr)) * HARTREE_TO_KCM / B_TO_ANG;
}

void orc_diat_scale(int model, double r, double* sv, double* sdv) {
  double rang = r * B_TO_ANG;
  if (model == ORC_DIAT_N2_UMN_PIPNN_FORN4) {
    n2p_scale(rang, sv, sdv);
    *sv *= KCM_TO_HARTREE;
    *sdv *= KCM_TO_HARTREE * B_TO_ANG;
    return;
  }
  if (model == ORC_DIAT_O2_UMN) {
    double a = 0.0, d = 0.0;
    for (int k = 0; k <= 7; ++k) {
      double ab = O2_ALPHA * powi_gf(O2_BETA, k);
      double e = exp(-(ab * (rang * rang)));
      a += fabs(O2_A[k]) * e;
      d += 2.0 * fabs(O2_A[k]) * ab * rang * e * (1.0 + ab * rang * rang);
    }
    double rb = rang / B_TO_ANG, e6, e8, e6dr, e8dr;
    o2_edisp(rb, &e6, &e8, &e6dr, &e8dr);
    *sv = a * 1.e-3 + e6 + 2.0 * e8;
    *sdv = (d * 1.e-3) * B_TO_ANG + fabs(e6dr) + 2.0 * fabs(e8dr);
  } else {
    double r3 = (rang * rang) * rang, r4 = r3 * rang, ts = r4 + N2_RED4;
    double y = (r4 - N2_RED4) / ts, fa = 0.0, fy = 0.0, yi = 1.0, dfa = 0.0, yj = 1.0;
    for (int i = 0; i < 7; ++i) { fa += fabs(N2_CS[i]) * fabs(yi); fy += N2_CS[i] * yi; yi *= y; }
    for (int i = 1; i < 7; ++i) { dfa += i * fabs(N2_CS[i]) * fabs(yj); yj *= y; }
    double dydr = 8.0 * r3 * N2_RED4 / (ts * ts);
    double u = exp(-(fy * (rang - N2_RED))), minu = 1.0 - u, dr = fabs(rang - N2_RED);
    double arg = fa * dr * (1.0 + fabs(fy * (rang - N2_RED)));   /* error of u is u times this (relative) */
    *sv = (N2_DE * (minu * minu) + N2_DE + 2.0 * N2_DE * fabs(minu) * u * arg) * KCM_TO_HARTREE;
    *sdv = 2.0 * N2_DE * (fabs(minu) + u) * u * (dfa * dydr * dr + fa) * (1.0 + arg) * KCM_TO_HARTREE * B_TO_ANG;
  }
}

/* ------------------------------------------------------------------------------------------ */
/* Generic PIP evaluator over the generated tables.  Follows EvMono/EvPoly/evbas and the      */
/* forward-mode EvdMdR/EvdPdr/evdbdr of N3_UMN_PES_Class.F90:677-2053 (same structure in      */
/* O4_UMN_PES_Class.F90:571-1962 and O3 Unified/UnifiedBis, O3_UMN_PES_Class.F90:336-638).   */
/* ------------------------------------------------------------------------------------------ */
typedef struct pip_tab {
  int nvar, nmono, npoly, nbasis;
  const short *mo, *ma, *mb, *po, *pa, *pb, *poff, *plen, *plist, *basis;
} pip_tab;

static pip_tab pip_table(int t) {
  pip_tab T;
  if (t == 0) {
    T.nvar = 3; T.nmono = PIP_O3_NMONO; T.npoly = PIP_O3_NPOLY; T.nbasis = PIP_O3_NBASIS;
    T.mo = pip_o3_mono_op; T.ma = pip_o3_mono_a; T.mb = pip_o3_mono_b; T.po = pip_o3_poly_op;
    T.pa = pip_o3_poly_a; T.pb = pip_o3_poly_b; T.poff = pip_o3_poly_off; T.plen = pip_o3_poly_len;
    T.plist = pip_o3_poly_list; T.basis = pip_o3_basis;
  } else if (t == 1) {
    T.nvar = 6; T.nmono = PIP_N4_NMONO; T.npoly = PIP_N4_NPOLY; T.nbasis = PIP_N4_NBASIS;
    T.mo = pip_n4_mono_op; T.ma = pip_n4_mono_a; T.mb = pip_n4_mono_b; T.po = pip_n4_poly_op;
    T.pa = pip_n4_poly_a; T.pb = pip_n4_poly_b; T.poff = pip_n4_poly_off; T.plen = pip_n4_poly_len;
    T.plist = pip_n4_poly_list; T.basis = pip_n4_basis;
  } else {
    T.nvar = 6; T.nmono = PIP_O4_NMONO; T.npoly = PIP_O4_NPOLY; T.nbasis = PIP_O4_NBASIS;
    T.mo = pip_o4_mono_op; T.ma = pip_o4_mono_a; T.mb = pip_o4_mono_b; T.po = pip_o4_poly_op;
    T.pa = pip_o4_poly_a; T.pb = pip_o4_poly_b; T.poff = pip_o4_poly_off; T.plen = pip_o4_poly_len;
    T.plist = pip_o4_poly_list; T.basis = pip_o4_basis;
  }
  return T;
}

/* table: 0 = O3 (3 variables), 1 = N4 PIP used by N3, 2 = O4.  V = V0 + sum_i C_i B_i and
 * dV[i] = sum_j C_j dB_j/dvar_i with dvar_i/dR_i = dmsdr_diag[i]. */
void orc_pip_eval(int table, const double* rms, const double* dmsdr_diag, int want_grad, const double* C,
                  double V0, double* V, double* dV) {
  pip_tab T = pip_table(table);
  double rm[128], p[480], dm[6][128], dp[6][480];
  for (int k = 0; k < T.nmono; ++k) {
    if (T.mo[k] == 0) rm[k] = 1.0;
    else if (T.mo[k] == 1) rm[k] = rms[T.ma[k]];
    else rm[k] = rm[T.ma[k]] * rm[T.mb[k]];
  }
  for (int k = 0; k < T.npoly; ++k) {
    const short* L = T.plist + T.poff[k];
    int n = T.plen[k];
    if (T.po[k] == 0) {
      double s = rm[L[0]];
      for (int i = 1; i < n; ++i) s = s + rm[L[i]];
      p[k] = s;
    } else {
      double s = p[T.pa[k]] * p[T.pb[k]];
      for (int i = 0; i < n; ++i) s = s - p[L[i]];
      p[k] = s;
    }
  }
  double v = V0;
  for (int i = 0; i < T.nbasis; ++i) v = v + C[i] * p[T.basis[i]];
  *V = v;
  if (!want_grad) return;
  for (int d = 0; d < T.nvar; ++d) {
    for (int k = 0; k < T.nmono; ++k) {
      if (T.mo[k] == 0) dm[d][k] = 0.0;
      else if (T.mo[k] == 1) dm[d][k] = (T.ma[k] == d) ? dmsdr_diag[d] : 0.0;
      else dm[d][k] = dm[d][T.ma[k]] * rm[T.mb[k]] + rm[T.ma[k]] * dm[d][T.mb[k]];
    }
    for (int k = 0; k < T.npoly; ++k) {
      const short* L = T.plist + T.poff[k];
      int n = T.plen[k];
      if (T.po[k] == 0) {
        double s = dm[d][L[0]];
        for (int i = 1; i < n; ++i) s = s + dm[d][L[i]];
        dp[d][k] = s;
      } else {
        double s = dp[d][T.pa[k]] * p[T.pb[k]] + p[T.pa[k]] * dp[d][T.pb[k]];
        for (int i = 0; i < n; ++i) s = s - dp[d][L[i]];
        dp[d][k] = s;
      }
    }
    double g = 0.0;
    for (int j = 0; j < T.nbasis; ++j) g = g + C[j] * dp[d][T.basis[j]];
    dV[d] = g;
  }
}

/* Basis functions B_1..B_nbasis at the variables x (EvMono/EvPoly/evbas order; bemsav49 and
 * bmx2b109 of N4_UMN_PIPNN_PES_Class.F90:1004-1466, 1753-1830 for table 1), and, if babs is given,
 * the same graph on absolute values (|p_a||p_b| + sum |p_c|), the scale of each basis function's
 * rounding error. */
void orc_pip_basis(int table, const double* x, double* b, double* babs) {
  pip_tab T = pip_table(table);
  double rm[128], p[480], ra[128], pa[480];
  for (int k = 0; k < T.nmono; ++k) {
    if (T.mo[k] == 0) { rm[k] = 1.0; ra[k] = 1.0; }
    else if (T.mo[k] == 1) { rm[k] = x[T.ma[k]]; ra[k] = fabs(x[T.ma[k]]); }
    else { rm[k] = rm[T.ma[k]] * rm[T.mb[k]]; ra[k] = ra[T.ma[k]] * ra[T.mb[k]]; }
  }
  for (int k = 0; k < T.npoly; ++k) {
    const short* L = T.plist + T.poff[k];
    const int n = T.plen[k];
    double s, sa = 0.0;
    if (T.po[k] == 0) {
      s = rm[L[0]];
      for (int i = 1; i < n; ++i) s = s + rm[L[i]];
      for (int i = 0; i < n; ++i) sa += ra[L[i]];
    } else {
      s = p[T.pa[k]] * p[T.pb[k]];
      for (int i = 0; i < n; ++i) s = s - p[L[i]];
      sa = pa[T.pa[k]] * pa[T.pb[k]];
      for (int i = 0; i < n; ++i) sa += pa[L[i]];
    }
    p[k] = s;
    pa[k] = sa;
  }
  for (int i = 0; i < T.nbasis; ++i) {
    b[i] = p[T.basis[i]];
    if (babs) babs[i] = pa[T.basis[i]];
  }
}

/* Condition scale of the PIP sum: the same graph evaluated on absolute values (|p_a||p_b| +
 * sum |p_c| at every node, and likewise for the derivatives), i.e. the standard bound on how
 * far any other evaluation order of these sums can move the result divided by the unit
 * roundoff.  scale[0] for V, scale[1 + d] for dV/dvar_d. */
void orc_pip_scale(int table, const double* rms, const double* dmsdr_diag, const double* C, double* scale) {
  pip_tab T = pip_table(table);
  double rm[128], p[480], dm[128], dp[480];
  for (int k = 0; k < T.nmono; ++k) {
    if (T.mo[k] == 0) rm[k] = 1.0;
    else if (T.mo[k] == 1) rm[k] = fabs(rms[T.ma[k]]);
    else rm[k] = rm[T.ma[k]] * rm[T.mb[k]];
  }
  for (int k = 0; k < T.npoly; ++k) {
    const short* L = T.plist + T.poff[k];
    double s = 0.0;
    if (T.po[k] == 0) { for (int i = 0; i < T.plen[k]; ++i) s += rm[L[i]]; }
    else { s = p[T.pa[k]] * p[T.pb[k]]; for (int i = 0; i < T.plen[k]; ++i) s += p[L[i]]; }
    p[k] = s;
  }
  double v = 0.0;
  for (int i = 0; i < T.nbasis; ++i) v += fabs(C[i]) * p[T.basis[i]];
  scale[0] = v;
  for (int d = 0; d < T.nvar; ++d) {
    for (int k = 0; k < T.nmono; ++k) {
      if (T.mo[k] == 0) dm[k] = 0.0;
      else if (T.mo[k] == 1) dm[k] = (T.ma[k] == d) ? fabs(dmsdr_diag[d]) : 0.0;
      else dm[k] = dm[T.ma[k]] * rm[T.mb[k]] + rm[T.ma[k]] * dm[T.mb[k]];
    }
    for (int k = 0; k < T.npoly; ++k) {
      const short* L = T.plist + T.poff[k];
      double s = 0.0;
      if (T.po[k] == 0) { for (int i = 0; i < T.plen[k]; ++i) s += dm[L[i]]; }
      else { s = dp[T.pa[k]] * p[T.pb[k]] + p[T.pa[k]] * dp[T.pb[k]]; for (int i = 0; i < T.plen[k]; ++i) s += dp[L[i]]; }
      dp[k] = s;
    }
    double g = 0.0;
    for (int j = 0; j < T.nbasis; ++j) g += fabs(C[j]) * dp[T.basis[j]];
    scale[1 + d] = g;
  }
}

/* Condition scale of a 3-atom surface evaluation at distances R [bohr]: scale[0] for V [Eh],
 * scale[1..3] for dV/dR [Eh/bohr] (PIP terms plus the diatomic terms' magnitudes). */
static void o3nn_scale(const orc_sys* s, const orc_pes* P, const double* R, double* scale);
static void n4pipnn_scale(const orc_pes* P, const double* R, double* scale);

void orc_pes_scale(const orc_sys* s, int ipes, const double* R, double* scale) {
  const orc_pes* P = &s->pes[ipes];
  double rms[6] = {0}, dms[6] = {0}, sc[7];
  if (P->model == ORC_PES_O3_NN || P->model == ORC_PES_O3_BNN) {
    o3nn_scale(s, P, R, scale);
    return;
  }
  if (P->model == ORC_PES_N4_PIPNN) {
    n4pipnn_scale(P, R, scale);
    return;
  }
  if (P->model == ORC_PES_O4_UMN || P->model == ORC_PES_N4_UMN) {   /* scale[0] for V, scale[1..6] per pair */
    const int n4 = P->model == ORC_PES_N4_UMN;
    for (int i = 0; i < 6; ++i) {
      double r = R[i] * B_TO_ANG;
      double d1 = n4 ? r - 1.098 : r - P->ra, d2 = n4 ? r - 1.098 : r - P->rb;
      double ia = n4 ? 1.0 : 1.0 / P->a, iab = n4 ? 1.0 / 1.5 : 1.0 / P->ab;
      double e = exp(-(d1 * ia) - (d2 * d2) * iab);
      rms[i] = e; dms[i] = (-(2.0 * d2 * iab) - ia) * e;
    }
    orc_pip_scale(n4 ? 1 : 2, rms, dms, P->coef, sc);
    scale[0] = (sc[0] + (n4 ? 457.4 : 0.0)) * KCM_TO_HARTREE;
    for (int i = 0; i < 6; ++i) {
      double sv, sdv;
      orc_diat_scale(s->diat, R[i], &sv, &sdv);
      scale[0] += sv;
      scale[1 + i] = sc[1 + i] * KCM_TO_HARTREE * B_TO_ANG + sdv;
    }
    return;
  }
  if (P->model == ORC_PES_O3_UMN) {
    for (int i = 0; i < 3; ++i) {
      double r = R[i] * B_TO_ANG, d1 = r - P->ra, d2 = r - P->rb;
      double e = exp(-(d1 / P->a) - (d2 * d2) / P->ab);
      rms[i] = e; dms[i] = (-(2.0 * d2 / P->ab) - 1.0 / P->a) * e;
    }
    orc_pip_scale(0, rms, dms, P->coef, sc);
    scale[0] = sc[0] * KCM_TO_HARTREE;
    for (int i = 0; i < 3; ++i) scale[1 + i] = sc[1 + i] * KCMANG_TO_HARTB;
  } else {
    double rt[6] = {R[0], R[1], 1.e3, R[2], 1.e3, 1.e3};
    for (int i = 0; i < 6; ++i) {
      double d = rt[i] * B_TO_ANG - 1.098, e = exp(-d - (d * d) / 1.5);
      rms[i] = e; dms[i] = (-(2.0 * d / 1.5) - 1.0) * e;
    }
    orc_pip_scale(1, rms, dms, P->coef, sc);
    scale[0] = (sc[0] + 457.4) * KCM_TO_HARTREE;
    scale[1] = sc[1] * KCM_TO_HARTREE * B_TO_ANG;
    scale[2] = sc[2] * KCM_TO_HARTREE * B_TO_ANG;
    scale[3] = sc[4] * KCM_TO_HARTREE * B_TO_ANG;
  }
  for (int i = 0; i < 3; ++i) {
    double sv, sdv;
    orc_diat_scale(s->diat, R[i], &sv, &sdv);
    scale[0] += sv;
    scale[1 + i] += sdv;
  }
}

/* ------------------------------------------------------------------------------------------ */
/* TransToCart (src/PESs/PES_Class.F90:252-360, implementation 2)                              */
/* ------------------------------------------------------------------------------------------ */
static void trans_to_cart_3(const double* mMiMn, const double* R, const double* Q, const double* dVdR,
                            double* m) {
  double Rx[3] = {Q[0] - Q[3], Q[0] - Q[6], Q[3] - Q[6]};
  double Ry[3] = {Q[1] - Q[4], Q[1] - Q[7], Q[4] - Q[7]};
  double Rz[3] = {Q[2] - Q[5], Q[2] - Q[8], Q[5] - Q[8]};
  double d[3];
  for (int i = 0; i < 3; ++i) d[i] = dVdR[i] / R[i];
  double m1 = mMiMn[0], m2 = mMiMn[1];
  m[0] = d[0] * Rx[0] + (1.0 - m1) * d[1] * Rx[1] - m1 * d[2] * Rx[2];
  m[1] = d[0] * Ry[0] + (1.0 - m1) * d[1] * Ry[1] - m1 * d[2] * Ry[2];
  m[2] = d[0] * Rz[0] + (1.0 - m1) * d[1] * Rz[1] - m1 * d[2] * Rz[2];
  m[3] = -(d[0] * Rx[0]) - m2 * d[1] * Rx[1] + (1.0 - m2) * d[2] * Rx[2];
  m[4] = -(d[0] * Ry[0]) - m2 * d[1] * Ry[1] + (1.0 - m2) * d[2] * Ry[2];
  m[5] = -(d[0] * Rz[0]) - m2 * d[1] * Rz[1] + (1.0 - m2) * d[2] * Rz[2];
}

static void trans_to_cart_4(const double* mMiMn, const double* R, const double* Q, const double* dVdR,
                            double* m) {
  double Rx[6] = {Q[0] - Q[3], Q[0] - Q[6], Q[0] - Q[9], Q[3] - Q[6], Q[3] - Q[9], Q[6] - Q[9]};
  double Ry[6] = {Q[1] - Q[4], Q[1] - Q[7], Q[1] - Q[10], Q[4] - Q[7], Q[4] - Q[10], Q[7] - Q[10]};
  double Rz[6] = {Q[2] - Q[5], Q[2] - Q[8], Q[2] - Q[11], Q[5] - Q[8], Q[5] - Q[11], Q[8] - Q[11]};
  double d[6];
  for (int i = 0; i < 6; ++i) d[i] = dVdR[i] / R[i];
  double m1 = mMiMn[0], m2 = mMiMn[1], m3 = mMiMn[2];
  const double* RR[3] = {Rx, Ry, Rz};
  for (int c = 0; c < 3; ++c) {
    const double* X = RR[c];
    m[0 + c] = d[0] * X[0] + d[1] * X[1] + (1.0 - m1) * d[2] * X[2] - m1 * d[4] * X[4] - m1 * d[5] * X[5];
    m[3 + c] = -(d[0] * X[0]) - m2 * d[2] * X[2] + d[3] * X[3] + (1.0 - m2) * d[4] * X[4] - m2 * d[5] * X[5];
    m[6 + c] = -(d[1] * X[1]) - m3 * d[2] * X[2] - d[3] * X[3] - m3 * d[4] * X[4] + (1.0 - m3) * d[5] * X[5];
  }
}

/* ------------------------------------------------------------------------------------------ */
/* Surfaces                                                                                   */
/* ------------------------------------------------------------------------------------------ */
/* O3 UMN: Compute_O3_UMN_PES_1d (O3_UMN_PES_Class.F90:259-326), O3_UMN_Potential_From_R (153-191) */
static void o3_compute(const orc_sys* s, const orc_pes* P, const double* R, const double* Qall, double* V,
                       double* dVdR, double* dVdQ) {
  double rang[3], rms[3], dms[3], vp, dvp[3];
  for (int i = 0; i < 3; ++i) {
    rang[i] = R[i] * B_TO_ANG;
    double d1 = rang[i] - P->ra, d2 = rang[i] - P->rb;
    double e = exp(-(d1 / P->a) - (d2 * d2) / P->ab);
    rms[i] = e;
    dms[i] = (-(2.0 * d2 / P->ab) - 1.0 / P->a) * e;
  }
  double vd[3], dvd[3];
  if (dVdR) {
    for (int i = 0; i < 3; ++i) orc_diat_VdV(s->diat, R[i], &vd[i], &dvd[i]);
  } else {
    for (int i = 0; i < 3; ++i) vd[i] = orc_diat_V(s->diat, R[i]);
  }
  double vdiat = (vd[0] + vd[1]) + vd[2];
  orc_pip_eval(0, rms, dms, dVdR != 0, P->coef, 0.0, &vp, dvp);
  *V = (vp * KCM_TO_HARTREE) + vdiat;
  if (!dVdR) return;
  for (int i = 0; i < 3; ++i) dVdR[i] = dvp[i] * KCMANG_TO_HARTB + dvd[i];
  trans_to_cart_3(s->mMiMn, R, Qall, dVdR, dVdQ);
}

/* N3 UMN: Compute_N3_UMN_PES_1d (N3_UMN_PES_Class.F90:332-382) -> n4pes (442-489) */
static void n3_compute(const orc_sys* s, const orc_pes* P, const double* R, const double* Qall, double* V,
                       double* dVdR, double* dVdQ) {
  const double a = 1.0, ab = 1.5, re = 1.098, totdiss = 457.4, eref = 0.0;
  double rt[6], rms[6], dms[6], vp, dvp[6];
  for (int i = 0; i < 6; ++i) rt[i] = 1.e3;             /* RTemp = 1.e3 (default-real literal) */
  rt[0] = R[0]; rt[1] = R[1]; rt[3] = R[2];
  for (int i = 0; i < 6; ++i) {
    double r = rt[i] * B_TO_ANG, d = r - re;
    double e = exp(-(d / a) - (d * d) / ab);          /* EvMorse 624-641 */
    rms[i] = e;
    dms[i] = (-(2.0 * d / ab) - 1.0 / a) * e;          /* EvdMsdR 646-672 */
  }
  double vdiat = 0.0, dd[3];
  for (int i = 0; i < 3; ++i) {
    double v;
    if (dVdR) orc_diat_VdV(s->diat, R[i], &v, &dd[i]);
    else v = orc_diat_V(s->diat, R[i]);
    vdiat = vdiat + v;
  }
  orc_pip_eval(1, rms, dms, dVdR != 0, P->coef, totdiss, &vp, dvp);
  double vt = (vp + eref) * KCM_TO_HARTREE;
  *V = vdiat + vt;
  if (!dVdR) return;
  for (int i = 0; i < 6; ++i) dvp[i] = dvp[i] * KCM_TO_HARTREE * B_TO_ANG;
  dVdR[0] = dd[0] + dvp[0];
  dVdR[1] = dd[1] + dvp[1];
  dVdR[2] = dd[2] + dvp[3];
  trans_to_cart_3(s->mMiMn, R, Qall, dVdR, dVdQ);
}

/* N4 UMN: Compute_N4_UMN_PES_1d (N4_UMN_PES_Class.F90:329-361) -> n4pes (373-417): the N4 PIP on
 * all six MEG variables, Eref = 0 (line 102), V = VTriat + VDiat. */
static void n4_compute(const orc_sys* s, const orc_pes* P, const double* R, const double* Qall, double* V,
                       double* dVdR, double* dVdQ) {
  const double a = 1.0, ab = 1.5, re = 1.098, totdiss = 457.4, eref = 0.0;
  double rms[6], dms[6], vp, dvp[6], vdiat = 0.0, dd[6];
  for (int i = 0; i < 6; ++i) {
    double v;
    if (dVdR) orc_diat_VdV(s->diat, R[i], &v, &dd[i]);
    else v = orc_diat_V(s->diat, R[i]);
    vdiat = vdiat + v;
  }
  for (int i = 0; i < 6; ++i) {
    double r = R[i] * B_TO_ANG, d = r - re;
    double e = exp(-(d / a) - (d * d) / ab);          /* EvMorse 551-568 */
    rms[i] = e;
    dms[i] = (-(2.0 * d / ab) - 1.0 / a) * e;          /* EvdMsdR 573-599 */
  }
  orc_pip_eval(1, rms, dms, dVdR != 0, P->coef, totdiss, &vp, dvp);
  double vt = vp * KCM_TO_HARTREE + eref;
  *V = vt + vdiat;
  if (!dVdR) return;
  for (int i = 0; i < 6; ++i) dVdR[i] = dvp[i] * KCM_TO_HARTREE * B_TO_ANG + dd[i];
  trans_to_cart_4(s->mMiMn, R, Qall, dVdR, dVdQ);
}

/* ------------------------------------------------------------------------------------------ */
/* N4 UMN PIPNN (N4_UMN_PIPNN_PES_Class.F90).  Packed as UseSurface(3), iFunc, NInput, NHid1, */
/* NHid2, NOutput, then networks a, b, c.  Initialize (176-330) reads the three networks into */
/* one set of layer sizes and one iFunc, so the last network's are the ones every network is  */
/* evaluated with.                                                                              */
/* ------------------------------------------------------------------------------------------ */
#define PIPNN_HDR 8
static const double PIPNN_VINF[3] = {-0.021346263746904, -0.196886061330806, -0.030606048118131};  /* 96 */

static int pipnn_net_size(int nin, int h1, int h2) { return 2 * (nin + 1) + nin * h1 + h1 + h1 * h2 + 2 * h2 + 1; }

static double pipnn_tranfun(double x, int ifunc) {          /* tranfun 962-984 */
  if (ifunc == 1) return tanh(x);
  if (ifunc == 2) return 1.0 / (1.0 + exp(-x));
  return x;
}

/* getpot (743-799): normalised input, hidden layers with iFunc, linear output, de-normalised */
double orc_pipnn_net(const double* c, int k, const double* x) {
  const int ifunc = (int)c[3], nin = (int)c[4], h1 = (int)c[5], h2 = (int)c[6];
  const double* pdel = c + PIPNN_HDR + k * pipnn_net_size(nin, h1, h2);
  const double *pavg = pdel + nin + 1, *W1 = pavg + nin + 1, *b1 = W1 + nin * h1, *W2 = b1 + h1, *b2 = W2 + h1 * h2,
               *W3 = b2 + h2, *b3 = W3 + h2;
  double y0[512], y1[64], y2[256];
  for (int i = 0; i < nin; ++i) y0[i] = (x[i] - pavg[i]) / pdel[i];
  for (int j = 0; j < h1; ++j) {
    double a = b1[j];
    for (int i = 0; i < nin; ++i) a = a + y0[i] * W1[i + nin * j];
    y1[j] = pipnn_tranfun(a, ifunc);
  }
  for (int j = 0; j < h2; ++j) {
    double a = b2[j];
    for (int i = 0; i < h1; ++i) a = a + y1[i] * W2[i + h1 * j];
    y2[j] = pipnn_tranfun(a, ifunc);
  }
  double o = b3[0];
  for (int i = 0; i < h2; ++i) o = o + y2[i] * W3[i];
  return o * pdel[nin] + pavg[nin];
}

/* Magnitude of network k's output sum at x: |pdel_out| (|b3| + sum |W3_k h2_k|) + |pavg_out|, the
 * scale of the cancellation in its de-normalised output. */
static double pipnn_net_magnitude(const double* c, int k, const double* x) {
  const int ifunc = (int)c[3], nin = (int)c[4], h1 = (int)c[5], h2 = (int)c[6];
  const double* pdel = c + PIPNN_HDR + k * pipnn_net_size(nin, h1, h2);
  const double *pavg = pdel + nin + 1, *W1 = pavg + nin + 1, *b1 = W1 + nin * h1, *W2 = b1 + h1, *b2 = W2 + h1 * h2,
               *W3 = b2 + h2, *b3 = W3 + h2;
  double y1[64];
  for (int j = 0; j < h1; ++j) {
    double a = b1[j];
    for (int i = 0; i < nin; ++i) a = a + ((x[i] - pavg[i]) / pdel[i]) * W1[i + nin * j];
    y1[j] = pipnn_tranfun(a, ifunc);
  }
  double s = fabs(b3[0]);
  for (int j = 0; j < h2; ++j) {
    double a = b2[j];
    for (int i = 0; i < h1; ++i) a = a + y1[i] * W2[i + h1 * j];
    s += fabs(W3[j] * pipnn_tranfun(a, ifunc));
  }
  return s * fabs(pdel[nin]) + fabs(pavg[nin]);
}

/* n4pipNN (450-657) energy in kcal/mol at the six bond lengths rb [Ang]: the N2 pair terms, the
 * basis of exp(-rb / alpha) (alpha = 1), the mean of the selected networks in eV, minus VInf. */
double orc_pipnn_kcal(const double* c, const double* rb) {
  double vn2 = 0.0, x[6], b[512];
  for (int i = 0; i < 6; ++i) {
    double v;
    n2p_ev2gm2(rb[i], &v, 0);
    vn2 = vn2 + v;
  }
  for (int i = 0; i < 6; ++i) x[i] = exp(-(rb[i] / 1.0));
  orc_pip_basis(1, x, b, 0);
  double vs[3] = {0.0, 0.0, 0.0}, vinf = 0.0;
  int nuse = 0;
  for (int k = 0; k < 3; ++k)
    if (c[k] == 1.0) {
      vs[k] = orc_pipnn_net(c, k, b);
      vinf = vinf + PIPNN_VINF[k];
      nuse += 1;
    }
  vinf = vinf / nuse;
  const double v = ((vs[0] + vs[1]) + vs[2]) / nuse;
  return (v * 23.0605 + vn2) - vinf;
}

/* Compute_N4_UMN_PIPNN_PES_1d (410-439): V, dVdR from n4pipNN's central differences (dr = 1e-5 Ang,
 * the bond lengthened, then shortened by 2 dr, then restored, one bond at a time), dVdQ = 0. */
static void n4pipnn_compute(const orc_sys* s, const orc_pes* P, const double* R, double* V, double* dVdR,
                            double* dVdQ) {
  double rb[6];
  for (int i = 0; i < 6; ++i) rb[i] = R[i] * B_TO_ANG;
  *V = orc_pipnn_kcal(P->coef, rb) * KCM_TO_HARTREE;
  if (!dVdR) return;
  const double dr = 1.0e-5;
  for (int i = 0; i < 6; ++i) {
    rb[i] = rb[i] + dr;
    const double vp = orc_pipnn_kcal(P->coef, rb);
    rb[i] = rb[i] - 2.0 * dr;
    const double vm = orc_pipnn_kcal(P->coef, rb);
    dVdR[i] = ((vp - vm) / (2.0 * dr)) * KCMANG_TO_HARTB;
    rb[i] = rb[i] + dr;
  }
  for (int i = 0; i < s->neqtvar; ++i) dVdQ[i] = 0.0;
}

/* Scale of the PIPNN energy [Eh]: the magnitudes of the terms summed at the top (the pair terms,
 * 23.0605 times the selected networks' output magnitudes, VInf), each carrying the cancellation
 * below it; and of each central difference [Eh/bohr]: that scale over 2 dr. */
static void n4pipnn_scale(const orc_pes* P, const double* R, double* scale) {
  const double* c = P->coef;
  double x[6], b[512], sv = 0.0;
  for (int i = 0; i < 6; ++i) {
    double a, d;
    const double rb = R[i] * B_TO_ANG;
    n2p_scale(rb, &a, &d);
    sv += a;
    x[i] = exp(-rb);
  }
  orc_pip_basis(1, x, b, 0);
  int nuse = 0;
  double sn = 0.0, vinf = 0.0;
  for (int k = 0; k < 3; ++k)
    if (c[k] == 1.0) { sn += pipnn_net_magnitude(c, k, b); vinf += fabs(PIPNN_VINF[k]); nuse += 1; }
  const double skcal = 23.0605 * sn / nuse + sv + vinf / nuse;
  scale[0] = skcal * KCM_TO_HARTREE;
  for (int i = 0; i < 6; ++i) scale[1 + i] = skcal / 2.0e-5 * KCMANG_TO_HARTB;
}

/* O4 UMN: Compute_O4_UMN_PES_1d (O4_UMN_PES_Class.F90:269-298) -> O4pes (310-370) */
static void o4_compute(const orc_sys* s, const orc_pes* P, const double* R, const double* Qall, double* V,
                       double* dVdR, double* dVdQ) {
  double rms[6], dms[6], vp, dvp[6];
  double vdiat = 0.0, dd[6];
  for (int i = 0; i < 6; ++i) {
    double v;
    if (dVdR) orc_diat_VdV(s->diat, R[i], &v, &dd[i]);
    else v = orc_diat_V(s->diat, R[i]);
    vdiat = vdiat + v;
  }
  for (int i = 0; i < 6; ++i) {
    double r = R[i] * B_TO_ANG, d1 = r - P->ra, d2 = r - P->rb;
    double e = exp(-(d1 / P->a) - (d2 * d2) / P->ab);  /* EvMorse 510-531 */
    rms[i] = e;
    dms[i] = (-(2.0 * d2 / P->ab) - 1.0 / P->a) * e;   /* EvdMsdR 536-566 */
  }
  orc_pip_eval(2, rms, dms, dVdR != 0, P->coef, 0.0, &vp, dvp);
  double vt = vp * KCM_TO_HARTREE;
  *V = vt + vdiat;
  if (!dVdR) return;
  for (int i = 0; i < 6; ++i) dVdR[i] = dvp[i] * KCM_TO_HARTREE * B_TO_ANG + dd[i];
  trans_to_cart_4(s->mMiMn, R, Qall, dVdR, dVdQ);
}


/* O3 NN (O3_NN_PES_Class.F90).  Compute (357-477) evaluates the six symmetric features
 * G = [sum p_i p_j, p1 p2 p3, sum p_i^2 p_j, sum p_i^3 p_j, p1 p2 p3 sum p_i, sum p_i^2 p_j^2] of
 * p = exp(-Lambda (R - re)) through the tanh-tanh-linear network; Potential (250-297), which the
 * Hamiltonian calls, evaluates three features, scaled by Scaling_MEAN/SD, through
 * dgemm(..., W1, 3, ...), i.e. on the leading 3 x NHL1 block of W1's storage read with leading
 * dimension 3.  The two therefore differ; both are kept as the reference has them. */
#define EV_TO_HARTREE (1.0 / 27.2113839712790)
typedef struct {
  int h1, h2, bnn;
  double lam, re, mean[3], sd[3], ysc, b3, noise;
  const double *W1, *b1, *W2, *b2, *W3;
} nn_view;

/* BNN_PES_Class.F90: one posterior sample (ReadParamPost_BNN, 686-770) is this layout followed by
 * its Noise; Compute (565-640) and Potential (395-442) are the NN's two networks with the output
 * passed through VExp = exp(V + Noise): V = (VExp - y_Scaling) eV_To_Hartree + sum(VDiat) and
 * dVdR = VExp sum(dVTemp) eV_To_Hartree + dVDiat. */
static nn_view nn_unpack(const double* c, int bnn) {
  nn_view v;
  v.bnn = bnn;
  v.h1 = (int)c[0]; v.h2 = (int)c[1];
  v.lam = c[2]; v.re = c[3];
  for (int i = 0; i < 3; ++i) { v.mean[i] = c[4 + i]; v.sd[i] = c[7 + i]; }
  v.ysc = c[10];
  const double* q = c + 11;
  v.W1 = q; q += 6 * v.h1;
  v.b1 = q; q += v.h1;
  v.W2 = q; q += v.h1 * v.h2;
  v.b2 = q; q += v.h2;
  v.W3 = q; q += v.h2;
  v.b3 = *q;
  v.noise = bnn ? q[1] : 0.0;
  return v;
}

int orc_o3bnn_ncoef(int h1, int h2) { return 13 + 7 * h1 + h1 * h2 + 2 * h2; }

int orc_o3nn_ncoef(int h1, int h2) { return 12 + 7 * h1 + h1 * h2 + 2 * h2; }

static void o3nn_compute(const orc_sys* s, const orc_pes* P, const double* R, const double* Qall, double* V,
                         double* dVdR, double* dVdQ) {
  const nn_view n = nn_unpack(P->coef, P->model == ORC_PES_O3_BNN);
  double vd[3], dvd[3], p[3];
  for (int i = 0; i < 3; ++i) orc_diat_VdV(s->diat, R[i], &vd[i], &dvd[i]);
  for (int i = 0; i < 3; ++i) p[i] = exp(-(n.lam * (R[i] - n.re)));
  const double gvp[3] = {p[0] * p[1], p[1] * p[2], p[2] * p[0]};
  const double gvs[3] = {p[1] + p[2], p[2] + p[0], p[0] + p[1]};
  const double gc[6] = {gvp[0] * p[0], gvp[0] * p[1], gvp[1] * p[1], gvp[1] * p[2], gvp[2] * p[0], gvp[2] * p[2]};
  const double gprod = (p[0] * p[1]) * p[2];
  double G[6];
  G[0] = (gvp[0] + gvp[1]) + gvp[2];
  G[1] = gprod;
  G[2] = ((((gc[0] + gc[1]) + gc[2]) + gc[3]) + gc[4]) + gc[5];
  G[3] = ((((gc[0] * p[0] + gc[1] * p[1]) + gc[2] * p[1]) + gc[3] * p[2]) + gc[4] * p[0]) + gc[5] * p[2];
  G[4] = (gc[0] * p[2] + gc[2] * p[0]) + gc[5] * p[1];
  G[5] = (gc[0] * p[1] + gc[2] * p[2]) + gc[4] * p[2];
  double psq[3], pcu[3];
  for (int i = 0; i < 3; ++i) { psq[i] = n.lam * (p[i] * p[i]); pcu[i] = n.lam * ((p[i] * p[i]) * p[i]); }
  const double psqs[3] = {psq[1] + psq[2], psq[2] + psq[0], psq[0] + psq[1]};
  const double pcus[3] = {pcu[1] + pcu[2], pcu[2] + pcu[0], pcu[0] + pcu[1]};
  const double gvps[3] = {-(n.lam * (gvp[0] + gvp[2])), -(n.lam * (gvp[1] + gvp[0])), -(n.lam * (gvp[2] + gvp[1]))};
  double dG[3][6];
  for (int r = 0; r < 3; ++r) {
    dG[r][0] = gvps[r];
    dG[r][1] = -(n.lam * gprod);
    dG[r][2] = -((2.0 * gvs[r]) * psq[r] + p[r] * psqs[r]);
    dG[r][3] = -((3.0 * gvs[r]) * pcu[r] + p[r] * pcus[r]);
    dG[r][4] = -((n.lam * gprod) * (2.0 * p[r] + gvs[r]));
    dG[r][5] = -(((2.0 * psq[r]) * psqs[r]) / n.lam);
  }
  double z1[64], y1[64], z2[64], y2[64];
  for (int j = 0; j < n.h1; ++j) {
    double acc = 0.0;
    for (int i = 0; i < 6; ++i) acc = acc + G[i] * n.W1[i + 6 * j];
    z1[j] = acc + n.b1[j];
    y1[j] = tanh(z1[j]);
  }
  for (int k = 0; k < n.h2; ++k) {
    double acc = 0.0;
    for (int j = 0; j < n.h1; ++j) acc = acc + y1[j] * n.W2[j + n.h1 * k];
    z2[k] = acc + n.b2[k];
    y2[k] = tanh(z2[k]);
  }
  double v = 0.0;
  for (int k = 0; k < n.h2; ++k) v = v + y2[k] * n.W3[k];
  v = v + n.b3;
  const double vexp = n.bnn ? exp(v + n.noise) : 1.0;
  *V = ((n.bnn ? vexp : v) - n.ysc) * EV_TO_HARTREE + ((vd[0] + vd[1]) + vd[2]);
  if (!dVdR) return;
  for (int r = 0; r < 3; ++r) {
    double dy1[64];
    for (int j = 0; j < n.h1; ++j) {
      double acc = 0.0;
      for (int i = 0; i < 6; ++i) acc = acc + dG[r][i] * n.W1[i + 6 * j];
      dy1[j] = (1.0 - y1[j] * y1[j]) * acc;
    }
    double sum = 0.0;
    for (int k = 0; k < n.h2; ++k) {
      double acc = 0.0;
      for (int j = 0; j < n.h1; ++j) acc = acc + n.W2[j + n.h1 * k] * dy1[j];
      sum = sum + (n.W3[k] * (1.0 - y2[k] * y2[k])) * acc;
    }
    dVdR[r] = (n.bnn ? vexp * sum * EV_TO_HARTREE : sum * EV_TO_HARTREE) + dvd[r];
  }
  trans_to_cart_3(s->mMiMn, R, Qall, dVdR, dVdQ);
}

static double o3nn_potential(const orc_sys* s, const orc_pes* P, const double* R) {
  const nn_view n = nn_unpack(P->coef, P->model == ORC_PES_O3_BNN);
  double vd[3], dvd[3], p[3];
  for (int i = 0; i < 3; ++i) orc_diat_VdV(s->diat, R[i], &vd[i], &dvd[i]);
  for (int i = 0; i < 3; ++i) p[i] = exp(-(n.lam * (R[i] - n.re)));
  const double gvp[3] = {p[0] * p[1], p[1] * p[2], p[2] * p[0]};
  const double gvs[3] = {p[0] + p[1], p[1] + p[2], p[2] + p[0]};
  double G[3];
  G[0] = (gvp[0] + gvp[1]) + gvp[2];
  G[1] = (p[0] * p[1]) * p[2];
  G[2] = (gvp[0] * gvs[0] + gvp[1] * gvs[1]) + gvp[2] * gvs[2];
  for (int i = 0; i < 3; ++i) G[i] = (G[i] - n.mean[i]) / n.sd[i];
  /* reference BLAS dgemm, alpha = beta = 1: C(1,j) += B(l,j) * A(1,l), l ascending */
  double y1[64];
  for (int j = 0; j < n.h1; ++j) {
    double z = n.b1[j];
    for (int l = 0; l < 3; ++l) z = z + n.W1[l + 3 * j] * G[l];
    y1[j] = tanh(z);
  }
  double v = 0.0;
  for (int k = 0; k < n.h2; ++k) {
    double z = n.b2[k];
    for (int j = 0; j < n.h1; ++j) z = z + n.W2[j + n.h1 * k] * y1[j];
    v = v + tanh(z) * n.W3[k];
  }
  v = v + n.b3;
  if (n.bnn) v = exp(v + n.noise);
  return (v - n.ysc) * EV_TO_HARTREE + ((vd[0] + vd[1]) + vd[2]);
}

/* Rounding-level scale of the O3 NN evaluation: the network evaluated on absolute values, with
 * the absolute error of each pre-activation carried through tanh (|tanh'| <= 1). */
static void o3nn_scale(const orc_sys* s, const orc_pes* P, const double* R, double* scale) {
  const nn_view n = nn_unpack(P->coef, P->model == ORC_PES_O3_BNN);
  double p[3];
  for (int i = 0; i < 3; ++i) p[i] = exp(-(n.lam * (R[i] - n.re)));
  double G[6] = {p[0] * p[1] + p[1] * p[2] + p[2] * p[0], p[0] * p[1] * p[2], 0, 0, 0, 0};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      if (i != j) { G[2] += p[i] * p[i] * p[j]; G[3] += p[i] * p[i] * p[i] * p[j]; }
  G[4] = G[1] * (p[0] + p[1] + p[2]);
  G[5] = p[0] * p[0] * p[1] * p[1] + p[1] * p[1] * p[2] * p[2] + p[0] * p[0] * p[2] * p[2];
  double a1[64], a2[64], w1g[6] = {0};
  for (int j = 0; j < n.h1; ++j) {
    double z = fabs(n.b1[j]);
    for (int i = 0; i < 6; ++i) z += fabs(G[i] * n.W1[i + 6 * j]);
    a1[j] = 1.0 + z;
  }
  double sv = fabs(n.b3) + fabs(n.ysc);
  for (int k = 0; k < n.h2; ++k) {
    double z = fabs(n.b2[k]);
    for (int j = 0; j < n.h1; ++j) z += fabs(n.W2[j + n.h1 * k]) * a1[j];
    a2[k] = 1.0 + z;
    sv += fabs(n.W3[k]) * a2[k];
  }
  /* gradient: |dG| |W1| (|W2| |W3| a2) with every factor on absolute values */
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < n.h1; ++j) {
      double t = 0.0;
      for (int k = 0; k < n.h2; ++k) t += fabs(n.W2[j + n.h1 * k]) * fabs(n.W3[k]) * a2[k];
      w1g[i] += fabs(n.W1[i + 6 * j]) * a1[j] * t;
    }
  /* BNN: VExp = exp(v + Noise) turns an absolute error e in v into VExp (e + u), and the gradient
   * carries VExp as a factor; VExp from the larger of the two networks' outputs */
  double vexp = 1.0, gfac = 1.0;
  if (n.bnn) {
    double vc, vdsum = 0.0, vdi, dvdi;
    o3nn_compute(s, P, R, 0, &vc, 0, 0);
    const double vp = o3nn_potential(s, P, R);
    for (int i = 0; i < 3; ++i) { orc_diat_VdV(s->diat, R[i], &vdi, &dvdi); vdsum += vdi; }
    const double ec = (vc - vdsum) / EV_TO_HARTREE + n.ysc, ep = (vp - vdsum) / EV_TO_HARTREE + n.ysc;
    vexp = fmax(fabs(ec), fabs(ep));
    gfac = vexp * (1.0 + sv);
    sv = vexp * (sv + fabs(n.noise) + 1.0) + fabs(n.ysc);
  }
  scale[0] = sv * EV_TO_HARTREE;
  for (int r = 0; r < 3; ++r) {
    double lp = fabs(n.lam) * 4.0 * (1.0 + p[r]) * (1.0 + p[r]) * (1.0 + p[r]);
    double t = 0.0;
    for (int i = 0; i < 6; ++i) t += lp * w1g[i];
    scale[1 + r] = t * gfac * EV_TO_HARTREE;
  }
  for (int i = 0; i < 3; ++i) {
    double sv, sdv;
    orc_diat_scale(s->diat, R[i], &sv, &sdv);
    scale[0] += sv;
    scale[1 + i] += sdv;
  }
}

void orc_pes_compute(const orc_sys* s, int ipes, const double* R, const double* Qall, double* V, double* dVdR,
                     double* dVdQ) {
  const orc_pes* P = &s->pes[ipes];
  if (P->model == ORC_PES_O3_UMN) o3_compute(s, P, R, Qall, V, dVdR, dVdQ);
  else if (P->model == ORC_PES_N3_UMN) n3_compute(s, P, R, Qall, V, dVdR, dVdQ);
  else if (P->model == ORC_PES_N4_UMN) n4_compute(s, P, R, Qall, V, dVdR, dVdQ);
  else if (P->model == ORC_PES_N4_PIPNN) n4pipnn_compute(s, P, R, V, dVdR, dVdQ);
  else if (P->model == ORC_PES_O3_NN || P->model == ORC_PES_O3_BNN) {
    if (dVdR) o3nn_compute(s, P, R, Qall, V, dVdR, dVdQ);
    else *V = o3nn_potential(s, P, R);
  } else o4_compute(s, P, R, Qall, V, dVdR, dVdQ);
}

double orc_pes_potential(const orc_sys* s, int ipes, const double* R) {
  double v;
  orc_pes_compute(s, ipes, R, 0, &v, 0, 0);
  return v;
}

double orc_const(const char* name) {
  if (!strcmp(name, "B_To_Ang")) return B_TO_ANG;
  if (!strcmp(name, "Kcm_To_Hartree")) return KCM_TO_HARTREE;
  if (!strcmp(name, "KcmAng_To_HartB")) return KCMANG_TO_HARTB;
  return 0.0;
}
