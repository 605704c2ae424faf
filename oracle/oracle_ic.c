/*
 * Oracle (test infrastructure): random-number streams and the diatom + atom initial-
 * condition sampler, restated from the CoarseAIR Fortran.  Build with -ffp-contract=off.
 */
#include <math.h>
#include <string.h>
#include "oracle.h"

#define TQ(M, i, j) (M)[(i) + 9 * (j)]
#define PI_ (acos(-1.0))

/* rand12 (src/Random/RandomVector_Module.F90:166-229): x <- a*x mod 2^64 computed in
 * base-256 digits in the reference (c = 0), then the digits are folded into a double by
 * Horner from the least-significant digit with bi = 1/256. */
double orc_rng_rand12(uint64_t* state) {
  const uint64_t a = 6364136223846793005ULL;
  *state = *state * a;
  uint64_t s = *state;
  const double bi = 3.90625E-3;
  double r = (double)(s & 0xFF);
  for (int i = 1; i < 8; ++i) r = (double)((s >> (8 * i)) & 0xFF) + r * bi;
  return r * bi;
}

/* RandsetVec (45-117): odd seed, 100-entry table warm-up */
void orc_rng_seed(orc_rng* r, int64_t iseed) {
  int64_t is = iseed;
  if (is % 2 == 0) is = is - 1;
  r->state = (uint64_t)is;
  for (int i = 0; i < 100; ++i) r->x[i] = orc_rng_rand12(&r->state);
}

/* RanddwsVec (120-163) */
double orc_rng_draw(orc_rng* r) {
  int i = (int)(99.0 * r->x[99]) + 1;
  double v = r->x[99];
  r->x[99] = r->x[i - 1];
  r->x[i - 1] = orc_rng_rand12(&r->state);
  return v;
}

/* RelativeTranslationEnergy_FromBoltzmann (Collision_Class.F90:1495-1553) */
double orc_boltzmann_er(double ttra, double randnum) {
  const double kelvin_to_hartree = 1.0 / 3.1577513E+05;
  double betai = ttra * kelvin_to_hartree;
  double er = 1.0;
  randnum = randnum - 1.0;
  for (int it = 0; it < 100000; ++it) {
    for (int k = 0; k < 4; ++k) er = (1.0 + er * (1.0 + er) + randnum * exp(er)) / er;
    double err = 0.0;
    double erri = ((1.0 + er * (1.0 + er) + randnum * exp(er)) / er) - er;
    if (erri > err) err = erri;
    er = er + erri;
    if (err <= 1.0E-5) break;
  }
  return betai * er;
}

/* ---- BondLength (StateInitDiatomAtom_Module.F90:543-730) ---- */
typedef struct bl_ctx { int diat; double xmui, vc_r2; } bl_ctx;
/* FuncRHS (837-861) */
static void bl_rhs(const void* c_, const double* r, double* d) {
  const bl_ctx* c = (const bl_ctx*)c_;
  double v, dv;
  orc_diat_VdV(c->diat, r[0], &v, &dv);
  d[0] = r[1];
  d[1] = -c->xmui * (dv - 2.0 * c->vc_r2 / ((r[0] * r[0]) * r[0]));
}
int orc_bs_generic_2(int nsteps, double relax, void (*f)(const void*, const double*, double*), const void* ctx,
                     double* y, double* x, double* h, const double* yscal);

void orc_bond_length(int diat, double xmui, double ro, double tau, double vc_r2, double vibphase, double* r,
                     double* rdot) {
  const double eps = 1.0E-08, epse = 1.0E-10;
  const int nsteps = 4, itermax = 10000;
  bl_ctx c = {diat, xmui, vc_r2};
  double tf = vibphase * tau, t = 0.0, dt = tf / 10.0;
  double y[2] = {ro, sqrt(2.0 * xmui * 0.0)};
  double ys[2];
  ys[0] = ro * epse;
  ys[1] = ys[0];
  int iter = 0;
  for (;;) {
    ++iter;
    double rem = tf - t;
    dt = dt < rem ? dt : rem;
    orc_bs_generic_2(nsteps, 0.5, bl_rhs, &c, y, &t, &dt, ys);
    if (fabs(t - tf) < eps) break;
    if (iter > itermax) break;
  }
  *r = y[0];
  *rdot = y[1];
}

/* ---- One diatom: ComputeKineticEnergy (draws for quasi-bound levels), BondLength (vibrational
 * phase draw) and Compute_Coordinates_Velocities (three orientation draws), StateInitDiatomAtom_Module.F90
 * 236-348, 543-833; atoms a, b of masses ma, mb; q, qd [dir][atom] relative to the diatom's centre. */
static void diatom_ic(const orc_sys* s, orc_rng* rng, const orc_level* L, double ma, double mb, double q[3][2],
                      double qd[3][2]) {
  double redmass_d = ma * mb / (ma + mb);
  double xmui = 1.0 / redmass_d, xmui2 = 0.5 * xmui;
  double jh = (double)L->jqn + 0.5;
  double vc_r2 = xmui2 * (jh * jh);
  if (L->egam != 0.0) {
    for (int it = 1; it < 100000; ++it) {
      double ra = orc_rng_draw(rng), rb = orc_rng_draw(rng);
      double v1 = 2.0 * ra - 1.0, v2 = 2.0 * rb - 1.0, r = v1 * v1 + v2 * v2;
      if (r >= 1.0) continue;
      double fac = sqrt(-2.0 * log(r) / r);
      double g1 = v1 * fac, g2 = v2 * fac;
      double ek = L->egam * g1 + L->eint;
      if (ek < 0.0 || ek >= L->vmax) {
        ek = L->egam * g2 + L->eint;
        if (ek < 0.0 || ek >= L->vmax) continue;
      }
      break;
    }
  }
  double vibphase = orc_rng_draw(rng);
  double bl, dbl;
  orc_bond_length(s->diat, xmui, L->ro, L->tau, vc_r2, vibphase, &bl, &dbl);
  double omega = 2.0 * sqrt(vc_r2 * xmui2) / (bl * bl);
  double fa = mb / (ma + mb), fb = -ma / (ma + mb);
  double rA = orc_rng_draw(rng), rB = orc_rng_draw(rng), rC = orc_rng_draw(rng);
  double twopi = PI_ * 2.0;
  double gam = rA * twopi, bet = acos(2.0 * (rB - 0.5)), alp = rC * twopi;
  double cb = cos(bet), sb = sin(bet), ca = cos(alp), sa = sin(alp), cg = cos(gam), sg = sin(gam);
  double u1 = cb * ca * cg - sa * sg, u2 = -(cb * ca * sg) - sa * cg;
  double w1 = cb * sa * cg + sg * ca, w2 = -(cb * sa * sg) + ca * cg;
  double uu1 = -(cb * sg * ca) - sa * cg;
  double ro_ = bl * omega;
  q[0][0] = fa * bl * u1;
  q[1][0] = fa * bl * u2;
  q[2][0] = fa * bl * sb * ca;
  q[0][1] = fb * bl * u1;
  q[1][1] = fb * bl * u2;
  q[2][1] = fb * bl * sb * ca;
  qd[0][0] = fa * (dbl * u1 + ro_ * w1);
  qd[1][0] = fa * (dbl * uu1 + ro_ * w2);
  qd[2][0] = fa * (dbl * (sb * ca) + ro_ * sb * sa);
  qd[0][1] = fb * (dbl * u1 + ro_ * w1);
  qd[1][1] = fb * (dbl * uu1 + ro_ * w2);
  qd[2][1] = fb * (dbl * (sb * ca) + ro_ * sb * sa);
}

/* ---- SetIniCondForward (Collision_Class.F90:1065-1211) for diatom (atoms 1,2) + diatom (atoms 3,4):
 * SetInitialState_DiatomDiatom (StateInitDiatomDiatom_Module.F90:86-219; state-specific: no level
 * draw) for each molecule, then CoordVeloc_FreeTotAngMom, ComputeCoordinatesVelocities,
 * ShiftCoordinates and SetPaQ (1216-1314, 1591-1849) with the projectile's atom 4 eliminated. ---- */
/* SETTING THE IMPACT PARAMETER (Collision_Class.F90:1276-1296): Traj%b is the ring's input value;
 * a negative one is replaced by a draw according to ImpParStrataType, with bmin the previous
 * ring's input value (GetImpactParamValue, ImpactParameter_Class.F90:202-221). */
static double impact_parameter(const orc_ic_cfg* cfg, orc_rng* rng) {
  double tb = -cfg->bmax, bmin = -cfg->bmin;
  if (tb < 0.0) {
    double randnum = orc_rng_draw(rng);
    if (cfg->b_mode == 0) tb = -sqrt(randnum) * tb;                          /* Circles */
    else if (cfg->b_mode == 1) tb = sqrt(bmin * bmin + randnum * (tb * tb - bmin * bmin));  /* Rings */
    else tb = bmin + randnum * (-tb - bmin);                                  /* Segments */
  }
  return tb;
}

int orc_sample_ic4(const orc_sys* s, orc_rng* rng, const orc_level* lev1, const orc_level* lev2,
                   const orc_ic_cfg* cfg, int ipes, double* paq, double* paq0, double* H0, double* erra,
                   double* bout, double* er_out) {
  const double* m = s->mass;
  double q1[3][2], qd1[3][2], q2[3][2], qd2[3][2];
  diatom_ic(s, rng, lev1, m[0], m[1], q1, qd1);
  diatom_ic(s, rng, lev2, m[2], m[3], q2, qd2);
  double er = orc_boltzmann_er(cfg->ttra, orc_rng_draw(rng));
  double b = impact_parameter(cfg, rng);
  double mt = m[0] + m[1], mp = m[2] + m[3];
  double redmass = mt * mp / (mt + mp);
  double fA = -mp / (mt + mp), fB = mt / (mt + mp);
  double qx1 = fA * cfg->dinit, qx2 = fB * cfg->dinit;
  double ver = sqrt(2.0 * er / redmass);
  double ratio = b / cfg->dinit;
  double verx = -ver * sqrt(1.0 - ratio * ratio);
  double verz = -ver * ratio;
  for (int a = 0; a < 2; ++a) {
    q1[0][a] = q1[0][a] + qx1; q1[1][a] = q1[1][a] + 0.0; q1[2][a] = q1[2][a] + 0.0;
    qd1[0][a] = qd1[0][a] + fA * verx; qd1[1][a] = qd1[1][a] + 0.0; qd1[2][a] = qd1[2][a] + fA * verz;
    q2[0][a] = q2[0][a] + qx2; q2[1][a] = q2[1][a] + 0.0; q2[2][a] = q2[2][a] + 0.0;
    qd2[0][a] = qd2[0][a] + fB * verx; qd2[1][a] = qd2[1][a] + 0.0; qd2[2][a] = qd2[2][a] + fB * verz;
  }
  int nv = s->neqtvar;   /* 9 */
  double dq[9];
  for (int d = 0; d < 3; ++d) {
    paq[nv + d] = q1[d][0]; dq[d] = qd1[d][0];
    paq[nv + 3 + d] = q1[d][1]; dq[3 + d] = qd1[d][1];
    paq[nv + 6 + d] = q2[d][0]; dq[6 + d] = qd2[d][0];
  }
  for (int i = 0; i < nv; ++i) paq[i] = 0.0;
  for (int ip = 0; ip < nv; ++ip)
    for (int i = 0; i < nv; ++i) paq[i] = paq[i] + TQ(s->Tqp, ip, i) * dq[ip];
  double Rpi[6];
  orc_hamiltonian(s, ipes, paq, H0, Rpi);
  orc_error_factor(s, s->eps, paq, erra);
  for (int i = 0; i < nv; ++i) { paq0[i] = dq[i]; paq0[nv + i] = paq[nv + i]; }
  *bout = b;
  if (er_out) *er_out = er;
  return 0;
}

/* ---- SetIniCondForward (Collision_Class.F90:1065-1211) for diatom (atoms 1,2) + atom (3) ---- */
int orc_sample_ic(const orc_sys* s, orc_rng* rng, const orc_level* levels, int nlevels, const orc_ic_cfg* cfg,
                  int ipes, double* paq, double* paq0, double* H0, double* erra, double* bout, int* ilevel,
                  double* er_out) {
  (void)ipes;
  const double* m = s->mass;
  /* SetInitialState_DiatomAtom (StateInitDiatomAtom_Module.F90:90-231) */
  int il = 0;
  double rn = orc_rng_draw(rng);
  if (!cfg->state_specific) {
    int i;
    for (i = 0; i < nlevels; ++i)
      if (levels[i].rlim >= rn) break;
    il = i < nlevels ? i : nlevels - 1;
  }
  const orc_level* L = &levels[il];
  double redmass_d = m[0] * m[1] / (m[0] + m[1]);    /* Initialize_*_DiatomicPotential: RedMass */
  double xmui = 1.0 / redmass_d, xmui2 = 0.5 * xmui;
  double jh = (double)L->jqn + 0.5;
  double vc_r2 = xmui2 * (jh * jh);
  /* ComputeKineticEnergy (236-348): draws only for quasi-bound levels (egam /= 0) */
  if (L->egam != 0.0) {
    for (int it = 1; it < 100000; ++it) {
      double ra = orc_rng_draw(rng), rb = orc_rng_draw(rng);
      double v1 = 2.0 * ra - 1.0, v2 = 2.0 * rb - 1.0, r = v1 * v1 + v2 * v2;
      if (r >= 1.0) continue;
      double fac = sqrt(-2.0 * log(r) / r);
      double g1 = v1 * fac, g2 = v2 * fac;
      double ek = L->egam * g1 + L->eint;
      if (ek < 0.0 || ek >= L->vmax) {
        ek = L->egam * g2 + L->eint;
        if (ek < 0.0 || ek >= L->vmax) continue;
      }
      break;
    }
  }
  /* BondLength with Ekin = 0 (the kinetic energy is overwritten before the call) */
  double vibphase = orc_rng_draw(rng);
  double bl, dbl;
  orc_bond_length(s->diat, xmui, L->ro, L->tau, vc_r2, vibphase, &bl, &dbl);
  double omega = 2.0 * sqrt(vc_r2 * xmui2) / (bl * bl);
  /* Compute_Coordinates_Velocities (735-833) */
  double ma = m[0], mb = m[1];
  double fa = mb / (ma + mb), fb = -ma / (ma + mb);
  double rA = orc_rng_draw(rng), rB = orc_rng_draw(rng), rC = orc_rng_draw(rng);
  double twopi = PI_ * 2.0;
  double gam = rA * twopi, bet = acos(2.0 * (rB - 0.5)), alp = rC * twopi;
  double cb = cos(bet), sb = sin(bet), ca = cos(alp), sa = sin(alp), cg = cos(gam), sg = sin(gam);
  double q[3][4], qd[3][4]; /* [dir][atom 0..2]; target atoms 0,1; projectile atom 2 */
  double u1 = cb * ca * cg - sa * sg, u2 = -(cb * ca * sg) - sa * cg;
  double w1 = cb * sa * cg + sg * ca, w2 = -(cb * sa * sg) + ca * cg;
  double ro_ = bl * omega;
  q[0][0] = fa * bl * u1;
  q[1][0] = fa * bl * u2;
  q[2][0] = fa * bl * sb * ca;
  q[0][1] = fb * bl * u1;
  q[1][1] = fb * bl * u2;
  q[2][1] = fb * bl * sb * ca;
  double uu1 = -(cb * sg * ca) - sa * cg;
  qd[0][0] = fa * (dbl * u1 + ro_ * w1);
  qd[1][0] = fa * (dbl * uu1 + ro_ * w2);
  qd[2][0] = fa * (dbl * (sb * ca) + ro_ * sb * sa);
  qd[0][1] = fb * (dbl * u1 + ro_ * w1);
  qd[1][1] = fb * (dbl * uu1 + ro_ * w2);
  qd[2][1] = fb * (dbl * (sb * ca) + ro_ * sb * sa);
  for (int d = 0; d < 3; ++d) { q[d][2] = 0.0; qd[d][2] = 0.0; }
  /* CoordVeloc_FreeTotAngMom (1216-1314) */
  double er = orc_boltzmann_er(cfg->ttra, orc_rng_draw(rng));
  double b = impact_parameter(cfg, rng);
  /* ComputeCoordinatesVelocities (1591-1670) */
  double mt = m[0] + m[1], mp = m[2];
  double redmass = mt * mp / (mt + mp);
  double fA = -mp / (mt + mp), fB = mt / (mt + mp);
  double qx1 = fA * cfg->dinit, qx2 = fB * cfg->dinit;
  double ver = sqrt(2.0 * er / redmass);
  double ratio = b / cfg->dinit;
  double verx = -ver * sqrt(1.0 - ratio * ratio);
  double verz = -ver * ratio;
  /* ShiftCoordinates (1675-1761) */
  for (int a = 0; a < 2; ++a) {
    q[0][a] = q[0][a] + qx1; q[1][a] = q[1][a] + 0.0; q[2][a] = q[2][a] + 0.0;
    qd[0][a] = qd[0][a] + fA * verx; qd[1][a] = qd[1][a] + 0.0; qd[2][a] = qd[2][a] + fA * verz;
  }
  q[0][2] = q[0][2] + qx2; q[1][2] = q[1][2] + 0.0; q[2][2] = q[2][2] + 0.0;
  qd[0][2] = qd[0][2] + fB * verx; qd[1][2] = qd[1][2] + 0.0; qd[2][2] = qd[2][2] + fB * verz;
  /* SetPaQ (1766-1849) */
  int nv = s->neqtvar;
  double dq[9];
  for (int a = 0; a < 2; ++a)
    for (int d = 0; d < 3; ++d) { paq[nv + 3 * a + d] = q[d][a]; dq[3 * a + d] = qd[d][a]; }
  for (int i = 0; i < nv; ++i) paq[i] = 0.0;
  for (int ip = 0; ip < nv; ++ip)
    for (int i = 0; i < nv; ++i) paq[i] = paq[i] + TQ(s->Tqp, ip, i) * dq[ip];
  /* Hamiltonian_0d, SetErrorFactor, SetInitialPaQ */
  double Rpi[6];
  orc_hamiltonian(s, ipes, paq, H0, Rpi);
  orc_error_factor(s, s->eps, paq, erra);
  for (int i = 0; i < nv; ++i) { paq0[i] = dq[i]; paq0[nv + i] = paq[nv + i]; }
  *bout = b;
  *ilevel = il;
  if (er_out) *er_out = er;
  return 0;
}
