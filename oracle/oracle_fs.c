/*
 * Oracle (test infrastructure): final-state analysis -- trajectory-point geometry,
 * product-pair selection and the semiclassical (v, J, arrangement) assignment --
 * restated from the CoarseAIR Fortran.  Build with -ffp-contract=off.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

#define PI_ (acos(-1.0))
static const double EPS_STAT_PTS = 1.0E-10;  /* DiatomicPotential_Class.F90:73 */
static const double RSTEP_STAT_PTS = 0.005;  /* DiatomicPotential_Class.F90:74 */
static const double EPSS = 1.0E-5;           /* Parameters_Module.F90:52 */

static double eff_pot(int diat, double r, double vc_r2) { return orc_diat_V(diat, r) + vc_r2 / (r * r); }

/* TurningPoint (DiatomicPotential_Class.F90:626-700).  Returns ier. */
int orc_turning_point(int diat, double ra, double rc, double vc_r2, double eint, int nbis, int nnew, double* rt_out) {
  double rt = 0.0;
  if (nbis > 0) {
    double va = eff_pot(diat, ra, vc_r2) - eint;
    double vc = eff_pot(diat, rc, vc_r2) - eint;
    double v2 = vc * va;
    if (v2 > 0.0 && v2 > EPS_STAT_PTS) { *rt_out = 0.0; return 1; }
    for (int it = 0; it < nbis; ++it) {
      rt = 0.5 * (ra + rc);
      double vb = eff_pot(diat, rt, vc_r2) - eint;
      v2 = vb * va;
      if (v2 > 0.0) { ra = rt; va = vb; }
      else { rc = rt; vc = vb; }
    }
  }
  for (int it = 0; it < nnew; ++it) {
    double vcen = vc_r2 / (rt * rt), vb, dvb;
    orc_diat_VdV(diat, rt, &vb, &dvb);
    double v = vb + vcen;
    double dv = dvb - 2.0 * vcen / rt;
    rt = rt + (eint - v) / dv;
  }
  *rt_out = rt;
  return 0;
}

/* GAUSSQ kind 3 (Chebyshev, second kind; GaussQuadrature_Module.F90:9-168) followed by
 * w = w / sqrt(1 - x**2) (DiatomicPotential_Class.F90:735).  The reference obtains the nodes
 * as eigenvalues of the Jacobi matrix (GBTQL2); here the closed form of the same nodes and
 * weights is used: x_k = cos(k pi/(n+1)) ascending, w_k = pi/(n+1) sin^2(k pi/(n+1)). */
static void cheb2_nodes(int n, double* x, double* w) {
  double pi = PI_;
  for (int i = 0; i < n; ++i) {
    int k = n - i;
    double th = (double)k * pi / (double)(n + 1);
    double s = sin(th);
    x[i] = cos(th);
    w[i] = pi / (double)(n + 1) * (s * s);
    w[i] = w[i] / sqrt(1.0 - x[i] * x[i]);
  }
}

/* ActionIntegral (DiatomicPotential_Class.F90:705-796), QuadratureType = 3 */
double orc_action_integral(int diat, double ri, double ro, double vc_r2, double eint, int n, double twomu) {
  double x[256], w[256];
  cheb2_nodes(n, x, w);
  double rm = (ro - ri) * 0.5;
  double rp = (ro + ri) * 0.5 + rm * x[0];
  double act = 0.0;
  for (int i = 0; i < n; ++i) {
    double ve = eff_pot(diat, rp, vc_r2);
    double e = eint - ve;
    if (!(e > 0.0)) e = -e;
    act = act + sqrt(e) * w[i];
    if (i != n - 1) rp = rp + rm * (x[i + 1] - x[i]);
  }
  return 2.0 * sqrt(twomu) * act * rm;
}

/* FindExtremum (DiatomicPotential_Class.F90:928-1009).  Returns ierr. */
int orc_find_extremum(int diat, double sig, double re, double rlim, double vc_r2, double tol, double* rout,
                      double* vout) {
  const double factor = 0.3819660115;
  double ra = re - RSTEP_STAT_PTS;
  double va = eff_pot(diat, ra, vc_r2) * sig;
  double vlast = eff_pot(diat, re, vc_r2) * sig;
  double ri = re, vtry;
  (void)va;
  for (;;) {
    ri = ri + RSTEP_STAT_PTS;
    if (ri >= rlim) {
      *rout = ri - RSTEP_STAT_PTS;
      *vout = vlast * sig;
      return 1;
    }
    vtry = eff_pot(diat, ri, vc_r2) * sig;
    if (vtry > vlast) break;
    vlast = vtry;
  }
  double rb = ri - RSTEP_STAT_PTS, vb = vlast, rc = ri, vc = vtry;
  ra = rb - RSTEP_STAT_PTS;
  (void)vc;
  for (int it = 0; it < 100000; ++it) {
    double rt1, vt1;
    if (rb - ra > rc - rb) {
      rt1 = (ra - rb) * factor + rb;
      vt1 = eff_pot(diat, rt1, vc_r2) * sig;
      if (vb < vt1) ra = rt1;
      else { rc = rb; vc = vb; rb = rt1; vb = vt1; }
    } else {
      rt1 = (rc - rb) * factor + rb;
      vt1 = eff_pot(diat, rt1, vc_r2) * sig;
      if (vb < vt1) { rc = rt1; vc = vt1; }
      else { ra = rb; va = vb; rb = rt1; vb = vt1; }
    }
    if (fabs(rc - ra) <= tol) break;
  }
  *rout = rb;
  *vout = vb * sig;
  return 0;
}

/* GammaFct (MolecularState_Class.F90:393-429) */
static double gamma_fct(double y) {
  const double g1 = -1.963510026021423;
  double sum = g1 * y;
  if (y == 0.0) return sum;
  for (int it = 0; it <= 1000000; ++it) {
    double t1 = y / (0.5 + it);
    double term = t1 - atan(t1);
    sum = sum + term;
    if (fabs(term / sum) < 1.0E-06) return sum;
  }
  return sum;
}

/* FindState (MolecularState_Class.F90:61-388).  x, xdot: [3][2] = (dir, atom). */
void orc_find_state(const orc_sys* s, int ipair, int ia, int ib, const double* X, const double* XD,
                    orc_molstate* m) {
  int diat = s->diat;
  double xma = s->mass[ia], xmb = s->mass[ib];
  double fa = xma / (xma + xmb), fb = xmb / (xma + xmb);
  double x[3][2], xd[3][2], xcm[3], xdcm[3];
  for (int i = 0; i < 3; ++i) {
    xcm[i] = fa * X[2 * i + 0] + fb * X[2 * i + 1];
    xdcm[i] = fa * XD[2 * i + 0] + fb * XD[2 * i + 1];
  }
  int itype = 1;
  double eint = 0.0, rbond = 0.0;
  for (int i = 0; i < 3; ++i) {
    x[i][0] = X[2 * i + 0] - xcm[i];
    x[i][1] = X[2 * i + 1] - xcm[i];
    xd[i][0] = XD[2 * i + 0] - xdcm[i];
    xd[i][1] = XD[2 * i + 1] - xdcm[i];
    double dd = x[i][0] - x[i][1];
    rbond = rbond + dd * dd;
    eint = eint + 0.5 * (xma * (xd[i][0] * xd[i][0]) + xmb * (xd[i][1] * xd[i][1]));
  }
  rbond = sqrt(rbond);
  double tx = 0.0, ty = 0.0, tz = 0.0;
  for (int a = 0; a < 2; ++a) {
    double mass = a == 0 ? xma : xmb;
    tx = tx + (x[1][a] * xd[2][a] - x[2][a] * xd[1][a]) * mass;
    ty = ty + (x[2][a] * xd[0][a] - x[0][a] * xd[2][a]) * mass;
    tz = tz + (x[0][a] * xd[1][a] - x[1][a] * xd[0][a]) * mass;
  }
  double tis = tx * tx + ty * ty + tz * tz;
  double angmom = sqrt(tis);
  double rms = xma * xmb / (xma + xmb);
  double twomu = rms * 2.0;
  double vc_r2 = 0.5 * tis / rms;
  double eps = EPSS;
  double vinf = orc_diat_V(diat, 1.0E+03);     /* InitializeMolecularStateParam: Vinf */
  double rmin, vmin, rmax = 0.0, vmax = 0.0, viba = 0.5;
  int ierr = orc_find_extremum(diat, 1.0, s->rsmal, s->rcent, vc_r2, eps, &rmin, &vmin);
  int imin = 1;
  if (ierr != 0) { rmin = (s->rsmal + s->rcent) * 0.5; imin = 0; }
  if (imin == 1) {
    ierr = orc_find_extremum(diat, -1.0, rmin, s->rcent, vc_r2, eps, &rmax, &vmax);
    if (ierr != 0) rmax = s->rcent;
  }
  double rb = rbond;
  if (imin == 0 || rb > rmax) {
    itype = 3;
    viba = 0.5;
  } else {
    double vib = orc_diat_V(diat, rb);
    eint = eint + vib;
    itype = (eint < vinf) ? 1 : 2;
    double r1 = rmin;
    if (eint > vmax) {
      viba = 0.5;
      itype = 3;
    } else {
      double r00 = s->rsmal, ri = 0.0, ro = 0.0;
      for (int itry = 1; itry <= 10; ++itry) {
        orc_turning_point(diat, r00, r1, vc_r2, eint, 4, 4, &ri);
        if (ri != 0.0) break;
        r00 = r00 * 0.5;
      }
      orc_turning_point(diat, r1, rmax, vc_r2, eint, 10, 4, &ro);
      viba = orc_action_integral(diat, ri, ro, vc_r2, eint, s->nquad, twomu);
      if (eint > vinf) {
        double rga = rmax, rgb = rmax * 2.0, r3 = 0.0;
        for (int ip = 1; ip <= 10; ++ip) {
          int e = orc_turning_point(diat, rga, rgb, vc_r2, eint, 10, 4, &r3);
          if (e == 0) break;
          rga = rgb;
          rgb = rgb * 2.0;
        }
        double eint_p = eint + EPSS;
        if (eint_p > vmax) eint_p = eint + 0.5 * (vmax - eint);
        double deint = eint_p - eint, rip, rop, rim, rom;
        orc_turning_point(diat, r00, r1, vc_r2, eint_p, 4, 4, &rip);
        orc_turning_point(diat, r1, rmax, vc_r2, eint_p, 10, 4, &rop);
        double act_p = orc_action_integral(diat, rip, rop, vc_r2, eint_p, s->nquad, twomu);
        double eint_m = eint - deint;
        orc_turning_point(diat, r00, r1, vc_r2, eint_m, 4, 4, &rim);
        orc_turning_point(diat, r1, rmax, vc_r2, eint_m, 10, 4, &rom);
        double act_m = orc_action_integral(diat, rim, rom, vc_r2, eint_m, s->nquad, twomu);
        double dade = 0.5 * (act_p - act_m) / deint;
        double act = orc_action_integral(diat, ro, r3, vc_r2, eint, s->nquad, twomu);
        double prob = exp(-act);
        double gam = prob / dade;
        double xlife = 1.0 / gam;
        if (xlife < s->tthresau) itype = 4;
        act = orc_action_integral(diat, ro, r3, vc_r2, eint, s->nquad, twomu) * 0.5 / PI_;
        double rho2 = gamma_fct(act) - act * (log(fabs(act)) - 1.0);
        viba = viba + rho2 * s->rfact;
      }
      viba = viba * 0.5 / PI_;
    }
  }
  itype = itype - 1;
  if (itype == 2) angmom = 0.5;
  m->ipair = ipair;
  m->itype = itype;
  m->eint = eint;
  m->angmom = angmom;
  m->viba = viba;
}

/* Analyze (TrajectoryPoint_Class.F90:128-374) with ComputeCoordAndVeloc (379-412) and
 * SetPairs (417-495); 3- and 4-atom systems. */
void orc_analyze(const orc_sys* s, const double* paq, orc_traj_point* out) {
  int n = s->natoms, nv = s->neqtvar;
  double xx[3][4], xd[3][4];
  for (int a = 0; a < n - 1; ++a)
    for (int d = 0; d < 3; ++d) { xd[d][a] = paq[d + 3 * a]; xx[d][a] = paq[d + 3 * a + nv]; }
  for (int d = 0; d < 3; ++d) {
    xd[d][n - 1] = 0.0;
    xx[d][n - 1] = 0.0;
    for (int a = 0; a < n - 1; ++a) {
      xd[d][n - 1] = xd[d][n - 1] + s->mMiMn[a] * paq[d + 3 * a];
      xx[d][n - 1] = xx[d][n - 1] + s->mMiMn[a] * paq[d + 3 * a + nv];
    }
  }
  static const int pa3[3] = {0, 0, 1}, pb3[3] = {1, 2, 2};
  static const int pa4[6] = {0, 0, 0, 1, 1, 2}, pb4[6] = {1, 2, 3, 2, 3, 3};
  const int* pa = n == 3 ? pa3 : pa4;
  const int* pb = n == 3 ? pb3 : pb4;
  int np = s->npairs;
  double rbs[6];
  int irbs[6];
  for (int p = 0; p < np; ++p) {
    double a = xx[0][pa[p]] - xx[0][pb[p]], b = xx[1][pa[p]] - xx[1][pb[p]], c = xx[2][pa[p]] - xx[2][pb[p]];
    rbs[p] = a * a + b * b + c * c;
    irbs[p] = p + 1;
  }
  /* hpsort (Sorting_Module.F90:20-83): ascending order with index */
  for (int i = 1; i < np; ++i)
    for (int j = i; j > 0 && rbs[j - 1] > rbs[j]; --j) {
      double t = rbs[j]; rbs[j] = rbs[j - 1]; rbs[j - 1] = t;
      int k = irbs[j]; irbs[j] = irbs[j - 1]; irbs[j - 1] = k;
    }
  int ip1, ip2 = 0;
  if (n == 3) {
    ip1 = irbs[0];
  } else {
    if (rbs[1] > 100.0) {
      ip1 = irbs[0] <= 3 ? irbs[0] : 7 - irbs[0];
    } else if (rbs[2] < 25.0) {   /* rmaxCluster (Input_Class.F90:166): a cluster, SetPairs 456-460 */
      out->nmol = 2;
      out->b = 0.0;
      out->xkin = 0.0;
      for (int d = 0; d < 3; ++d) out->vrel[d] = 0.0;
      for (int im = 0; im < 2; ++im) {   /* AnalyzeTrajectoryPoint 355-364 */
        out->mol[im].ipair = -1;
        out->mol[im].itype = -10;
        out->mol[im].eint = 0.0;
        out->mol[im].angmom = -1.0;
        out->mol[im].viba = -1.0;
      }
      return;
    } else {
      ip1 = irbs[0] < irbs[1] ? irbs[0] : irbs[1];
      if (ip1 > 3) ip1 = 7 - ip1;
    }
    ip2 = 7 - ip1;                               /* OppositePair_4At = [6,5,4,3,2,1] */
  }
  out->nmol = (n == 3) ? 1 : 2;
  int m1a = pa[ip1 - 1], m1b = pb[ip1 - 1];
  /* centres of mass of the molecule and of the rest */
  double cm[3][2] = {{0}}, cmd[3][2] = {{0}};
  for (int d = 0; d < 3; ++d)
    for (int j = 0; j < n; ++j) {
      int k = (j == m1a || j == m1b) ? 0 : 1;
      cm[d][k] = cm[d][k] + s->mass[j] * xx[d][j];
      cmd[d][k] = cmd[d][k] + s->mass[j] * xd[d][j];
    }
  double xp = 0.0, xt = 0.0;
  for (int j = 0; j < n; ++j) {
    if (j == m1a || j == m1b) xp = xp + s->mass[j];
    else xt = xt + s->mass[j];
  }
  double xpi = 1.0 / xp, xti = 1.0 / xt, xrel[3];
  for (int d = 0; d < 3; ++d) {
    cm[d][0] *= xpi; cm[d][1] *= xti; cmd[d][0] *= xpi; cmd[d][1] *= xti;
  }
  for (int d = 0; d < 3; ++d) { xrel[d] = cm[d][0] - cm[d][1]; out->vrel[d] = cmd[d][0] - cmd[d][1]; }
  double xnum = xrel[0] * out->vrel[0] + xrel[1] * out->vrel[1] + xrel[2] * out->vrel[2];
  double v = out->vrel[0] * out->vrel[0] + out->vrel[1] * out->vrel[1] + out->vrel[2] * out->vrel[2];
  double t = -xnum / v;
  double e0 = xrel[0] + t * out->vrel[0], e1 = xrel[1] + t * out->vrel[1], e2 = xrel[2] + t * out->vrel[2];
  out->b = sqrt(e0 * e0 + e1 * e1 + e2 * e2);
  out->xkin = 0.0;
  for (int d = 0; d < 3; ++d)
    out->xkin = out->xkin + 0.5 * xp * (cmd[d][0] * cmd[d][0]) + 0.5 * xt * (cmd[d][1] * cmd[d][1]);
  for (int im = 0; im < out->nmol; ++im) {
    int ip = im == 0 ? ip1 : ip2;
    int a = pa[ip - 1], b = pb[ip - 1];
    double X[6], XD[6];
    for (int d = 0; d < 3; ++d) {
      X[2 * d] = xx[d][a]; X[2 * d + 1] = xx[d][b];
      XD[2 * d] = xd[d][a]; XD[2 * d + 1] = xd[d][b];
    }
    orc_find_state(s, ip, a, b, X, XD, &out->mol[im]);
  }
  if (out->nmol == 1) memset(&out->mol[1], 0, sizeof(orc_molstate));
}
