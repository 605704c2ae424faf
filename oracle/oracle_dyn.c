/*
 * Oracle (test infrastructure): collision geometry, Hamilton's equations, the
 * Bulirsch-Stoer step and the end-of-collision loop, restated from the CoarseAIR
 * Fortran (src/Collision/...).  Build with -ffp-contract=off.
 */
#include <math.h>
#include <float.h>
#include <string.h>
#include "oracle.h"

#define TQ(M, i, j) (M)[(i) + 9 * (j)]

/* Gauss-Jordan inverse with partial pivoting.  The reference inverts Tqp with LAPACK
 * DGETRF/DGETRI (src/Collision/Matrix_Inversion_Module.F90:40-82); the two agree to
 * rounding.  Tpq is also accepted as an input by the CUDA library, so a caller can
 * pass the exact matrix its own LAPACK produced. */
static int invert(int n, const double* A, double* Ainv) {
  double M[9][18];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 2 * n; ++j) M[i][j] = (j < n) ? TQ(A, i, j) : (j - n == i ? 1.0 : 0.0);
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (fabs(M[r][c]) > fabs(M[p][c])) p = r;
    if (M[p][c] == 0.0) return -1;
    if (p != c)
      for (int j = 0; j < 2 * n; ++j) { double t = M[p][j]; M[p][j] = M[c][j]; M[c][j] = t; }
    double piv = M[c][c];
    for (int j = 0; j < 2 * n; ++j) M[c][j] /= piv;
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      double f = M[r][c];
      if (f == 0.0) continue;
      for (int j = 0; j < 2 * n; ++j) M[r][j] -= f * M[c][j];
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) TQ(Ainv, i, j) = M[i][n + j];
  return 0;
}

/* InitializeCollision (Collision_Class.F90:439-444) + Initialize_Transformation
 * (Transformation_Class.F90:53-128) */
int orc_sys_init(orc_sys* s) {
  int na = s->natoms;
  s->neqtvar = 3 * (na - 1);
  s->neqttot = 2 * s->neqtvar;
  s->npairs = na * (na - 1) / 2;
  for (int i = 0; i < na - 1; ++i) s->mMiMn[i] = -s->mass[i] / s->mass[na - 1];
  int N = s->neqtvar;
  memset(s->Tqp, 0, sizeof(s->Tqp));
  double xmi = 1.0 / s->mass[na - 1];
  int ic = 0;
  for (int i = 0; i < na - 1; ++i) {
    double temp1 = s->mass[i] * xmi;
    double temp = (s->mass[na - 1] + s->mass[i]) * temp1;
    for (int j = 0; j < 3; ++j) {
      TQ(s->Tqp, ic, ic) = temp;
      for (int ip = i + 1; ip < na - 1; ++ip) {
        double temp2 = temp1 * s->mass[ip];
        TQ(s->Tqp, ic, ip * 3 + j) = temp2;
        TQ(s->Tqp, ip * 3 + j, ic) = temp2;
      }
      ++ic;
    }
  }
  return invert(N, s->Tqp, s->Tpq);
}

/* Compute_Rp_CartCoord_3Atoms / _4Atoms (Collision_Class.F90:2244-2316) */
void orc_rp(const orc_sys* s, const double* Q, double* X, double* Rp) {
  const double* m = s->mMiMn;
  if (s->natoms == 3) {
    for (int c = 0; c < 3; ++c) X[c] = m[0] * Q[c] + m[1] * Q[3 + c];
    double a, b, c;
    a = Q[0] - Q[3]; b = Q[1] - Q[4]; c = Q[2] - Q[5];
    Rp[0] = sqrt(a * a + b * b + c * c);
    a = Q[0] - X[0]; b = Q[1] - X[1]; c = Q[2] - X[2];
    Rp[1] = sqrt(a * a + b * b + c * c);
    a = Q[3] - X[0]; b = Q[4] - X[1]; c = Q[5] - X[2];
    Rp[2] = sqrt(a * a + b * b + c * c);
  } else {
    for (int c = 0; c < 3; ++c) X[c] = m[0] * Q[c] + m[1] * Q[3 + c] + m[2] * Q[6 + c];
    const double* P[4] = {Q, Q + 3, Q + 6, X};
    static const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
    for (int k = 0; k < 6; ++k) {
      double a = P[pa[k]][0] - P[pb[k]][0], b = P[pa[k]][1] - P[pb[k]][1], c = P[pa[k]][2] - P[pb[k]][2];
      Rp[k] = sqrt(a * a + b * b + c * c);
    }
  }
}

/* HamiltonODESystem (src/Collision/ODE/ODE_System.F90:45-96) with Compute_PES_1d
 * (Collision_Class.F90:2148-2195).  y = [p(NEqtVar), q(NEqtVar)]. */
void orc_rhs(const orc_sys* s, int ipes, const double* y, double* yp) {
  int nv = s->neqtvar;
  for (int i = 0; i < nv; ++i) yp[nv + i] = 0.0;
  for (int i = 1; i <= nv; ++i) {
    int jmin = i % 3;
    if (jmin == 0) jmin = 3;
    for (int j = jmin; j <= nv; j += 3) yp[nv + j - 1] = yp[nv + j - 1] + TQ(s->Tpq, j - 1, i - 1) * y[i - 1];
  }
  double Qall[12], Rp[6], V, dVdR[6], dVdQ[9];
  for (int i = 0; i < nv; ++i) Qall[i] = y[nv + i];
  orc_rp(s, Qall, Qall + nv, Rp);
  orc_pes_compute(s, ipes, Rp, Qall, &V, dVdR, dVdQ);
  for (int i = 0; i < nv; ++i) yp[i] = -dVdQ[i];
}

/* Hamiltonian_0d (Collision_Class.F90:1985-2040) / Hamiltonian_1d (2046-2111) */
void orc_hamiltonian(const orc_sys* s, int ipes, const double* paq, double* H, double* Rpi) {
  int nv = s->neqtvar;
  double eki[9] = {0};
  for (int i = 1; i <= nv; ++i) {
    int jmin = i % 3;
    if (jmin == 0) jmin = 3;
    for (int j = jmin; j <= nv; j += 3) eki[i - 1] = eki[i - 1] + TQ(s->Tpq, j - 1, i - 1) * paq[j - 1];
  }
  double h = 0.0;
  for (int i = 0; i < nv; ++i) h = h + paq[i] * eki[i];
  double Q[12], Rp[6];
  for (int i = 0; i < nv; ++i) Q[i] = paq[nv + i];
  orc_rp(s, Q, Q + nv, Rp);
  double V = orc_pes_potential(s, ipes, Rp);
  for (int k = 0; k < s->npairs; ++k) Rpi[k] = 1.0 / Rp[k];
  *H = h * 0.5 + V;
}

/* SetErrorFactor (Collision_Class.F90:2320-2352): both halves use the RMS of the momenta. */
void orc_error_factor(const orc_sys* s, double eps, const double* paq, double* erra) {
  int nv = s->neqtvar;
  double ep = 0.0, eq = 0.0;
  for (int i = 0; i < nv; ++i) { ep = ep + paq[i] * paq[i]; eq = eq + paq[i] * paq[i]; }
  ep = eps * sqrt(ep / nv);
  eq = eps * sqrt(eq / nv);
  for (int i = 0; i < nv; ++i) { erra[i] = ep; erra[nv + i] = eq; }
}

/* ApplyTransformation (Collision_Class.F90:2406-2432): momenta -> velocities */
void orc_apply_transformation(const orc_sys* s, const double* paq, double* out) {
  int nv = s->neqtvar;
  for (int i = 0; i < 2 * nv; ++i) out[i] = paq[i];
  for (int i = 0; i < nv; ++i) {
    double a = 0.0;
    for (int j = 0; j < nv; ++j) a = a + TQ(s->Tpq, i, j) * paq[j];
    out[i] = a;
  }
}

/* ------------------------------------------------------------------------------------------ */
/* Bulirsch-Stoer (src/Collision/ODE/ODE_Solver.F90)                                           */
/* ------------------------------------------------------------------------------------------ */
static const int NSEQ[11] = {2, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96};

typedef void (*rhs_fn)(const void* ctx, const double* y, double* yp);

typedef struct rhs_ctx { const orc_sys* s; int ipes; } rhs_ctx;
static void rhs_traj(const void* ctx, const double* y, double* yp) {
  const rhs_ctx* c = (const rhs_ctx*)ctx;
  orc_rhs(c->s, c->ipes, y, yp);
}

/* mmidv (363-462) */
static void mmidv(int ne, rhs_fn f, const void* ctx, const double* y, const double* dydx, double htot, int nstep,
                  double* yout) {
  double yn[3][18];
  double htemp = 1.0 / (double)nstep;
  double h = htot * htemp;
  double h2 = 2.0 * h;
  for (int i = 0; i < ne; ++i) { yn[0][i] = y[i]; yn[1][i] = y[i] + h * dydx[i]; }
  int iym = 0, iyn = 1, iys = 2;
  f(ctx, yn[iyn], yout);
  for (int n = 2; n <= nstep; ++n) {
    for (int i = 0; i < ne; ++i) yn[iys][i] = yn[iym][i] + h2 * yout[i];
    int t = iym; iym = iyn; iyn = iys; iys = t;
    f(ctx, yn[iyn], yout);
  }
  for (int i = 0; i < ne; ++i) yout[i] = 0.5 * (yn[iym][i] + yn[iyn][i] + h * yout[i]);
}

/* RatPolExtrap (467-541); d is [ne][nsteps], x is [imax] */
static void ratpol(int ne, int nsteps, int iest, double xest, const double* yest, double* yz, double* d,
                   double* x) {
  const double eps = 1.0E-40;
  double fx[12];
  x[iest - 1] = xest;
  if (iest == 1) {
    for (int j = 0; j < ne; ++j) { yz[j] = yest[j]; d[j * nsteps + 0] = yest[j]; }
    return;
  }
  int m1 = iest < nsteps ? iest : nsteps;
  for (int k = 1; k <= m1 - 1; ++k) fx[k + 1] = x[iest - k - 1] / xest;
  for (int j = 0; j < ne; ++j) {
    double yy = yest[j], v = d[j * nsteps + 0], c = yy;
    d[j * nsteps + 0] = yy;
    for (int k = 2; k <= m1; ++k) {
      double b1 = fx[k] * v;
      double b = (c - v) / ((b1 - c) + eps);
      double ddy = c * b;
      c = b1 * b;
      v = d[j * nsteps + k - 1];
      d[j * nsteps + k - 1] = ddy;
      yy = yy + ddy;
      yz[j] = yy;
    }
  }
}

/* Integrate_ODE_1d (225-358) for one system of ne equations.  Returns 1 if an error term
 * was NaN (the reference stops there), else 0. */
static int bs_generic(int ne, int nsteps, int incstp, double relax, rhs_fn f, const void* ctx, double* y,
                      double* x, double* h, const double* yscal, double* smax, double* smin, int* irej,
                      int* iste) {
  double dydx[18], yseq[18], ytry[8][18], d[18 * 8], x2[11], errmax[8];
  f(ctx, y, dydx);
  memset(d, 0, sizeof(d));
  memset(x2, 0, sizeof(x2));
  for (int is = 1; is <= nsteps; ++is) {
    mmidv(ne, f, ctx, y, dydx, *h, NSEQ[is - 1], yseq);
    double htemp = 1.0 / (double)NSEQ[is - 1];
    double hh = *h * htemp;
    double fv1 = hh * hh;
    ratpol(ne, nsteps, is, fv1, yseq, ytry[is - 1], d, x2);
  }
  int nan = 0;
  for (int is = 1; is <= nsteps - 1; ++is) {
    errmax[is - 1] = 0.0;
    for (int i = 0; i < ne; ++i) {
      double e = fabs((ytry[is - 1][i] - ytry[nsteps - 1][i]) / yscal[i]);
      if (e != e) nan = 1;
      if (e > errmax[is - 1]) errmax[is - 1] = e;
    }
  }
  int iconv = 0;
  for (int is = 2; is <= nsteps; ++is) {
    int j = nsteps + 1 - is;
    if (errmax[j - 1] >= 1.0) break;
    iconv = j;
  }
  if (errmax[nsteps - 2] < 1.0) {
    *x = *x + *h;
    for (int i = 0; i < ne; ++i) y[i] = ytry[nsteps - 1][i];
    if (smin) *smin = (*smin < *h) ? *smin : *h;
    if (smax) *smax = (*smax > *h) ? *smax : *h;
    if (iste) *iste += 1;
    if (iconv < nsteps - 1 && incstp)
      *h = *h * ((double)NSEQ[nsteps - 1] / (double)NSEQ[iconv] + relax) / (1.0 + relax);
  } else {
    int k = nsteps / 2;
    if (k < 1) k = 1;
    *h = *h / (double)NSEQ[k - 1];
    if (irej) *irej += 1;
  }
  return nan;
}

int orc_bs_attempt(const orc_sys* s, int ipes, double* y, double* x, double* h, const double* yscal, double* smax,
                   double* smin, int* irej, int* iste) {
  rhs_ctx c = {s, ipes};
  return bs_generic(s->neqttot, s->nsteps, s->incstpsz, s->relax, rhs_traj, &c, y, x, h, yscal, smax, smin, irej,
                    iste);
}

/* Fixed number of BS attempts without end checks (for phase-space parity tests). */
int orc_bs_attempts(const orc_sys* s, int n, const int* ipes, double* paq, double* t, double* dt,
                    const double* erra, int nattempts) {
  int ne = s->neqttot;
  for (int k = 0; k < n; ++k) {
    for (int a = 0; a < nattempts; ++a)
      orc_bs_attempt(s, ipes[k], paq + (size_t)k * ne, t + k, dt + k, erra + (size_t)k * ne, 0, 0, 0, 0);
  }
  return n;
}

/* Integrator%Integrate (Integrator_Class.F90:422-466) for each trajectory independently:
 * ncall attempts, then Hamiltonian_1d and AssessConvergence (Trajectories_Class.F90:240-280).
 * Trajectories advance in lockstep in the reference, and each one's attempts and checks
 * depend only on its own state, so per-trajectory processing is equivalent. */
int orc_integrate(const orc_sys* s, int n, const int* ipes, double* paq, double* t, double* dt,
                  const double* erra, double* H, double* smax, double* smin, int* irej, int* iste, int* status,
                  int64_t max_attempts) {
  int ne = s->neqttot;
  double rpimax = 1.0 / s->rmax;
  for (int k = 0; k < n; ++k) {
    double* y = paq + (size_t)k * ne;
    int64_t att = 0;
    status[k] = 1;
    for (;;) {
      int bad = 0;
      for (int c = 0; c < s->ncall; ++c) {
        bad |= orc_bs_attempt(s, ipes[k], y, t + k, dt + k, erra + (size_t)k * ne, smax + k, smin + k, irej + k,
                              iste + k);
        ++att;
      }
      double Rpi[6];
      orc_hamiltonian(s, ipes[k], y, H + k, Rpi);
      if (bad) { status[k] = 2; break; }
      int conv = t[k] > s->tmax;
      for (int p = 0; p < s->npairs && !conv; ++p)
        if (Rpi[p] < rpimax) conv = 1;
      if (conv) { status[k] = 0; break; }
      if (att >= max_attempts) { status[k] = 1; break; }
    }
  }
  return n;
}

/* exposed for the IC sampler's 1-D BondLength integration (StateInitDiatomAtom_Module.F90:543-730) */
int orc_bs_generic_2(int nsteps, double relax, void (*f)(const void*, const double*, double*), const void* ctx,
                     double* y, double* x, double* h, const double* yscal) {
  return bs_generic(2, nsteps, 1, relax, f, ctx, y, x, h, yscal, 0, 0, 0, 0);
}
