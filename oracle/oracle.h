/*
 * CPU oracle for the CoarseAIR trajectory hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library is a line-by-line C restatement of the reference Fortran for the
 * path RunTrajectories -> Integrator%Integrate -> ODE (Bulirsch-Stoer) ->
 * HamiltonODESystem -> Collision%Compute_PES -> PES%Compute, plus the initial-
 * condition sampler and the final-state analysis that feed and judge it.  It is
 * the checker for the CUDA library: only the tests, the smoke check and the
 * bench's CPU-baseline leg load it.  Nothing in the product links against it.
 *
 * Every function cites the reference file:line it follows (paths relative to
 * the CoarseAIR tree).  Operation order follows the Fortran (left-to-right
 * sums, no fused multiply-add: build with -ffp-contract=off).
 *
 * Parity pinned in part.  The reference ships no golden values for these surfaces
 * or the integrator; its one independent source, the original UMN Fortran modules of
 * the O4, N4 (hence N3) and O3 2 5A' surfaces and their O2 and N2 diatomics (under
 * dtb/Systems/), pins the UMN evaluations here (tests/golden/umn_originals.json, made by
 * the script beside it).  Everything else is parity unpinned against reference outputs
 * and checked by
 * (1) the structural check of the PIP tables against the reference's own derivative
 * routines (gen_pip.py), (2) the shipped level lists read as known-answer tests of the
 * final-state chain (turning points, action integral -> v+1/2), (3) finite-difference,
 * permutation-symmetry and dissociation-limit checks of every surface, independent
 * numpy restatements of the NN and BNN networks, the random-number generator and the
 * impact-parameter rings, (4) energy conservation and time reversibility of the
 * integrator.
 */
#ifndef CAIR_ORACLE_H
#define CAIR_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_PES_O3_UMN = 1, ORC_PES_N3_UMN = 2, ORC_PES_O4_UMN = 3, ORC_PES_O3_NN = 4, ORC_PES_N4_UMN = 5,
       ORC_PES_O3_BNN = 6, ORC_PES_N4_PIPNN = 7 };
enum { ORC_DIAT_O2_UMN = 1, ORC_DIAT_N2_UMN_FORN4 = 2, ORC_DIAT_N2_UMN_PIPNN_FORN4 = 3 };

typedef struct orc_pes {
  int model;
  int ncoef;
  const double* coef;           /* UMN: C(1:ncoef) [kcal/mol].  O3 NN: NHL1, NHL2, Lambda, re,
                                   Scaling_MEAN(3), Scaling_SD(3), y_Scaling, W1(6,NHL1), b1, W2(NHL1,NHL2),
                                   b2, W3, b3 (column-major, as read by O3_NN_PES_Class.F90:74-232).
                                   N4 PIPNN: UseSurface(3), iFunc, NInput, NHid1, NHid2, NOutput, then per
                                   network pdel(NInput+1), pavg(NInput+1), W1(NInput,NHid1), b1, W2(NHid1,NHid2),
                                   b2, W3(NHid2), b3 (N4_UMN_PIPNN_PES_Class.F90:176-330) */
  double a, ab, ra, rb;         /* MEG parameters (O3, O4) */
  double eref, totdiss;         /* O4 */
} orc_pes;

typedef struct orc_sys {
  int natoms, neqtvar, neqttot, npairs;
  double mass[4];
  double mMiMn[3];
  double Tqp[81], Tpq[81];      /* column-major (i,j) -> [i + 9*j], NEqtVar x NEqtVar */
  int npes;
  orc_pes pes[64];
  int diat;
  /* integrator (Input keys "Initial time step", "Error control parameter", ...) */
  double dt0, eps, relax, rmax, tmax, hamabstol;
  int nsteps, incstpsz, ncall;
  /* final-state analysis */
  int nquad;
  double rsmal, rcent, rfact, tthresau;
} orc_sys;

/* ---- set-up ---- */
int  orc_sys_init(orc_sys* s);   /* fills neqtvar/neqttot/npairs, mMiMn, Tqp, Tpq from natoms/mass */

/* ---- diatomic potentials ---- */
double orc_diat_V(int model, double r);
void   orc_diat_VdV(int model, double r, double* v, double* dv);
void   orc_diat_scale(int model, double r, double* sv, double* sdv);   /* rounding-level scales */

/* ---- surfaces: V [Eh], dVdR [Eh/bohr], dVdQ (+dV/dq of the NAtoms-1 free atoms) ---- */
void   orc_pes_compute(const orc_sys* s, int ipes, const double* R, const double* Qall,
                       double* V, double* dVdR, double* dVdQ);
double orc_pes_potential(const orc_sys* s, int ipes, const double* R);
int    orc_o3nn_ncoef(int nhl1, int nhl2);
/* PIP part only (kcal/mol, derivatives wrt R in Angstrom), all six/three directions */
void   orc_pip_eval(int table, const double* rms, const double* dmsdr_diag, int want_grad,
                    const double* C, double V0, double* V, double* dV);

void   orc_pip_scale(int table, const double* rms, const double* dmsdr_diag, const double* C, double* scale);
/* the basis functions themselves (b[NBASIS]) and their absolute-value graph (same shape) */
void   orc_pip_basis(int table, const double* x, double* b, double* babs);
/* N4 UMN PIPNN: network k (0..2) at the basis values b, and the surface in kcal/mol at rb [Ang] */
double orc_pipnn_net(const double* coef, int k, const double* b);
double orc_pipnn_kcal(const double* coef, const double* rb);
void   orc_pes_scale(const orc_sys* s, int ipes, const double* R, double* scale);

/* ---- dynamics ---- */
void   orc_rp(const orc_sys* s, const double* Q, double* Rxyz, double* Rp);
void   orc_rhs(const orc_sys* s, int ipes, const double* y, double* yp);
void   orc_hamiltonian(const orc_sys* s, int ipes, const double* paq, double* H, double* Rpi);
int    orc_bs_attempt(const orc_sys* s, int ipes, double* y, double* x, double* h,
                      const double* yscal, double* smax, double* smin, int* irej, int* iste);
int    orc_bs_attempts(const orc_sys* s, int n, const int* ipes, double* paq, double* t, double* dt,
                       const double* erra, int nattempts);
/* Integrate trajectories to the end of the collision.  status: 0 converged, 1 attempt cap,
 * 2 non-finite error.  Returns the number of trajectories processed. */
int    orc_integrate(const orc_sys* s, int n, const int* ipes, double* paq, double* t, double* dt,
                     const double* erra, double* H, double* smax, double* smin, int* irej, int* iste,
                     int* status, int64_t max_attempts);
void   orc_error_factor(const orc_sys* s, double eps, const double* paq, double* erra);
void   orc_apply_transformation(const orc_sys* s, const double* paq, double* out);

/* ---- random numbers (Schwenke/Knuth MCG with shuffle table) ---- */
typedef struct orc_rng { uint64_t state; double x[100]; } orc_rng;
void   orc_rng_seed(orc_rng* r, int64_t iseed);
double orc_rng_draw(orc_rng* r);
double orc_rng_rand12(uint64_t* state);

/* ---- initial conditions (diatom + atom) ---- */
typedef struct orc_level {
  int vqn, jqn;
  double eint, egam, rmin, rmax, vmin, vmax, tau, ri, ro, rlim;
} orc_level;

typedef struct orc_ic_cfg {
  double ttra;          /* translational temperature [K] (Boltzmann model) */
  double bmax;          /* -(the ring's input b): > 0 sampled, < 0 the fixed value -bmax */
  double dinit;         /* initial separation [bohr] */
  int    state_specific;
  int    b_mode;        /* ImpParStrataType: 0 Circles, 1 Rings, 2 Segments */
  double bmin;          /* -(the previous ring's input b), 0 for the first ring */
} orc_ic_cfg;

/* Sample one trajectory's initial condition from the stream `rng` (draw order as the
 * reference).  Outputs PaQ (momenta+coords), PaQ0 (velocities+coords), H0, erra, b, level. */
int    orc_sample_ic(const orc_sys* s, orc_rng* rng, const orc_level* levels, int nlevels,
                     const orc_ic_cfg* cfg, int ipes,
                     double* paq, double* paq0, double* H0, double* erra, double* b, int* ilevel,
                     double* er_out);
/* diatom (atoms 1, 2; level lev1) + diatom (atoms 3, 4; level lev2), state-specific */
int    orc_sample_ic4(const orc_sys* s, orc_rng* rng, const orc_level* lev1, const orc_level* lev2,
                      const orc_ic_cfg* cfg, int ipes, double* paq, double* paq0, double* H0, double* erra,
                      double* bout, double* er_out);
void   orc_bond_length(int diat, double xmui, double ro, double tau, double vc_r2, double vibphase,
                       double* r, double* rdot);
double orc_boltzmann_er(double ttra, double randnum);

/* ---- final-state analysis ---- */
typedef struct orc_molstate {
  int ipair;            /* 1-based pair index of the molecule (0: none) */
  int itype;            /* 0 bound, 1 quasi-bound, 2 dissociated(-ish), 3 short-lived q.b. */
  double eint, angmom, viba;
} orc_molstate;

typedef struct orc_traj_point {
  orc_molstate mol[2];
  double b, xkin, vrel[3];
  int nmol;
} orc_traj_point;

/* PaQ here holds velocities + coordinates (after ApplyTransformation). */
void   orc_analyze(const orc_sys* s, const double* paq_vel, orc_traj_point* out);
void   orc_find_state(const orc_sys* s, int ipair, int ia, int ib, const double* x /*3x2*/,
                      const double* xdot /*3x2*/, orc_molstate* m);
/* Level-list known-answer helpers */
int    orc_turning_point(int diat, double ra, double rc, double vc_r2, double eint, int nbis, int nnew,
                         double* rt);
double orc_action_integral(int diat, double ri, double ro, double vc_r2, double eint, int n, double twomu);
int    orc_find_extremum(int diat, double sig, double r0, double rlim, double vc_r2, double tol,
                         double* rout, double* vout);

/* ---- statistics of one state-specific run (Histogram assignment) ---- */
int    orc_statistics(int nrows, int ncond, const int* iskip, const int* pres, int qnmax, const double* bmax,
                      const double* bsamp, const double* qini, const double* qfin, int cap, long long* codes,
                      int* fincond, int* inistate, long long* counts, double* cross, double* cross_sd);
double orc_mean_velocity(double ttra, double xmu);

/* ---- constants ---- */
double orc_const(const char* name);

#ifdef __cplusplus
}
#endif
#endif
