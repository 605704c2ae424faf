/*
 * cair_gpu.h -- C ABI of the GB300 (sm_103a) trajectory library for CoarseAIR's
 * quasi-classical trajectory hot path.
 *
 * The library replaces, for one process on one GPU, the path
 *   app/RunTrajectories/RunTrajectories.F90:277  call Integrator%Integrate(Input, Collision)
 *   -> src/Collision/Integrator_Class.F90:231-579  (batch loop, end checks, compaction)
 *   -> src/Collision/ODE/ODE_Solver.F90:225-541    (Bulirsch-Stoer step, mmidv, RatPolExtrap)
 *   -> src/Collision/ODE/ODE_System.F90:45-96      (Hamilton's equations)
 *   -> src/Collision/Collision_Class.F90:2148-2316 (Compute_PES_1d, pair distances)
 *   -> src/PESs/PES_Class.F90:43-72,252-360        (PES_Type%Compute / Potential, TransToCart)
 * and the final-state analysis of
 *   src/Collision/Trajectories/TrajectoryPoint_Class.F90:128-495 and
 *   src/Collision/MolecularState/MolecularState_Class.F90:61-429;
 * on either side of it, the initial conditions (Collision_Class.F90:1065-1849, with the
 * impact-parameter rings of ImpactParameter_Class.F90), the final-state statistics and rates
 * (app/TrajectoriesStats/Statistics_Class.F90, Process_Class.F90:122-209), and the
 * trajectories.out / trajectories.bin writers and MergeTrajectories (Integrator_Class.F90:884-933,
 * Statistics_Class.F90:283-314, scripts/executing/ComputeRates.sh:406-472).
 *
 * Conventions (those of the Fortran arrays, so a Fortran ISO_C_BINDING shim passes its
 * arrays unchanged):
 *   - FP64 everywhere; atomic units (bohr, hartree, a.u. of time, electron masses).
 *   - PaQ is stored per trajectory contiguously: paq[k*NEqtTot + i], i.e. the Fortran
 *     column-major PaQ(NEqtTot, NTraj).  PaQ = [p(1:NEqtVar), q(1:NEqtVar)], where q are
 *     the Cartesian coordinates of atoms 1..NAtoms-1 (the last atom is eliminated through
 *     the centre of mass) and p the conjugate momenta.
 *   - Pair order: 3 atoms (1-2, 1-3, 2-3); 4 atoms (1-2, 1-3, 1-4, 2-3, 2-4, 3-4).
 *   - PES indices `ipes` are 0-based here (the Fortran Traj%iPES is 1-based).
 *   - Pointers named *_host are host memory; the *_dev entry points take device pointers
 *     and a cudaStream_t passed as void*.
 *
 * Errors: every entry point returns 0 on success or a cair_status code; the message is
 * available from cair_last_error() until the next call on the same handle.  The library
 * never calls exit() or abort().  Per-trajectory numerical outcomes are reported in the
 * status[] arrays (cair_traj_status).
 *
 * Threading: a handle is used by one host thread at a time; distinct handles may be used
 * concurrently from distinct threads.  Calls are synchronous unless named *_dev: those run
 * on the given stream and return before it completes, except the statistics entry points,
 * which return their results in host memory and so synchronise with it.
 */
#ifndef CAIR_GPU_H
#define CAIR_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CAIR_MAX_PES 64
#define CAIR_ABI_VERSION 6

/* Surface models (PES_Factory_Class.F90:46-329, System x PES_Model strings). */
enum cair_pes_model {
  CAIR_PES_O3_UMN = 1, /* O3_UMN_PES_Class.F90  (System O3, Model UMN_*)            */
  CAIR_PES_N3_UMN = 2, /* N3_UMN_PES_Class.F90  (System N3, Model UMN)              */
  CAIR_PES_O4_UMN = 3, /* O4_UMN_PES_Class.F90  (System O4, Model UMN_Singlet/...)  */
  CAIR_PES_O3_NN = 4,  /* O3_NN_PES_Class.F90   (System O3, Model NN_*)             */
  CAIR_PES_N4_UMN = 5, /* N4_UMN_PES_Class.F90  (System N4, Model UMN; 4 atoms)     */
  CAIR_PES_O3_BNN = 6, /* BNN_PES_Class.F90     (System O3, Model BNN; one surface
                          per posterior sample, StochPESFlg)                        */
  CAIR_PES_N4_PIPNN = 7 /* N4_UMN_PIPNN_PES_Class.F90 (System N4, Model UMN_PIPNN,
                          UMN_PIPNN_A/_B/_C; 4 atoms)                               */
};

/* Diatomic potentials of the pairs (DiatomicPotential_Factory_Class.F90:115-229). */
enum cair_diat_model {
  CAIR_DIAT_O2_UMN = 1,            /* O2_UMN_DiatomicPotential_Class.F90             */
  CAIR_DIAT_N2_UMN_FORN4 = 2,      /* N2_UMN_ForN4_DiatomicPotential_Class.F90       */
  CAIR_DIAT_N2_UMN_PIPNN_FORN4 = 3 /* N2_UMN_PIPNN_ForN4_DiatomicPotential_Class.F90
                                      (with CAIR_PES_N4_PIPNN only)                  */
};

enum cair_status {
  CAIR_OK = 0,
  CAIR_EINVAL = 1,      /* bad argument (null pointer, size, model)            */
  CAIR_ECUDA = 2,       /* CUDA runtime error (no device, launch failure, ...) */
  CAIR_ETIMEOUT = 3,    /* host watchdog expired while waiting for the GPU     */
  CAIR_ENONFINITE = 4,  /* non-finite input                                    */
  CAIR_EUNSUPPORTED = 5 /* combination not built (e.g. 4-atom final states)    */
};

/* Per-trajectory outcome of cair_integrate. */
enum cair_traj_status {
  CAIR_TRAJ_DONE = 0,        /* t > tmax or a pair beyond rmax at an end check      */
  CAIR_TRAJ_ATTEMPT_CAP = 1, /* max_attempts reached (reference: IterMax*ncall)      */
  CAIR_TRAJ_NONFINITE = 2    /* NaN in the error estimate (reference: stop in ODE)   */
};

/* One surface: linear coefficients and MEG parameters.  Replaces the data a
 * PES%Initialize reads (O3_UMN_PES_Class.F90:67-135, O4_UMN_PES_Class.F90:118-210;
 * the N3 coefficients are inline in N3_UMN_PES_Class.F90:108-201).
 * CAIR_PES_O3_NN packs what Initialize_O3_NN_PES reads (O3_NN_PES_Class.F90:74-232) into coef:
 *   NHL1, NHL2, Lambda, re, Scaling_MEAN(3), Scaling_SD(3), y_Scaling, W1(6,NHL1), b1(NHL1),
 *   W2(NHL1,NHL2), b2(NHL2), W3(NHL2), b3
 * (matrices column-major as in Fortran), ncoef = 12 + 7 NHL1 + NHL1 NHL2 + 2 NHL2; the kernels
 * hold NHL1 <= 20, NHL2 <= 10.  CAIR_PES_O3_BNN packs one posterior sample the same way
 * (Initialize_BNN_PES and ReadParamPost_BNN, BNN_PES_Class.F90:95-200, 640-760: ScalingValues.csv
 * and CalibratedParams/<name>.csv.<sample>) followed by its Noise, ncoef one more.
 * CAIR_PES_N4_PIPNN packs what Initialize_N4_UMN_PIPNN_PES reads from Weights.dat and Biases.dat
 * (N4_UMN_PIPNN_PES_Class.F90:176-330) with the PES model's UseSurface (PES_Factory_Class.F90:276-296):
 *   UseSurface(3) (0/1), iFunc, NInput, NHid1, NHid2, NOutput, then for networks a, b, c
 *   pdel(NInput+1), pavg(NInput+1), W1(NInput,NHid1), b1, W2(NHid1,NHid2), b2, W3(NHid2), b3
 * (weight(inode2, inode1) column-major as in Fortran; one iFunc and one set of layer sizes for the
 * three networks, the last ones read, as the reference keeps them), ncoef = 8 + 3 x 2570 for the
 * shipped 276-5-90-1 networks, the only shape built.  Its Compute returns dVdQ = 0, so its
 * trajectories feel no force from it (cair_rhs gives dp/dt = -0); cair_pes_eval returns dVdR by the
 * reference's central differences (1e-5 Ang).  The MEG fields are unused. */
typedef struct cair_pes_desc {
  int32_t model;       /* cair_pes_model                                      */
  int32_t ncoef;       /* 56 (O3), 276 (N3, N4), 430 (O4), see above (NN, BNN, PIPNN) */
  const double* coef;  /* C(1:ncoef) [kcal/mol], copied at cair_create        */
  double a, ab, ra, rb;/* MEG parameters [Ang, Ang^2, Ang, Ang] (O3, O4)      */
  double eref;         /* O4 file value (unused by the energy, as in the reference) */
  double totdiss;      /* O4 file value (unused by the energy, as in the reference) */
} cair_pes_desc;

/* Everything Collision%Initialize and Integrator%Initialize derive from the input file
 * for this path (Input_Class.F90:1192-1241 ODE keys; 1079 nquad; masses; surfaces). */
typedef struct cair_system_desc {
  int32_t abi_version;   /* CAIR_ABI_VERSION                                      */
  int32_t natoms;        /* 3 or 4                                                */
  int32_t npes;          /* 1..CAIR_MAX_PES                                       */
  int32_t diat_model;    /* cair_diat_model of every pair                         */
  double mass[4];        /* atom masses [a.u.]                                    */
  const double* tpq;     /* optional Tpq(NEqtVar,NEqtVar) column-major, e.g. the
                            matrix the caller's LAPACK produced; NULL: computed   */
  cair_pes_desc pes[CAIR_MAX_PES];
  /* "Initial time step", "Error control parameter", "Stepsize increase damping factor",
     "Nb of extrapolation steps", "Try to increase stepsize?",
     "Nb of integration between end checking", "Max distance between atom pair [bohr]",
     "Max trajectory time [a.u.]", "Tolerance on Hamiltonian" */
  double dt0, eps, relax, rmax, tmax, ham_abs_tol;
  int32_t nsteps, inc_step, ncall;
  /* final-state analysis: "Nb of Quadrature Pts for Action Integral", "Lower/Upper Bound
     for Position of Centrifugal Barrier Max", "Factor for q.b. Levels",
     "Time threshold for q.b. Levels [Eh]" */
  int32_t nquad;
  double rsmal, rcent, rfact, tthresau;
} cair_system_desc;

/* Final state of one molecule (MolecularState_Type after FindState). */
typedef struct cair_mol_state {
  int32_t ipair;   /* 1-based pair index of the molecule                          */
  int32_t itype;   /* 0 bound, 1 quasi-bound, 2 dissociated/unbound, 3 short-lived */
  double eint;     /* internal energy [Eh]                                        */
  double angmom;   /* |L| (= J + 1/2 semiclassically), 1/2 when itype == 2         */
  double viba;     /* action / 2 pi (= v + 1/2)                                     */
} cair_mol_state;

/* Analysed trajectory point (TrajectoryPoint_Type after Analyze). */
typedef struct cair_traj_point {
  cair_mol_state mol[2];
  double b;        /* impact parameter of the relative motion [bohr]              */
  double xkin;     /* relative kinetic energy [Eh]                                */
  double vrel[3];  /* relative velocity                                           */
  int32_t nmol;
  int32_t pad;
} cair_traj_point;

/* One row of a level list (LevelsContainer_Class.F90:86-262; columns of FromUMN_Sorted.inp). */
typedef struct cair_level {
  int32_t vqn, jqn;
  double eint, egam, rmin, rmax, vmin, vmax, tau, ri, ro;
} cair_level;

/* One state-specific run of RunTrajectories: ntraj trajectories from one initial level at one
 * translational temperature, drawn from their own random-number stream (the per-process
 * stream of Collision_Class.F90:286-313).  Its trajectories occupy rows
 * [first, first + ntraj) of the batch arrays. */
typedef struct cair_work_item {
  int32_t ilevel;   /* row of the level table                                  */
  int32_t ipes;     /* 0-based surface                                          */
  int64_t first;    /* first row of this item in the batch arrays               */
  int64_t ntraj;    /* number of trajectories                                   */
  int64_t seed;     /* stream seed ("Initial Random Nb Seed" mapped per process) */
  double ttra;      /* translational temperature [K] (Boltzmann model)         */
  double bmax;      /* the ring's bound [bohr] = -(the ring's input "b"): > 0 sampled by b_mode,
                       < 0 the fixed impact parameter -bmax (no random number drawn) */
  double dinit;     /* initial separation [bohr]                               */
  int32_t ilevel2;  /* diatom + diatom: row of the projectile's level (atoms 3, 4) */
  int32_t b_mode;   /* "Impact Parameter Strata Type" (Collision_Class.F90:1276-1296), U uniform:
                       0 Circles:  b = sqrt(U) bmax
                       1 Rings:    b = sqrt(bmin^2 + U (bmax^2 - bmin^2))
                       2 Segments: b = -bmin + U (bmax + bmin)                              */
  double bmin;      /* -(the previous ring's input "b"), 0 for the first ring (GetImpactParamValue) */
  int64_t skip;     /* trajectories of the same stream before this item's first: the earlier rings
                       of a stratified run (Ring%iTrajMax of the previous ring); rows are numbered
                       from skip + 1.  An item with the previous item's seed and skip = that item's
                       skip + ntraj continues its stream (one thread draws the rings in order, each
                       with its own b rule); any other item with skip > 0 draws and drops skip
                       trajectories under its own b rule first */
} cair_work_item;

/* One row of trajectories.out (Integrator_Class.F90:884-933) plus diagnostics. */
typedef struct cair_traj_result {
  int64_t idx;      /* index in its item's stream, 1-based: skip + k + 1 (Traj%Idx)   */
  int32_t item;     /* work item                                                   */
  int32_t ipes;     /* 0-based surface                                              */
  int32_t status;   /* cair_traj_status                                             */
  int32_t iste;     /* accepted Bulirsch-Stoer steps                                 */
  int32_t irej;     /* rejected attempts                                             */
  int32_t pad;
  double bmax, b;   /* ring bound and impact parameter of the analysed initial point */
  double j_i, v_i, arr_i;  /* AngMom, viba, 16*iPair + itype + 1/2 of the initial point */
  double j_f, v_f, arr_f;  /* the same for the final point                             */
  double t;         /* final time [a.u.]                                            */
  double dH;        /* H_final - H0 [Eh]; |dH| > HamAbsTol goes to the HNotCons file */
  double j2_i, v2_i, j2_f, v2_f;  /* four atoms: the second molecule's AngMom, viba; the
                                     arrangement is then 16 iPair1 + itype1 + 4 itype2 + 1/2 */
} cair_traj_result;

typedef struct cair_handle cair_handle;

/* Create a handle on the current CUDA device: copies the surfaces to device memory and
 * computes Tqp/Tpq (Transformation_Class.F90:53-128) unless sys->tpq is given.
 * Replaces PES_Factory%Construct_PES + Transformation%Initialize + ODE%Initialize. */
int cair_create(cair_handle** h, const cair_system_desc* sys);
void cair_destroy(cair_handle* h);
const char* cair_last_error(const cair_handle* h);
/* NEqtVar, NEqtTot, NPairs of the handle's system */
int cair_dims(const cair_handle* h, int32_t* neqtvar, int32_t* neqttot, int32_t* npairs);
/* Tpq(NEqtVar,NEqtVar) column-major as used by the kernels */
int cair_get_tpq(const cair_handle* h, double* tpq_host);

/* Batched PES%Compute (PES_Class.F90:43-72; e.g. Compute_N3_UMN_PES_1d,
 * N3_UMN_PES_Class.F90:332-382) for n geometries:
 *   R[n][NPairs] pair distances [bohr], Qall[n][3*NAtoms] Cartesian coordinates of all
 *   atoms (the last atom included, as Compute_PES_1d builds QAll) ->
 *   V[n] [Eh], dVdR[n][NPairs] [Eh/bohr], dVdQ[n][NEqtVar] (+dV/dq, before the sign flip
 *   of Compute_PES_1d).  dVdR == NULL and dVdQ == NULL gives the energy-only
 *   PES%Potential (O3_UMN_PES_Class.F90:153-191). */
int cair_pes_eval(cair_handle* h, int64_t n, const int32_t* ipes, const double* R, const double* Qall,
                  double* V, double* dVdR, double* dVdQ);

/* Batched HamiltonODESystem (ODE_System.F90:45-96) -- the RHS_Evaluation interface of
 * ODE_Solver.F90:53-60: y[n][NEqtTot] -> yp[n][NEqtTot]. */
int cair_rhs(cair_handle* h, int64_t n, const int32_t* ipes, const double* y, double* yp);

/* Batched Hamiltonian_1d (Collision_Class.F90:2046-2111): H[n], Rpi[n][NPairs]. */
int cair_hamiltonian(cair_handle* h, int64_t n, const int32_t* ipes, const double* paq, double* H,
                     double* Rpi);

/* Exactly `nattempts` Bulirsch-Stoer attempts (Integrate_ODE_1d, ODE_Solver.F90:225-358)
 * per trajectory, without end checks.  paq, t, dt are updated in place. */
int cair_bs_steps(cair_handle* h, int64_t n, const int32_t* ipes, double* paq, double* t, double* dt,
                  const double* erra, int32_t nattempts);

/* Propagate each trajectory to the end of the collision (Integrator_Class.F90:422-466 and
 * AssessConvergence, Trajectories_Class.F90:240-280): repeat {ncall attempts; Hamiltonian;
 * stop if t > tmax or any 1/Rp < 1/rmax} up to max_attempts attempts.  In/out: paq, t, dt,
 * smax, smin, irej, iste (initialise as SetIniCondForward does: t = 0, dt = dt0,
 * smin = +huge, smax = -huge, irej = iste = 0).  Out: H (last end check), status.
 * One GPU thread owns one trajectory; a persistent kernel refills finished threads from a
 * device work queue, so a batch of any length runs in one launch. */
int cair_integrate(cair_handle* h, int64_t n, const int32_t* ipes, double* paq, double* t, double* dt,
                   const double* erra, double* H, double* smax, double* smin, int32_t* irej, int32_t* iste,
                   int32_t* status, int64_t max_attempts);

/* Same as cair_integrate on device pointers, asynchronous on `stream` (cudaStream_t). */
int cair_integrate_dev(cair_handle* h, int64_t n, const int32_t* ipes, double* paq, double* t, double* dt,
                       const double* erra, double* H, double* smax, double* smin, int32_t* irej, int32_t* iste,
                       int32_t* status, int64_t max_attempts, void* stream);

/* Final-state analysis of n trajectory points (TrajectoryPoint%Analyze + SetPairs + FindState);
 * four-atom points fill both molecules of cair_traj_point (a cluster gives iPair = -1).
 * paq_vel[n][NEqtTot] holds VELOCITIES and coordinates, i.e. PaQ after
 * Collision%ApplyTransformation (Collision_Class.F90:2406-2432) or PaQ0. */
int cair_find_state(cair_handle* h, int64_t n, const double* paq_vel, cair_traj_point* out);

/* ApplyTransformation on device: momenta -> velocities, in place on a copy. */
int cair_apply_transformation(cair_handle* h, int64_t n, const double* paq, double* paq_vel);

/* Initial conditions on the device (SetIniCondForward, Collision_Class.F90:1065-1211: level,
 * BondLength vibrational phase, orientation, Boltzmann translational energy, impact parameter,
 * momenta, H0, error scales) for diatom + atom systems (SetInitialState_DiatomAtom,
 * StateInitDiatomAtom_Module.F90:90-231) and diatom + diatom systems (SetInitialState_DiatomDiatom,
 * StateInitDiatomDiatom_Module.F90:86-219; the projectile's level is items[].ilevel2).  One device
 * thread per work item runs the item's random-number stream in the reference's draw order; one
 * thread per trajectory does the rest.  Host arrays of NEqtTot columns; ntot = sum of items[].ntraj. */
int cair_sample_ics(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                    const cair_work_item* items, int64_t ntot, double* paq, double* paq0, double* erra,
                    double* H0, double* b, int32_t* ipes);
int cair_sample_ics_dev(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                        const cair_work_item* items, int64_t ntot, double* paq, double* paq0, double* erra,
                        double* H0, double* b, int32_t* ipes, int32_t* item_of, void* stream);

/* RunTrajectories for a set of work items, end to end on the GPU: initial conditions,
 * propagation (persistent kernel), ApplyTransformation, analysis of the initial and final
 * points and the trajectories.out rows.  Host arrays: results[ntot].  Put every (level,
 * temperature, surface) run of a computation into one call: the queue is ordered longest-first
 * across all of them, which hides each run's slowest trajectories behind the others' work. */
int cair_run_queue(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                   const cair_work_item* items, int64_t ntot, int64_t max_attempts, cair_traj_result* results);
/* The same on device pointers (levels, items, results on the device), asynchronous on
 * `stream` (a cudaStream_t; NULL is the default stream).  The batch state lives in
 * `workspace` (device memory of cair_queue_workspace_bytes(ntot) bytes, 256-byte aligned),
 * so calls with distinct workspaces may run concurrently on distinct streams; a NULL
 * workspace uses the handle's own arena (one call at a time).  The queue is ordered
 * longest-first by the predicted duration (initial relative speed) of each trajectory. */
int cair_run_queue_dev(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                       const cair_work_item* items, int64_t ntot, int64_t max_attempts, cair_traj_result* results,
                       void* workspace, void* stream);
int64_t cair_queue_workspace_bytes(int64_t ntot);

/* No counterpart in the reference.  cair_run_queue_dev for callers that cannot allocate device
 * memory once they are running (a host whose GPU memory is handed out by its own pool at
 * start-up, or code that must not trigger cudaMalloc's implicit synchronisation while it
 * runs): the batch state lives in a file-scope static device array of
 * CAIR_STATIC_QUEUE_MAX_TRAJ diatom + atom trajectories (about 8 MB that every GPU loading the
 * library keeps until exit; it holds about two thirds as many diatom + diatom ones), and the call
 * allocates nothing.  A batch beyond the array is rejected with CAIR_EINVAL.  The first call on a device looks up the array's device address,
 * so make it before any stream capture; the handle's device must be current.  All calls share
 * the array, so calls that overlap on the GPU race; the array keeps the last call's contents. */
#define CAIR_STATIC_QUEUE_MAX_TRAJ 16384
int cair_run_queue_static_dev(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                              const cair_work_item* items, int64_t ntot, int64_t max_attempts,
                              cair_traj_result* results, void* stream);

/* CUDA graph of the queue path (no counterpart in the reference): cair_queue_graph_create captures
 * cair_run_queue_dev(h, ..., workspace, stream) -- the eight kernel launches and the memsets between
 * them -- once and instantiates it; cair_queue_graph_launch replays it on `stream`, reading the level
 * table and work items and writing the result rows through the same device pointers every time
 * (refill them between replays to run other batches of the same size).  The workspace is required
 * (nothing may be allocated while capturing); replays on one workspace must not overlap.  The graph
 * does not record cair_set_integrate_timing events. */
typedef struct cair_queue_graph cair_queue_graph;
int cair_queue_graph_create(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                            const cair_work_item* items, int64_t ntot, int64_t max_attempts,
                            cair_traj_result* results, void* workspace, cair_queue_graph** graph);
int cair_queue_graph_launch(cair_handle* h, cair_queue_graph* graph, void* stream);
void cair_queue_graph_destroy(cair_queue_graph* graph);

/* Final-state statistics of state-specific runs (app/TrajectoriesStats/Statistics_Class.F90,
 * "Final States Assigment Mthd = Histogram", "Identical Diatoms? = no"; three conditions J, v,
 * arrangement for diatom + atom, five J1, v1, J2, v2, arrangement for diatom + diatom) and rate
 * coefficients (Process_Class.F90:122-209 with the Boltzmann mean velocity of
 * Collision_Class.F90:576-595).  A run is what the reference's statistics read for one initial
 * state: the rows of every surface and impact-parameter ring of one level and temperature, merged
 * (item_run maps each work item to its run; NULL makes every item its own run).  Rows counted are
 * the finished trajectories whose |dH| <= ham_abs_tol (the rest are the HNotCons rows).  The
 * rings of a run are the distinct |bmax| of its items that have counted rows (SetRings, within
 * 1e-3), and each row falls in the ring its sampled b lies in, as AddFinState assigns it. */
typedef struct cair_stats_params {
  int32_t qn_max;            /* QuantumNumberMax (300 in the reference)                         */
  int32_t ncond;             /* "Nb of Final Conditions": 3 (J, v, arr) or 5 (J1, v1, J2, v2, arr) */
  int32_t iskip[5];          /* "Iskip for Condition 1..ncond"                                  */
  int32_t pres_even_odd[5];  /* "Preserving Even / Oddness of Condition 1..ncond?" (0/1)       */
  double ham_abs_tol;        /* "Tolerance on Hamiltonian" [Eh]                                 */
  double xmu;                /* reduced mass of the relative translation [a.u.] (RedMass)      */
} cair_stats_params;

/* One line of the statistics output (FinCondVec, IniState, Cross, CrossSD) plus its rate;
 * conditions beyond ncond are zero. */
typedef struct cair_final_state {
  int32_t run;               /* run (the work item when item_run is NULL)                      */
  int32_t fin[5];            /* FinCondVec: J, v, arrangement or J1, v1, J2, v2, arrangement    */
  int32_t ini[5];            /* IniState                                                        */
  int32_t nrings;            /* impact-parameter rings of the run                               */
  int64_t count;             /* rows that ended in this state                                   */
  int64_t nrows;             /* rows of the run in the statistics (sum of TrajsPerb)            */
  double cross, cross_sd;    /* [bohr^2]                                                        */
  double rate, rate_sd;      /* cross sections x mean velocity [cm^3/s]                         */
} cair_final_state;

/* Statistics of `ntot` result rows already on the device (as cair_run_queue_dev leaves them),
 * counted on the GPU; the final states (at most `cap`, sorted by run then final-state code) and
 * their count come back to host memory.  Returns CAIR_EINVAL with the needed size in the message
 * when cap is too small, and when the items of one run differ in temperature or initial state.
 * `items` and `item_run` are host arrays. */
int cair_statistics_dev(cair_handle* h, int32_t nitems, const cair_work_item* items, const int32_t* item_run,
                        int64_t ntot, const cair_traj_result* results, const cair_stats_params* params,
                        cair_final_state* out, int64_t cap, int64_t* nout, void* stream);
/* The same from host rows. */
int cair_statistics(cair_handle* h, int32_t nitems, const cair_work_item* items, const int32_t* item_run, int64_t ntot,
                    const cair_traj_result* results, const cair_stats_params* params, cair_final_state* out,
                    int64_t cap, int64_t* nout);

/* Replicas: the statistics of processes or GPUs that ran the same runs from disjoint streams (the
 * reference's per-process outputs, merged by MergeTrajectories before TrajectoriesStats reads them),
 * without gathering their rows.  The only exchange between replicas is two host-side sums:
 *   1. cair_statistics_items(_dev) on every replica; sum item_rows and take the minimum of item_ini
 *      over replicas;
 *   2. cair_statistics_counts(_dev) on every replica with those totals, so that every replica uses the
 *      same rings; sum ring_rows (nruns x CAIR_STATS_MAX_RINGS) and the counts of equal (run, ring, code);
 *   3. cair_statistics_finish on the sums (host code, no handle or GPU).
 * On one replica the three steps give the lines of cair_statistics(_dev).  Runs are numbered as
 * item_run says (NULL: run = item); nruns = the largest run + 1. */
#define CAIR_STATS_MAX_RINGS 64
typedef struct cair_stats_count {
  int32_t run;
  int32_t ring;    /* 0-based ring of the run, rings ascending in bmax */
  int64_t code;    /* final-state code (iquse + 2) x QuantumNumberMax^c summed over the conditions */
  int64_t count;
} cair_stats_count;
/* Counted rows and the smallest initial-state code of every item (item_ini: INT64 max-like
 * 0x7f7f7f7f7f7f7f7f for an item without counted rows). */
int cair_statistics_items_dev(cair_handle* h, int32_t nitems, int64_t ntot, const cair_traj_result* results,
                              const cair_stats_params* params, uint64_t* item_rows, int64_t* item_ini,
                              void* stream);
int cair_statistics_items(cair_handle* h, int32_t nitems, int64_t ntot, const cair_traj_result* results,
                          const cair_stats_params* params, uint64_t* item_rows, int64_t* item_ini);
/* (run, ring, final-state code) counts of this replica's rows with the rings given by the totals of
 * step 1, at most `cap` entries (CAIR_EINVAL with the size needed in the message beyond), and the rows
 * per (run, ring) in ring_rows[run * CAIR_STATS_MAX_RINGS + ring] (host array of nruns x 64). */
int cair_statistics_counts_dev(cair_handle* h, int32_t nitems, const cair_work_item* items, const int32_t* item_run,
                               const uint64_t* item_rows, const int64_t* item_ini, int64_t ntot,
                               const cair_traj_result* results, const cair_stats_params* params,
                               cair_stats_count* out, int64_t cap, int64_t* nout, uint64_t* ring_rows, void* stream);
int cair_statistics_counts(cair_handle* h, int32_t nitems, const cair_work_item* items, const int32_t* item_run,
                           const uint64_t* item_rows, const int64_t* item_ini, int64_t ntot,
                           const cair_traj_result* results, const cair_stats_params* params, cair_stats_count* out,
                           int64_t cap, int64_t* nout, uint64_t* ring_rows);
/* The statistics lines from the summed totals and counts (host code).  Returns CAIR_EINVAL, with the
 * reason in msg when msg_cap > 0, for inconsistent input or a too-small cap. */
int cair_statistics_finish(int32_t nitems, const cair_work_item* items, const int32_t* item_run,
                           const uint64_t* item_rows, const int64_t* item_ini, const cair_stats_params* params,
                           int64_t n, const cair_stats_count* counts, const uint64_t* ring_rows,
                           cair_final_state* out, int64_t cap, int64_t* nout, char* msg, int32_t msg_cap);

/* trajectories.out rows (Integrator_Class.F90:884-933): format
 * (I10, ',', I5, 2(',', ES11.5), *(',', ES14.8)) with iTraj = idx_offset + idx, iPES 1-based, bmax,
 * b_i, then for nmol = 1 (NInitMolecules, diatom + atom) j_i, v_i, arr_i, j_f, v_f, arr_f and for
 * nmol = 2 (diatom + diatom) j1_i, v1_i, j2_i, v2_i, arr_i, j1_f, v1_f, j2_f, v2_f, arr_f; the header
 * line is the reference's for each (Integrator_Class.F90:183-189).  Fortran field overflow prints
 * asterisks.  Host code, no handle or GPU needed.  cair_format_rows fills buf (not NUL-terminated)
 * and sets *len; it returns CAIR_EINVAL with *len = the size needed when cap is too small. */
int cair_format_rows(const cair_traj_result* rows, int64_t n, int64_t idx_offset, int32_t nmol, int32_t with_header,
                     char* buf, int64_t cap, int64_t* len);
/* <dir>/trajectories.out (finished rows with |dH| <= ham_abs_tol) and <dir>/trajectories_HNotCons.out
 * (the rest: energy not conserved, and the attempt-capped or non-finite rows, where the reference
 * stops with an error), each with the reference's header line; counts[0..1] = rows written. */
int cair_write_trajectories(const char* dir, const cair_traj_result* rows, int64_t n, int64_t idx_offset, int32_t nmol,
                            double ham_abs_tol, int64_t* counts);
/* trajectories.bin: the stream Statistics_Class.F90:283-314 writes (NTraj, then per row Idx, iPES,
 * bMax, bSampled, Qini(NCond), Qfin(NCond); NCond = 3 for nmol = 1, 5 for nmol = 2; 8-byte integers
 * and reals) for the trajectories.out rows. */
int cair_write_trajectories_bin(const char* path, const cair_traj_result* rows, int64_t n, int64_t idx_offset,
                                int32_t nmol, double ham_abs_tol);

/* MergeTrajectories (scripts/executing/ComputeRates.sh:406-472): the trajectories.out of each
 * source directory (one per process or replica, in order) is appended to <out_dir>/trajectories.csv
 * -- whole when that file does not exist yet, without its header line otherwise -- and its
 * trajectories_HNotCons.out to <out_dir>/trajectories_HNotCons.out alike; directories without a
 * trajectories.out are skipped.  Writes <out_dir>/NConvTraj.dat (rows in trajectories.csv) and
 * sets *ntraj to that count.  Host code, no handle or GPU needed. */
int cair_merge_trajectories(int32_t nsrc, const char* const* src_dirs, const char* out_dir, int64_t* ntraj);

/* Algorithmic FP64 operation counts the library's kernels execute per PES energy+gradient
 * evaluation, per energy-only evaluation and per BS attempt (excluding the PES), for
 * roofline accounting.  `exp_per_eval` counts exponentials separately. */
int cair_flop_model(const cair_handle* h, int32_t ipes, double* flops_grad, double* flops_energy,
                    double* flops_attempt_overhead, double* exp_per_eval);

/* FP64 fused-multiply-add throughput of the handle's GPU in GFLOP/s (2 flops per DFMA),
 * measured with a register-resident DFMA kernel; the denominator of the FP64 roofline. */
int cair_fp64_peak_probe(cair_handle* h, double* gflops);

/* Kernel timing for roofline accounting (no counterpart in the reference).  While on, every
 * launch of the persistent integrator made by cair_integrate* / cair_run_queue* is bracketed by
 * CUDA events on the stream it runs on.  cair_integrate_timings waits for the recorded launches,
 * writes the first `cap` durations [ms] in launch order, sets *count to the number recorded and
 * starts a new record.  cair_set_integrate_timing also starts a new record. */
int cair_set_integrate_timing(cair_handle* h, int32_t on);
int cair_integrate_timings(cair_handle* h, float* ms, int32_t cap, int32_t* count);

/* Warp timeline of the persistent FP64 integrator (no counterpart in the reference; for measuring
 * the queue's tail): while set, each launch with at most cap_warps warps writes, per warp w of the
 * launch, to times_dev[4 w .. 4 w + 3] (device memory, cap_warps x 4 uint64): %globaltimer [ns] at its
 * start, %globaltimer when its last lane runs out of work, the sum over its ncall-attempt blocks of
 * the lanes that held a trajectory, and its number of blocks (so 1 - [2] / (32 [3]) is the warp's
 * idle lane-time).  cair_warp_timeline_count gives the warps of the last launch that recorded (0 if
 * it had more than cap_warps).  NULL stops it. */
int cair_set_warp_timeline(cair_handle* h, uint64_t* times_dev, int64_t cap_warps);
int64_t cair_warp_timeline_count(const cair_handle* h);

/* Launch shape of the persistent integrator (no counterpart in the reference, whose loop is
 * serial): threads per block (32, 64 or 128) and resident blocks per SM (0 = as many as fit). */
int cair_set_launch_shape(cair_handle* h, int32_t block, int32_t per_sm);
int cair_get_launch_shape(const cair_handle* h, int32_t* block, int32_t* per_sm);
/* Persistent integrator mode (no counterpart in the reference, whose loop is serial).
 * CAIR_INTEGRATOR_THREAD (default): every lane of a warp integrates its own trajectory -- the
 * throughput mode for queues of many more trajectories than the GPU has lanes.
 * CAIR_INTEGRATOR_WARP: a warp integrates one trajectory -- its half-warps run the modified-midpoint
 * sequences of an attempt side by side and its lanes evaluate each right-hand side together -- the
 * latency mode for small jobs, whose time is their longest trajectory's.  Same queue, end check and
 * outputs; built for the O3, N3, O4 and N4 UMN surfaces with their own diatomics (one surface model
 * per handle; diatom + diatom runs its sequences on the whole warp), NSteps 2..4; any other system
 * returns CAIR_EUNSUPPORTED.  An attached surrogate takes precedence over either. */
#define CAIR_INTEGRATOR_THREAD 0
#define CAIR_INTEGRATOR_WARP 1
/* CAIR_INTEGRATOR_AUTO: per launch, the warp integrator when the system has its programs and the launch
 * holds fewer trajectories than twice the lanes the thread integrator keeps resident (a smaller job is as
 * long as its longest trajectory on one lane), the thread integrator otherwise. */
#define CAIR_INTEGRATOR_AUTO 2
int cair_set_integrator_mode(cair_handle* h, int32_t mode);
int32_t cair_get_integrator_mode(const cair_handle* h);
/* The integrator the handle's last launch ran (CAIR_INTEGRATOR_THREAD or _WARP; THREAD too for a surrogate
 * launch, and for a thread launch that handed its tail to the warp integrator). */
int32_t cair_last_integrator(const cair_handle* h);
/* Tail hand-off of CAIR_INTEGRATOR_AUTO on launches the thread integrator runs: once the queue is empty and at
 * most `below` trajectories are still in flight, each is written back at its next end check and the warp
 * integrator finishes it, a warp per trajectory (same attempt counts and end checks).  below < 0: the warp
 * integrator's resident warps (the default); 0: off. */
int cair_set_tail_handoff(cair_handle* h, int64_t below);
/* Trajectories the handle's last launch handed to the warp integrator (synchronises the device). */
int64_t cair_last_handoffs(cair_handle* h);
/* Autotuner: runs a sample of about `sample` trajectories of the job's own work items (each item's
 * leading trajectories, same streams), capped at cap_attempts attempts each, once per launch shape
 * (block 32, 64, 128 x 1 .. the resident maximum per SM), and keeps on the handle the shape with the
 * most attempts per second of integrator time.  out[0 .. cap) receives the measured points,
 * *nout their number.  Host arrays; synchronous on the handle's stream.  Make the sample several
 * times the lanes a shape keeps resident (up to 32 x 8 warps per SM): a sample that ends in a
 * partial round of lanes favours the shapes with fewer lanes. */
typedef struct cair_tune_point {
  int32_t block, per_sm;
  double ms;                 /* integrator time of the sample */
  double attempts_per_s;
} cair_tune_point;
int cair_autotune(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                  const cair_work_item* items, int64_t sample, int64_t cap_attempts, cair_tune_point* out,
                  int32_t cap, int32_t* nout);

/* Device counters of the last cair_integrate*: total BS attempts, accepted, rejected,
 * PES gradient evaluations, PES energy evaluations.  Calls of cair_run_queue_dev with a caller
 * workspace (and cair_run_queue_static_dev) keep their counters in that workspace and leave these
 * unchanged. */
int cair_last_counters(cair_handle* h, int64_t* counters5);

/* ---------------------------------------------------------------------------------------------
 * Learned surrogate of the N3 UMN three-body term (no counterpart in the reference: the reference
 * has no learned surface on this path; its analogue of the dense layers is
 * O3_NN_PES_Class.F90:357-477).  The N3 UMN surface is sum_i V_N2(R_i) + (457.4 + sum C_k B_k(x))
 * kcal/mol (N3_UMN_PES_Class.F90:332-382); its polynomial part minus 457.4, V3, vanishes in every
 * asymptotic channel.  The surrogate keeps the FP64 diatomics and models V3 as D(x) y(f):
 *   x_i = exp(-d_i - d_i^2/1.5) (d_i = R_i in angstrom - 1.098) the surface's own MEG variables;
 *   f = the ten S3-orbit sums of x of degree 1..4, normalised ((raw - mu) isd), 5 zeros, 1;
 *   y = a 16 -> 128 -> 128 -> 128 -> 1 tanh network [eV], BF16 hidden weights, FP32 output layer;
 *   D = 1 - exp(-(x1 x2 + x1 x3 + x2 x3) / sigma_d), so V3_s = 0 exactly where V3 = 0.
 * Hidden layers run as tcgen05 BF16 MMAs with FP32 accumulation in tensor memory, each activation
 * split exactly into three BF16 parts (FP32-accurate products).  Two ensemble members (0 = A, the
 * one that drives the dynamics; 1 = B) are trained from different starts; an attempt whose start
 * has |D (yA - yB)| > gate_ev, or a feature outside [fmin, fmax] where D > gate_dmin, runs on the
 * FP64 surface instead.  Parameters: cair_sur_nparam() floats per member, in the order W1[128][16]
 * (column 15 is the first layer's bias), W2[128][128], W3[128][128] (row = output), b2, b3, w4
 * [128], b4. */
typedef struct cair_sur_sample {
  double R[3];   /* pair distances [bohr] */
  float e;       /* V3 [eV] */
  float g[3];    /* dV3/dR_i [eV/bohr] */
} cair_sur_sample;
typedef struct cair_sur_consts {
  float mu[10], isd[10];    /* feature normalisation */
  float fmin[10], fmax[10]; /* normalised feature range of the training set */
  float sigma_d;            /* damping scale */
  float gate_ev;            /* ensemble gate [eV] (1 meV = 1e-3) */
  float gate_dmin;          /* the range gate applies where D exceeds this */
} cair_sur_consts;
typedef struct cair_surrogate cair_surrogate;
int cair_sur_create(cair_surrogate** s, int32_t device);   /* CAIR_EUNSUPPORTED off sm_103 */
void cair_sur_destroy(cair_surrogate* s);
const char* cair_sur_last_error(const cair_surrogate* s);
int cair_sur_nparam(void);
int cair_sur_set_consts(cair_surrogate* s, const cair_sur_consts* c);
int cair_sur_get_consts(const cair_surrogate* s, cair_sur_consts* c);
/* Host parameters of one member; set also resets its Adam state. */
int cair_sur_set_params(cair_surrogate* s, int32_t member, const float* params);
int cair_sur_get_params(cair_surrogate* s, int32_t member, float* params);
/* Device pointers: at n geometries R[n][3], both members' y [eV], member A's dy/df g[n][16], and
 * the surrogate's V3 [Eh] and dV3/dR [n][3] [Eh/bohr].  Synchronises `stream`. */
int cair_sur_eval_dev(cair_surrogate* s, int64_t n, const double* R, float* ya, float* yb, float* g, double* v3,
                      double* dv3, void* stream);
/* Training, device pointers: adds to the member's gradient the parameter gradient of
 * (w_e (D y - e)^2 + w_f |d(D y)/dR - g|^2) averaged over samples[idx[0..nbatch)]; the loss parts
 * accumulate until cair_sur_take_loss.  cair_sur_adam_dev applies one Adam step (beta 0.9, 0.999,
 * eps 1e-8) with learning rate lr and clears the gradient.  cair_sur_get_grad copies the gradient
 * to the host (synchronising). */
int cair_sur_grad_dev(cair_surrogate* s, int32_t member, int64_t nbatch, const cair_sur_sample* samples,
                      const int64_t* idx, float w_e, float w_f, void* stream);
int cair_sur_adam_dev(cair_surrogate* s, int32_t member, float lr, void* stream);
int cair_sur_get_grad(cair_surrogate* s, int32_t member, float* grad);
int cair_sur_take_loss(cair_surrogate* s, double* loss2, void* stream);
/* Gate counters since the last reset: attempts on the FP64 surface, on the surrogate, range-gated,
 * ensemble-gated. */
int cair_sur_counters(cair_surrogate* s, int64_t* counters4, int32_t reset);
/* Training targets from the handle's FP64 N3 surface at n geometries (device pointers). */
int cair_sur_targets_dev(cair_handle* h, int64_t n, const double* R, cair_sur_sample* out, void* stream);
/* Every integrator launch of the handle (cair_integrate*, cair_run_queue*, graphs captured after the
 * call) runs on the surrogate s; NULL restores the FP64 surface.  The handle must be N3 UMN with
 * NSteps = 3; s must outlive its use. */
int cair_sur_attach(cair_handle* h, cair_surrogate* s);
/* Geometry recorder of the FP64 integrator (the training set along the method's own trajectories):
 * at every end check of a trajectory whose middle pair distance is below rcut [bohr], with
 * probability 1/modulus (a hash of trajectory and attempt count), its three pair distances are
 * appended to rec_dev[cap][3] (device).  rec_dev NULL stops recording.  cair_recorded_samples
 * returns the number appended since the recorder was set (it may exceed cap; the excess is
 * dropped). */
int cair_record_samples(cair_handle* h, double* rec_dev, int64_t cap, int32_t modulus, double rcut);
int64_t cair_recorded_samples(cair_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* CAIR_GPU_H */
