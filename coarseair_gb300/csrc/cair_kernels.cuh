// GB300 kernels of the trajectory path: batched surface evaluation, right-hand side,
// Hamiltonian, fixed-count Bulirsch-Stoer attempts, the persistent end-to-end integrator
// and the final-state analysis.  One thread owns one trajectory.
#pragma once
#include "cair_device.cuh"

namespace cair {

// ------------------------------------------------------------------------------------------
// Batched PES%Compute / PES%Potential.  R[n][NP], Qall[n][3 NA], dVdR[n][NP], dVdQ[n][NV].
// ------------------------------------------------------------------------------------------
template <int MODEL, bool GRAD>
__global__ void __launch_bounds__(128) k_pes_eval(DevSys S, int64_t n, const int32_t* __restrict__ ipes,
                                                  const double* __restrict__ Rin, const double* __restrict__ Qin,
                                                  double* __restrict__ V, double* __restrict__ dVdR,
                                                  double* __restrict__ dVdQ) {
  using T = Traits<MODEL>;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const DevPes& P = S.pes[ipes ? ipes[k] : 0];
    double R[T::NP], Ri[T::NP], Q[3 * T::NA], v, g[T::NP], m[T::NV];
#pragma unroll
    for (int i = 0; i < T::NP; ++i) { R[i] = Rin[T::NP * k + i]; Ri[i] = 1.0 / R[i]; }
#pragma unroll
    for (int i = 0; i < 3 * T::NA; ++i) Q[i] = Qin[3 * T::NA * k + i];
    pes<MODEL, GRAD>(S, P, R, Ri, Q, v, g, m);
    V[k] = v;
    if (GRAD) {
#pragma unroll
      for (int i = 0; i < T::NP; ++i) dVdR[T::NP * k + i] = g[i];
#pragma unroll
      for (int i = 0; i < T::NV; ++i) dVdQ[T::NV * k + i] = m[i];
    }
  }
}

template <int MODEL>
__global__ void __launch_bounds__(128) k_rhs(DevSys S, int64_t n, const int32_t* __restrict__ ipes,
                                             const double* __restrict__ y, double* __restrict__ yp) {
  constexpr int NE = Traits<MODEL>::NE;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    Rhs<MODEL> f(S, S.pes[ipes ? ipes[k] : 0]);
    double a[NE], b[NE];
#pragma unroll
    for (int i = 0; i < NE; ++i) a[i] = y[NE * k + i];
    f(a, b);
#pragma unroll
    for (int i = 0; i < NE; ++i) yp[NE * k + i] = b[i];
  }
}

template <int MODEL>
__global__ void __launch_bounds__(128) k_hamiltonian(DevSys S, int64_t n, const int32_t* __restrict__ ipes,
                                                     const double* __restrict__ paq, double* __restrict__ H,
                                                     double* __restrict__ Rpi) {
  using T = Traits<MODEL>;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    double y[T::NE], r[T::NP];
#pragma unroll
    for (int i = 0; i < T::NE; ++i) y[i] = paq[T::NE * k + i];
    H[k] = hamiltonian<MODEL>(S, S.pes[ipes ? ipes[k] : 0], y, r);
    if (Rpi) {
#pragma unroll
      for (int i = 0; i < T::NP; ++i) Rpi[T::NP * k + i] = r[i];
    }
  }
}

template <int MODEL, int NS>
__global__ void __launch_bounds__(128) k_bs_steps(DevSys S, int64_t n, const int32_t* __restrict__ ipes,
                                                  double* __restrict__ paq, double* __restrict__ t,
                                                  double* __restrict__ dt, const double* __restrict__ erra,
                                                  int32_t nattempts) {
  constexpr int NE = Traits<MODEL>::NE;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    Rhs<MODEL> f(S, S.pes[ipes ? ipes[k] : 0]);
    double y[NE];
#pragma unroll
    for (int i = 0; i < NE; ++i) y[i] = paq[NE * k + i];
    double x = t[k], h = dt[k], smax = 0.0, smin = 0.0;
    int irej = 0, iste = 0;
#pragma unroll 1
    for (int a = 0; a < nattempts; ++a)
      bs_attempt<NE, NS>(f, y, x, h, erra + NE * k, S.relax, S.incstp != 0, smax, smin, irej, iste);
#pragma unroll
    for (int i = 0; i < NE; ++i) paq[NE * k + i] = y[i];
    t[k] = x;
    dt[k] = h;
  }
}

// ------------------------------------------------------------------------------------------
// Persistent integrator: every thread takes a trajectory from the device work queue,
// integrates it to the end of the collision (ncall attempts, then the end check of
// Integrator_Class.F90:457-465) and takes the next one.  Finished threads refill
// immediately, so the attempt loop of a warp stays converged while trajectory lengths
// differ by orders of magnitude.
// ------------------------------------------------------------------------------------------
struct IntegrateArgs {
  int64_t n;
  const int32_t* ipes;
  double* paq;
  double* t;
  double* dt;
  const double* erra;
  double* H;
  double* smax;
  double* smin;
  int32_t* irej;
  int32_t* iste;
  int32_t* status;
  int64_t max_attempts;
  unsigned long long* queue;    // next queue position
  unsigned long long* counters; // attempts, accepted, rejected, grad evals, energy evals
  const int32_t* order;         // queue position -> trajectory (NULL: identity)
  // geometry recorder (cair_record_samples; NULL: off): pair distances at end checks
  double* rec;
  unsigned long long* nrec;
  unsigned long long rec_cap;
  unsigned long long rec_mod;
  double rec_rcut;
  // warp timeline (cair_set_warp_timeline; NULL: off): per warp w of the launch, at [4 w .. 4 w + 3],
  // %globaltimer [ns] when it starts and when its last lane runs out of work, the sum over its
  // ncall blocks of the lanes with a trajectory, and its ncall blocks
  unsigned long long* warp_times;
  // tail hand-off to the warp integrator (hand NULL: off).  Once the queue is empty and at most
  // hand_below trajectories are in flight, a lane writes its trajectory back at its next end check,
  // records the attempts it has made (hand_att[k]) and appends k to hand[]; hctl[0] counts the
  // trajectories in flight, hctl[1] the hand-offs.
  int32_t* hand;
  long long* hand_att;
  unsigned long long* hctl;
  long long hand_below;
  // the warp integrator over a hand-off list: the number of entries read from *n_dev (A.n bounds it),
  // each trajectory's earlier attempts from att0[k]
  const unsigned long long* n_dev;
  const long long* att0;
};

// The GPU's nanosecond clock (0 where this source is compiled for the host by the test harness).
__device__ __forceinline__ unsigned long long globaltimer_ns() {
#ifdef __CUDA_ARCH__
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
#else
  return 0;
#endif
}

// Keep one in `mod` end checks, by a hash of trajectory and attempt count (splitmix64 finaliser).
__device__ __forceinline__ bool rec_pick(unsigned long long k, long long att, unsigned long long mod) {
  unsigned long long z = k * 0x9E3779B97F4A7C15ull + (unsigned long long)att;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return z % mod == 0;
}

// Minimum resident blocks per SM the register allocation must allow (1: up to 255 registers per
// thread, 8 warps per SM fit).  Blocks of 32, 64 or 128 threads; cair_autotune picks the block size
// and the blocks per SM at run time.
#ifndef CAIR_INTEGRATE_MIN_BLOCKS
#define CAIR_INTEGRATE_MIN_BLOCKS 1
#endif

template <int MODEL, int NS>
__global__ void __launch_bounds__(128, CAIR_INTEGRATE_MIN_BLOCKS) k_integrate(DevSys S, IntegrateArgs A) {
  constexpr int NE = Traits<MODEL>::NE, NP = Traits<MODEL>::NP;
  unsigned long long c_att = 0, c_acc = 0, c_rej = 0;
  const bool incstp = S.incstp != 0;
  const int ncall = S.ncall;
  // Lane state.  A lane takes a new trajectory only at an ncall-block boundary, where the whole
  // warp meets (__syncwarp), so the warp's active lanes always run their attempts in lockstep;
  // each trajectory still gets its end check after every ncall attempts of its own.
  unsigned long long k = 0;
  bool active = false;
  int ip = 0, irej = 0, iste = 0, irej0 = 0, iste0 = 0;
  int64_t att = 0;
  double y[NE], x = 0.0, h = 0.0, smax = 0.0, smin = 0.0, H = 0.0;
  auto take = [&]() {
    const unsigned long long q = atomicAdd(A.queue, 1ull);
    active = q < (unsigned long long)A.n;
    if (!active) return;
    if (A.hand) atomicAdd(A.hctl, 1ull);
    k = A.order ? (unsigned long long)A.order[q] : q;
    ip = A.ipes ? A.ipes[k] : 0;
#pragma unroll
    for (int i = 0; i < NE; ++i) y[i] = A.paq[NE * k + i];
    x = A.t[k]; h = A.dt[k]; smax = A.smax[k]; smin = A.smin[k]; H = 0.0;
    irej = irej0 = A.irej[k];
    iste = iste0 = A.iste[k];
    att = 0;
  };
  const unsigned long long warp_id = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
  if (A.warp_times && (threadIdx.x & 31) == 0) {
    A.warp_times[4 * warp_id] = globaltimer_ns();
  }
  unsigned long long lane_blocks = 0, blocks = 0;
  take();
#pragma unroll 1
  for (;;) {
    const unsigned busy = __ballot_sync(0xffffffffu, active);
    if (!busy) break;
    lane_blocks += __popc(busy);
    ++blocks;
    if (active) {
      const DevPes& P = S.pes[ip];
      Rhs<MODEL> f(S, P);
      int bad = 0;
#pragma unroll 1
      for (int c = 0; c < ncall; ++c)
        bad |= bs_attempt<NE, NS>(f, y, x, h, A.erra + NE * k, S.relax, incstp, smax, smin, irej, iste);
      att += ncall;
      double rpi[NP];
      H = hamiltonian<MODEL>(S, P, y, rpi);
      bool conv = x > S.tmax;
#pragma unroll
      for (int p = 0; p < NP; ++p) conv = conv || (rpi[p] < S.rpimax);
      if constexpr (NP == 3) {
        if (A.rec) {
          const double r0 = 1.0 / rpi[0], r1 = 1.0 / rpi[1], r2 = 1.0 / rpi[2];
          const double mid = fmax(fmin(r0, r1), fmin(fmax(r0, r1), r2));
          if (mid < A.rec_rcut && rec_pick(k, att, A.rec_mod)) {
            const unsigned long long slot = atomicAdd(A.nrec, 1ull);
            if (slot < A.rec_cap) {
              A.rec[3 * slot] = r0;
              A.rec[3 * slot + 1] = r1;
              A.rec[3 * slot + 2] = r2;
            }
          }
        }
      }
      if (bad || conv || att >= A.max_attempts) {
#pragma unroll
        for (int i = 0; i < NE; ++i) A.paq[NE * k + i] = y[i];
        A.t[k] = x;
        A.dt[k] = h;
        A.H[k] = H;
        A.smax[k] = smax;
        A.smin[k] = smin;
        A.irej[k] = irej;
        A.iste[k] = iste;
        A.status[k] = bad ? CAIR_TRAJ_NONFINITE : (conv ? CAIR_TRAJ_DONE : CAIR_TRAJ_ATTEMPT_CAP);
        c_att += att;
        c_acc += iste - iste0;
        c_rej += irej - irej0;
        if (A.hand) atomicAdd(A.hctl, ~0ull);  // one fewer in flight
        take();
      } else if (A.hand && *(volatile unsigned long long*)A.queue >= (unsigned long long)A.n &&
                 (long long)*(volatile unsigned long long*)A.hctl <= A.hand_below) {
        // the queue's tail: the warp integrator finishes this trajectory from this end check
#pragma unroll
        for (int i = 0; i < NE; ++i) A.paq[NE * k + i] = y[i];
        A.t[k] = x;
        A.dt[k] = h;
        A.H[k] = H;
        A.smax[k] = smax;
        A.smin[k] = smin;
        A.irej[k] = irej;
        A.iste[k] = iste;
        A.hand_att[k] = att;
        c_att += att;
        c_acc += iste - iste0;
        c_rej += irej - irej0;
        A.hand[atomicAdd(A.hctl + 1, 1ull)] = (int32_t)k;
        active = false;
      }
    }
    __syncwarp();
  }
  if (A.warp_times && (threadIdx.x & 31) == 0) {
    A.warp_times[4 * warp_id + 1] = globaltimer_ns();
    A.warp_times[4 * warp_id + 2] = lane_blocks;
    A.warp_times[4 * warp_id + 3] = blocks;
  }
  if (c_att) {
    atomicAdd(A.counters + 0, c_att);
    atomicAdd(A.counters + 1, c_acc);
    atomicAdd(A.counters + 2, c_rej);
    atomicAdd(A.counters + 3, c_att * (unsigned long long)nseq_total(NS));
    atomicAdd(A.counters + 4, c_att / (unsigned long long)(ncall > 0 ? ncall : 1));
  }
}

// ApplyTransformation (Collision_Class.F90:2406-2432), any NEqtVar
#ifndef CAIR_MODEL_TU  // model-independent: built once, in the API translation unit
__global__ void k_apply_transformation(DevSys S, int64_t n, const double* __restrict__ paq,
                                       double* __restrict__ out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int nv = S.nv, ne = S.ne;
    for (int i = 0; i < ne; ++i) out[ne * k + i] = paq[ne * k + i];
    for (int i = 0; i < nv; ++i) {
      double a = 0.0;
      for (int j = 0; j < nv; ++j) a = a + S.Tpq[i + 9 * j] * paq[ne * k + j];
      out[ne * k + i] = a;
    }
  }
}
#endif

// ------------------------------------------------------------------------------------------
// Final-state analysis (TrajectoryPoint_Class.F90:128-495, MolecularState_Class.F90:61-429,
// DiatomicPotential_Class.F90:626-1009)
// ------------------------------------------------------------------------------------------
struct FsArgs {
  int32_t nquad;
  double rsmal, rcent, rfact, tthresau, vinf;
  const double* gx;   // Chebyshev-2 nodes (ascending)
  const double* gw;   // weights already divided by sqrt(1 - x^2)
  double mass[4];
};

__device__ __forceinline__ double diat_v(const DevSys& S, double r) {
  double v, dv;
  diat_any<false>(S, r, v, dv);
  return v;
}
__device__ __forceinline__ double eff_pot(const DevSys& S, double r, double vc_r2) {
  return diat_v(S, r) + vc_r2 / (r * r);
}

static __device__ int turning_point(const DevSys& S, double ra, double rc, double vc_r2, double eint, int nbis, int nnew,
                             double& rt_out) {
  double rt = 0.0;
  if (nbis > 0) {
    double va = eff_pot(S, ra, vc_r2) - eint;
    double vc = eff_pot(S, rc, vc_r2) - eint;
    double v2 = vc * va;
    if (v2 > 0.0 && v2 > 1.0E-10) { rt_out = 0.0; return 1; }
    for (int it = 0; it < nbis; ++it) {
      rt = 0.5 * (ra + rc);
      double vb = eff_pot(S, rt, vc_r2) - eint;
      v2 = vb * va;
      if (v2 > 0.0) { ra = rt; va = vb; } else { rc = rt; vc = vb; }
    }
  }
  for (int it = 0; it < nnew; ++it) {
    double vcen = vc_r2 / (rt * rt), vb, dvb;
    diat_any<true>(S, rt, vb, dvb);
    double v = vb + vcen;
    double dv = dvb - 2.0 * vcen / rt;
    rt = rt + (eint - v) / dv;
  }
  rt_out = rt;
  return 0;
}

static __device__ double action_integral(const DevSys& S, const FsArgs& F, double ri, double ro, double vc_r2,
                                  double eint, double twomu) {
  const int n = F.nquad;
  double rm = (ro - ri) * 0.5;
  double rp = (ro + ri) * 0.5 + rm * F.gx[0];
  double act = 0.0;
  for (int i = 0; i < n; ++i) {
    double e = eint - eff_pot(S, rp, vc_r2);
    if (!(e > 0.0)) e = -e;
    act = act + sqrt(e) * F.gw[i];
    if (i != n - 1) rp = rp + rm * (F.gx[i + 1] - F.gx[i]);
  }
  return 2.0 * sqrt(twomu) * act * rm;
}

static __device__ int find_extremum(const DevSys& S, double sig, double re, double rlim, double vc_r2, double tol,
                             double& rout, double& vout) {
  const double factor = 0.3819660115, step = 0.005;
  double vlast = eff_pot(S, re, vc_r2) * sig;
  double ri = re, vtry = 0.0;
  for (;;) {
    ri = ri + step;
    if (ri >= rlim) { rout = ri - step; vout = vlast * sig; return 1; }
    vtry = eff_pot(S, ri, vc_r2) * sig;
    if (vtry > vlast) break;
    vlast = vtry;
  }
  double rb = ri - step, vb = vlast, rc = ri, ra = rb - step;
  for (int it = 0; it < 100000; ++it) {
    double rt1, vt1;
    if (rb - ra > rc - rb) {
      rt1 = (ra - rb) * factor + rb;
      vt1 = eff_pot(S, rt1, vc_r2) * sig;
      if (vb < vt1) ra = rt1; else { rc = rb; rb = rt1; vb = vt1; }
    } else {
      rt1 = (rc - rb) * factor + rb;
      vt1 = eff_pot(S, rt1, vc_r2) * sig;
      if (vb < vt1) rc = rt1; else { ra = rb; rb = rt1; vb = vt1; }
    }
    if (fabs(rc - ra) <= tol) break;
  }
  rout = rb;
  vout = vb * sig;
  return 0;
}

static __device__ double gamma_fct(double y) {
  double sum = -1.963510026021423 * y;
  if (y == 0.0) return sum;
  for (int it = 0; it <= 1000000; ++it) {
    double t1 = y / (0.5 + it);
    double term = t1 - atan(t1);
    sum = sum + term;
    if (fabs(term / sum) < 1.0E-06) return sum;
  }
  return sum;
}

static __device__ void find_state(const DevSys& S, const FsArgs& F, int ipair, int ia, int ib, const double* X,
                           const double* XD, cair_mol_state& m) {
  const double PI = 3.141592653589793;
  double xma = F.mass[ia], xmb = F.mass[ib];
  double fa = xma / (xma + xmb), fb = xmb / (xma + xmb);
  double x[3][2], xd[3][2];
  double eint = 0.0, rbond = 0.0;
  for (int i = 0; i < 3; ++i) {
    double xc = fa * X[2 * i] + fb * X[2 * i + 1];
    double xdc = fa * XD[2 * i] + fb * XD[2 * i + 1];
    x[i][0] = X[2 * i] - xc; x[i][1] = X[2 * i + 1] - xc;
    xd[i][0] = XD[2 * i] - xdc; xd[i][1] = XD[2 * i + 1] - xdc;
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
  const double eps = 1.0E-5;
  double rmin, vmin, rmax = 0.0, vmax = 0.0, viba = 0.5;
  int itype = 1;
  int ierr = find_extremum(S, 1.0, F.rsmal, F.rcent, vc_r2, eps, rmin, vmin);
  int imin = 1;
  if (ierr != 0) { rmin = (F.rsmal + F.rcent) * 0.5; imin = 0; }
  if (imin == 1) {
    ierr = find_extremum(S, -1.0, rmin, F.rcent, vc_r2, eps, rmax, vmax);
    if (ierr != 0) rmax = F.rcent;
  }
  if (imin == 0 || rbond > rmax) {
    itype = 3;
    viba = 0.5;
  } else {
    eint = eint + diat_v(S, rbond);
    itype = (eint < F.vinf) ? 1 : 2;
    double r1 = rmin;
    if (eint > vmax) {
      viba = 0.5;
      itype = 3;
    } else {
      double r00 = F.rsmal, ri = 0.0, ro = 0.0;
      for (int itry = 1; itry <= 10; ++itry) {
        turning_point(S, r00, r1, vc_r2, eint, 4, 4, ri);
        if (ri != 0.0) break;
        r00 = r00 * 0.5;
      }
      turning_point(S, r1, rmax, vc_r2, eint, 10, 4, ro);
      viba = action_integral(S, F, ri, ro, vc_r2, eint, twomu);
      if (eint > F.vinf) {
        double rga = rmax, rgb = rmax * 2.0, r3 = 0.0;
        for (int ip = 1; ip <= 10; ++ip) {
          if (turning_point(S, rga, rgb, vc_r2, eint, 10, 4, r3) == 0) break;
          rga = rgb;
          rgb = rgb * 2.0;
        }
        double eint_p = eint + 1.0E-5;
        if (eint_p > vmax) eint_p = eint + 0.5 * (vmax - eint);
        double deint = eint_p - eint, rip, rop, rim, rom;
        turning_point(S, r00, r1, vc_r2, eint_p, 4, 4, rip);
        turning_point(S, r1, rmax, vc_r2, eint_p, 10, 4, rop);
        double act_p = action_integral(S, F, rip, rop, vc_r2, eint_p, twomu);
        double eint_m = eint - deint;
        turning_point(S, r00, r1, vc_r2, eint_m, 4, 4, rim);
        turning_point(S, r1, rmax, vc_r2, eint_m, 10, 4, rom);
        double act_m = action_integral(S, F, rim, rom, vc_r2, eint_m, twomu);
        double dade = 0.5 * (act_p - act_m) / deint;
        double act = action_integral(S, F, ro, r3, vc_r2, eint, twomu);
        double gam = exp(-act) / dade;
        if (1.0 / gam < F.tthresau) itype = 4;
        act = act * 0.5 / PI;
        double rho2 = gamma_fct(act) - act * (log(fabs(act)) - 1.0);
        viba = viba + rho2 * F.rfact;
      }
      viba = viba * 0.5 / PI;
    }
  }
  itype = itype - 1;
  if (itype == 2) angmom = 0.5;
  m.ipair = ipair;
  m.itype = itype;
  m.eint = eint;
  m.angmom = angmom;
  m.viba = viba;
}

// Analyze for 3 atoms (the atom-diatom systems); p = velocities + coordinates
static __device__ void analyze3(const DevSys& S, const FsArgs& F, const double* __restrict__ p, cair_traj_point& o) {
  double xx[3][3], xd[3][3];
  for (int a = 0; a < 2; ++a)
    for (int d = 0; d < 3; ++d) { xd[d][a] = p[d + 3 * a]; xx[d][a] = p[d + 3 * a + 6]; }
  for (int d = 0; d < 3; ++d) {
    xd[d][2] = (0.0 + S.mMiMn[0] * p[d]) + S.mMiMn[1] * p[d + 3];
    xx[d][2] = (0.0 + S.mMiMn[0] * p[d + 6]) + S.mMiMn[1] * p[d + 9];
  }
  const int pa[3] = {0, 0, 1}, pb[3] = {1, 2, 2};
  double rbs[3];
  for (int q = 0; q < 3; ++q) {
    double a = xx[0][pa[q]] - xx[0][pb[q]], b = xx[1][pa[q]] - xx[1][pb[q]], c = xx[2][pa[q]] - xx[2][pb[q]];
    rbs[q] = a * a + b * b + c * c;
  }
  int ip = 1;
  if (rbs[1] < rbs[ip - 1]) ip = 2;
  if (rbs[2] < rbs[ip - 1]) ip = 3;
  int m1a = pa[ip - 1], m1b = pb[ip - 1];
  double cm[3][2], cmd[3][2];
  for (int d = 0; d < 3; ++d) {
    cm[d][0] = cm[d][1] = cmd[d][0] = cmd[d][1] = 0.0;
    for (int j = 0; j < 3; ++j) {
      int w = (j == m1a || j == m1b) ? 0 : 1;
      cm[d][w] = cm[d][w] + F.mass[j] * xx[d][j];
      cmd[d][w] = cmd[d][w] + F.mass[j] * xd[d][j];
    }
  }
  double xp = 0.0, xt = 0.0;
  for (int j = 0; j < 3; ++j) {
    if (j == m1a || j == m1b) xp = xp + F.mass[j];
    else xt = xt + F.mass[j];
  }
  double xpi = 1.0 / xp, xti = 1.0 / xt, xrel[3], vrel[3];
  for (int d = 0; d < 3; ++d) {
    cm[d][0] *= xpi; cm[d][1] *= xti; cmd[d][0] *= xpi; cmd[d][1] *= xti;
    xrel[d] = cm[d][0] - cm[d][1];
    vrel[d] = cmd[d][0] - cmd[d][1];
  }
  double xnum = xrel[0] * vrel[0] + xrel[1] * vrel[1] + xrel[2] * vrel[2];
  double v = vrel[0] * vrel[0] + vrel[1] * vrel[1] + vrel[2] * vrel[2];
  double tt = -xnum / v;
  double e0 = xrel[0] + tt * vrel[0], e1 = xrel[1] + tt * vrel[1], e2 = xrel[2] + tt * vrel[2];
  o.b = sqrt(e0 * e0 + e1 * e1 + e2 * e2);
  o.xkin = 0.0;
  for (int d = 0; d < 3; ++d) o.xkin = o.xkin + 0.5 * xp * (cmd[d][0] * cmd[d][0]) + 0.5 * xt * (cmd[d][1] * cmd[d][1]);
  for (int d = 0; d < 3; ++d) o.vrel[d] = vrel[d];
  o.nmol = 1;
  o.pad = 0;
  double X[6], XD[6];
  for (int d = 0; d < 3; ++d) {
    X[2 * d] = xx[d][m1a]; X[2 * d + 1] = xx[d][m1b];
    XD[2 * d] = xd[d][m1a]; XD[2 * d + 1] = xd[d][m1b];
  }
  find_state(S, F, ip, m1a, m1b, X, XD, o.mol[0]);
  o.mol[1].ipair = 0; o.mol[1].itype = 0; o.mol[1].eint = 0.0; o.mol[1].angmom = 0.0; o.mol[1].viba = 0.0;
}

// Analyze for 4 atoms (TrajectoryPoint_Class.F90:128-374 with SetPairs 417-495): the closest pair
// (mapped onto a pair of atom 1) and its opposite pair are the two molecules, unless the third
// closest squared distance is below rmaxCluster (25 bohr^2, Input_Class.F90:166), a cluster: then
// both molecules get iPair = -1, itype = -10, viba = AngMom = -1.
constexpr double kRmaxCluster = 25.0;

static __device__ void analyze4(const DevSys& S, const FsArgs& F, const double* __restrict__ p, cair_traj_point& o) {
  double xx[3][4], xd[3][4];
  for (int a = 0; a < 3; ++a)
    for (int d = 0; d < 3; ++d) { xd[d][a] = p[d + 3 * a]; xx[d][a] = p[d + 3 * a + 9]; }
  for (int d = 0; d < 3; ++d) {
    xd[d][3] = ((0.0 + S.mMiMn[0] * p[d]) + S.mMiMn[1] * p[d + 3]) + S.mMiMn[2] * p[d + 6];
    xx[d][3] = ((0.0 + S.mMiMn[0] * p[d + 9]) + S.mMiMn[1] * p[d + 12]) + S.mMiMn[2] * p[d + 15];
  }
  const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
  double rbs[6];
  int irbs[6];
  for (int q = 0; q < 6; ++q) {
    double a = xx[0][pa[q]] - xx[0][pb[q]], b = xx[1][pa[q]] - xx[1][pb[q]], c = xx[2][pa[q]] - xx[2][pb[q]];
    rbs[q] = a * a + b * b + c * c;
    irbs[q] = q + 1;
  }
  for (int i = 1; i < 6; ++i)  // ascending with index (hpsort, Sorting_Module.F90:20-83)
    for (int j = i; j > 0 && rbs[j - 1] > rbs[j]; --j) {
      double t = rbs[j]; rbs[j] = rbs[j - 1]; rbs[j - 1] = t;
      int k = irbs[j]; irbs[j] = irbs[j - 1]; irbs[j - 1] = k;
    }
  o.nmol = 2;
  o.pad = 0;
  int ip1;
  if (rbs[1] > 100.0) {
    ip1 = irbs[0] <= 3 ? irbs[0] : 7 - irbs[0];
  } else if (rbs[2] < kRmaxCluster) {
    o.b = 0.0;
    o.xkin = 0.0;
    for (int d = 0; d < 3; ++d) o.vrel[d] = 0.0;
    for (int im = 0; im < 2; ++im) {
      o.mol[im].ipair = -1; o.mol[im].itype = -10; o.mol[im].eint = 0.0;
      o.mol[im].angmom = -1.0; o.mol[im].viba = -1.0;
    }
    return;
  } else {
    ip1 = irbs[0] < irbs[1] ? irbs[0] : irbs[1];
    if (ip1 > 3) ip1 = 7 - ip1;
  }
  const int ip2 = 7 - ip1;  // opposite pair
  const int m1a = pa[ip1 - 1], m1b = pb[ip1 - 1];
  double cm[3][2], cmd[3][2];
  for (int d = 0; d < 3; ++d) {
    cm[d][0] = cm[d][1] = cmd[d][0] = cmd[d][1] = 0.0;
    for (int j = 0; j < 4; ++j) {
      int w = (j == m1a || j == m1b) ? 0 : 1;
      cm[d][w] = cm[d][w] + F.mass[j] * xx[d][j];
      cmd[d][w] = cmd[d][w] + F.mass[j] * xd[d][j];
    }
  }
  double xp = 0.0, xt = 0.0;
  for (int j = 0; j < 4; ++j) {
    if (j == m1a || j == m1b) xp = xp + F.mass[j];
    else xt = xt + F.mass[j];
  }
  double xpi = 1.0 / xp, xti = 1.0 / xt, xrel[3], vrel[3];
  for (int d = 0; d < 3; ++d) {
    cm[d][0] *= xpi; cm[d][1] *= xti; cmd[d][0] *= xpi; cmd[d][1] *= xti;
    xrel[d] = cm[d][0] - cm[d][1];
    vrel[d] = cmd[d][0] - cmd[d][1];
  }
  double xnum = xrel[0] * vrel[0] + xrel[1] * vrel[1] + xrel[2] * vrel[2];
  double v = vrel[0] * vrel[0] + vrel[1] * vrel[1] + vrel[2] * vrel[2];
  double tt = -xnum / v;
  double e0 = xrel[0] + tt * vrel[0], e1 = xrel[1] + tt * vrel[1], e2 = xrel[2] + tt * vrel[2];
  o.b = sqrt(e0 * e0 + e1 * e1 + e2 * e2);
  o.xkin = 0.0;
  for (int d = 0; d < 3; ++d) o.xkin = o.xkin + 0.5 * xp * (cmd[d][0] * cmd[d][0]) + 0.5 * xt * (cmd[d][1] * cmd[d][1]);
  for (int d = 0; d < 3; ++d) o.vrel[d] = vrel[d];
  for (int im = 0; im < 2; ++im) {
    const int ip = im == 0 ? ip1 : ip2, a = pa[ip - 1], b = pb[ip - 1];
    double X[6], XD[6];
    for (int d = 0; d < 3; ++d) {
      X[2 * d] = xx[d][a]; X[2 * d + 1] = xx[d][b];
      XD[2 * d] = xd[d][a]; XD[2 * d + 1] = xd[d][b];
    }
    find_state(S, F, ip, a, b, X, XD, o.mol[im]);
  }
}

template <int NA>
__device__ __forceinline__ void analyze(const DevSys& S, const FsArgs& F, const double* __restrict__ p,
                                        cair_traj_point& o) {
  if (NA == 3) analyze3(S, F, p, o);
  else analyze4(S, F, p, o);
}

#ifndef CAIR_MODEL_TU  // model-independent: built once, in the API translation unit
template <int NA>
__global__ void __launch_bounds__(128) k_find_state(DevSys S, FsArgs F, int64_t n, const double* __restrict__ paq,
                                                    cair_traj_point* __restrict__ out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    cair_traj_point o;
    analyze<NA>(S, F, paq + 6 * (NA - 1) * k, o);
    out[k] = o;
  }
}
#endif

}  // namespace cair
