// Warp integrator: one warp integrates one trajectory (the latency mode of the persistent integrator).
//
// The thread integrator (k_integrate) gives every lane its own trajectory, which is the fastest use
// of the FP64 pipe while the queue holds many more trajectories than lanes.  A small job, or the
// long trajectories a queue ends on, leave it with lanes that advance one trajectory each: GB300
// issues an FP64 warp instruction every 64 cycles per sub-partition, and a dependent one completes
// 64 cycles later, whatever the active lanes -- a lone lane makes ~2,500 Bulirsch-Stoer attempts per
// second.  Here a warp owns a trajectory:
//
//  * a group of W lanes evaluates a right-hand side together: the lane-parallel programs of
//    generated/warp_prog.h (Tpq p, distances, MEG variables, diatomics, the PIP and its adjoint,
//    TransToCart) run level by level from shared memory (cair_warp.cuh);
//  * diatom + atom (W = 16): the two half-warps run different modified-midpoint sequences of the
//    same attempt side by side (NSteps 3: the n = 6 sequence on one, n = 2 then n = 4 on the other),
//    so an attempt takes 1 + 6 right-hand-side latencies instead of 13; diatom + diatom (W = 32,
//    NE = 18) runs its sequences one after the other on the whole warp;
//  * lane l < NE of each group holds equation l of the state (y, the sequences' midpoint values); the
//    extrapolation (RatPolExtrap) and step control run on every lane with warp-wide error reductions
//    (__all_sync), so the state stays replicated without broadcasts.
//
// Trajectories come from the same device queue, with the same end-of-collision check every ncall
// attempts (the energy program gives H and 1/R_p) and the same outputs as k_integrate.
#include <cuda_runtime.h>

#include <type_traits>

#define CAIR_MODEL_TU  // model-independent kernels are built in the API translation unit
#include "cair_kernels.cuh"
#include "cair_warp.cuh"
#include "cair_warp_launch.h"

namespace cair {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// Warps (trajectories) per CTA: the CTA shares one shared-memory copy of the programs.  Diatom + atom:
// 4 (several CTAs per SM); diatom + diatom, whose programs take over 100 KB: one CTA per SM with as
// many warps as its slot arrays leave room for.
template <int MODEL>
struct WLaunch {
  static constexpr int W = WCfg<MODEL>::W, NG = WCfg<MODEL>::NG;
  static constexpr size_t PROG_BYTES = (size_t)WCfg<MODEL>::NLEV * W * 32;
  static constexpr size_t WARP_BYTES = (size_t)NG * WCfg<MODEL>::NSLOT * 8;
  // as many warps as the shared memory left after the programs holds (about 220 KB per SM), up to 8
  static constexpr int FIT = (int)((225 * 1024 - PROG_BYTES) / WARP_BYTES);
  static constexpr int CTA = W == 16 ? 4 : (FIT < 8 ? FIT : 8);
  static constexpr size_t SMEM = PROG_BYTES + (size_t)CTA * WARP_BYTES;
  static_assert(CTA >= 1, "programs too large for shared memory");
};

// Sequence schedule: the stage (1-based) group grp runs as its i-th sequence, 0 when it has none
// left.  Two groups: both take the same number of right-hand sides.  One group: stages in order.
template <int NS, int NG>
__device__ __forceinline__ int wstage(int grp, int i) {
  if (NG == 1) return i < NS ? i + 1 : 0;
  if (NS == 2) return i == 0 ? (grp == 0 ? 2 : 1) : 0;
  if (NS == 3) return grp == 0 ? (i == 0 ? 3 : 0) : (i == 0 ? 1 : i == 1 ? 2 : 0);
  return grp == 0 ? (i == 0 ? 4 : i == 1 ? 1 : 0) : (i == 0 ? 3 : i == 1 ? 2 : 0);
}
template <int NS, int NG>
__host__ __device__ constexpr int wrounds() {
  return NG == 1 ? nseq_total(NS) - 1 : NS == 2 ? 4 : NS == 3 ? 6 : 10;
}
template <int NS, int NG>
__device__ __forceinline__ int wowner(int stage) {
  if (NG == 1) return 0;
  if (NS == 2) return stage == 2 ? 0 : 1;
  if (NS == 3) return stage == 3 ? 0 : 1;
  return (stage == 4 || stage == 1) ? 0 : 1;
}

// The grad and energy programs copied into shared memory (`tab`), returned pointing there.
__device__ __forceinline__ void stage_programs(unsigned* tab, WModel& M, int W) {
  int off = 0;
  auto copy = [&](WProg& p) {
    const int n16 = 2 * W * p.nlev;  // 16-byte halves of the 32-byte records
    const uint4* src = reinterpret_cast<const uint4*>(p.rec);
    uint4* dst = reinterpret_cast<uint4*>(tab + off);
    for (int i = threadIdx.x; i < n16; i += blockDim.x) dst[i] = src[i];
    p.rec = tab + off;
    off += 4 * n16;
  };
  copy(M.grad);
  copy(M.energy);
}

// The levels of a program on a group of W lanes: lane gl runs its record of each level (the next
// level's record is loaded while this one computes), the warp meets between levels.
template <int W>
__device__ __forceinline__ void run_levels(const WProg& p, double* s, int gl) {
  const uint4* R = reinterpret_cast<const uint4*>(p.rec) + 2 * gl;
  char* sb = reinterpret_cast<char*>(s);
  uint4 c0 = R[0], c1 = R[1];
#pragma unroll 2
  for (int L = 0; L < p.nlev; ++L) {
    uint4 n0 = c0, n1 = c1;
    if (L + 1 < p.nlev) {
      n0 = R[2 * W * (L + 1)];
      n1 = R[2 * W * (L + 1) + 1];
    }
    if (c0.x >> 31) *reinterpret_cast<double*>(sb + c0.y) = wp_eval(c0, c1, sb);
    __syncwarp();
    c0 = n0;
    c1 = n1;
  }
}

// Constants of surface P into every group's slots, then the const program on each.
template <int W, int NG>
__device__ __forceinline__ void load_constants(const WModel& M, const DevSys& S, const DevPes& P, double* slots,
                                               double* s, int lane, int gl) {
  for (int i = lane; i < M.nconst; i += 32) {
    const double v = wp_const(M, S, P, i);
#pragma unroll
    for (int g = 0; g < NG; ++g) slots[g * M.nslot + i] = v;
  }
  __syncwarp();
  run_levels<W>(M.cprog, s, gl);
}

// One program on every group: lane gl < NE puts its input, the levels run, it reads its output.
template <int W>
__device__ __forceinline__ double run_program(const WProg& p, double* s, int gl, bool io, int in, int out,
                                              double v) {
  if (io) s[in] = v;
  __syncwarp();
  run_levels<W>(p, s, gl);
  return io ? s[out] : 0.0;
}

template <int S1, int NS>
__device__ __forceinline__ void extrap_one(const double (&est)[NS], const double (&xs)[NS], double (&d)[NS - 1][1],
                                           double (&yt)[NS - 1][1], double (&ylast)[1]) {
  if constexpr (S1 <= NS) {
    const double e[1] = {est[S1 - 1]};
    extrap_stage<S1, 1, NS>(e, xs, d, yt, ylast);
    extrap_one<S1 + 1, NS>(est, xs, d, yt, ylast);
  }
}

// One Bulirsch-Stoer attempt of the warp's trajectory (Integrate_ODE_1d, ODE_Solver.F90:225-358, with
// the same arithmetic per equation as bs_attempt) from dydx = f(y).  Returns bit 0 when a difference of
// extrapolants is NaN, bit 1 when the step was accepted (a rejected step leaves y, and so f(y), as
// they were: the caller reuses dydx).
template <int W, int NG, int NS>
__device__ __forceinline__ int warp_attempt(const WProg& G, double* s, int gl, int grp, bool io, int in, int out,
                                            double dydx, double& y, double& x, double& h, double yscal,
                                            double relax, bool incstp, double& smax, double& smin, int& irej,
                                            int& iste) {
  double est[NS];
#pragma unroll
  for (int j = 0; j < NS; ++j) est[j] = 0.0;
  int si = 0, stage = wstage<NS, NG>(grp, 0);
  int nst = nseq_of(stage - 1), sub = 1;
  double hs = h * htemp_of(stage), h2 = 2.0 * hs;
  double ym = y, yn = y + hs * dydx;
#pragma unroll 1
  for (int r = 0; r < wrounds<NS, NG>(); ++r) {
    const double fo = run_program<W>(G, s, gl, io, in, out, yn);
    if (stage > 0) {
      if (sub == nst) {
        // end of mmidv: yout = Half*(ym + yn + h*yout)
        const double e = 0.5 * (ym + yn + hs * fo);
#pragma unroll
        for (int j = 0; j < NS; ++j)
          if (j == stage - 1) est[j] = e;
        stage = wstage<NS, NG>(grp, ++si);
        if (stage > 0) {
          nst = nseq_of(stage - 1);
          hs = h * htemp_of(stage);
          h2 = 2.0 * hs;
          sub = 1;
          ym = y;
          yn = y + hs * dydx;
        }
      } else {
        const double ys = ym + h2 * fo;
        ym = yn;
        yn = ys;
        ++sub;
      }
    }
  }
  // every lane gets every sequence's estimate of its equation
  if (NG == 2) {
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      const double o = __shfl_xor_sync(kFull, est[j], 16);
      if (wowner<NS, NG>(j + 1) != grp) est[j] = o;
    }
  }
  double xs[NS];
#pragma unroll
  for (int st = 1; st <= NS; ++st) {
    const double hh = h * htemp_of(st);
    xs[st - 1] = hh * hh;
  }
  double d[NS - 1][1], yt[NS - 1][1], ylast[1];
  extrap_one<1, NS>(est, xs, d, yt, ylast);
  // errmax(k) < 1 for k = 1..NS-1, over the NE equations
  bool below[NS - 1];
  int nan = 0;
#pragma unroll
  for (int k = 0; k < NS - 1; ++k) {
    bool ok = true;
    if (io) {
      const double dd = yt[k][0] - ylast[0];
      if (is_nan_bits(dd)) nan = 1;
      ok = err_below_one(dd, yscal);
    }
    below[k] = __all_sync(kFull, ok);
  }
  nan = __any_sync(kFull, nan);
  int iconv = 0;
#pragma unroll
  for (int is = 2; is <= NS; ++is) {
    const int j = NS + 1 - is;
    if (!below[j - 1]) break;
    iconv = j;
  }
  const bool accept = below[NS - 2];
  if (accept) {
    x = x + h;
    y = ylast[0];
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
  return nan | (accept ? 2 : 0);
}

template <int MODEL, int NS>
__global__ void __launch_bounds__(32 * WLaunch<MODEL>::CTA, 1) k_integrate_warp(DevSys S, IntegrateArgs A) {
  constexpr int NE = Traits<MODEL>::NE, NP = Traits<MODEL>::NP;
  constexpr int W = WCfg<MODEL>::W, NG = WCfg<MODEL>::NG;
  static_assert(NE <= W, "a group holds one equation per lane");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned* tab = reinterpret_cast<unsigned*>(smem_raw);
  WModel M = wmodel<MODEL>();
  stage_programs(tab, M, W);
  const int lane = threadIdx.x & 31, grp = lane / W, gl = lane % W;
  double* slots = reinterpret_cast<double*>(smem_raw + WLaunch<MODEL>::PROG_BYTES) +
                  (size_t)(threadIdx.x >> 5) * NG * M.nslot;
  double* s = slots + grp * M.nslot;
  __syncthreads();
  const bool io = gl < NE;
  const int gin = io ? M.gin[gl] : 0, gout = io ? M.gout[gl] : 0, ein = io ? M.ein[gl] : 0;
  int eR[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) eR[p] = M.eout[1 + p];
  const int eH = M.eout[0];
  const bool incstp = S.incstp != 0;
  const int ncall = S.ncall;
  unsigned long long c_att = 0, c_acc = 0, c_rej = 0, blocks = 0;
  const unsigned long long warp_id = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) >> 5;
  if (A.warp_times && lane == 0) A.warp_times[4 * warp_id] = globaltimer_ns();
  int loaded = -1;
  // a hand-off list's length is known only on the device
  const unsigned long long ntraj = A.n_dev ? *A.n_dev : (unsigned long long)A.n;
#pragma unroll 1
  for (;;) {
    unsigned long long q = 0;
    if (lane == 0) q = atomicAdd(A.queue, 1ull);
    q = __shfl_sync(kFull, q, 0);
    if (q >= ntraj) break;
    const unsigned long long k = A.order ? (unsigned long long)A.order[q] : q;
    const int ip = A.ipes ? A.ipes[k] : 0;
    if (ip != loaded) {
      load_constants<W, NG>(M, S, S.pes[ip], slots, s, lane, gl);
      loaded = ip;
    }
    double y = io ? A.paq[NE * k + gl] : 0.0;
    const double yscal = io ? A.erra[NE * k + gl] : 1.0;
    double x = A.t[k], h = A.dt[k], smax = A.smax[k], smin = A.smin[k], H = 0.0;
    int irej = A.irej[k], iste = A.iste[k];
    const int irej0 = irej, iste0 = iste;
    int64_t att = A.att0 ? A.att0[k] : 0;
    const int64_t att_start = att;
    double dydx = 0.0;
    bool fresh = false;  // dydx = f(y) of the current y
#pragma unroll 1
    for (;;) {
      int bad = 0;
#pragma unroll 1
      for (int c = 0; c < ncall; ++c) {
        if (!fresh) dydx = run_program<W>(M.grad, s, gl, io, gin, gout, y);
        const int r = warp_attempt<W, NG, NS>(M.grad, s, gl, grp, io, gin, gout, dydx, y, x, h, yscal, S.relax,
                                              incstp, smax, smin, irej, iste);
        bad |= r & 1;
        fresh = !(r & 2);
      }
      att += ncall;
      ++blocks;
      // end check (Integrator_Class.F90:457-465): H and 1/R_p of the new point
      run_program<W>(M.energy, s, gl, io, ein, 0, y);
      H = s[eH];
      double rpi[NP];
#pragma unroll
      for (int p = 0; p < NP; ++p) rpi[p] = s[eR[p]];
      bool conv = x > S.tmax;
#pragma unroll
      for (int p = 0; p < NP; ++p) conv = conv || (rpi[p] < S.rpimax);
      if constexpr (NP == 3) {
        if (A.rec && lane == 0) {
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
        if (io && grp == 0) A.paq[NE * k + gl] = y;
        if (lane == 0) {
          A.t[k] = x;
          A.dt[k] = h;
          A.H[k] = H;
          A.smax[k] = smax;
          A.smin[k] = smin;
          A.irej[k] = irej;
          A.iste[k] = iste;
          A.status[k] = bad ? CAIR_TRAJ_NONFINITE : (conv ? CAIR_TRAJ_DONE : CAIR_TRAJ_ATTEMPT_CAP);
          c_att += att - att_start;
          c_acc += iste - iste0;
          c_rej += irej - irej0;
        }
        break;
      }
    }
    __syncwarp();
  }
  if (lane == 0) {
    if (A.warp_times) {
      A.warp_times[4 * warp_id + 1] = globaltimer_ns();
      A.warp_times[4 * warp_id + 2] = 32ull * blocks;
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
}

// n points y[n][NE] -> dy/dt, H and 1/R_p through the lane-parallel programs, one point per group
// (the parity tests' entry to the programs on the GPU).
template <int MODEL>
__global__ void __launch_bounds__(32 * WLaunch<MODEL>::CTA, 1) k_warp_eval(DevSys S, int64_t n,
                                                                           const int32_t* __restrict__ ipes,
                                                                           const double* __restrict__ y,
                                                                           double* __restrict__ yp,
                                                                           double* __restrict__ H,
                                                                           double* __restrict__ Ri) {
  constexpr int NE = Traits<MODEL>::NE, NP = Traits<MODEL>::NP;
  constexpr int W = WCfg<MODEL>::W, NG = WCfg<MODEL>::NG;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned* tab = reinterpret_cast<unsigned*>(smem_raw);
  WModel M = wmodel<MODEL>();
  stage_programs(tab, M, W);
  const int lane = threadIdx.x & 31, grp = lane / W, gl = lane % W;
  double* s = reinterpret_cast<double*>(smem_raw + WLaunch<MODEL>::PROG_BYTES) +
              (size_t)(threadIdx.x >> 5) * NG * M.nslot + grp * M.nslot;
  __syncthreads();
  const bool io = gl < NE;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t base = NG * ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5); base < n; base += NG * nwarps) {
    const int64_t k = base + grp < n ? base + grp : base;
    const int ip = ipes ? ipes[k] : 0;
    const bool ok = ip >= 0 && ip < S.npes;  // a surface index out of range gives NaN, not a read past S.pes
    const DevPes& P = S.pes[ok ? ip : 0];
    for (int i = gl; i < M.nconst; i += W) s[i] = ok ? wp_const(M, S, P, i) : __longlong_as_double(0x7ff8000000000000ll);
    __syncwarp();
    run_levels<W>(M.cprog, s, gl);
    const double v = io ? y[NE * k + gl] : 0.0;
    const double f = run_program<W>(M.grad, s, gl, io, io ? M.gin[gl] : 0, io ? M.gout[gl] : 0, v);
    const bool mine = base + grp < n;
    if (io && mine) yp[NE * k + gl] = f;
    run_program<W>(M.energy, s, gl, io, io ? M.ein[gl] : 0, 0, v);
    if (mine && gl <= NP) {
      const double e = s[M.eout[gl]];
      if (gl == 0) H[k] = e;
      else Ri[NP * k + gl - 1] = e;
    }
    __syncwarp();
  }
}

template <class K>
int fit_smem(K kern, size_t smem) {
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 1;
  return 0;
}

template <int MODEL, int NS>
int launch_ns(int nsm, int per_sm_cap, cudaStream_t st, const DevSys& S, IntegrateArgs A, int64_t warp_times_cap,
              int64_t* nwarps) {
  using LW = WLaunch<MODEL>;
  auto kern = k_integrate_warp<MODEL, NS>;
  if (fit_smem(kern, LW::SMEM)) return 1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * LW::CTA, LW::SMEM) != cudaSuccess) return 1;
  if (per_sm_cap > 0 && per_sm_cap < per_sm) per_sm = per_sm_cap;
  if (per_sm < 1) per_sm = 1;
  int64_t g = (int64_t)nsm * per_sm;
  const int64_t need = (A.n + LW::CTA - 1) / LW::CTA;
  if (g > need) g = need;
  if (g < 1) g = 1;
  // the warp timeline records only when it has room for every warp of the launch
  if (g * LW::CTA > warp_times_cap) A.warp_times = nullptr;
  if (nwarps) *nwarps = A.warp_times ? g * LW::CTA : 0;
  kern<<<(unsigned)g, 32 * LW::CTA, LW::SMEM, st>>>(S, A);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

template <int MODEL>
int launch_model(int nsm, int per_sm_cap, cudaStream_t st, const DevSys& S, const IntegrateArgs& A,
                 int64_t warp_times_cap, int64_t* nwarps) {
  if (S.nsteps == 2) return launch_ns<MODEL, 2>(nsm, per_sm_cap, st, S, A, warp_times_cap, nwarps);
  if (S.nsteps == 4) return launch_ns<MODEL, 4>(nsm, per_sm_cap, st, S, A, warp_times_cap, nwarps);
  return launch_ns<MODEL, 3>(nsm, per_sm_cap, st, S, A, warp_times_cap, nwarps);
}

template <int MODEL>
int eval_model(int nsm, cudaStream_t st, const DevSys& S, int64_t n, const int32_t* ipes, const double* y,
               double* yp, double* H, double* Ri) {
  using LW = WLaunch<MODEL>;
  auto kern = k_warp_eval<MODEL>;
  if (fit_smem(kern, LW::SMEM)) return 1;
  const int per_cta = LW::CTA * LW::NG;
  int64_t g = (n + per_cta - 1) / per_cta;
  if (g > 4 * (int64_t)nsm) g = 4 * (int64_t)nsm;
  if (g < 1) g = 1;
  kern<<<(unsigned)g, 32 * LW::CTA, LW::SMEM, st>>>(S, n, ipes, y, yp, H, Ri);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

template <class F>
int with_warp_model(const DevSys& S, F f) {
  switch (S.pes[0].model) {
    case CAIR_PES_O3_UMN: return f(std::integral_constant<int, CAIR_PES_O3_UMN>{});
    case CAIR_PES_N3_UMN: return f(std::integral_constant<int, CAIR_PES_N3_UMN>{});
    case CAIR_PES_O4_UMN: return f(std::integral_constant<int, CAIR_PES_O4_UMN>{});
    case CAIR_PES_N4_UMN: return f(std::integral_constant<int, CAIR_PES_N4_UMN>{});
    case CAIR_PES_O3_NN: return f(std::integral_constant<int, CAIR_PES_O3_NN>{});
    default: return f(std::integral_constant<int, CAIR_PES_O3_BNN>{});
  }
}

}  // namespace

bool warp_integrate_supported(const DevSys& S) {
  if (S.nsteps < 2 || S.nsteps > 4 || S.npes < 1) return false;
  for (int p = 0; p < S.npes; ++p)
    if (!warp_model_built(S.pes[p].model) || S.pes[p].model != S.pes[0].model) return false;
  return S.diat == warp_model_diat(S.pes[0].model);
}

int warp_integrate_launch(int nsm, int per_sm_cap, cudaStream_t st, const DevSys& S, const IntegrateArgs& A,
                          int64_t warp_times_cap, int64_t* nwarps) {
  if (!warp_integrate_supported(S)) return 2;
  return with_warp_model(S, [&](auto m) {
    return launch_model<decltype(m)::value>(nsm, per_sm_cap, st, S, A, warp_times_cap, nwarps);
  });
}

int warp_eval_launch(int nsm, cudaStream_t st, const DevSys& S, int64_t n, const int32_t* ipes, const double* y,
                     double* yp, double* H, double* Ri) {
  if (!warp_integrate_supported(S)) return 2;
  return with_warp_model(S, [&](auto m) { return eval_model<decltype(m)::value>(nsm, st, S, n, ipes, y, yp, H, Ri); });
}

int64_t warp_resident_warps(int nsm, const DevSys& S) {
  if (!warp_integrate_supported(S)) return 0;
  return with_warp_model(S, [&](auto m) {
    using LW = WLaunch<decltype(m)::value>;
    auto kern = k_integrate_warp<decltype(m)::value, 3>;
    int per_sm = 0;
    if (fit_smem(kern, LW::SMEM) ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * LW::CTA, LW::SMEM) != cudaSuccess)
      return 0;
    return (int)((int64_t)nsm * per_sm * LW::CTA);
  });
}

}  // namespace cair
