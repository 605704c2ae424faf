// Host build of the library's device surface code -- TEST INFRASTRUCTURE ONLY.
//
// coarseair_gb300/csrc/cair_device.cuh is included unchanged: the CUDA qualifiers are defined away and
// the four device intrinsics it uses get host equivalents with the same bit-level meaning.  The
// tests fill the DevSys through the library's own setup (cair_internal_setup_system) and compare
// these evaluations with the oracle, so surface code can be checked without a GPU.  Arithmetic
// differs from the GPU's only where nvcc contracts a * b + c into a fused multiply-add.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#define __device__
#define __host__
#define __forceinline__ inline
#define __constant__
#define __global__
static inline int __double2loint(double d) {
  uint64_t u;
  std::memcpy(&u, &d, 8);
  return (int)(uint32_t)u;
}
static inline int __double2hiint(double d) {
  uint64_t u;
  std::memcpy(&u, &d, 8);
  return (int)(uint32_t)(u >> 32);
}
static inline double __hiloint2double(int hi, int lo) {
  const uint64_t u = ((uint64_t)(uint32_t)hi << 32) | (uint32_t)lo;
  double d;
  std::memcpy(&d, &u, 8);
  return d;
}
static inline long long __double_as_longlong(double d) {
  long long u;
  std::memcpy(&u, &d, 8);
  return u;
}
template <class T>
static inline T __ldg(const T* p) {
  return *p;
}
static inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }
using std::max;
using std::min;
struct uint4 {
  unsigned x, y, z, w;
};
// one host "thread" that owns a 1 x 1 grid: the kernels' grid-stride loops then visit every element
struct HostDim {
  unsigned x, y, z;
};
static const HostDim threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0}, blockDim = {1, 1, 1}, gridDim = {1, 1, 1};
#define __launch_bounds__(...)
template <class T>
static inline T atomicAdd(T* p, T v) {
  const T o = *p;
  *p = o + v;
  return o;
}
static inline void __syncwarp(unsigned = 0xffffffffu) {}
static inline int __any_sync(unsigned, int pred) { return pred; }
// one host lane: the ballot holds only its own bit
static inline unsigned __ballot_sync(unsigned, int pred) { return pred ? 1u : 0u; }
static inline int __popc(unsigned x) { return __builtin_popcount(x); }
template <class T>
static inline T atomicExch(T* p, T v) {
  const T o = *p;
  *p = v;
  return o;
}
template <class T>
static inline T atomicMin(T* p, T v) {
  const T o = *p;
  if (v < o) *p = v;
  return o;
}
template <class T>
static inline T atomicCAS(T* p, T cmp, T v) {
  const T o = *p;
  if (o == cmp) *p = v;
  return o;
}

#include "../../coarseair_gb300/csrc/cair_ic.cuh"
#include "../../coarseair_gb300/csrc/cair_stats.cuh"
#include "../../coarseair_gb300/csrc/cair_warp.cuh"

#include <vector>

using namespace cair;

template <int MODEL>
static void eval(const DevSys& S, int64_t n, const int32_t* ipes, const double* Rin, const double* Qin, double* V,
                 double* dVdR, double* dVdQ, int grad) {
  using T = Traits<MODEL>;
  for (int64_t k = 0; k < n; ++k) {
    const DevPes& P = S.pes[ipes ? ipes[k] : 0];
    double R[T::NP], Ri[T::NP], Q[3 * T::NA], v, g[T::NP], m[T::NV];
    for (int i = 0; i < T::NP; ++i) {
      R[i] = Rin[T::NP * k + i];
      Ri[i] = 1.0 / R[i];
    }
    for (int i = 0; i < 3 * T::NA; ++i) Q[i] = Qin[3 * T::NA * k + i];
    if (grad) pes<MODEL, true>(S, P, R, Ri, Q, v, g, m);
    else pes<MODEL, false>(S, P, R, Ri, Q, v, g, m);
    V[k] = v;
    if (grad) {
      for (int i = 0; i < T::NP; ++i) dVdR[T::NP * k + i] = g[i];
      for (int i = 0; i < T::NV; ++i) dVdQ[T::NV * k + i] = m[i];
    }
  }
}

// k_bs_steps on the host: nattempts Bulirsch-Stoer attempts per trajectory with the device's Rhs and
// bs_attempt.
template <int MODEL, int NS>
static void bs_steps(const DevSys& S, int64_t n, const int32_t* ipes, double* paq, double* t, double* dt,
                     const double* erra, int nattempts) {
  constexpr int NE = Traits<MODEL>::NE;
  for (int64_t k = 0; k < n; ++k) {
    Rhs<MODEL> f(S, S.pes[ipes ? ipes[k] : 0]);
    double y[NE];
    for (int i = 0; i < NE; ++i) y[i] = paq[NE * k + i];
    double x = t[k], h = dt[k], smax = 0.0, smin = 0.0;
    int irej = 0, iste = 0;
    for (int a = 0; a < nattempts; ++a)
      bs_attempt<NE, NS>(f, y, x, h, erra + NE * k, S.relax, S.incstp != 0, smax, smin, irej, iste);
    for (int i = 0; i < NE; ++i) paq[NE * k + i] = y[i];
    t[k] = x;
    dt[k] = h;
  }
}

template <int MODEL>
static int bs_steps_ns(const DevSys& S, int64_t n, const int32_t* ipes, double* paq, double* t, double* dt,
                       const double* erra, int nattempts) {
  switch (S.nsteps) {
    case 2: bs_steps<MODEL, 2>(S, n, ipes, paq, t, dt, erra, nattempts); return 0;
    case 3: bs_steps<MODEL, 3>(S, n, ipes, paq, t, dt, erra, nattempts); return 0;
    case 4: bs_steps<MODEL, 4>(S, n, ipes, paq, t, dt, erra, nattempts); return 0;
    default: return 1;
  }
}

extern "C" int pes_host_bs_steps(const void* devsys, const double* packed, const int64_t* offsets, int64_t n,
                                 const int32_t* ipes, double* paq, double* t, double* dt, const double* erra,
                                 int nattempts) {
  DevSys S;
  std::memcpy(&S, devsys, sizeof S);
  for (int p = 0; p < S.npes; ++p) S.pes[p].coef = packed + offsets[p];
  switch (S.pes[0].model) {
    case CAIR_PES_O3_UMN: return bs_steps_ns<CAIR_PES_O3_UMN>(S, n, ipes, paq, t, dt, erra, nattempts);
    case CAIR_PES_N3_UMN: return bs_steps_ns<CAIR_PES_N3_UMN>(S, n, ipes, paq, t, dt, erra, nattempts);
    case CAIR_PES_O4_UMN: return bs_steps_ns<CAIR_PES_O4_UMN>(S, n, ipes, paq, t, dt, erra, nattempts);
    case CAIR_PES_O3_NN: return bs_steps_ns<CAIR_PES_O3_NN>(S, n, ipes, paq, t, dt, erra, nattempts);
    case CAIR_PES_N4_UMN: return bs_steps_ns<CAIR_PES_N4_UMN>(S, n, ipes, paq, t, dt, erra, nattempts);
    case CAIR_PES_O3_BNN: return bs_steps_ns<CAIR_PES_O3_BNN>(S, n, ipes, paq, t, dt, erra, nattempts);
    case CAIR_PES_N4_PIPNN: return bs_steps_ns<CAIR_PES_N4_PIPNN>(S, n, ipes, paq, t, dt, erra, nattempts);
    default: return 1;
  }
}

// Initial conditions of a batch of work items on the host: the streams drawn as k_ic_draws draws them
// (one per stream head, rings continuing their stream), then the body of k_sample_ic3 / k_sample_ic4
// over every trajectory.
template <int MODEL>
static void sample(const DevSys& S, int64_t ntot, const cair_work_item* items, const cair_level* levels,
                   const double* draws, const int32_t* item_of, double* paq, double* paq0, double* erra, double* H0,
                   double* b, int32_t* ipes, double* key) {
  if (Traits<MODEL>::NA == 3)
    k_sample_ic3<MODEL>(S, ntot, items, levels, draws, item_of, paq, paq0, erra, H0, b, ipes, key);
  else
    k_sample_ic4<MODEL>(S, ntot, items, levels, draws, item_of, paq, paq0, erra, H0, b, ipes, key);
}

extern "C" int ic_host_sample(const void* devsys, const double* packed, const int64_t* offsets,
                              const cair_level* levels, int32_t nitems, const cair_work_item* items, int64_t ntot,
                              double* paq, double* paq0, double* erra, double* H0, double* b, int32_t* ipes) {
  DevSys S;
  std::memcpy(&S, devsys, sizeof S);
  for (int p = 0; p < S.npes; ++p) S.pes[p].coef = packed + offsets[p];
  const int nmol = S.natoms == 4 ? 2 : 1;
  double* draws = new double[kDraws * (ntot > 0 ? ntot : 1)];
  int32_t* item_of = new int32_t[ntot > 0 ? ntot : 1];
  double* key = new double[ntot > 0 ? ntot : 1];
  for (int i = 0; i < nitems; ++i)
    if (!continues_stream(items, i)) stream_draws(items, nitems, i, nmol, levels, draws, item_of);
  int rc = 0;
  switch (S.pes[0].model) {
    case CAIR_PES_O3_UMN: sample<CAIR_PES_O3_UMN>(S, ntot, items, levels, draws, item_of, paq, paq0, erra, H0, b, ipes, key); break;
    case CAIR_PES_N3_UMN: sample<CAIR_PES_N3_UMN>(S, ntot, items, levels, draws, item_of, paq, paq0, erra, H0, b, ipes, key); break;
    case CAIR_PES_O4_UMN: sample<CAIR_PES_O4_UMN>(S, ntot, items, levels, draws, item_of, paq, paq0, erra, H0, b, ipes, key); break;
    case CAIR_PES_O3_NN: sample<CAIR_PES_O3_NN>(S, ntot, items, levels, draws, item_of, paq, paq0, erra, H0, b, ipes, key); break;
    case CAIR_PES_N4_UMN: sample<CAIR_PES_N4_UMN>(S, ntot, items, levels, draws, item_of, paq, paq0, erra, H0, b, ipes, key); break;
    case CAIR_PES_O3_BNN: sample<CAIR_PES_O3_BNN>(S, ntot, items, levels, draws, item_of, paq, paq0, erra, H0, b, ipes, key); break;
    case CAIR_PES_N4_PIPNN: sample<CAIR_PES_N4_PIPNN>(S, ntot, items, levels, draws, item_of, paq, paq0, erra, H0, b, ipes, key); break;
    default: rc = 1;
  }
  delete[] draws;
  delete[] item_of;
  delete[] key;
  return rc;
}

// cair_statistics_dev's steps on the host: the two counting kernels and the compaction over a 1 x 1
// grid on host arrays, with the library's host half (stats_runs, stats_rings, stats_finish) between
// and after them.
extern "C" int stats_host_run(const cair_stats_params* P, int32_t nitems, const cair_work_item* items,
                              const int32_t* item_run, int64_t ntot, const cair_traj_result* rows,
                              cair_final_state* out, int64_t cap, int64_t* nout) {
  StatsRuns runs;
  if (!stats_runs(nitems, items, item_run, runs).empty()) return 1;
  unsigned long long tsize = 1024;
  while (tsize < 2ull * (unsigned long long)ntot) tsize <<= 1;
  std::vector<unsigned long long> keys(tsize, kStatsEmpty), counts(tsize, 0), okeys(tsize), ocounts(tsize);
  std::vector<unsigned long long> item_rows(nitems, 0);
  std::vector<long long> item_ini(nitems, 0x7f7f7f7f7f7f7f7fll);
  std::vector<double> ring_b((size_t)runs.nruns * kMaxRings, 0.0);
  std::vector<unsigned long long> ring_rows((size_t)runs.nruns * kMaxRings, 0);
  std::vector<int32_t> run_of(runs.run_of), nring(runs.nruns, 0);
  int err = 0;
  StatsArgs A{};
  A.ntot = ntot;
  A.rows = rows;
  A.qnmax = P->qn_max;
  for (int q = 0; q < 5; ++q) {
    A.iskip[q] = P->iskip[q];
    A.pres[q] = P->pres_even_odd[q];
  }
  A.ham_abs_tol = P->ham_abs_tol;
  A.item_run = run_of.data();
  A.ring_b = ring_b.data();
  A.nring = nring.data();
  A.nruns = runs.nruns;
  A.R = 1;
  A.keys = keys.data();
  A.counts = counts.data();
  A.mask = tsize - 1;
  A.item_rows = item_rows.data();
  A.item_inicode = item_ini.data();
  A.ring_rows = ring_rows.data();
  A.error = &err;
  if (P->ncond == 3) k_stats_items<3>(A);
  else k_stats_items<5>(A);
  if (err) return 2;
  if (!stats_rings(*P, nitems, items, item_rows.data(), item_ini.data(), runs).empty()) return 3;
  std::copy(runs.ring_b.begin(), runs.ring_b.end(), ring_b.begin());
  std::copy(runs.nring.begin(), runs.nring.end(), nring.begin());
  A.R = runs.R;
  if (P->ncond == 3) k_stats_count<3>(A);
  else k_stats_count<5>(A);
  if (err) return 4;
  unsigned long long n = 0;
  k_stats_compact(keys.data(), counts.data(), tsize, okeys.data(), ocounts.data(), tsize, &n);
  return stats_finish(*P, runs, (int64_t)n, okeys.data(), ocounts.data(), ring_rows.data(), out, cap, nout).empty()
             ? 0
             : 5;
}

// cair_run_queue_dev's pipeline on the host, one lane: the streams and k_sample_ic3/4, the state of
// cair_k_init_state, k_integrate over the queue in item order (the GPU's longest-first order changes
// only the schedule), and k_results.  The final-state parameters come from the caller; the
// Chebyshev-2 nodes and Vinf are formed as cair_create forms them.
template <int MODEL, int NS>
static void queue_run(const DevSys& S, const FsArgs& F, int64_t ntot, const cair_work_item* items, int32_t* item_of,
                      double* paq, const double* paq0, const double* erra, const double* H0, const int32_t* ipes,
                      int64_t max_attempts, cair_traj_result* out) {
  constexpr int NE = Traits<MODEL>::NE;
  std::vector<double> t(ntot, 0.0), dt(ntot, S.dt0), smax(ntot, -1.7976931348623157e308),
      smin(ntot, 1.7976931348623157e308), H(ntot, 0.0);
  std::vector<int32_t> irej(ntot, 0), iste(ntot, 0), status(ntot, 0);
  unsigned long long ctl[6] = {0, 0, 0, 0, 0, 0};
  IntegrateArgs A{ntot, ipes, paq, t.data(), dt.data(), erra, H.data(), smax.data(), smin.data(), irej.data(),
                  iste.data(), status.data(), max_attempts, ctl, ctl + 1, nullptr};
  k_integrate<MODEL, NS>(S, A);
  (void)NE;
  if (Traits<MODEL>::NA == 3)
    k_results<3>(S, F, ntot, paq0, paq, H0, H.data(), t.data(), status.data(), iste.data(), irej.data(), item_of,
                 items, out);
  else
    k_results<4>(S, F, ntot, paq0, paq, H0, H.data(), t.data(), status.data(), iste.data(), irej.data(), item_of,
                 items, out);
}

template <int MODEL>
static int queue_run_ns(const DevSys& S, const FsArgs& F, int64_t ntot, const cair_work_item* items, int32_t* item_of,
                        double* paq, const double* paq0, const double* erra, const double* H0, const int32_t* ipes,
                        int64_t max_attempts, cair_traj_result* out) {
  switch (S.nsteps) {
    case 2: queue_run<MODEL, 2>(S, F, ntot, items, item_of, paq, paq0, erra, H0, ipes, max_attempts, out); return 0;
    case 3: queue_run<MODEL, 3>(S, F, ntot, items, item_of, paq, paq0, erra, H0, ipes, max_attempts, out); return 0;
    case 4: queue_run<MODEL, 4>(S, F, ntot, items, item_of, paq, paq0, erra, H0, ipes, max_attempts, out); return 0;
    default: return 1;
  }
}

extern "C" int queue_host_run(const void* devsys, const double* packed, const int64_t* offsets,
                              const cair_level* levels, int32_t nitems, const cair_work_item* items, int64_t ntot,
                              int64_t max_attempts, int32_t nquad, double rsmal, double rcent, double rfact,
                              double tthresau, cair_traj_result* out) {
  DevSys S;
  std::memcpy(&S, devsys, sizeof S);
  for (int p = 0; p < S.npes; ++p) S.pes[p].coef = packed + offsets[p];
  const int ne = S.ne, nmol = S.natoms == 4 ? 2 : 1;
  std::vector<double> draws(kDraws * ntot), paq(ne * ntot), paq0(ne * ntot), erra(ne * ntot), H0(ntot), b(ntot),
      key(ntot);
  std::vector<int32_t> item_of(ntot), ipes(ntot);
  for (int i = 0; i < nitems; ++i)
    if (!continues_stream(items, i)) stream_draws(items, nitems, i, nmol, levels, draws.data(), item_of.data());
  // final-state parameters (cair_create: GAUSSQ kind 3 in closed form, Vinf = the diatomic at 1e3 bohr)
  std::vector<double> gx(nquad), gw(nquad);
  const double pi = std::acos(-1.0);
  for (int i = 0; i < nquad; ++i) {
    const int k = nquad - i;
    const double th = (double)k * pi / (double)(nquad + 1), sn = std::sin(th);
    gx[i] = std::cos(th);
    gw[i] = pi / (double)(nquad + 1) * (sn * sn);
    gw[i] = gw[i] / std::sqrt(1.0 - gx[i] * gx[i]);
  }
  FsArgs F{};
  F.nquad = nquad;
  F.rsmal = rsmal;
  F.rcent = rcent;
  F.rfact = rfact;
  F.tthresau = tthresau;
  F.gx = gx.data();
  F.gw = gw.data();
  for (int i = 0; i < 4; ++i) F.mass[i] = S.mass[i];
  F.vinf = diat_v(S, 1.0E+03);
  int rc = 0;
#define QUEUE(M)                                                                                              \
  sample<M>(S, ntot, items, levels, draws.data(), item_of.data(), paq.data(), paq0.data(), erra.data(),        \
            H0.data(), b.data(), ipes.data(), key.data());                                                     \
  rc = queue_run_ns<M>(S, F, ntot, items, item_of.data(), paq.data(), paq0.data(), erra.data(), H0.data(),     \
                       ipes.data(), max_attempts, out);
  switch (S.pes[0].model) {
    case CAIR_PES_O3_UMN: QUEUE(CAIR_PES_O3_UMN) break;
    case CAIR_PES_N3_UMN: QUEUE(CAIR_PES_N3_UMN) break;
    case CAIR_PES_O4_UMN: QUEUE(CAIR_PES_O4_UMN) break;
    case CAIR_PES_O3_NN: QUEUE(CAIR_PES_O3_NN) break;
    case CAIR_PES_N4_UMN: QUEUE(CAIR_PES_N4_UMN) break;
    case CAIR_PES_O3_BNN: QUEUE(CAIR_PES_O3_BNN) break;
    case CAIR_PES_N4_PIPNN: QUEUE(CAIR_PES_N4_PIPNN) break;
    default: rc = 1;
  }
#undef QUEUE
  return rc;
}

extern "C" int64_t pes_host_devsys_size(void) { return (int64_t)sizeof(DevSys); }

// V, dV/dR and -dV/dQ of n points as the library's k_pes_eval computes them (surface model of
// surface 0; ipes may be null).
extern "C" int pes_host_eval(const void* devsys, const double* packed, const int64_t* offsets, int64_t n,
                             const int32_t* ipes, const double* R, const double* Q, double* V, double* dVdR,
                             double* dVdQ, int grad) {
  DevSys S;
  std::memcpy(&S, devsys, sizeof S);
  for (int p = 0; p < S.npes; ++p) S.pes[p].coef = packed + offsets[p];
  switch (S.pes[0].model) {
    case CAIR_PES_O3_UMN: eval<CAIR_PES_O3_UMN>(S, n, ipes, R, Q, V, dVdR, dVdQ, grad); break;
    case CAIR_PES_N3_UMN: eval<CAIR_PES_N3_UMN>(S, n, ipes, R, Q, V, dVdR, dVdQ, grad); break;
    case CAIR_PES_O4_UMN: eval<CAIR_PES_O4_UMN>(S, n, ipes, R, Q, V, dVdR, dVdQ, grad); break;
    case CAIR_PES_O3_NN: eval<CAIR_PES_O3_NN>(S, n, ipes, R, Q, V, dVdR, dVdQ, grad); break;
    case CAIR_PES_N4_UMN: eval<CAIR_PES_N4_UMN>(S, n, ipes, R, Q, V, dVdR, dVdQ, grad); break;
    case CAIR_PES_O3_BNN: eval<CAIR_PES_O3_BNN>(S, n, ipes, R, Q, V, dVdR, dVdQ, grad); break;
    case CAIR_PES_N4_PIPNN: eval<CAIR_PES_N4_PIPNN>(S, n, ipes, R, Q, V, dVdR, dVdQ, grad); break;
    default: return 1;
  }
  return 0;
}

// The warp integrator's lane-parallel programs run one instruction after the other: constants of each
// point's surface, the const program, then the grad program (y -> dy/dt) and the energy program
// (y -> H, 1/R_p) at n phase-space points y[n][NE].
template <int MODEL>
static void warp_eval(const DevSys& S, int64_t n, const int32_t* ipes, const double* y, double* yp, double* H,
                      double* Ri) {
  constexpr int NE = Traits<MODEL>::NE, NP = Traits<MODEL>::NP, W = WCfg<MODEL>::W;
  const WModel M = wmodel<MODEL>();
  std::vector<double> s(M.nslot);
  int loaded = -1;
  for (int64_t k = 0; k < n; ++k) {
    const int ip = ipes ? ipes[k] : 0;
    if (ip != loaded) {
      for (int i = 0; i < M.nconst; ++i) s[i] = wp_const(M, S, S.pes[ip], i);
      wp_run_serial(M.cprog, W, s.data());
      loaded = ip;
    }
    for (int i = 0; i < NE; ++i) s[M.gin[i]] = y[NE * k + i];
    wp_run_serial(M.grad, W, s.data());
    for (int i = 0; i < NE; ++i) yp[NE * k + i] = s[M.gout[i]];
    for (int i = 0; i < NE; ++i) s[M.ein[i]] = y[NE * k + i];
    wp_run_serial(M.energy, W, s.data());
    H[k] = s[M.eout[0]];
    for (int p = 0; p < NP; ++p) Ri[NP * k + p] = s[M.eout[1 + p]];
  }
}

extern "C" int warp_host_eval(const void* devsys, const double* packed, const int64_t* offsets, int64_t n,
                              const int32_t* ipes, const double* y, double* yp, double* H, double* Ri) {
  DevSys S;
  std::memcpy(&S, devsys, sizeof S);
  for (int p = 0; p < S.npes; ++p) S.pes[p].coef = packed + offsets[p];
  switch (S.pes[0].model) {
    case CAIR_PES_O3_UMN: warp_eval<CAIR_PES_O3_UMN>(S, n, ipes, y, yp, H, Ri); return 0;
    case CAIR_PES_N3_UMN: warp_eval<CAIR_PES_N3_UMN>(S, n, ipes, y, yp, H, Ri); return 0;
    case CAIR_PES_O4_UMN: warp_eval<CAIR_PES_O4_UMN>(S, n, ipes, y, yp, H, Ri); return 0;
    case CAIR_PES_N4_UMN: warp_eval<CAIR_PES_N4_UMN>(S, n, ipes, y, yp, H, Ri); return 0;
    case CAIR_PES_O3_NN: warp_eval<CAIR_PES_O3_NN>(S, n, ipes, y, yp, H, Ri); return 0;
    case CAIR_PES_O3_BNN: warp_eval<CAIR_PES_O3_BNN>(S, n, ipes, y, yp, H, Ri); return 0;
    default: return 1;
  }
}

// The library's table-driven exponential (cair_device.cuh fexp) at n points.
extern "C" void host_fexp(int64_t n, const double* x, double* y) {
  for (int64_t i = 0; i < n; ++i) y[i] = fexp(x[i]);
}

// The thread integrator with its tail hand-off on the host (one lane): n diatom + atom trajectories from
// paq/erra; once the queue is empty and at most hand_below are in flight, a trajectory is written back at its
// end check and listed in hand[] (hctl: in flight, hand-offs).  status[] is left as the caller set it for a
// handed-off trajectory.
template <int MODEL>
static void handoff_run(const DevSys& S, int64_t n, double* paq, const double* erra, int64_t max_attempts,
                        long long hand_below, double* t, double* dt, double* H, int32_t* irej, int32_t* iste,
                        int32_t* status, int32_t* hand, long long* hand_att, unsigned long long* hctl) {
  std::vector<double> smax(n, -1.7976931348623157e308), smin(n, 1.7976931348623157e308);
  for (int64_t k = 0; k < n; ++k) {
    t[k] = 0.0;
    dt[k] = S.dt0;
    irej[k] = iste[k] = 0;
  }
  unsigned long long ctl[6] = {0, 0, 0, 0, 0, 0};
  IntegrateArgs A{n, nullptr, paq, t, dt, erra, H, smax.data(), smin.data(), irej, iste, status, max_attempts,
                  ctl, ctl + 1, nullptr};
  A.hand = hand;
  A.hand_att = hand_att;
  A.hctl = hctl;
  A.hand_below = hand_below;
  k_integrate<MODEL, 3>(S, A);
}

extern "C" int handoff_host_run(const void* devsys, const double* packed, const int64_t* offsets, int64_t n,
                                double* paq, const double* erra, int64_t max_attempts, long long hand_below,
                                double* t, double* dt, double* H, int32_t* irej, int32_t* iste, int32_t* status,
                                int32_t* hand, long long* hand_att, unsigned long long* hctl) {
  DevSys S;
  std::memcpy(&S, devsys, sizeof S);
  for (int p = 0; p < S.npes; ++p) S.pes[p].coef = packed + offsets[p];
  if (S.nsteps != 3) return 1;
  switch (S.pes[0].model) {
    case CAIR_PES_O3_UMN:
      handoff_run<CAIR_PES_O3_UMN>(S, n, paq, erra, max_attempts, hand_below, t, dt, H, irej, iste, status, hand,
                                   hand_att, hctl);
      return 0;
    case CAIR_PES_N3_UMN:
      handoff_run<CAIR_PES_N3_UMN>(S, n, paq, erra, max_attempts, hand_below, t, dt, H, irej, iste, status, hand,
                                   hand_att, hctl);
      return 0;
    default: return 1;
  }
}

// The system's diatomic as the initial-condition and final-state kernels evaluate it (diat_any)
extern "C" void diat_host_eval(const void* devsys, int64_t n, const double* r, double* v, double* dv) {
  DevSys S;
  std::memcpy(&S, devsys, sizeof S);
  for (int64_t k = 0; k < n; ++k) diat_any<true>(S, r[k], v[k], dv[k]);
}
