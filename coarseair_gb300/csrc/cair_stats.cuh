// Final-state statistics on the device (app/TrajectoriesStats/Statistics_Class.F90, Histogram
// assignment, conditions J, v, arrangement or J1, v1, J2, v2, arrangement): each finished
// trajectory's row is turned into its initial- and final-state codes where it lies in HBM, and the
// rows are counted per (run, final state, impact-parameter ring) in an open-addressing table, so
// the cross sections need only the table back on the host instead of the million
// trajectories.out rows.
#pragma once
#include "cair_device.cuh"
#include "cair_stats_host.h"

namespace cair {

constexpr int kMaxRings = kStatsMaxRings;  // impact-parameter rings per run

struct StatsArgs {
  int64_t ntot;
  const cair_traj_result* rows;
  int32_t qnmax;
  int32_t iskip[5];
  int32_t pres[5];
  double ham_abs_tol;
  const int32_t* item_run;        // run of each work item
  const double* ring_b;           // ascending ring bounds of each run, kMaxRings per run
  const int32_t* nring;           // rings of each run
  long long nruns, R;             // table key = (final-state code x nruns + run) x R + ring
  unsigned long long* keys;       // ~0 = empty
  unsigned long long* counts;
  unsigned long long mask;        // table size - 1 (a power of two)
  unsigned long long* item_rows;  // counted rows of each item
  long long* item_inicode;        // smallest initial-state code of each item (IniStateCode(1))
  unsigned long long* ring_rows;  // rows of each (run, ring): TrajsPerb
  int* error;                     // 1: a quantum number at or above qnmax; 2: an unrepresentable key;
                                  // 3: a counted row whose bmax is not its item's
  const double* item_bmax;        // |bmax| of each work item (null: not checked)
};

constexpr unsigned long long kStatsEmpty = ~0ull;
constexpr double kStatsBmaxTol = 1.0e-3;  // SetRings' tolerance for one ring (Statistics_Class.F90:534-545)

// The NC conditions of a row, in trajectories.csv order: J, v, arr (3 atoms) or J1, v1, J2, v2, arr.
template <int NC>
__host__ __device__ __forceinline__ void stats_conditions(const cair_traj_result& r, double (&qi)[NC], double (&qf)[NC]) {
  if (NC == 3) {
    qi[0] = r.j_i; qi[1] = r.v_i; qi[NC - 1] = r.arr_i;
    qf[0] = r.j_f; qf[1] = r.v_f; qf[NC - 1] = r.arr_f;
  } else {
    qi[0] = r.j_i; qi[1] = r.v_i; qi[2 % NC] = r.j2_i; qi[3 % NC] = r.v2_i; qi[NC - 1] = r.arr_i;
    qf[0] = r.j_f; qf[1] = r.v_f; qf[2 % NC] = r.j2_f; qf[3 % NC] = r.v2_f; qf[NC - 1] = r.arr_f;
  }
}

// IdentifyInitialStates (Statistics_Class.F90:591-680) for one row and the final-state code of
// AddFinState's Histogram branch (935-1282).  Fortran nint rounds half away from zero (llround);
// Fortran mod takes the sign of the dividend, as C's % does.
template <int NC>
__host__ __device__ __forceinline__ void stats_codes(const StatsArgs& A, const cair_traj_result& r, long long& ini_code,
                                            long long& fin_code, bool& bad) {
  double qi[NC], qf[NC];
  stats_conditions<NC>(r, qi, qf);
  const long long qnmax = A.qnmax;
  const int ipair_ini = (int)((qi[NC - 1] - 0.49) / 16);
  const int ipair_fin = (int)((qf[NC - 1] - 0.49) / 16);
  long long ifact = 1, isum = 0;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    qi[c] = qi[c] - 0.5;
    long long ini = llround(qi[c]);
    if (ini >= qnmax) bad = true;
    const double fin_raw = qf[c];
    qf[c] = qf[c] - 0.5;
    if (A.pres[c] && ipair_ini == ipair_fin) {
      if (ini % 2 == 1) {
        qf[c] = qf[c] - 1.0;
        if (llround(qf[c] * 0.5) < 0 && fin_raw > 0.0) qf[c] = qf[c] + 2.0;
      }
      qf[c] = qf[c] * 0.5;
    }
    ini = ini + 2;
    isum = isum + (A.iskip[c] != 0 ? ini : 2) * ifact;
    ifact = ifact * qnmax;
  }
  ini_code = isum;
  long long fsum = 0;
  ifact = 1;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    long long iquse = llround(qf[c]) * A.iskip[c];
    if (iquse + 2 > qnmax) iquse = 0;
    if (A.iskip[c] != 0 || c == NC - 1) fsum = fsum + (iquse + 2) * ifact;
    ifact = ifact * qnmax;
  }
  fin_code = fsum;
}

__device__ __forceinline__ unsigned long long stats_hash(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

__host__ __device__ __forceinline__ bool stats_counted(const StatsArgs& A, const cair_traj_result& r) {
  // finished trajectories whose energy is conserved (the others go to trajectories_HNotCons.out,
  // Integrator_Class.F90:755-776, 884-888)
  return r.status == CAIR_TRAJ_DONE && fabs(r.dH) <= A.ham_abs_tol;
}

// A counted row's ring from its sampled b (AddFinState: ring iR + 1 when
// bRings(iR) < b <= bRings(iR+1), else the first) and its table key (code x nruns + run) x R + ring.
// |fc| < 70 qnmax^NC (a cluster's arrangement code is negative) and 70 qnmax^NC x nruns x R < 2^62 is
// checked on the host: the key is a two's-complement 64-bit number.
__host__ __device__ __forceinline__ unsigned long long stats_key(const StatsArgs& A, const cair_traj_result& r,
                                                                 long long fc, int& run, int& ring) {
  run = A.item_run[r.item];
  const double* e = A.ring_b + (size_t)run * kMaxRings;
  const int nr = A.nring[run];
  ring = 0;
  for (int q = 0; q < nr - 1; ++q)
    if (!(r.b > e[q + 1] || r.b <= e[q])) {
      ring = q + 1;
      break;
    }
  return (unsigned long long)((fc * A.nruns + run) * A.R + ring);
}

#ifndef CAIR_MODEL_TU

// Pass 1: rows and the initial-state code of each item (the rings of a run are the bMax values
// its rows carry, SetRings, Statistics_Class.F90:511-586).
template <int NC>
__global__ void __launch_bounds__(256) k_stats_items(StatsArgs A) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < A.ntot; k += (int64_t)gridDim.x * blockDim.x) {
    const cair_traj_result r = A.rows[k];
    if (!stats_counted(A, r)) continue;
    long long ic, fc;
    bool bad = false;
    stats_codes<NC>(A, r, ic, fc, bad);
    if (bad) atomicExch(A.error, 1);
    atomicAdd(A.item_rows + r.item, 1ull);
    atomicMin(A.item_inicode + r.item, ic);
  }
}

// Pass 2: each row's ring from its sampled b (AddFinState: ring iR + 1 when
// bRings(iR) < b <= bRings(iR+1), else the first) and its (run, final state, ring) count.
template <int NC>
__global__ void __launch_bounds__(256) k_stats_count(StatsArgs A) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < A.ntot; k += (int64_t)gridDim.x * blockDim.x) {
    const cair_traj_result r = A.rows[k];
    if (!stats_counted(A, r)) continue;
    long long ic, fc;
    bool bad = false;
    stats_codes<NC>(A, r, ic, fc, bad);
    // the rings are the items' |bmax|; SetRings takes them from the rows' bMax, which the queue
    // copies from the items, so a row carrying another bmax cannot be ringed as the reference would
    if (A.item_bmax && !(fabs(fabs(r.bmax) - A.item_bmax[r.item]) < kStatsBmaxTol)) {
      atomicExch(A.error, 3);
      continue;
    }
    int run, ring;
    const unsigned long long key = stats_key(A, r, fc, run, ring);
    atomicAdd(A.ring_rows + (size_t)run * kMaxRings + ring, 1ull);
    if (key == kStatsEmpty) {  // the key -1: not representable in the table
      atomicExch(A.error, 2);
      continue;
    }
    unsigned long long h = stats_hash(key) & A.mask;
    for (unsigned long long probe = 0; probe <= A.mask; ++probe) {  // the table is at least twice the rows
      const unsigned long long old = atomicCAS(A.keys + h, kStatsEmpty, key);
      if (old == kStatsEmpty || old == key) {
        atomicAdd(A.counts + h, 1ull);
        break;
      }
      h = (h + 1) & A.mask;
    }
  }
}

__global__ void __launch_bounds__(256) k_stats_compact(const unsigned long long* keys, const unsigned long long* counts,
                                                       unsigned long long size, unsigned long long* out_keys,
                                                       unsigned long long* out_counts, unsigned long long cap,
                                                       unsigned long long* nout) {
  for (unsigned long long s = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; s < size;
       s += (unsigned long long)gridDim.x * blockDim.x) {
    if (keys[s] == kStatsEmpty) continue;
    const unsigned long long i = atomicAdd(nout, 1ull);
    if (i < cap) {
      out_keys[i] = keys[s];
      out_counts[i] = counts[s];
    }
  }
}
#endif

}  // namespace cair
