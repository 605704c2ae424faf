// C-ABI implementation (include/cair_gpu.h): handle management, host<->device staging and
// kernel dispatch.  No CPU fallback: every numerical entry point runs on the GPU and
// returns CAIR_ECUDA when no device is usable.  The cair_internal_* functions at the end are not
// part of the ABI: they run the random-number stream and the statistics' per-row code (the same
// source the kernels run) on the host, for tests without a GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "cair_ic.cuh"
#include "cair_launch.h"
#include "cair_stats.cuh"
#include "cair_sur_launch.h"
#include "cair_warp_launch.h"

using namespace cair;

struct cair_handle {
  int device = 0;
  int nsm = 0;
  DevSys sys;
  FsArgs fs;
  double* d_coef[CAIR_MAX_PES] = {nullptr};
  double nnets[CAIR_MAX_PES] = {0.0};      // N4 PIPNN: networks selected per surface (flop model)
  double* d_gauss = nullptr;
  double tqp[81], tpq[81];
  double mass[4];
  std::string err;
  cudaStream_t stream = nullptr;
  void* d_scratch = nullptr;     // staging of host-pointer calls
  size_t scratch_bytes = 0;
  void* d_work = nullptr;        // batch state of the *_dev / queue paths
  size_t work_bytes = 0;
  unsigned long long* d_ctl = nullptr;   // [0] queue, [1..5] counters
  long long last_counters[5] = {0, 0, 0, 0, 0};
  double watchdog_s = 0.0;
  void* d_stats = nullptr;                  // statistics table and its compaction
  size_t stats_bytes = 0;
  bool time_integrate = false;              // bracket every integrator launch with events
  std::vector<cudaEvent_t> tev;             // pairs (start, end), reused across calls
  size_t ntev = 0;                          // pairs recorded since the last read
  int tune_block = 64;                      // persistent integrator launch shape (cair_autotune)
  int tune_per_sm = 0;                      // resident blocks per SM; 0 = as many as fit
  int mode = CAIR_INTEGRATOR_THREAD;        // persistent integrator: a lane or a warp per trajectory
  int last_integrator = CAIR_INTEGRATOR_THREAD;  // the one the last launch ran
  long long hand_below = -1;                // AUTO's tail hand-off: -1 the warp integrator's resident warps, 0 off
  int64_t hand_cap = 0;                     // hand-off buffers of the cair_integrate* paths
  void* d_hand = nullptr;
  unsigned long long* last_hctl = nullptr;  // hand-off counters of the last launch (NULL: none)
  unsigned long long* warp_times = nullptr; // warp timeline of the next integrator launches
  int64_t warp_times_cap = 0;
  int64_t warp_times_n = 0;                 // warps of the last launch that recorded
  cair_surrogate* sur = nullptr;            // attached surrogate: integrator launches run on it
  double* rec = nullptr;                    // geometry recorder of the FP64 integrator
  unsigned long long* d_nrec = nullptr;
  unsigned long long rec_cap = 0, rec_mod = 1;
  double rec_rcut = 0.0;
};

namespace {

int fail(cair_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

#define CUDA_TRY(h, call)                                                                        \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess)                                                                       \
      return fail(h, CAIR_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_));            \
  } while (0)

// libgfortran's pow_r8_i4 (binary powering), as the reference evaluates beta**k
double powi_gf(double a, int b) {
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

// Gauss-Jordan inverse with partial pivoting (the reference uses LAPACK DGETRF/DGETRI;
// callers that need its exact matrix pass it through cair_system_desc::tpq)
int invert(int n, const double* A, double* Ainv) {
  double M[9][18];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 2 * n; ++j) M[i][j] = (j < n) ? A[i + 9 * j] : (j - n == i ? 1.0 : 0.0);
  for (int c = 0; c < n; ++c) {
    int p = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(M[r][c]) > std::fabs(M[p][c])) p = r;
    if (M[p][c] == 0.0) return -1;
    if (p != c)
      for (int j = 0; j < 2 * n; ++j) std::swap(M[p][j], M[c][j]);
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
    for (int j = 0; j < n; ++j) Ainv[i + 9 * j] = M[i][n + j];
  return 0;
}

int grid_for(const cair_handle* h, int64_t n, int block = 128) {
  int64_t g = (n + block - 1) / block;
  int64_t cap = (int64_t)h->nsm * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

// Device scratch arena: one allocation reused across calls, grown on demand.
int ensure_scratch(cair_handle* h, size_t bytes) {
  if (bytes <= h->scratch_bytes) return 0;
  if (h->d_scratch) cudaFree(h->d_scratch);
  h->d_scratch = nullptr;
  h->scratch_bytes = 0;
  size_t b = bytes + bytes / 4 + (1 << 20);
  CUDA_TRY(h, cudaMalloc(&h->d_scratch, b));
  h->scratch_bytes = b;
  return 0;
}

int ensure_work(cair_handle* h, size_t bytes) {
  if (bytes <= h->work_bytes) return 0;
  if (h->d_work) cudaFree(h->d_work);
  h->d_work = nullptr;
  h->work_bytes = 0;
  size_t b = bytes + bytes / 8 + (1 << 20);
  CUDA_TRY(h, cudaMalloc(&h->d_work, b));
  h->work_bytes = b;
  return 0;
}

struct Carver {
  char* base;
  size_t off = 0;
  template <class T>
  T* take(size_t count) {
    off = (off + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base + off);
    off += count * sizeof(T);
    return p;
  }
};

int wait_stream(cair_handle* h) {
  if (h->watchdog_s <= 0.0) {
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return 0;
  }
  auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaStreamQuery(h->stream);
    if (e == cudaSuccess) return 0;
    if (e != cudaErrorNotReady) return fail(h, CAIR_ECUDA, std::string("stream: ") + cudaGetErrorString(e));
    double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (dt > h->watchdog_s) return fail(h, CAIR_ETIMEOUT, "watchdog: GPU work did not finish in time");
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  }
}

int check_launch(cair_handle* h) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(h, CAIR_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return 0;
}

bool three_atoms(const cair_handle* h) { return h->sys.natoms == 3; }

int model_of(const cair_handle* h) { return h->sys.pes[0].model; }

// Run f(ModelLaunch<model>{}) for the handle's surface model, then check the launch.
template <class F>
int with_model(cair_handle* h, F&& f) {
  switch (model_of(h)) {
#define CAIR_CASE(M) \
  case M:            \
    f(ModelLaunch<M>{}); \
    break;
    CAIR_FOR_EACH_MODEL(CAIR_CASE)
#undef CAIR_CASE
    default:
      return fail(h, CAIR_EUNSUPPORTED, "no kernels for this surface model in this library");
  }
  return check_launch(h);
}

// O3 NN: the reference's arrays (Initialize_O3_NN_PES, O3_NN_PES_Class.F90:139-230, packed as the
// header states) -> the kernels' fixed 20 x 10 layout (CAIR_NN_* offsets in cair_device.cuh),
// padded with zeros, plus W1's storage as Potential's dgemm reads it: a 3 x NHL1 matrix with
// leading dimension 3 (O3_NN_PES_Class.F90:281).
// A BNN sample (BNN_PES_Class.F90) is packed the same way with its Noise appended.
int pack_o3nn(const double* c, int32_t ncoef, bool bnn, std::vector<double>& out) {
  const double fh1 = c[0], fh2 = c[1];
  if (!(fh1 >= 1 && fh1 <= CAIR_NN_H1 && fh2 >= 1 && fh2 <= CAIR_NN_H2)) return CAIR_EINVAL;
  const int h1 = (int)fh1, h2 = (int)fh2;
  if (h1 != fh1 || h2 != fh2 || ncoef != 12 + 7 * h1 + h1 * h2 + 2 * h2 + (bnn ? 1 : 0)) return CAIR_EINVAL;
  const double* W1 = c + 11;
  const double* b1 = W1 + 6 * h1;
  const double* W2 = b1 + h1;
  const double* b2 = W2 + h1 * h2;
  const double* W3 = b2 + h2;
  const double b3 = W3[h2];
  out.assign(bnn ? CAIR_BNN_NCOEF : CAIR_NN_NCOEF, 0.0);
  if (bnn) out[CAIR_BNN_NOISE] = W3[h2 + 1];
  out[CAIR_NN_LAM] = c[2];
  out[CAIR_NN_RE] = c[3];
  for (int i = 0; i < 3; ++i) {
    out[CAIR_NN_MEAN + i] = c[4 + i];
    out[CAIR_NN_SD + i] = c[7 + i];
  }
  out[CAIR_NN_YSC] = c[10];
  out[CAIR_NN_B3] = b3;
  for (int j = 0; j < h1; ++j) {
    for (int i = 0; i < 6; ++i) out[CAIR_NN_W1 + i + 6 * j] = W1[i + 6 * j];
    for (int l = 0; l < 3; ++l) out[CAIR_NN_W1P + l + 3 * j] = W1[l + 3 * j];
    out[CAIR_NN_B1 + j] = b1[j];
    for (int k = 0; k < h2; ++k) out[CAIR_NN_W2 + j + CAIR_NN_H1 * k] = W2[j + h1 * k];
  }
  for (int k = 0; k < h2; ++k) {
    out[CAIR_NN_B2 + k] = b2[k];
    out[CAIR_NN_W3 + k] = W3[k];
  }
  return 0;
}

int check_ipes(cair_handle* h, int64_t n, const int32_t* ipes) {
  if (!ipes) return 0;
  for (int64_t k = 0; k < n; ++k)
    if (ipes[k] < 0 || ipes[k] >= h->sys.npes) return fail(h, CAIR_EINVAL, "ipes out of range");
  return 0;
}

}  // namespace

// SetIniCondForward's per-trajectory integrator state (Collision_Class.F90:1102-1108)
__global__ void cair_k_init_state(int64_t n, double dt0, double* t, double* dt, double* smax, double* smin,
                                  int32_t* irej, int32_t* iste) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    t[k] = 0.0;
    dt[k] = dt0;
    smax[k] = -1.7976931348623157e308;
    smin[k] = 1.7976931348623157e308;
    irej[k] = 0;
    iste[k] = 0;
  }
}

// Queue ordering: 256 buckets of log2(initial relative speed), slowest (longest) first.
__device__ __forceinline__ int speed_bucket(double v) {
  double l = log2(v > 1e-300 ? v : 1e-300);
  int b = (int)floor((l + 20.0) * 8.0);
  return b < 0 ? 0 : (b > 255 ? 255 : b);
}
__global__ void cair_k_bucket_count(int64_t n, const double* __restrict__ key, unsigned long long* counts) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(counts + speed_bucket(key[k]), 1ull);
}
__global__ void cair_k_bucket_scan(const unsigned long long* counts, unsigned long long* offsets) {
  __shared__ unsigned long long c[256];
  c[threadIdx.x] = counts[threadIdx.x];
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long acc = 0;
    for (int i = 0; i < 256; ++i) { unsigned long long v = c[i]; c[i] = acc; acc += v; }
  }
  __syncthreads();
  offsets[threadIdx.x] = c[threadIdx.x];
}
__global__ void cair_k_bucket_scatter(int64_t n, const double* __restrict__ key, unsigned long long* offsets,
                                      int32_t* __restrict__ order) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long pos = atomicAdd(offsets + speed_bucket(key[k]), 1ull);
    order[pos] = (int32_t)k;
  }
}

// Register-resident DFMA chains: the FP64 pipe's throughput
__global__ void cair_k_dfma_probe(double* out, int iters, double a, double b) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  double x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = 1.0 + 1e-3 * (tid & 7) + 1e-4 * i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  out[tid] = s;
}

// 1-thread helper used at create time for Vinf
__global__ void cair_k_diat_v(DevSys S, const double* r, double* v, int64_t n) {
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n) v[k] = diat_v(S, r[k]);
}

// Everything cair_create derives from the system description without the GPU: the DevSys fields, Tqp and its
// inverse Tpq (Transformation_Class.F90:53-128), the O2 UMN exponent factors, and every surface checked and packed
// into its device layout (packed_out[p]; P.coef is left for the caller to point at the device copy).  Returns ""
// or the error with its code.
std::string setup_system(const cair_system_desc* d, DevSys& S, double* tqp, double* tpq,
                         std::vector<std::vector<double>>& packed_out, int& code) {
  auto fail_setup = [](int& c, int e, const std::string& msg) {
    c = e;
    return msg;
  };
  packed_out.assign(d->npes, {});
  std::memset(&S, 0, sizeof(S));
  S.natoms = d->natoms;
  S.nv = 3 * (d->natoms - 1);
  S.ne = 2 * S.nv;
  S.npairs = d->natoms * (d->natoms - 1) / 2;
  S.npes = d->npes;
  S.nsteps = d->nsteps;
  S.ncall = d->ncall;
  S.incstp = d->inc_step;
  S.diat = d->diat_model;
  if (d->diat_model < CAIR_DIAT_O2_UMN || d->diat_model > CAIR_DIAT_N2_UMN_PIPNN_FORN4)
    return fail_setup(code, CAIR_EINVAL, "unknown diatomic model");
  if (d->diat_model == CAIR_DIAT_N2_UMN_PIPNN_FORN4 && d->pes[0].model != CAIR_PES_N4_PIPNN)
    return fail_setup(code, CAIR_EUNSUPPORTED, "the UMN_PIPNN_ForN4 diatomic is built for the N4 UMN PIPNN surface");
  S.relax = d->relax;
  S.eps = d->eps;
  S.dt0 = d->dt0;
  for (int i = 0; i < 4; ++i) S.mass[i] = d->mass[i];
  S.rmax = d->rmax;
  S.tmax = d->tmax;
  S.rpimax = 1.0 / d->rmax;
  for (int i = 0; i < d->natoms - 1; ++i) S.mMiMn[i] = -d->mass[i] / d->mass[d->natoms - 1];
  // Tqp (Transformation_Class.F90:53-128)
  std::memset(tqp, 0, 81 * sizeof(double));
  double xmi = 1.0 / d->mass[d->natoms - 1];
  int ic = 0;
  for (int i = 0; i < d->natoms - 1; ++i) {
    double temp1 = d->mass[i] * xmi;
    double temp = (d->mass[d->natoms - 1] + d->mass[i]) * temp1;
    for (int j = 0; j < 3; ++j) {
      tqp[ic + 9 * ic] = temp;
      for (int ip = i + 1; ip < d->natoms - 1; ++ip) {
        double temp2 = temp1 * d->mass[ip];
        tqp[ic + 9 * (ip * 3 + j)] = temp2;
        tqp[(ip * 3 + j) + 9 * ic] = temp2;
      }
      ++ic;
    }
  }
  if (d->tpq) {
    std::memset(tpq, 0, 81 * sizeof(double));
    for (int j = 0; j < S.nv; ++j)
      for (int i = 0; i < S.nv; ++i) tpq[i + 9 * j] = d->tpq[i + S.nv * j];
  } else if (invert(S.nv, tqp, tpq) != 0) {
    return fail_setup(code, CAIR_EINVAL, "mass matrix is singular");
  }
  std::memcpy(S.Tpq, tpq, sizeof(S.Tpq));
  std::memcpy(S.Tqp, tqp, sizeof(S.Tqp));
  // O2 UMN exponent factors (O2_UMN_DiatomicPotential_Class.F90 Ev2gm2/_Grad)
  {
    const double a[8] = {-1.488979427684798e3, 1.881435846488955e4, -1.053475425838226e5,
                         2.755135591229064e5,  -4.277588997761775e5, 4.404104009614092e5,
                         -2.946204062950765e5, 1.176861219078620e5};
    const double alpha = 9.439784362354936e-1, beta = 1.262242998506810;
    for (int k = 0; k < 8; ++k) {
      double bk = powi_gf(beta, k);
      S.o2_ab[k] = alpha * bk;
      S.o2_cd[k] = 2.0 * a[k] * alpha * bk;
    }
  }
  for (int p = 0; p < d->npes; ++p) {
    const cair_pes_desc& src = d->pes[p];
    int expect = src.model == CAIR_PES_O3_UMN ? 56 : (src.model == CAIR_PES_N3_UMN || src.model == CAIR_PES_N4_UMN) ? 276
                 : src.model == CAIR_PES_O4_UMN ? 430 : (src.model == CAIR_PES_O3_NN || src.model == CAIR_PES_O3_BNN) ? 0
                 : src.model == CAIR_PES_N4_PIPNN ? CAIR_PIPNN_HDR + 3 * CAIR_PIPNN_NET
                 : -1;
    if (expect < 0) return fail_setup(code, CAIR_EINVAL, "unknown surface model");
    std::vector<double> packed;
    if (src.model == CAIR_PES_O3_NN || src.model == CAIR_PES_O3_BNN) {
      const bool bnn = src.model == CAIR_PES_O3_BNN;
      if (!src.coef || src.ncoef < 12) return fail_setup(code, CAIR_EINVAL, "O3 NN: coefficient array too short");
      if (int e = pack_o3nn(src.coef, src.ncoef, bnn, packed))
        return fail_setup(code, e, bnn ? "O3 BNN: hidden layers must be 1..20 and 1..10 neurons and ncoef = 13 + 7 NHL1 + NHL1 NHL2 "
                            "+ 2 NHL2"
                          : "O3 NN: hidden layers must be 1..20 and 1..10 neurons and ncoef = 12 + 7 NHL1 + NHL1 NHL2 "
                            "+ 2 NHL2");
      if (d->natoms != 3) return fail_setup(code, CAIR_EINVAL, "surface/atom count mismatch");
    } else if (src.ncoef != expect || !src.coef) {
      return fail_setup(code, CAIR_EINVAL, "wrong coefficient count for surface");
    } else if (src.model == CAIR_PES_N4_PIPNN) {
      // UseSurface(3) of 0/1, at least one set; iFunc 1..3; the 276-5-90-1 networks of the shipped fit
      const double* c = src.coef;
      const bool use_ok = (c[0] == 0.0 || c[0] == 1.0) && (c[1] == 0.0 || c[1] == 1.0) &&
                          (c[2] == 0.0 || c[2] == 1.0) && c[0] + c[1] + c[2] >= 1.0;
      if (!use_ok) return fail_setup(code, CAIR_EINVAL, "N4 PIPNN: UseSurface must be 0/1 with one network selected");
      if (!(c[3] == 1.0 || c[3] == 2.0 || c[3] == 3.0)) return fail_setup(code, CAIR_EINVAL, "N4 PIPNN: iFunc must be 1, 2 or 3");
      if (c[4] != CAIR_PIPNN_NIN || c[5] != CAIR_PIPNN_H1 || c[6] != CAIR_PIPNN_H2 || c[7] != 1.0)
        return fail_setup(code, CAIR_EUNSUPPORTED, "N4 PIPNN: the kernels are built for 276-5-90-1 networks");
      for (int i = 0; i < src.ncoef; ++i)
        if (!std::isfinite(c[i])) return fail_setup(code, CAIR_ENONFINITE, "N4 PIPNN: non-finite coefficient");
      packed.assign(src.coef, src.coef + src.ncoef);
    } else {
      packed.assign(src.coef, src.coef + src.ncoef);
    }
    if (src.model != d->pes[0].model) return fail_setup(code, CAIR_EUNSUPPORTED, "all surfaces of a handle must share a model");
    if ((src.model == CAIR_PES_O4_UMN || src.model == CAIR_PES_N4_UMN || src.model == CAIR_PES_N4_PIPNN) != (d->natoms == 4))
      return fail_setup(code, CAIR_EINVAL, "surface/atom count mismatch");
    DevPes& P = S.pes[p];
    P.model = src.model;
    P.ncoef = (int32_t)packed.size();
    P.a = src.a; P.ab = src.ab; P.ra = src.ra; P.rb = src.rb;
    P.inv_a = (src.a != 0.0) ? 1.0 / src.a : 0.0;
    P.inv_ab = (src.ab != 0.0) ? 1.0 / src.ab : 0.0;
    packed_out[p] = std::move(packed);
  }
  return "";
}

extern "C" {

int cair_create(cair_handle** out, const cair_system_desc* d) {
  if (!out || !d) return CAIR_EINVAL;
  *out = nullptr;
  cair_handle* h = new cair_handle();
  auto bad = [&](int code, const std::string& msg) {
    h->err = msg;
    *out = h;  // caller reads the message, then destroys
    return code;
  };
  if (d->abi_version != CAIR_ABI_VERSION) return bad(CAIR_EINVAL, "abi_version mismatch");
  if (d->natoms != 3 && d->natoms != 4) return bad(CAIR_EINVAL, "natoms must be 3 or 4");
  if (d->npes < 1 || d->npes > CAIR_MAX_PES) return bad(CAIR_EINVAL, "npes out of range");
  if (d->nsteps < 2 || d->nsteps > 4) return bad(CAIR_EUNSUPPORTED, "Nb of extrapolation steps must be 2..4");
  if (d->natoms == 4 && d->nsteps != 3)
    return bad(CAIR_EUNSUPPORTED, "Nb of extrapolation steps 2 and 4 are built for diatom + atom surfaces only");
  if (d->ncall < 1) return bad(CAIR_EINVAL, "ncall must be >= 1");
  if (d->nquad < 1 || d->nquad > 256) return bad(CAIR_EINVAL, "nquad must be 1..256");
  for (int i = 0; i < d->natoms; ++i)
    if (!(d->mass[i] > 0.0)) return bad(CAIR_EINVAL, "atom masses must be positive");
  int ndev = 0;
  cudaError_t ce = cudaGetDeviceCount(&ndev);
  if (ce != cudaSuccess || ndev == 0) return bad(CAIR_ECUDA, "no CUDA device available");
  cudaGetDevice(&h->device);
  cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device);
  if (const char* w = std::getenv("CAIR_WATCHDOG_S")) h->watchdog_s = std::atof(w);

  DevSys& S = h->sys;
  for (int i = 0; i < 4; ++i) h->mass[i] = d->mass[i];
  {
    std::vector<std::vector<double>> packed;
    int code = CAIR_OK;
    const std::string msg = setup_system(d, S, h->tqp, h->tpq, packed, code);
    if (!msg.empty()) return bad(code, msg);
    for (int p = 0; p < d->npes; ++p) {
      DevPes& P = S.pes[p];
      if (cudaMalloc(&h->d_coef[p], sizeof(double) * packed[p].size()) != cudaSuccess)
        return bad(CAIR_ECUDA, "cudaMalloc");
      if (cudaMemcpy(h->d_coef[p], packed[p].data(), sizeof(double) * packed[p].size(), cudaMemcpyHostToDevice) !=
          cudaSuccess)
        return bad(CAIR_ECUDA, "cudaMemcpy coefficients");
      P.coef = h->d_coef[p];
      if (P.model == CAIR_PES_N4_PIPNN) h->nnets[p] = packed[p][0] + packed[p][1] + packed[p][2];
    }
  }
  // final-state analysis parameters and Chebyshev-2 nodes (GAUSSQ kind 3)
  FsArgs& F = h->fs;
  F.nquad = d->nquad;
  F.rsmal = d->rsmal;
  F.rcent = d->rcent;
  F.rfact = d->rfact;
  F.tthresau = d->tthresau;
  for (int i = 0; i < 4; ++i) F.mass[i] = d->mass[i];
  {
    // Vinf = DiatomicPotential(1.0E+03) of the target (MolecularStateParam_Class.F90:94)
    std::vector<double> gx(d->nquad), gw(d->nquad);
    const double pi = std::acos(-1.0);
    for (int i = 0; i < d->nquad; ++i) {
      int k = d->nquad - i;
      double th = (double)k * pi / (double)(d->nquad + 1);
      double s = std::sin(th);
      gx[i] = std::cos(th);
      gw[i] = pi / (double)(d->nquad + 1) * (s * s);
      gw[i] = gw[i] / std::sqrt(1.0 - gx[i] * gx[i]);
    }
    if (cudaMalloc(&h->d_gauss, sizeof(double) * 2 * d->nquad) != cudaSuccess) return bad(CAIR_ECUDA, "cudaMalloc");
    cudaMemcpy(h->d_gauss, gx.data(), sizeof(double) * d->nquad, cudaMemcpyHostToDevice);
    cudaMemcpy(h->d_gauss + d->nquad, gw.data(), sizeof(double) * d->nquad, cudaMemcpyHostToDevice);
    F.gx = h->d_gauss;
    F.gw = h->d_gauss + d->nquad;
    F.vinf = 0.0;  // filled below on the device
  }
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) return bad(CAIR_ECUDA, "stream");
  if (cudaMalloc(&h->d_ctl, sizeof(unsigned long long) * 8) != cudaSuccess) return bad(CAIR_ECUDA, "cudaMalloc");
  // Vinf on the device with the same diatomic code as the kernels
  {
    double* dv = nullptr;
    if (cudaMalloc(&dv, sizeof(double)) != cudaSuccess) return bad(CAIR_ECUDA, "cudaMalloc");
    double r = 1.0E+03, *dr = nullptr;
    cudaMalloc(&dr, sizeof(double));
    cudaMemcpy(dr, &r, sizeof(double), cudaMemcpyHostToDevice);
    cair_k_diat_v<<<1, 32, 0, h->stream>>>(S, dr, dv, 1);
    cudaStreamSynchronize(h->stream);
    cudaError_t e = cudaMemcpy(&F.vinf, dv, sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(dv);
    cudaFree(dr);
    if (e != cudaSuccess) return bad(CAIR_ECUDA, std::string("Vinf: ") + cudaGetErrorString(e));
  }
  *out = h;
  return CAIR_OK;
}

void cair_destroy(cair_handle* h) {
  if (!h) return;
  for (int p = 0; p < CAIR_MAX_PES; ++p)
    if (h->d_coef[p]) cudaFree(h->d_coef[p]);
  if (h->d_gauss) cudaFree(h->d_gauss);
  if (h->d_scratch) cudaFree(h->d_scratch);
  if (h->d_work) cudaFree(h->d_work);
  if (h->d_ctl) cudaFree(h->d_ctl);
  if (h->d_hand) cudaFree(h->d_hand);
  if (h->d_stats) cudaFree(h->d_stats);
  if (h->d_nrec) cudaFree(h->d_nrec);
  if (h->stream) cudaStreamDestroy(h->stream);
  for (cudaEvent_t e : h->tev) cudaEventDestroy(e);
  delete h;
}

const char* cair_last_error(const cair_handle* h) { return h ? h->err.c_str() : "null handle"; }

int cair_dims(const cair_handle* h, int32_t* nv, int32_t* ne, int32_t* np) {
  if (!h) return CAIR_EINVAL;
  if (nv) *nv = h->sys.nv;
  if (ne) *ne = h->sys.ne;
  if (np) *np = h->sys.npairs;
  return 0;
}

int cair_get_tpq(const cair_handle* h, double* tpq) {
  if (!h || !tpq) return CAIR_EINVAL;
  int nv = h->sys.nv;
  for (int j = 0; j < nv; ++j)
    for (int i = 0; i < nv; ++i) tpq[i + nv * j] = h->tpq[i + 9 * j];
  return 0;
}

int cair_pes_eval(cair_handle* h, int64_t n, const int32_t* ipes, const double* R, const double* Qall, double* V,
                  double* dVdR, double* dVdQ) {
  if (!h || n < 0 || !R || !Qall || !V) return fail(h, CAIR_EINVAL, "cair_pes_eval: bad argument");
  if (n == 0) return 0;
  if (int e = check_ipes(h, n, ipes)) return e;
  bool grad = dVdR != nullptr;
  if (grad && !dVdQ) return fail(h, CAIR_EINVAL, "cair_pes_eval: dVdQ required with dVdR");
  const int np = h->sys.npairs, na3 = 3 * h->sys.natoms, nv = h->sys.nv;
  size_t bytes = n * (sizeof(int32_t) + sizeof(double) * (np + na3 + 1 + np + nv)) + 8 * 256;
  if (int e = ensure_scratch(h, bytes)) return e;
  Carver c{(char*)h->d_scratch};
  int32_t* d_ip = ipes ? c.take<int32_t>(n) : nullptr;
  double *d_R = c.take<double>(n * np), *d_Q = c.take<double>(n * na3), *d_V = c.take<double>(n);
  double *d_g = c.take<double>(n * np), *d_m = c.take<double>(n * nv);
  if (d_ip) CUDA_TRY(h, cudaMemcpyAsync(d_ip, ipes, n * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(d_R, R, n * np * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(d_Q, Qall, n * na3 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int g = grid_for(h, n);
  if (int e = with_model(h, [&](auto L) { L.pes_eval(grad, g, h->stream, h->sys, n, d_ip, d_R, d_Q, d_V, d_g, d_m); }))
    return e;
  CUDA_TRY(h, cudaMemcpyAsync(V, d_V, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (grad) {
    CUDA_TRY(h, cudaMemcpyAsync(dVdR, d_g, n * np * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaMemcpyAsync(dVdQ, d_m, n * nv * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  }
  return wait_stream(h);
}

int cair_rhs(cair_handle* h, int64_t n, const int32_t* ipes, const double* y, double* yp) {
  if (!h || n < 0 || !y || !yp) return fail(h, CAIR_EINVAL, "cair_rhs: bad argument");
  if (n == 0) return 0;
  if (int e = check_ipes(h, n, ipes)) return e;
  const int ne = h->sys.ne;
  if (int e = ensure_scratch(h, n * (4 + 2 * ne * 8) + 1024)) return e;
  Carver c{(char*)h->d_scratch};
  int32_t* d_ip = ipes ? c.take<int32_t>(n) : nullptr;
  double *d_y = c.take<double>(n * ne), *d_yp = c.take<double>(n * ne);
  if (d_ip) CUDA_TRY(h, cudaMemcpyAsync(d_ip, ipes, n * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(d_y, y, n * ne * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int g = grid_for(h, n);
  if (int e = with_model(h, [&](auto L) { L.rhs(g, h->stream, h->sys, n, d_ip, d_y, d_yp); })) return e;
  CUDA_TRY(h, cudaMemcpyAsync(yp, d_yp, n * ne * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return wait_stream(h);
}

int cair_hamiltonian(cair_handle* h, int64_t n, const int32_t* ipes, const double* paq, double* H, double* Rpi) {
  if (!h || n < 0 || !paq || !H) return fail(h, CAIR_EINVAL, "cair_hamiltonian: bad argument");
  if (n == 0) return 0;
  if (int e = check_ipes(h, n, ipes)) return e;
  const int ne = h->sys.ne, np = h->sys.npairs;
  if (int e = ensure_scratch(h, n * (4 + (ne + 1 + np) * 8) + 1024)) return e;
  Carver c{(char*)h->d_scratch};
  int32_t* d_ip = ipes ? c.take<int32_t>(n) : nullptr;
  double *d_y = c.take<double>(n * ne), *d_H = c.take<double>(n), *d_r = c.take<double>(n * np);
  if (d_ip) CUDA_TRY(h, cudaMemcpyAsync(d_ip, ipes, n * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(d_y, paq, n * ne * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int g = grid_for(h, n);
  if (int e = with_model(h, [&](auto L) { L.hamiltonian(g, h->stream, h->sys, n, d_ip, d_y, d_H, d_r); }))
    return e;
  CUDA_TRY(h, cudaMemcpyAsync(H, d_H, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (Rpi) CUDA_TRY(h, cudaMemcpyAsync(Rpi, d_r, n * np * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return wait_stream(h);
}

int cair_bs_steps(cair_handle* h, int64_t n, const int32_t* ipes, double* paq, double* t, double* dt,
                  const double* erra, int32_t nattempts) {
  if (!h || n < 0 || !paq || !t || !dt || !erra || nattempts < 0)
    return fail(h, CAIR_EINVAL, "cair_bs_steps: bad argument");
  if (n == 0) return 0;
  if (int e = check_ipes(h, n, ipes)) return e;
  const int ne = h->sys.ne;
  if (int e = ensure_scratch(h, n * (4 + (2 * ne + 2) * 8) + 2048)) return e;
  Carver c{(char*)h->d_scratch};
  int32_t* d_ip = ipes ? c.take<int32_t>(n) : nullptr;
  double *d_y = c.take<double>(n * ne), *d_t = c.take<double>(n), *d_dt = c.take<double>(n),
         *d_e = c.take<double>(n * ne);
  if (d_ip) CUDA_TRY(h, cudaMemcpyAsync(d_ip, ipes, n * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(d_y, paq, n * ne * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(d_t, t, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(d_dt, dt, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(d_e, erra, n * ne * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  int g = grid_for(h, n);
  if (int e = with_model(h, [&](auto L) { L.bs_steps(g, h->stream, h->sys, n, d_ip, d_y, d_t, d_dt, d_e, nattempts); }))
    return e;
  CUDA_TRY(h, cudaMemcpyAsync(paq, d_y, n * ne * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(t, d_t, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(h, cudaMemcpyAsync(dt, d_dt, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return wait_stream(h);
}

// Device buffers of a launch's tail hand-off: the list, the attempts by trajectory, 3 control words
// (zeroed by the caller with the rest of its control block).
struct HandBufs {
  int32_t* hand;
  long long* att;
  unsigned long long* ctl;
};

static int launch_integrate(cair_handle* h, const IntegrateArgs& A0, cudaStream_t st, const HandBufs* hb = nullptr) {
  IntegrateArgs A = A0;
  h->last_hctl = nullptr;
  if (h->rec && !h->sur) {
    A.rec = h->rec;
    A.nrec = h->d_nrec;
    A.rec_cap = h->rec_cap;
    A.rec_mod = h->rec_mod;
    A.rec_rcut = h->rec_rcut;
  }
  bool warp = h->mode == CAIR_INTEGRATOR_WARP;
  if (!h->sur && h->mode == CAIR_INTEGRATOR_AUTO && warp_integrate_supported(h->sys)) {
    int resident = 0;
    if (int e = with_model(h, [&](auto L) { resident = L.integrate_blocks_per_sm(h->tune_block, h->sys.nsteps); }))
      return e;
    if (h->tune_per_sm > 0 && h->tune_per_sm < resident) resident = h->tune_per_sm;
    warp = A.n < 2 * (int64_t)h->nsm * (resident > 0 ? resident : 1) * h->tune_block;
  }
  h->last_integrator = (!h->sur && warp) ? CAIR_INTEGRATOR_WARP : CAIR_INTEGRATOR_THREAD;
  if (!h->sur && warp) {
    // a warp per trajectory: as many CTAs as fit on every SM
    cudaEvent_t w0 = nullptr, w1 = nullptr;
    if (h->time_integrate) {
      if (2 * h->ntev + 2 > h->tev.size()) {
        for (int k = 0; k < 2; ++k) {
          cudaEvent_t e;
          CUDA_TRY(h, cudaEventCreate(&e));
          h->tev.push_back(e);
        }
      }
      w0 = h->tev[2 * h->ntev];
      w1 = h->tev[2 * h->ntev + 1];
      ++h->ntev;
      CUDA_TRY(h, cudaEventRecord(w0, st));
    }
    int64_t nw = 0;
    if (h->warp_times) A.warp_times = h->warp_times;
    const int rc = warp_integrate_launch(h->nsm, 0, st, h->sys, A, h->warp_times ? h->warp_times_cap : 0, &nw);
    if (rc == 2) return fail(h, CAIR_EUNSUPPORTED, "warp integrator: no lane-parallel programs for this system");
    if (rc) return fail(h, CAIR_ECUDA, std::string("warp integrator launch: ") + cudaGetErrorString(cudaGetLastError()));
    if (h->warp_times && nw > 0) h->warp_times_n = nw;
    if (w1) CUDA_TRY(h, cudaEventRecord(w1, st));
    return 0;
  }
  // launch shape: 64-thread blocks by default (a block holding one long trajectory frees the rest
  // of its SM for the next batch on another stream), or what cair_autotune measured best
  int block = h->tune_block, per_sm = 0;
  if (!h->sur)
    if (int e = with_model(h, [&](auto L) { per_sm = L.integrate_blocks_per_sm(block, h->sys.nsteps); })) return e;
  if (h->tune_per_sm > 0 && h->tune_per_sm < per_sm) per_sm = h->tune_per_sm;
  if (per_sm < 1) per_sm = 1;
  int64_t g = (int64_t)h->nsm * per_sm;
  int64_t need = (A.n + block - 1) / block;
  if (g > need) g = need;
  if (g < 1) g = 1;
  if (h->warp_times && !h->sur && g * block / 32 <= h->warp_times_cap) {
    A.warp_times = h->warp_times;
    h->warp_times_n = g * block / 32;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (h->time_integrate) {
    if (2 * h->ntev + 2 > h->tev.size()) {
      for (int k = 0; k < 2; ++k) {
        cudaEvent_t e;
        CUDA_TRY(h, cudaEventCreate(&e));
        h->tev.push_back(e);
      }
    }
    e0 = h->tev[2 * h->ntev];
    e1 = h->tev[2 * h->ntev + 1];
    ++h->ntev;
    CUDA_TRY(h, cudaEventRecord(e0, st));
  }
  // AUTO on a large launch: the thread integrator hands its tail to the warp integrator
  const bool handoff = !h->sur && hb && h->mode == CAIR_INTEGRATOR_AUTO && h->hand_below != 0 &&
                       warp_integrate_supported(h->sys);
  if (handoff) {
    A.hand = hb->hand;
    A.hand_att = hb->att;
    A.hctl = hb->ctl;
    A.hand_below = h->hand_below > 0 ? h->hand_below : warp_resident_warps(h->nsm, h->sys);
  }
  if (h->sur) {
    if (sur_integrate_launch(h->sur, h->nsm, st, h->sys, A))
      return fail(h, CAIR_ECUDA, std::string("surrogate integrator launch: ") + cudaGetErrorString(cudaGetLastError()));
  } else if (int e = with_model(h, [&](auto L) { L.integrate((int)g, block, st, h->sys, A); })) {
    return e;
  }
  if (handoff) {
    // the handed-off trajectories, at most the lanes the thread launch had, each on a warp
    IntegrateArgs W = A;
    W.n = std::min<int64_t>(A.n, g * (int64_t)block);
    W.order = hb->hand;
    W.queue = hb->ctl + 2;
    W.n_dev = hb->ctl + 1;
    W.att0 = hb->att;
    W.hand = nullptr;
    W.warp_times = nullptr;
    int64_t nw = 0;
    if (warp_integrate_launch(h->nsm, 0, st, h->sys, W, 0, &nw))
      return fail(h, CAIR_ECUDA, std::string("warp integrator launch: ") + cudaGetErrorString(cudaGetLastError()));
    h->last_hctl = hb->ctl;
  }
  if (e1) CUDA_TRY(h, cudaEventRecord(e1, st));
  return 0;
}

// Hand-off buffers for the cair_integrate* paths (the queue paths carve theirs from the batch).
static const HandBufs* integrate_handbufs(cair_handle* h, int64_t n, HandBufs& hb, cudaStream_t st) {
  if (h->mode != CAIR_INTEGRATOR_AUTO || h->hand_below == 0 || !warp_integrate_supported(h->sys)) return nullptr;
  if (n > h->hand_cap) {
    if (h->d_hand) cudaFree(h->d_hand);
    h->d_hand = nullptr;
    h->hand_cap = 0;
    if (cudaMalloc(&h->d_hand, (size_t)n * 12 + 64) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    h->hand_cap = n;
  }
  char* base = (char*)h->d_hand;
  hb.ctl = (unsigned long long*)base;
  hb.att = (long long*)(base + 64);
  hb.hand = (int32_t*)(base + 64 + 8 * (size_t)n);
  if (cudaMemsetAsync(hb.ctl, 0, 64, st) != cudaSuccess) return nullptr;
  return &hb;
}

int cair_integrate_dev(cair_handle* h, int64_t n, const int32_t* ipes, double* paq, double* t, double* dt,
                       const double* erra, double* H, double* smax, double* smin, int32_t* irej, int32_t* iste,
                       int32_t* status, int64_t max_attempts, void* stream) {
  if (!h || n < 0 || !paq || !t || !dt || !erra || !H || !smax || !smin || !irej || !iste || !status ||
      max_attempts < 1)
    return fail(h, CAIR_EINVAL, "cair_integrate_dev: bad argument");
  if (n == 0) return 0;
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(h, cudaMemsetAsync(h->d_ctl, 0, sizeof(unsigned long long) * 8, st));
  IntegrateArgs A{n, ipes, paq, t, dt, erra, H, smax, smin, irej, iste, status, max_attempts, h->d_ctl,
                  h->d_ctl + 1, nullptr};
  HandBufs hb;
  return launch_integrate(h, A, st, integrate_handbufs(h, n, hb, st));
}

int cair_integrate(cair_handle* h, int64_t n, const int32_t* ipes, double* paq, double* t, double* dt,
                   const double* erra, double* H, double* smax, double* smin, int32_t* irej, int32_t* iste,
                   int32_t* status, int64_t max_attempts) {
  if (!h || n < 0 || !paq || !t || !dt || !erra || !H || !smax || !smin || !irej || !iste || !status ||
      max_attempts < 1)
    return fail(h, CAIR_EINVAL, "cair_integrate: bad argument");
  if (n == 0) return 0;
  if (int e = check_ipes(h, n, ipes)) return e;
  const int ne = h->sys.ne;
  size_t bytes = n * (3 * sizeof(int32_t) + sizeof(int32_t) + sizeof(double) * (2 * ne + 5)) + 16 * 256;
  if (int e = ensure_scratch(h, bytes)) return e;
  Carver c{(char*)h->d_scratch};
  int32_t* d_ip = ipes ? c.take<int32_t>(n) : nullptr;
  double *d_y = c.take<double>(n * ne), *d_e = c.take<double>(n * ne), *d_t = c.take<double>(n),
         *d_dt = c.take<double>(n), *d_H = c.take<double>(n), *d_smax = c.take<double>(n),
         *d_smin = c.take<double>(n);
  int32_t *d_irej = c.take<int32_t>(n), *d_iste = c.take<int32_t>(n), *d_st = c.take<int32_t>(n);
  cudaStream_t st = h->stream;
  if (d_ip) CUDA_TRY(h, cudaMemcpyAsync(d_ip, ipes, n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_y, paq, n * ne * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_e, erra, n * ne * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_t, t, n * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_dt, dt, n * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_smax, smax, n * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_smin, smin, n * sizeof(double), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_irej, irej, n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_iste, iste, n * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemsetAsync(h->d_ctl, 0, sizeof(unsigned long long) * 8, st));
  IntegrateArgs A{n, d_ip, d_y, d_t, d_dt, d_e, d_H, d_smax, d_smin, d_irej, d_iste, d_st, max_attempts,
                  h->d_ctl, h->d_ctl + 1, nullptr};
  HandBufs hb;
  if (int e = launch_integrate(h, A, st, integrate_handbufs(h, n, hb, st))) return e;
  CUDA_TRY(h, cudaMemcpyAsync(paq, d_y, n * ne * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(t, d_t, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(dt, d_dt, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(H, d_H, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(smax, d_smax, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(smin, d_smin, n * sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(irej, d_irej, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(iste, d_iste, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(status, d_st, n * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  unsigned long long ctr[5];
  CUDA_TRY(h, cudaMemcpyAsync(ctr, h->d_ctl + 1, sizeof(ctr), cudaMemcpyDeviceToHost, st));
  if (int e = wait_stream(h)) return e;
  for (int i = 0; i < 5; ++i) h->last_counters[i] = (long long)ctr[i];
  return 0;
}

int cair_sur_attach(cair_handle* h, cair_surrogate* s) {
  if (!h) return CAIR_EINVAL;
  if (s && (h->sys.npes != 1 || h->sys.pes[0].model != CAIR_PES_N3_UMN || h->sys.nsteps != 3))
    return fail(h, CAIR_EUNSUPPORTED, "cair_sur_attach: the surrogate is built for N3 UMN (one surface) with NSteps = 3");
  h->sur = s;
  return 0;
}

int cair_sur_targets_dev(cair_handle* h, int64_t n, const double* R, cair_sur_sample* out, void* stream) {
  if (!h || n < 0 || (n > 0 && (!R || !out))) return fail(h, CAIR_EINVAL, "cair_sur_targets_dev: bad argument");
  if (h->sys.pes[0].model != CAIR_PES_N3_UMN) return fail(h, CAIR_EUNSUPPORTED, "cair_sur_targets_dev: N3 UMN only");
  if (n == 0) return 0;
  if (sur_targets_launch(h->sys, h->nsm, (cudaStream_t)stream, n, R, out))
    return fail(h, CAIR_ECUDA, std::string("cair_sur_targets_dev: ") + cudaGetErrorString(cudaGetLastError()));
  return 0;
}

int cair_record_samples(cair_handle* h, double* rec_dev, int64_t cap, int32_t modulus, double rcut) {
  if (!h || (rec_dev && (cap < 1 || modulus < 1))) return fail(h, CAIR_EINVAL, "cair_record_samples: bad argument");
  if (rec_dev && h->sys.natoms != 3) return fail(h, CAIR_EUNSUPPORTED, "cair_record_samples: three atoms only");
  if (!h->d_nrec) CUDA_TRY(h, cudaMalloc(&h->d_nrec, sizeof(unsigned long long)));
  CUDA_TRY(h, cudaMemset(h->d_nrec, 0, sizeof(unsigned long long)));
  h->rec = rec_dev;
  h->rec_cap = (unsigned long long)cap;
  h->rec_mod = (unsigned long long)(modulus > 0 ? modulus : 1);
  h->rec_rcut = rcut;
  return 0;
}

int64_t cair_recorded_samples(cair_handle* h) {
  if (!h || !h->d_nrec) return 0;
  unsigned long long n = 0;
  if (cudaMemcpy(&n, h->d_nrec, sizeof n, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return (int64_t)n;
}

int cair_last_counters(cair_handle* h, int64_t* c5) {
  if (!h || !c5) return CAIR_EINVAL;
  unsigned long long ctr[5];
  CUDA_TRY(h, cudaMemcpy(ctr, h->d_ctl + 1, sizeof(ctr), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 5; ++i) c5[i] = (int64_t)ctr[i];
  return 0;
}

int cair_apply_transformation(cair_handle* h, int64_t n, const double* paq, double* out) {
  if (!h || n < 0 || !paq || !out) return fail(h, CAIR_EINVAL, "cair_apply_transformation: bad argument");
  if (n == 0) return 0;
  const int ne = h->sys.ne;
  if (int e = ensure_scratch(h, n * 2 * ne * 8 + 1024)) return e;
  Carver c{(char*)h->d_scratch};
  double *d_a = c.take<double>(n * ne), *d_b = c.take<double>(n * ne);
  CUDA_TRY(h, cudaMemcpyAsync(d_a, paq, n * ne * 8, cudaMemcpyHostToDevice, h->stream));
  k_apply_transformation<<<grid_for(h, n), 128, 0, h->stream>>>(h->sys, n, d_a, d_b);
  if (int e = check_launch(h)) return e;
  CUDA_TRY(h, cudaMemcpyAsync(out, d_b, n * ne * 8, cudaMemcpyDeviceToHost, h->stream));
  return wait_stream(h);
}

int cair_find_state(cair_handle* h, int64_t n, const double* paq_vel, cair_traj_point* out) {
  if (!h || n < 0 || !paq_vel || !out) return fail(h, CAIR_EINVAL, "cair_find_state: bad argument");
  if (n == 0) return 0;
  const int ne = h->sys.ne;
  if (int e = ensure_scratch(h, n * (ne * 8 + sizeof(cair_traj_point)) + 1024)) return e;
  Carver c{(char*)h->d_scratch};
  double* d_p = c.take<double>(n * ne);
  cair_traj_point* d_o = c.take<cair_traj_point>(n);
  CUDA_TRY(h, cudaMemcpyAsync(d_p, paq_vel, n * ne * 8, cudaMemcpyHostToDevice, h->stream));
  if (three_atoms(h)) k_find_state<3><<<grid_for(h, n), 128, 0, h->stream>>>(h->sys, h->fs, n, d_p, d_o);
  else k_find_state<4><<<grid_for(h, n), 128, 0, h->stream>>>(h->sys, h->fs, n, d_p, d_o);
  if (int e = check_launch(h)) return e;
  CUDA_TRY(h, cudaMemcpyAsync(out, d_o, n * sizeof(cair_traj_point), cudaMemcpyDeviceToHost, h->stream));
  return wait_stream(h);
}

namespace {
// control words of a batch: [0] queue head, [1..5] counters, [8..8+511] bucket counts and offsets,
// [520..522] the tail hand-off's (in flight, hand-offs, the warp integrator's queue over them)
constexpr int kCtl = 8 + 2 * 256 + 8, kHandCtl = 8 + 2 * 256;
struct BatchBufs {
  unsigned long long* ctl;
  double *paq, *paq0, *erra, *t, *dt, *H, *H0, *smax, *smin, *b, *draws, *key;
  int32_t *irej, *iste, *status, *ipes, *item_of, *order;
};

// Batch state of n trajectories of ne equations (12: diatom + atom, 18: diatom + diatom)
constexpr size_t batch_bytes(int64_t n, int ne) {
  return (size_t)n * (sizeof(double) * (ne * 3 + 9 + kDraws) + sizeof(int32_t) * 6) + 40 * 256 +
         sizeof(unsigned long long) * kCtl;
}

void carve_into(char* base, int64_t n, int ne, BatchBufs& B) {
  Carver c{base};
  B.ctl = c.take<unsigned long long>(kCtl);
  B.paq = c.take<double>(n * ne); B.paq0 = c.take<double>(n * ne); B.erra = c.take<double>(n * ne);
  B.t = c.take<double>(n); B.dt = c.take<double>(n); B.H = c.take<double>(n); B.H0 = c.take<double>(n);
  B.smax = c.take<double>(n); B.smin = c.take<double>(n); B.b = c.take<double>(n);
  B.draws = c.take<double>(n * kDraws); B.key = c.take<double>(n);
  B.irej = c.take<int32_t>(n); B.iste = c.take<int32_t>(n); B.status = c.take<int32_t>(n);
  B.ipes = c.take<int32_t>(n); B.item_of = c.take<int32_t>(n); B.order = c.take<int32_t>(n);
}

int carve_batch(cair_handle* h, int64_t n, bool with_state, BatchBufs& B) {
  (void)with_state;
  if (int e = ensure_work(h, batch_bytes(n, h->sys.ne))) return e;
  carve_into((char*)h->d_work, n, h->sys.ne, B);
  return 0;
}

int sample_ics_into(cair_handle* h, int32_t nitems, const cair_work_item* d_items, const cair_level* d_levels,
                    int64_t ntot, double* paq, double* paq0, double* erra, double* H0, double* b, int32_t* ipes,
                    int32_t* item_of, double* draws, cudaStream_t st, double* key = nullptr) {
  k_ic_draws<<<(nitems + 63) / 64, 64, 0, st>>>(nitems, h->sys.natoms == 4 ? 2 : 1, d_items, d_levels, draws,
                                                item_of);
  if (int e = check_launch(h)) return e;
  int g = grid_for(h, ntot);
  return with_model(h, [&](auto L) {
    L.sample_ic(g, st, h->sys, ntot, d_items, d_levels, draws, item_of, paq, paq0, erra, H0, b, ipes, key);
  });
}

int validate_items(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                   const cair_work_item* items, int64_t ntot) {
  int64_t sum = 0;
  for (int i = 0; i < nitems; ++i) {
    const cair_work_item& w = items[i];
    if (w.ilevel < 0 || w.ilevel >= nlevels) return fail(h, CAIR_EINVAL, "work item level out of range");
    if (h->sys.natoms == 4 && (w.ilevel2 < 0 || w.ilevel2 >= nlevels))
      return fail(h, CAIR_EINVAL, "work item projectile level out of range");
    if (w.ipes < 0 || w.ipes >= h->sys.npes) return fail(h, CAIR_EINVAL, "work item surface out of range");
    if (w.ntraj < 0 || w.first != sum) return fail(h, CAIR_EINVAL, "work items must tile [0, ntot) in order");
    if (!(w.dinit > 0.0) || std::fabs(w.bmax) > w.dinit || std::fabs(w.bmin) > w.dinit)
      return fail(h, CAIR_EINVAL, "impact parameter exceeds Dinit");
    if (w.b_mode < 0 || w.b_mode > 2) return fail(h, CAIR_EINVAL, "b_mode must be 0 (Circles), 1 (Rings) or 2 (Segments)");
    if (w.skip < 0) return fail(h, CAIR_EINVAL, "work item skip must be >= 0");
    if (!(w.ttra > 0.0)) return fail(h, CAIR_EINVAL, "translational temperature must be positive");
    sum += w.ntraj;
  }
  if (sum != ntot) return fail(h, CAIR_EINVAL, "ntot differs from the sum of the items' ntraj");
  for (int i = 0; i < nlevels; ++i)
    if (!(levels[i].tau > 0.0) || !(levels[i].ro > 0.0)) return fail(h, CAIR_EINVAL, "level with tau or ro <= 0");
  return 0;
}
}  // namespace

int cair_sample_ics_dev(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                        const cair_work_item* items, int64_t ntot, double* paq, double* paq0, double* erra,
                        double* H0, double* b, int32_t* ipes, int32_t* item_of, void* stream) {
  if (!h || nlevels < 1 || nitems < 0 || ntot < 0 || !levels || !items || !paq || !paq0 || !erra || !H0 || !b ||
      !ipes || !item_of)
    return fail(h, CAIR_EINVAL, "cair_sample_ics_dev: bad argument");
  if (ntot == 0) return 0;
  if (int e = ensure_scratch(h, ntot * kDraws * sizeof(double) + 1024)) return e;
  cudaStream_t st = (cudaStream_t)stream;
  return sample_ics_into(h, nitems, items, levels, ntot, paq, paq0, erra, H0, b, ipes, item_of,
                         (double*)h->d_scratch, st);
}

int cair_sample_ics(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                    const cair_work_item* items, int64_t ntot, double* paq, double* paq0, double* erra,
                    double* H0, double* b, int32_t* ipes) {
  if (!h || nlevels < 1 || nitems < 0 || ntot < 0 || !levels || !items || !paq || !paq0 || !erra || !H0 || !b ||
      !ipes)
    return fail(h, CAIR_EINVAL, "cair_sample_ics: bad argument");
  if (ntot == 0) return 0;
  if (int e = validate_items(h, nlevels, levels, nitems, items, ntot)) return e;
  BatchBufs B;
  if (int e = carve_batch(h, ntot, false, B)) return e;
  if (int e = ensure_scratch(h, nlevels * sizeof(cair_level) + nitems * sizeof(cair_work_item) + 1024)) return e;
  Carver c{(char*)h->d_scratch};
  cair_level* d_lv = c.take<cair_level>(nlevels);
  cair_work_item* d_it = c.take<cair_work_item>(nitems > 0 ? nitems : 1);
  cudaStream_t st = h->stream;
  CUDA_TRY(h, cudaMemcpyAsync(d_lv, levels, nlevels * sizeof(cair_level), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_it, items, nitems * sizeof(cair_work_item), cudaMemcpyHostToDevice, st));
  if (int e = sample_ics_into(h, nitems, d_it, d_lv, ntot, B.paq, B.paq0, B.erra, B.H0, B.b, B.ipes, B.item_of,
                              B.draws, st))
    return e;
  const int ne = h->sys.ne;
  CUDA_TRY(h, cudaMemcpyAsync(paq, B.paq, ntot * ne * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(paq0, B.paq0, ntot * ne * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(erra, B.erra, ntot * ne * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(H0, B.H0, ntot * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(b, B.b, ntot * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(ipes, B.ipes, ntot * 4, cudaMemcpyDeviceToHost, st));
  return wait_stream(h);
}

int64_t cair_queue_workspace_bytes(int64_t ntot) { return ntot < 0 ? 0 : (int64_t)batch_bytes(ntot, 18); }

int cair_run_queue_dev(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                       const cair_work_item* items, int64_t ntot, int64_t max_attempts, cair_traj_result* results,
                       void* workspace, void* stream) {
  if (!h || nlevels < 1 || nitems < 0 || ntot < 0 || !levels || !items || !results || max_attempts < 1)
    return fail(h, CAIR_EINVAL, "cair_run_queue_dev: bad argument");
  if (ntot == 0) return 0;
  if (workspace && ((uintptr_t)workspace & 255)) return fail(h, CAIR_EINVAL, "workspace must be 256-byte aligned");
  BatchBufs B;
  if (workspace) carve_into((char*)workspace, ntot, h->sys.ne, B);
  else if (int e = carve_batch(h, ntot, true, B)) return e;
  cudaStream_t st = (cudaStream_t)stream;
  if (int e = sample_ics_into(h, nitems, items, levels, ntot, B.paq, B.paq0, B.erra, B.H0, B.b, B.ipes, B.item_of,
                              B.draws, st, B.key))
    return e;
  // queue order: longest predicted duration first (bucketed by initial relative speed)
  CUDA_TRY(h, cudaMemsetAsync(B.ctl, 0, sizeof(unsigned long long) * kCtl, st));
  const int g = grid_for(h, ntot);
  cair_k_bucket_count<<<g, 256, 0, st>>>(ntot, B.key, B.ctl + 8);
  cair_k_bucket_scan<<<1, 256, 0, st>>>(B.ctl + 8, B.ctl + 8 + 256);
  cair_k_bucket_scatter<<<g, 256, 0, st>>>(ntot, B.key, B.ctl + 8 + 256, B.order);
  cair_k_init_state<<<g, 128, 0, st>>>(ntot, h->sys.dt0, B.t, B.dt, B.smax, B.smin, B.irej, B.iste);
  if (int e = check_launch(h)) return e;
  IntegrateArgs A{ntot, B.ipes, B.paq, B.t, B.dt, B.erra, B.H, B.smax, B.smin, B.irej, B.iste, B.status,
                  max_attempts, B.ctl, B.ctl + 1, B.order};
  // the initial-condition draws are spent: their space holds the tail hand-off's list and attempt counts
  static_assert(kDraws >= 2, "hand-off list and attempts fit in the draws");
  HandBufs hb{reinterpret_cast<int32_t*>(B.draws + ntot), reinterpret_cast<long long*>(B.draws), B.ctl + kHandCtl};
  if (int e = launch_integrate(h, A, st, &hb)) return e;
  if (three_atoms(h))
    k_results<3><<<g, 128, 0, st>>>(h->sys, h->fs, ntot, B.paq0, B.paq, B.H0, B.H, B.t, B.status, B.iste, B.irej,
                                    B.item_of, items, results);
  else
    k_results<4><<<g, 128, 0, st>>>(h->sys, h->fs, ntot, B.paq0, B.paq, B.H0, B.H, B.t, B.status, B.iste, B.irej,
                                    B.item_of, items, results);
  if (int e = check_launch(h)) return e;
  if (!workspace)
    CUDA_TRY(h, cudaMemcpyAsync(h->d_ctl + 1, B.ctl + 1, sizeof(unsigned long long) * 5, cudaMemcpyDeviceToDevice, st));
  return 0;
}

}  // extern "C"

// -----------------------------------------------------------------------------------------
// Allocation-free variant of the queue path.  The batch state of up to
// CAIR_STATIC_QUEUE_MAX_TRAJ trajectories lives in this file-scope device array, which every
// GPU that loads the library holds until the process exits.  In host code the array's name is
// only a host-side stand-in, so its device address is looked up once per device with
// cudaGetSymbolAddress (on the first call made with that device current) and passed to the
// kernels like any workspace.  Every call shares the array: the queue head and counters are
// cleared at the start of each call, and calls that overlap on the GPU race.
// -----------------------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_cair_static_queue_ws[batch_bytes(CAIR_STATIC_QUEUE_MAX_TRAJ, 12)];
static std::mutex g_static_ws_mutex;
static void* g_static_ws_ptr[64] = {nullptr};

extern "C" {

int cair_run_queue_static_dev(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                              const cair_work_item* items, int64_t ntot, int64_t max_attempts,
                              cair_traj_result* results, void* stream) {
  if (!h) return CAIR_EINVAL;
  if (ntot < 0 || batch_bytes(ntot, h->sys.ne) > sizeof(g_cair_static_queue_ws))
    return fail(h, CAIR_EINVAL, "cair_run_queue_static_dev: ntot exceeds the static workspace (at most " +
                                    std::to_string(CAIR_STATIC_QUEUE_MAX_TRAJ) +
                                    " diatom + atom trajectories per call, fewer of four atoms)");
  int dev = -1;
  CUDA_TRY(h, cudaGetDevice(&dev));
  if (dev != h->device || dev < 0 || dev >= 64)
    return fail(h, CAIR_EINVAL, "cair_run_queue_static_dev: the current device is not the handle's device");
  void* ws = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_static_ws_mutex);
    if (!g_static_ws_ptr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_cair_static_queue_ws);
      if (e != cudaSuccess || !p)
        return fail(h, CAIR_ECUDA, std::string("cudaGetSymbolAddress of the static workspace: ") +
                                       cudaGetErrorString(e));
      g_static_ws_ptr[dev] = p;
    }
    ws = g_static_ws_ptr[dev];
  }
  return cair_run_queue_dev(h, nlevels, levels, nitems, items, ntot, max_attempts, results, ws, stream);
}

int cair_run_queue(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                   const cair_work_item* items, int64_t ntot, int64_t max_attempts, cair_traj_result* results) {
  if (!h || nlevels < 1 || nitems < 0 || ntot < 0 || !levels || !items || !results || max_attempts < 1)
    return fail(h, CAIR_EINVAL, "cair_run_queue: bad argument");
  if (ntot == 0) return 0;
  if (int e = validate_items(h, nlevels, levels, nitems, items, ntot)) return e;
  if (int e = ensure_scratch(h, nlevels * sizeof(cair_level) + nitems * sizeof(cair_work_item) +
                                     ntot * sizeof(cair_traj_result) + 4096))
    return e;
  Carver c{(char*)h->d_scratch};
  cair_level* d_lv = c.take<cair_level>(nlevels);
  cair_work_item* d_it = c.take<cair_work_item>(nitems > 0 ? nitems : 1);
  cair_traj_result* d_res = c.take<cair_traj_result>(ntot);
  cudaStream_t st = h->stream;
  CUDA_TRY(h, cudaMemcpyAsync(d_lv, levels, nlevels * sizeof(cair_level), cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_it, items, nitems * sizeof(cair_work_item), cudaMemcpyHostToDevice, st));
  if (int e = cair_run_queue_dev(h, nlevels, d_lv, nitems, d_it, ntot, max_attempts, d_res, nullptr, st)) return e;
  CUDA_TRY(h, cudaMemcpyAsync(results, d_res, ntot * sizeof(cair_traj_result), cudaMemcpyDeviceToHost, st));
  unsigned long long ctr[5];
  CUDA_TRY(h, cudaMemcpyAsync(ctr, h->d_ctl + 1, sizeof(ctr), cudaMemcpyDeviceToHost, st));
  if (int e = wait_stream(h)) return e;
  for (int i = 0; i < 5; ++i) h->last_counters[i] = (long long)ctr[i];
  return 0;
}

int cair_set_warp_timeline(cair_handle* h, uint64_t* times_dev, int64_t cap_warps) {
  if (!h || (times_dev && cap_warps < 1)) return fail(h, CAIR_EINVAL, "cair_set_warp_timeline: bad argument");
  h->warp_times = (unsigned long long*)times_dev;
  h->warp_times_cap = times_dev ? cap_warps : 0;
  h->warp_times_n = 0;
  return 0;
}

int64_t cair_warp_timeline_count(const cair_handle* h) { return h ? h->warp_times_n : 0; }

int cair_set_launch_shape(cair_handle* h, int32_t block, int32_t per_sm) {
  if (!h || (block != 32 && block != 64 && block != 128) || per_sm < 0)
    return fail(h, CAIR_EINVAL, "cair_set_launch_shape: block must be 32, 64 or 128, per_sm >= 0");
  h->tune_block = block;
  h->tune_per_sm = per_sm;
  return 0;
}

int cair_get_launch_shape(const cair_handle* h, int32_t* block, int32_t* per_sm) {
  if (!h || !block || !per_sm) return CAIR_EINVAL;
  *block = h->tune_block;
  *per_sm = h->tune_per_sm;
  return 0;
}

int cair_set_integrator_mode(cair_handle* h, int32_t mode) {
  if (!h || (mode != CAIR_INTEGRATOR_THREAD && mode != CAIR_INTEGRATOR_WARP && mode != CAIR_INTEGRATOR_AUTO))
    return fail(h, CAIR_EINVAL, "cair_set_integrator_mode: mode must be CAIR_INTEGRATOR_THREAD, _WARP or _AUTO");
  if (mode == CAIR_INTEGRATOR_WARP && !warp_integrate_supported(h->sys))
    return fail(h, CAIR_EUNSUPPORTED,
                "cair_set_integrator_mode: the warp integrator is built for the O3, N3, O4 and N4 UMN surfaces with "
                "their own diatomics (one model per handle) and NSteps 2..4");
  h->mode = mode;
  return 0;
}

int32_t cair_get_integrator_mode(const cair_handle* h) { return h ? h->mode : CAIR_INTEGRATOR_THREAD; }

int32_t cair_last_integrator(const cair_handle* h) { return h ? h->last_integrator : CAIR_INTEGRATOR_THREAD; }

int cair_set_tail_handoff(cair_handle* h, int64_t below) {
  if (!h) return CAIR_EINVAL;
  h->hand_below = below < 0 ? -1 : below;
  return 0;
}

int64_t cair_last_handoffs(cair_handle* h) {
  if (!h || !h->last_hctl) return 0;
  unsigned long long n = 0;
  if (cudaStreamSynchronize(h->stream) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
      cudaMemcpy(&n, h->last_hctl + 1, sizeof n, cudaMemcpyDeviceToHost) != cudaSuccess)
    return -1;
  return (int64_t)n;
}

// Calibration of the persistent integrator's launch shape on the job's own work: every item keeps
// the leading fraction of its trajectories (same streams) so that about `sample` trajectories run,
// each capped at `cap_attempts` attempts so that every lane stays busy, once per candidate shape
// (blocks of 32, 64 and 128 threads, 1 .. the resident maximum per SM); the shape with the most
// Bulirsch-Stoer attempts per second of integrator time is kept on the handle.
int cair_autotune(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                  const cair_work_item* items, int64_t sample, int64_t cap_attempts, cair_tune_point* out,
                  int32_t cap, int32_t* nout) {
  if (!h || nlevels < 1 || nitems < 1 || !levels || !items || sample < 1 || cap_attempts < 1 || !nout ||
      (cap > 0 && !out))
    return fail(h, CAIR_EINVAL, "cair_autotune: bad argument");
  if (h->sur) return fail(h, CAIR_EUNSUPPORTED, "cair_autotune: the surrogate integrator has one launch shape");
  int64_t ntot = 0;
  for (int i = 0; i < nitems; ++i) ntot += items[i].ntraj;
  if (ntot < 1) return fail(h, CAIR_EINVAL, "cair_autotune: no trajectories");
  std::vector<cair_work_item> smp(items, items + nitems);
  const double f = std::min(1.0, (double)sample / (double)ntot);
  int64_t first = 0;
  for (auto& it : smp) {
    it.ntraj = it.ntraj > 0 ? std::max<int64_t>(1, (int64_t)std::llround(it.ntraj * f)) : 0;
    it.first = first;
    first += it.ntraj;
  }
  const int64_t n = first;
  std::vector<cair_traj_result> rows((size_t)n);
  const int keep_block = h->tune_block, keep_per_sm = h->tune_per_sm;
  const bool keep_timing = h->time_integrate;
  double best = -1.0;
  int best_block = keep_block, best_per_sm = keep_per_sm;
  int32_t k = 0;
  int rc = 0;
  for (int block : {32, 64, 128}) {
    int occ = 0;
    if (int e = with_model(h, [&](auto L) { occ = L.integrate_blocks_per_sm(block, h->sys.nsteps); })) return e;
    for (int per_sm = 1; per_sm <= occ; ++per_sm) {
      h->tune_block = block;
      h->tune_per_sm = per_sm;
      h->time_integrate = true;
      h->ntev = 0;
      rc = cair_run_queue(h, nlevels, levels, nitems, smp.data(), n, cap_attempts, rows.data());
      float ms = 0.0f;
      int32_t cnt = 0;
      if (!rc) rc = cair_integrate_timings(h, &ms, 1, &cnt);
      if (rc) break;
      const double rate = (double)h->last_counters[0] / (ms * 1e-3);
      if (k < cap) out[k] = cair_tune_point{block, per_sm, (double)ms, rate};
      ++k;
      if (rate > best) {
        best = rate;
        best_block = block;
        best_per_sm = per_sm;
      }
    }
    if (rc) break;
  }
  h->time_integrate = keep_timing;
  h->ntev = 0;
  h->tune_block = rc ? keep_block : best_block;
  h->tune_per_sm = rc ? keep_per_sm : best_per_sm;
  *nout = k;
  return rc;
}

int cair_flop_model(const cair_handle* h, int32_t ipes, double* fg, double* fe, double* fa, double* ex) {
  if (!h || ipes < 0 || ipes >= h->sys.npes) return CAIR_EINVAL;
  // FP64 operations of the executed formulation, counted from the device code (an FMA counts
  // two, exp / division / sqrt one each): PIP part from the generator's counts of the gradient
  // formulation compiled in (adjoint sweep unless CAIR_PIP_FORWARD); per pair the
  // diatomic (O2 UMN 107 with gradient, 64 energy only; N2 UMN_ForN4 64 / 40) and the MEG
  // variable (11 / 7); pair distances 36, TransToCart 46, Hamilton's equations 18, assembly 15.
  const int m = h->sys.pes[ipes].model;
  const bool o2 = h->sys.diat == CAIR_DIAT_O2_UMN;
  const double diat_g = o2 ? 107 : 64, diat_e = o2 ? 64 : 40, meg_g = 11, meg_e = 7;
#ifdef CAIR_PIP_FORWARD
  const double pip_g = m == CAIR_PES_O3_UMN ? PIP_O3_EVAL_FLOPS : PIP_N3_EVAL_FLOPS;
#else
  const double pip_g = m == CAIR_PES_O3_UMN ? PIP_O3_EVAL_REV_FLOPS : PIP_N3_EVAL_REV_FLOPS;
#endif
  const double pip_e = m == CAIR_PES_O3_UMN ? PIP_O3_VALUE_FLOPS : PIP_N3_VALUE_FLOPS;
  if (m == CAIR_PES_O3_NN || m == CAIR_PES_O3_BNN) {
    // pes_o3nn: MEG-like variables 9, features 41, layer 1 20 x 14, layer 2 and output 10 x 47,
    // output 6, adjoint sweep 20 x 35, dG/dR contraction 148 (tanh counted as one operation);
    // the energy-only network (Potential) 9 + 21 + 20 x 7 + 10 x 43 + 4.  Diatomics with gradient
    // in both (Compute_Vd_dVd).  BNN: exp(v + Noise) and its factor on the gradient, 2 + 4.
    const double bo = m == CAIR_PES_O3_BNN ? 1.0 : 0.0;
    if (fg) *fg = 9 + 3 * diat_g + 41 + 280 + 470 + 6 + 700 + 148 + 36 + 46 + 18 + 15 + 6 * bo;
    if (fe) *fe = 9 + 3 * diat_g + 21 + 140 + 430 + 4 + 36 + 30 + 8 + 2 * bo;
    if (fa) *fa = 811;
    if (ex) *ex = 3.0 * ((o2 ? 8 : 1) + 1) + CAIR_NN_H1 + CAIR_NN_H2 + bo;
    return 0;
  }
  if (m == CAIR_PES_N4_PIPNN) {
    // no force from the surface (dVdQ = 0): Hamilton's equations 45 and the assembly of zeros; the
    // energy: six pair terms (~60 each), six exponentials, the 276-function basis and per selected
    // network 276 normalisations (2) and 5 x 276 + 90 x 5 + 90 multiply-adds (2), 95 activations (~12)
    const double nuse = h->nnets[ipes];
    if (fg) *fg = 45 + 15;
    if (fe) *fe = 6 * 60 + 6 + PIP_N4_BASIS_FLOPS + nuse * (2 * 276 + 2 * (5 * 276 + 90 * 5 + 90) + 95 * 12 + 2) + 72 + 45 + 8;
    if (fa) *fa = 811.0 * 18.0 / 12.0;
    if (ex) *ex = 6.0 + nuse * 95.0;
    return 0;
  }
  if (m == CAIR_PES_O4_UMN || m == CAIR_PES_N4_UMN) {
    // six pairs: distances 72, TransToCart_4 110, Hamilton's equations 45, assembly 15; BS
    // bookkeeping scales with the 18 equations
    const double pg = m == CAIR_PES_O4_UMN ? PIP_O4_EVAL_REV_FLOPS : PIP_N4_EVAL_REV_FLOPS;
    const double pe = m == CAIR_PES_O4_UMN ? PIP_O4_VALUE_FLOPS : PIP_N4_VALUE_FLOPS;
    if (fg) *fg = pg + 6 * (diat_g + meg_g) + 72 + 110 + 45 + 15;
    if (fe) *fe = pe + 6 * (diat_e + meg_e) + 72 + 45 + 8;
    if (fa) *fa = 811.0 * 18.0 / 12.0;
    if (ex) *ex = 6.0 * ((o2 ? 8 : 1) + 1);
    return 0;
  }
  if (fg) *fg = pip_g + 3 * (diat_g + meg_g) + 36 + 46 + 18 + 15;
  if (fe) *fe = pip_e + 3 * (diat_e + meg_e) + 36 + 30 + 8;
  // per attempt outside the right-hand side: modified-midpoint updates (432), rational
  // extrapolation (297), error norms and step control (82)
  if (fa) *fa = 811;
  if (ex) *ex = 3.0 * ((o2 ? 8 : 1) + 1);
  return 0;
}

// The device rings a run by its items' |bmax|.  SetRings (Statistics_Class.F90:534-581) rings by the
// rows' bMax; the queue writes each row's bmax from its item, so the two agree unless the rows were
// edited or merged from elsewhere, and then the statistics refuse them instead of ringing them apart
// from the reference.
static const char* kBmaxMismatch =
    "cair_statistics: a counted row's bmax differs from its work item's |bmax| by 1e-3 or more (the rings are "
    "the items' bmax)";

int cair_statistics_dev(cair_handle* h, int32_t nitems, const cair_work_item* items, const int32_t* item_run,
                        int64_t ntot, const cair_traj_result* results, const cair_stats_params* params,
                        cair_final_state* out, int64_t cap, int64_t* nout, void* stream) {
  if (!h || nitems < 1 || !items || ntot < 0 || (ntot > 0 && !results) || !params || cap < 0 || (cap > 0 && !out) ||
      !nout)
    return fail(h, CAIR_EINVAL, "cair_statistics: bad argument");
  const cair_stats_params& P = *params;
  const int nc = P.ncond;
  if (nc != 3 && nc != 5) return fail(h, CAIR_EINVAL, "cair_statistics: ncond must be 3 or 5");
  if (nc != (h->sys.natoms == 4 ? 5 : 3))
    return fail(h, CAIR_EINVAL, "cair_statistics: ncond must be 3 for diatom + atom, 5 for diatom + diatom");
  if (P.qn_max < 2) return fail(h, CAIR_EINVAL, "cair_statistics: qn_max out of range");
  StatsRuns runs;
  if (std::string e = stats_runs(nitems, items, item_run, runs); !e.empty()) return fail(h, CAIR_EINVAL, e);
  const int32_t nruns = runs.nruns;
  *nout = 0;
  if (ntot == 0) return 0;
  // table at least twice the rows, so linear probing always finds a slot
  unsigned long long tsize = 1024;
  while (tsize < 2ull * (unsigned long long)ntot) tsize <<= 1;
  const size_t per_run = (size_t)kMaxRings * 16 + 16;
  const size_t need = tsize * 32 + (size_t)nitems * 32 + (size_t)nruns * per_run + 9 * 256;
  if (h->stats_bytes < need) {
    if (h->d_stats) cudaFree(h->d_stats);
    h->d_stats = nullptr;
    h->stats_bytes = 0;
    CUDA_TRY(h, cudaMalloc(&h->d_stats, need));
    h->stats_bytes = need;
  }
  Carver c{(char*)h->d_stats};
  unsigned long long* keys = c.take<unsigned long long>(tsize);
  unsigned long long* counts = c.take<unsigned long long>(tsize);
  unsigned long long* okeys = c.take<unsigned long long>(tsize);
  unsigned long long* ocounts = c.take<unsigned long long>(tsize);
  unsigned long long* item_rows = c.take<unsigned long long>(nitems);
  long long* item_ini = c.take<long long>(nitems);
  double* ring_b = c.take<double>((size_t)nruns * kMaxRings);
  unsigned long long* ring_rows = c.take<unsigned long long>((size_t)nruns * kMaxRings);
  int32_t* d_run = c.take<int32_t>(nitems);
  int32_t* d_nring = c.take<int32_t>(nruns);
  double* d_ibmax = c.take<double>(nitems);
  unsigned long long* dn = c.take<unsigned long long>(2);
  int* derr = (int*)(dn + 1);
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<double> ibmax(nitems);
  for (int i = 0; i < nitems; ++i) ibmax[i] = std::fabs(items[i].bmax);
  CUDA_TRY(h, cudaMemsetAsync(keys, 0xff, tsize * 8, st));
  CUDA_TRY(h, cudaMemsetAsync(counts, 0, tsize * 8, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_ibmax, ibmax.data(), (size_t)nitems * 8, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemsetAsync(item_rows, 0, (size_t)nitems * 8, st));
  CUDA_TRY(h, cudaMemsetAsync(item_ini, 0x7f, (size_t)nitems * 8, st));
  CUDA_TRY(h, cudaMemsetAsync(ring_rows, 0, (size_t)nruns * kMaxRings * 8, st));
  CUDA_TRY(h, cudaMemsetAsync(dn, 0, 16, st));
  StatsArgs A{ntot,
              results,
              P.qn_max,
              {P.iskip[0], P.iskip[1], P.iskip[2], P.iskip[3], P.iskip[4]},
              {P.pres_even_odd[0], P.pres_even_odd[1], P.pres_even_odd[2], P.pres_even_odd[3], P.pres_even_odd[4]},
              P.ham_abs_tol,
              d_run,
              ring_b,
              d_nring,
              nruns,
              1,
              keys,
              counts,
              tsize - 1,
              item_rows,
              item_ini,
              ring_rows,
              derr,
              d_ibmax};
  // pass 1: rows and initial-state codes of each item
  if (nc == 3) k_stats_items<3><<<grid_for(h, ntot), 256, 0, st>>>(A);
  else k_stats_items<5><<<grid_for(h, ntot), 256, 0, st>>>(A);
  if (int e = check_launch(h)) return e;
  int err = 0;
  std::vector<unsigned long long> rows(nitems);
  std::vector<long long> ini(nitems);
  CUDA_TRY(h, cudaMemcpyAsync(&err, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(rows.data(), item_rows, (size_t)nitems * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(ini.data(), item_ini, (size_t)nitems * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaStreamSynchronize(st));
  if (err == 1) return fail(h, CAIR_EINVAL, "cair_statistics: a quantum number is at or above qn_max");
  if (std::string e = stats_rings(P, nitems, items, rows.data(), ini.data(), runs); !e.empty())
    return fail(h, CAIR_EINVAL, e);
  // pass 2: (run, final state, ring) counts
  A.R = runs.R;
  CUDA_TRY(h, cudaMemcpyAsync(ring_b, runs.ring_b.data(), runs.ring_b.size() * 8, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_nring, runs.nring.data(), (size_t)nruns * 4, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_run, runs.run_of.data(), (size_t)nitems * 4, cudaMemcpyHostToDevice, st));
  if (nc == 3) k_stats_count<3><<<grid_for(h, ntot), 256, 0, st>>>(A);
  else k_stats_count<5><<<grid_for(h, ntot), 256, 0, st>>>(A);
  k_stats_compact<<<grid_for(h, (int64_t)tsize), 256, 0, st>>>(keys, counts, tsize, okeys, ocounts, tsize, dn);
  if (int e = check_launch(h)) return e;
  unsigned long long n = 0;
  std::vector<unsigned long long> perb((size_t)nruns * kMaxRings);
  CUDA_TRY(h, cudaMemcpyAsync(&n, dn, 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(&err, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(perb.data(), ring_rows, perb.size() * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaStreamSynchronize(st));
  if (err == 3) return fail(h, CAIR_EINVAL, kBmaxMismatch);
  if (err) return fail(h, CAIR_EINVAL, "cair_statistics: a final-state key of -1 (not representable)");
  std::vector<unsigned long long> k(n), cnt(n);
  if (n) {
    CUDA_TRY(h, cudaMemcpyAsync(k.data(), okeys, n * 8, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(h, cudaMemcpyAsync(cnt.data(), ocounts, n * 8, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(h, cudaStreamSynchronize(st));
  }
  if (std::string e = stats_finish(P, runs, (int64_t)n, k.data(), cnt.data(), perb.data(), out, cap, nout); !e.empty())
    return fail(h, CAIR_EINVAL, e);
  return 0;
}

int cair_statistics(cair_handle* h, int32_t nitems, const cair_work_item* items, const int32_t* item_run, int64_t ntot,
                    const cair_traj_result* results, const cair_stats_params* params, cair_final_state* out,
                    int64_t cap, int64_t* nout) {
  if (!h || ntot < 0 || (ntot > 0 && !results)) return fail(h, CAIR_EINVAL, "cair_statistics: bad argument");
  if (int e = ensure_scratch(h, (size_t)ntot * sizeof(cair_traj_result) + 256)) return e;
  if (ntot > 0)
    CUDA_TRY(h, cudaMemcpyAsync(h->d_scratch, results, (size_t)ntot * sizeof(cair_traj_result),
                                cudaMemcpyHostToDevice, h->stream));
  return cair_statistics_dev(h, nitems, items, item_run, ntot, (const cair_traj_result*)h->d_scratch, params, out,
                             cap, nout, h->stream);
}

// Statistics of replicas, step 1: counted rows and the smallest initial-state code per item (pass 1).
int cair_statistics_items_dev(cair_handle* h, int32_t nitems, int64_t ntot, const cair_traj_result* results,
                              const cair_stats_params* params, uint64_t* item_rows, int64_t* item_ini,
                              void* stream) {
  if (!h || nitems < 1 || ntot < 0 || (ntot > 0 && !results) || !params || !item_rows || !item_ini)
    return fail(h, CAIR_EINVAL, "cair_statistics_items: bad argument");
  const cair_stats_params& P = *params;
  const int nc = P.ncond;
  if (nc != (h->sys.natoms == 4 ? 5 : 3))
    return fail(h, CAIR_EINVAL, "cair_statistics_items: ncond must be 3 for diatom + atom, 5 for diatom + diatom");
  if (P.qn_max < 2) return fail(h, CAIR_EINVAL, "cair_statistics_items: qn_max out of range");
  const size_t need = (size_t)nitems * 16 + 4 * 256;
  if (h->stats_bytes < need) {
    if (h->d_stats) cudaFree(h->d_stats);
    h->d_stats = nullptr;
    h->stats_bytes = 0;
    CUDA_TRY(h, cudaMalloc(&h->d_stats, need));
    h->stats_bytes = need;
  }
  Carver c{(char*)h->d_stats};
  unsigned long long* d_rows = c.take<unsigned long long>(nitems);
  long long* d_ini = c.take<long long>(nitems);
  int* derr = c.take<int>(2);
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(h, cudaMemsetAsync(d_rows, 0, (size_t)nitems * 8, st));
  CUDA_TRY(h, cudaMemsetAsync(d_ini, 0x7f, (size_t)nitems * 8, st));
  CUDA_TRY(h, cudaMemsetAsync(derr, 0, 8, st));
  if (ntot > 0) {
    StatsArgs A{};
    A.ntot = ntot;
    A.rows = results;
    A.qnmax = P.qn_max;
    for (int q = 0; q < 5; ++q) {
      A.iskip[q] = P.iskip[q];
      A.pres[q] = P.pres_even_odd[q];
    }
    A.ham_abs_tol = P.ham_abs_tol;
    A.item_rows = d_rows;
    A.item_inicode = d_ini;
    A.error = derr;
    if (nc == 3) k_stats_items<3><<<grid_for(h, ntot), 256, 0, st>>>(A);
    else k_stats_items<5><<<grid_for(h, ntot), 256, 0, st>>>(A);
    if (int e = check_launch(h)) return e;
  }
  int err = 0;
  CUDA_TRY(h, cudaMemcpyAsync(&err, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(item_rows, d_rows, (size_t)nitems * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(item_ini, d_ini, (size_t)nitems * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaStreamSynchronize(st));
  if (err == 1) return fail(h, CAIR_EINVAL, "cair_statistics_items: a quantum number is at or above qn_max");
  return 0;
}

// Statistics of replicas, step 2: this replica's (run, ring, code) counts under the rings of the
// replicas' totals (pass 2).
int cair_statistics_counts_dev(cair_handle* h, int32_t nitems, const cair_work_item* items, const int32_t* item_run,
                               const uint64_t* item_rows, const int64_t* item_ini, int64_t ntot,
                               const cair_traj_result* results, const cair_stats_params* params,
                               cair_stats_count* out, int64_t cap, int64_t* nout, uint64_t* ring_rows,
                               void* stream) {
  if (!h || nitems < 1 || !items || !item_rows || !item_ini || ntot < 0 || (ntot > 0 && !results) || !params ||
      cap < 0 || (cap > 0 && !out) || !nout || !ring_rows)
    return fail(h, CAIR_EINVAL, "cair_statistics_counts: bad argument");
  const cair_stats_params& P = *params;
  const int nc = P.ncond;
  if (nc != (h->sys.natoms == 4 ? 5 : 3))
    return fail(h, CAIR_EINVAL, "cair_statistics_counts: ncond must be 3 for diatom + atom, 5 for diatom + diatom");
  if (P.qn_max < 2) return fail(h, CAIR_EINVAL, "cair_statistics_counts: qn_max out of range");
  StatsRuns runs;
  if (std::string e = stats_runs(nitems, items, item_run, runs); !e.empty()) return fail(h, CAIR_EINVAL, e);
  if (std::string e = stats_rings(P, nitems, items, (const unsigned long long*)item_rows, (const long long*)item_ini,
                                  runs);
      !e.empty())
    return fail(h, CAIR_EINVAL, e);
  const int32_t nruns = runs.nruns;
  *nout = 0;
  std::memset(ring_rows, 0, (size_t)nruns * kMaxRings * sizeof(uint64_t));
  if (ntot == 0) return 0;
  unsigned long long tsize = 1024;
  while (tsize < 2ull * (unsigned long long)ntot) tsize <<= 1;
  const size_t need = tsize * 32 + (size_t)nitems * 16 + (size_t)nruns * ((size_t)kMaxRings * 16 + 16) + 9 * 256;
  if (h->stats_bytes < need) {
    if (h->d_stats) cudaFree(h->d_stats);
    h->d_stats = nullptr;
    h->stats_bytes = 0;
    CUDA_TRY(h, cudaMalloc(&h->d_stats, need));
    h->stats_bytes = need;
  }
  Carver c{(char*)h->d_stats};
  unsigned long long* keys = c.take<unsigned long long>(tsize);
  unsigned long long* counts = c.take<unsigned long long>(tsize);
  unsigned long long* okeys = c.take<unsigned long long>(tsize);
  unsigned long long* ocounts = c.take<unsigned long long>(tsize);
  double* ring_b = c.take<double>((size_t)nruns * kMaxRings);
  unsigned long long* d_ring_rows = c.take<unsigned long long>((size_t)nruns * kMaxRings);
  int32_t* d_run = c.take<int32_t>(nitems);
  int32_t* d_nring = c.take<int32_t>(nruns);
  double* d_ibmax = c.take<double>(nitems);
  unsigned long long* dn = c.take<unsigned long long>(2);
  int* derr = (int*)(dn + 1);
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<double> ibmax(nitems);
  for (int i = 0; i < nitems; ++i) ibmax[i] = std::fabs(items[i].bmax);
  CUDA_TRY(h, cudaMemsetAsync(keys, 0xff, tsize * 8, st));
  CUDA_TRY(h, cudaMemsetAsync(counts, 0, tsize * 8, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_ibmax, ibmax.data(), (size_t)nitems * 8, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemsetAsync(d_ring_rows, 0, (size_t)nruns * kMaxRings * 8, st));
  CUDA_TRY(h, cudaMemsetAsync(dn, 0, 16, st));
  CUDA_TRY(h, cudaMemcpyAsync(ring_b, runs.ring_b.data(), runs.ring_b.size() * 8, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_nring, runs.nring.data(), (size_t)nruns * 4, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_run, runs.run_of.data(), (size_t)nitems * 4, cudaMemcpyHostToDevice, st));
  StatsArgs A{};
  A.ntot = ntot;
  A.rows = results;
  A.qnmax = P.qn_max;
  for (int q = 0; q < 5; ++q) {
    A.iskip[q] = P.iskip[q];
    A.pres[q] = P.pres_even_odd[q];
  }
  A.ham_abs_tol = P.ham_abs_tol;
  A.item_run = d_run;
  A.ring_b = ring_b;
  A.nring = d_nring;
  A.nruns = nruns;
  A.R = runs.R;
  A.keys = keys;
  A.counts = counts;
  A.mask = tsize - 1;
  A.ring_rows = d_ring_rows;
  A.error = derr;
  A.item_bmax = d_ibmax;
  if (nc == 3) k_stats_count<3><<<grid_for(h, ntot), 256, 0, st>>>(A);
  else k_stats_count<5><<<grid_for(h, ntot), 256, 0, st>>>(A);
  k_stats_compact<<<grid_for(h, (int64_t)tsize), 256, 0, st>>>(keys, counts, tsize, okeys, ocounts, tsize, dn);
  if (int e = check_launch(h)) return e;
  unsigned long long n = 0;
  int err = 0;
  CUDA_TRY(h, cudaMemcpyAsync(&n, dn, 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(&err, derr, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(ring_rows, d_ring_rows, (size_t)nruns * kMaxRings * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaStreamSynchronize(st));
  if (err == 3) return fail(h, CAIR_EINVAL, kBmaxMismatch);
  if (err) return fail(h, CAIR_EINVAL, "cair_statistics_counts: a final-state key of -1 (not representable)");
  if ((int64_t)n > cap)
    return fail(h, CAIR_EINVAL, "cair_statistics_counts: cap too small, " + std::to_string(n) + " counts");
  std::vector<unsigned long long> k(n), cnt(n);
  if (n) {
    CUDA_TRY(h, cudaMemcpyAsync(k.data(), okeys, n * 8, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(h, cudaMemcpyAsync(cnt.data(), ocounts, n * 8, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(h, cudaStreamSynchronize(st));
  }
  const std::vector<StatsEntry> ent = stats_decode(runs, (int64_t)n, k.data(), cnt.data());
  for (size_t q = 0; q < ent.size(); ++q)
    out[q] = cair_stats_count{ent[q].run, ent[q].ring, (int64_t)ent[q].code, (int64_t)ent[q].count};
  *nout = (int64_t)n;
  return 0;
}

int cair_statistics_items(cair_handle* h, int32_t nitems, int64_t ntot, const cair_traj_result* results,
                          const cair_stats_params* params, uint64_t* item_rows, int64_t* item_ini) {
  if (!h || ntot < 0 || (ntot > 0 && !results)) return fail(h, CAIR_EINVAL, "cair_statistics_items: bad argument");
  if (int e = ensure_scratch(h, (size_t)ntot * sizeof(cair_traj_result) + 256)) return e;
  if (ntot > 0)
    CUDA_TRY(h, cudaMemcpyAsync(h->d_scratch, results, (size_t)ntot * sizeof(cair_traj_result),
                                cudaMemcpyHostToDevice, h->stream));
  return cair_statistics_items_dev(h, nitems, ntot, (const cair_traj_result*)h->d_scratch, params, item_rows, item_ini,
                                   h->stream);
}

int cair_statistics_counts(cair_handle* h, int32_t nitems, const cair_work_item* items, const int32_t* item_run,
                           const uint64_t* item_rows, const int64_t* item_ini, int64_t ntot,
                           const cair_traj_result* results, const cair_stats_params* params, cair_stats_count* out,
                           int64_t cap, int64_t* nout, uint64_t* ring_rows) {
  if (!h || ntot < 0 || (ntot > 0 && !results)) return fail(h, CAIR_EINVAL, "cair_statistics_counts: bad argument");
  if (int e = ensure_scratch(h, (size_t)ntot * sizeof(cair_traj_result) + 256)) return e;
  if (ntot > 0)
    CUDA_TRY(h, cudaMemcpyAsync(h->d_scratch, results, (size_t)ntot * sizeof(cair_traj_result),
                                cudaMemcpyHostToDevice, h->stream));
  return cair_statistics_counts_dev(h, nitems, items, item_run, item_rows, item_ini, ntot,
                                    (const cair_traj_result*)h->d_scratch, params, out, cap, nout, ring_rows,
                                    h->stream);
}

struct cair_queue_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

int cair_queue_graph_create(cair_handle* h, int32_t nlevels, const cair_level* levels, int32_t nitems,
                            const cair_work_item* items, int64_t ntot, int64_t max_attempts,
                            cair_traj_result* results, void* workspace, cair_queue_graph** out) {
  if (!h || !out || !workspace) return fail(h, CAIR_EINVAL, "cair_queue_graph_create: bad argument (workspace required)");
  *out = nullptr;
  cudaStream_t st = nullptr;
  CUDA_TRY(h, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  const bool timing = h->time_integrate;
  h->time_integrate = false;  // event pairs are per call, not per replay
  cudaGraph_t graph = nullptr;
  int rc = 0;
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    rc = fail(h, CAIR_ECUDA, std::string("cudaStreamBeginCapture: ") + cudaGetErrorString(e));
  } else {
    rc = cair_run_queue_dev(h, nlevels, levels, nitems, items, ntot, max_attempts, results, workspace, st);
    e = cudaStreamEndCapture(st, &graph);  // always ends the capture, also after a failed call
    if (rc == 0 && e != cudaSuccess) rc = fail(h, CAIR_ECUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
  }
  h->time_integrate = timing;
  cudaGraphExec_t exec = nullptr;
  if (rc == 0) {
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) rc = fail(h, CAIR_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  }
  cudaStreamDestroy(st);
  if (rc != 0) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return rc;
  }
  *out = new cair_queue_graph{graph, exec};
  return 0;
}

int cair_queue_graph_launch(cair_handle* h, cair_queue_graph* g, void* stream) {
  if (!h || !g || !g->exec) return fail(h, CAIR_EINVAL, "cair_queue_graph_launch: bad argument");
  CUDA_TRY(h, cudaGraphLaunch(g->exec, (cudaStream_t)stream));
  return 0;
}

void cair_queue_graph_destroy(cair_queue_graph* g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
}

int cair_set_integrate_timing(cair_handle* h, int32_t on) {
  if (!h) return CAIR_EINVAL;
  h->time_integrate = on != 0;
  h->ntev = 0;
  return 0;
}

int cair_integrate_timings(cair_handle* h, float* ms, int32_t cap, int32_t* count) {
  if (!h || !count || cap < 0 || (cap > 0 && !ms)) return CAIR_EINVAL;
  const int32_t n = (int32_t)h->ntev;
  for (int32_t k = 0; k < n && k < cap; ++k) {
    CUDA_TRY(h, cudaEventSynchronize(h->tev[2 * k + 1]));
    CUDA_TRY(h, cudaEventElapsedTime(&ms[k], h->tev[2 * k], h->tev[2 * k + 1]));
  }
  *count = n;
  h->ntev = 0;
  return 0;
}

int cair_fp64_peak_probe(cair_handle* h, double* gflops) {
  if (!h || !gflops) return CAIR_EINVAL;
  const int block = 256, grid = h->nsm * 8, iters = 4096;
  double* d = nullptr;
  CUDA_TRY(h, cudaMalloc(&d, sizeof(double) * grid * block));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0, h->stream);
    cair_k_dfma_probe<<<grid, block, 0, h->stream>>>(d, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, h->stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    double gf = 2.0 * 8.0 * iters * (double)grid * block / (ms * 1e-3) / 1e9;
    if (rep > 0 && gf > best) best = gf;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (int e = check_launch(h)) return e;
  *gflops = best;
  return 0;
}

}  // extern "C"


// Internal (not in include/cair_gpu.h): k_ic_draws' stream code and each trajectory's impact
// parameter run on the host, so that tests can check the stream order (level pick, diatom draws,
// the earlier rings' trajectories, a fixed b without a draw) against the oracle without a GPU.
extern "C" int cair_internal_ic_draws(int32_t natoms, int32_t nlevels, const cair_level* levels, int32_t nitems,
                                      const cair_work_item* items, int64_t ntot, double* draws, int32_t* item_of,
                                      double* b) {
  if ((natoms != 3 && natoms != 4) || nlevels < 1 || !levels || nitems < 1 || !items || !draws || !item_of || !b)
    return CAIR_EINVAL;
  int64_t sum = 0;
  for (int i = 0; i < nitems; ++i) {
    const cair_work_item& w = items[i];
    if (w.first != sum || w.ntraj < 0 || w.skip < 0 || w.ilevel < 0 || w.ilevel >= nlevels ||
        (natoms == 4 && (w.ilevel2 < 0 || w.ilevel2 >= nlevels)))
      return CAIR_EINVAL;
    sum += w.ntraj;
  }
  if (sum != ntot) return CAIR_EINVAL;
  const int nmol = natoms == 4 ? 2 : 1;
  for (int i = 0; i < nitems; ++i)
    if (!cair::continues_stream(items, i)) cair::stream_draws(items, nitems, i, nmol, levels, draws, item_of);
  for (int64_t g = 0; g < ntot; ++g)
    b[g] = cair::impact_parameter(items[item_of[g]], draws[cair::kDraws * g + 4 * nmol + 1]);
  return 0;
}

// Internal (not in include/cair_gpu.h): the statistics' per-row device code (stats_counted,
// stats_codes, stats_key, as k_stats_items and k_stats_count run them) on the host, with the rings
// from the host half, so that tests can check each row's codes, ring and key without a GPU.
extern "C" int cair_internal_stats_rows(const cair_stats_params* P, int32_t nitems, const cair_work_item* items,
                                        const int32_t* item_run, const unsigned long long* item_rows,
                                        const long long* item_ini, int64_t n, const cair_traj_result* rows,
                                        int32_t* counted, long long* ic, long long* fc, int32_t* ring,
                                        unsigned long long* key) {
  if (!P || (P->ncond != 3 && P->ncond != 5) || nitems < 1 || !items || n < 0 || (n > 0 && !rows)) return CAIR_EINVAL;
  cair::StatsRuns runs;
  if (!cair::stats_runs(nitems, items, item_run, runs).empty()) return CAIR_EINVAL;
  if (!cair::stats_rings(*P, nitems, items, item_rows, item_ini, runs).empty()) return CAIR_EINVAL;
  int err = 0;
  cair::StatsArgs A{n,
                    rows,
                    P->qn_max,
                    {P->iskip[0], P->iskip[1], P->iskip[2], P->iskip[3], P->iskip[4]},
                    {P->pres_even_odd[0], P->pres_even_odd[1], P->pres_even_odd[2], P->pres_even_odd[3],
                     P->pres_even_odd[4]},
                    P->ham_abs_tol,
                    runs.run_of.data(),
                    runs.ring_b.data(),
                    runs.nring.data(),
                    runs.nruns,
                    runs.R,
                    nullptr,
                    nullptr,
                    0,
                    nullptr,
                    nullptr,
                    nullptr,
                    &err};
  for (int64_t k = 0; k < n; ++k) {
    const cair_traj_result& r = rows[k];
    counted[k] = cair::stats_counted(A, r) ? 1 : 0;
    ic[k] = fc[k] = 0;
    ring[k] = 0;
    key[k] = 0;
    if (!counted[k]) continue;
    bool bad = false;
    if (P->ncond == 3) cair::stats_codes<3>(A, r, ic[k], fc[k], bad);
    else cair::stats_codes<5>(A, r, ic[k], fc[k], bad);
    if (bad) return CAIR_EINVAL;
    int run;
    key[k] = cair::stats_key(A, r, fc[k], run, ring[k]);
  }
  return 0;
}

// Internal (not in include/cair_gpu.h): surface 0 of the handle through the parity build
// (cair_parity.cu: no fused multiply-adds, CUDA's exp, forward-mode PIP gradients) at n points, host
// arrays as cair_pes_eval's.  For tests that separate this library's reordering from the surfaces'
// own conditioning.
extern "C" int cair_internal_pes_eval_parity(cair_handle* h, int64_t n, const double* R, const double* Q, double* V,
                                             double* dVdR, double* dVdQ) {
  if (!h || n < 1 || !R || !Q || !V || !dVdR || !dVdQ) return CAIR_EINVAL;
  const int np = h->sys.npairs, nq = 3 * h->sys.natoms, nv = h->sys.nv;
  if (int e = ensure_scratch(h, (size_t)n * 8 * (2 * np + nq + 1 + nv) + 4096)) return e;
  Carver c{(char*)h->d_scratch};
  double *d_R = c.take<double>(n * np), *d_Q = c.take<double>(n * nq), *d_V = c.take<double>(n),
         *d_g = c.take<double>(n * np), *d_m = c.take<double>(n * nv);
  cudaStream_t st = h->stream;
  CUDA_TRY(h, cudaMemcpyAsync(d_R, R, n * np * 8, cudaMemcpyHostToDevice, st));
  CUDA_TRY(h, cudaMemcpyAsync(d_Q, Q, n * nq * 8, cudaMemcpyHostToDevice, st));
  if (int e = parity_pes_launch(h->sys, grid_for(h, n), st, n, d_R, d_Q, d_V, d_g, d_m)) return fail(h, e, "parity build");
  CUDA_TRY(h, cudaMemcpyAsync(V, d_V, n * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(dVdR, d_g, n * np * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaMemcpyAsync(dVdQ, d_m, n * nv * 8, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(h, cudaStreamSynchronize(st));
  return 0;
}

// Internal (not in include/cair_gpu.h): what cair_create sets up, without a GPU -- the DevSys
// (surface coefficient pointers left null) and every surface's packed device-layout coefficients,
// concatenated, surface p at packed[offsets[p] .. offsets[p + 1]).  For tests that run the device
// surface code on the host.
// Internal: dy/dt, H and 1/R_p of n points y[n][NE] through the warp integrator's lane-parallel
// programs (device pointers; ipes may be null), synchronous on the handle's stream.
extern "C" int cair_internal_warp_eval(cair_handle* h, int64_t n, const int32_t* ipes, const double* y, double* yp,
                                       double* H, double* Ri) {
  if (!h || n < 0 || !y || !yp || !H || !Ri) return CAIR_EINVAL;
  if (n == 0) return 0;
  const int rc = warp_eval_launch(h->nsm, h->stream, h->sys, n, ipes, y, yp, H, Ri);
  if (rc == 2) return fail(h, CAIR_EUNSUPPORTED, "warp programs: not built for this system");
  if (rc) return fail(h, CAIR_ECUDA, std::string("warp programs: ") + cudaGetErrorString(cudaGetLastError()));
  return wait_stream(h);
}

extern "C" int64_t cair_internal_devsys_size(void) { return (int64_t)sizeof(DevSys); }

extern "C" int cair_internal_setup_system(const cair_system_desc* d, void* devsys, int64_t devsys_bytes,
                                          double* packed, int64_t packed_cap, int64_t* offsets, char* err,
                                          int errcap) {
  if (!d || !devsys || devsys_bytes != (int64_t)sizeof(DevSys) || !offsets || d->npes < 1 || d->npes > CAIR_MAX_PES)
    return CAIR_EINVAL;
  DevSys S;
  double tqp[81], tpq[81];
  std::vector<std::vector<double>> pk;
  int code = CAIR_OK;
  const std::string msg = setup_system(d, S, tqp, tpq, pk, code);
  if (!msg.empty()) {
    if (err && errcap > 0) {
      std::strncpy(err, msg.c_str(), (size_t)errcap - 1);
      err[errcap - 1] = 0;
    }
    return code;
  }
  int64_t off = 0;
  for (int p = 0; p < d->npes; ++p) {
    offsets[p] = off;
    if (off + (int64_t)pk[p].size() > packed_cap) return CAIR_EINVAL;
    if (packed) std::memcpy(packed + off, pk[p].data(), pk[p].size() * sizeof(double));
    off += (int64_t)pk[p].size();
  }
  offsets[d->npes] = off;
  std::memcpy(devsys, &S, sizeof S);
  return 0;
}
