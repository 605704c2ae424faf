// Host-side launchers of the kernels that are templated on the surface model.  cair_model.cu
// is compiled once per model (CAIR_MODEL_ID) and instantiates ModelLaunch<CAIR_MODEL_ID>, so
// the surfaces build in parallel translation units; cair_api.cu dispatches on the handle's
// model.  Every launcher only enqueues work on `st`; errors surface through cudaGetLastError.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "../../include/cair_gpu.h"

namespace cair {

struct DevSys;
struct IntegrateArgs;

template <int MODEL>
struct ModelLaunch {
  static void pes_eval(bool grad, int grid, cudaStream_t st, const DevSys& S, int64_t n, const int32_t* ipes,
                       const double* R, const double* Q, double* V, double* dVdR, double* dVdQ);
  static void rhs(int grid, cudaStream_t st, const DevSys& S, int64_t n, const int32_t* ipes, const double* y,
                  double* yp);
  static void hamiltonian(int grid, cudaStream_t st, const DevSys& S, int64_t n, const int32_t* ipes,
                          const double* paq, double* H, double* Rpi);
  static void bs_steps(int grid, cudaStream_t st, const DevSys& S, int64_t n, const int32_t* ipes, double* paq,
                       double* t, double* dt, const double* erra, int32_t nattempts);
  static int integrate_blocks_per_sm(int block, int nsteps);
  static void integrate(int grid, int block, cudaStream_t st, const DevSys& S, const IntegrateArgs& A);
  static void sample_ic(int grid, cudaStream_t st, const DevSys& S, int64_t ntot, const cair_work_item* items,
                        const cair_level* levels, const double* draws, const int32_t* item_of, double* paq,
                        double* paq0, double* erra, double* H0, double* b, int32_t* ipes, double* key);
};

// The parity build of the three-atom surfaces (cair_parity.cu, compiled without fused multiply-adds):
// surface 0 of S at n points; 0, CAIR_EUNSUPPORTED for other models, or CAIR_ECUDA.
int parity_pes_launch(const DevSys& S, int grid, cudaStream_t st, int64_t n, const double* R, const double* Q,
                      double* V, double* dVdR, double* dVdQ);

// Surface models with kernels in this library (one cair_model.cu object each)
#define CAIR_FOR_EACH_MODEL(X) \
  X(CAIR_PES_O3_UMN) X(CAIR_PES_N3_UMN) X(CAIR_PES_O4_UMN) X(CAIR_PES_O3_NN) X(CAIR_PES_N4_UMN) X(CAIR_PES_O3_BNN) \
  X(CAIR_PES_N4_PIPNN)

}  // namespace cair
