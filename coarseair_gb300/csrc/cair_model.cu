// Kernels of one surface model (CAIR_MODEL_ID, set by the build), instantiated behind the
// launchers declared in cair_launch.h.
#ifndef CAIR_MODEL_ID
#error "compile with -DCAIR_MODEL_ID=<surface model>"
#endif
#define CAIR_MODEL_TU
#include "cair_ic.cuh"
#include "cair_launch.h"

namespace cair {

template <int MODEL>
void ModelLaunch<MODEL>::pes_eval(bool grad, int grid, cudaStream_t st, const DevSys& S, int64_t n,
                                  const int32_t* ipes, const double* R, const double* Q, double* V, double* dVdR,
                                  double* dVdQ) {
  if (grad) k_pes_eval<MODEL, true><<<grid, 128, 0, st>>>(S, n, ipes, R, Q, V, dVdR, dVdQ);
  else k_pes_eval<MODEL, false><<<grid, 128, 0, st>>>(S, n, ipes, R, Q, V, dVdR, dVdQ);
}

template <int MODEL>
void ModelLaunch<MODEL>::rhs(int grid, cudaStream_t st, const DevSys& S, int64_t n, const int32_t* ipes,
                             const double* y, double* yp) {
  k_rhs<MODEL><<<grid, 128, 0, st>>>(S, n, ipes, y, yp);
}

template <int MODEL>
void ModelLaunch<MODEL>::hamiltonian(int grid, cudaStream_t st, const DevSys& S, int64_t n, const int32_t* ipes,
                                     const double* paq, double* H, double* Rpi) {
  k_hamiltonian<MODEL><<<grid, 128, 0, st>>>(S, n, ipes, paq, H, Rpi);
}

// NSteps ("Nb of extrapolation steps") 2..4 are built for the three-atom surfaces; the four-atom
// surfaces, whose integrator kernels are the largest to compile, have NSteps = 3 only
// (cair_create refuses the others for them).
template <int MODEL>
constexpr bool kAllNSteps = Traits<MODEL>::NA == 3;

template <int MODEL>
void ModelLaunch<MODEL>::bs_steps(int grid, cudaStream_t st, const DevSys& S, int64_t n, const int32_t* ipes,
                                  double* paq, double* t, double* dt, const double* erra, int32_t nattempts) {
  if constexpr (kAllNSteps<MODEL>) {
    if (S.nsteps == 2) return (void)(k_bs_steps<MODEL, 2><<<grid, 128, 0, st>>>(S, n, ipes, paq, t, dt, erra, nattempts));
    if (S.nsteps == 4) return (void)(k_bs_steps<MODEL, 4><<<grid, 128, 0, st>>>(S, n, ipes, paq, t, dt, erra, nattempts));
  }
  k_bs_steps<MODEL, 3><<<grid, 128, 0, st>>>(S, n, ipes, paq, t, dt, erra, nattempts);
}

template <int MODEL>
int ModelLaunch<MODEL>::integrate_blocks_per_sm(int block, int nsteps) {
  int per_sm = 0;
  if constexpr (kAllNSteps<MODEL>) {
    if (nsteps == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_integrate<MODEL, 2>, block, 0);
    else if (nsteps == 4) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_integrate<MODEL, 4>, block, 0);
    if (nsteps != 3) return per_sm;
  }
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_integrate<MODEL, 3>, block, 0);
  return per_sm;
}

template <int MODEL>
void ModelLaunch<MODEL>::integrate(int grid, int block, cudaStream_t st, const DevSys& S, const IntegrateArgs& A) {
  if constexpr (kAllNSteps<MODEL>) {
    if (S.nsteps == 2) return (void)(k_integrate<MODEL, 2><<<grid, block, 0, st>>>(S, A));
    if (S.nsteps == 4) return (void)(k_integrate<MODEL, 4><<<grid, block, 0, st>>>(S, A));
  }
  k_integrate<MODEL, 3><<<grid, block, 0, st>>>(S, A);
}

template <int MODEL>
void ModelLaunch<MODEL>::sample_ic(int grid, cudaStream_t st, const DevSys& S, int64_t ntot,
                                   const cair_work_item* items, const cair_level* levels, const double* draws,
                                   const int32_t* item_of, double* paq, double* paq0, double* erra, double* H0,
                                   double* b, int32_t* ipes, double* key) {
  if constexpr (Traits<MODEL>::NA == 3)
    k_sample_ic3<MODEL><<<grid, 128, 0, st>>>(S, ntot, items, levels, draws, item_of, paq, paq0, erra, H0, b, ipes,
                                              key);
  else
    k_sample_ic4<MODEL><<<grid, 128, 0, st>>>(S, ntot, items, levels, draws, item_of, paq, paq0, erra, H0, b, ipes,
                                              key);
}

template struct ModelLaunch<CAIR_MODEL_ID>;

}  // namespace cair
