// Host launchers of the warp integrator (cair_warp.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace cair {
struct DevSys;
struct IntegrateArgs;

// True when every surface of the system has lane-parallel programs (the O3, N3, O4 and N4 UMN
// surfaces with their own diatomic, one model per system) and NSteps is 2..4.
bool warp_integrate_supported(const DevSys& S);
// The persistent warp integrator over A's queue: nsm x (resident CTAs per SM, capped by per_sm_cap
// when > 0) CTAs of 4 warps (diatom + atom) or of as many as shared memory holds, up to 8 (diatom + diatom).  A's warp timeline records only when warp_times_cap holds
// every warp of the launch; *nwarps receives the warps that record (0 when none).  0 on success, 2
// when unsupported, 1 on a launch error.
int warp_integrate_launch(int nsm, int per_sm_cap, cudaStream_t st, const DevSys& S, const IntegrateArgs& A,
                          int64_t warp_times_cap, int64_t* nwarps);
// dy/dt, H and 1/R_p of n points through the same programs (device pointers).
int warp_eval_launch(int nsm, cudaStream_t st, const DevSys& S, int64_t n, const int32_t* ipes, const double* y,
                     double* yp, double* H, double* Ri);
// Warps the warp integrator keeps resident on the GPU (0 when unsupported).
int64_t warp_resident_warps(int nsm, const DevSys& S);
}  // namespace cair
