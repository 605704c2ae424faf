// Launchers of the surrogate translation unit (cair_sur.cu) called from the API translation unit.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/cair_gpu.h"

namespace cair {

struct DevSys;
struct IntegrateArgs;

// The persistent surrogate integrator on `st` (N3 UMN, NSteps = 3); 0 or CAIR_ECUDA.
int sur_integrate_launch(cair_surrogate* s, int nsm, cudaStream_t st, const DevSys& S, const IntegrateArgs& A);
// Training targets from the FP64 N3 surface S; 0 or CAIR_ECUDA.
int sur_targets_launch(const DevSys& S, int nsm, cudaStream_t st, int64_t n, const double* R, cair_sur_sample* out);
const char* sur_last_error(const cair_surrogate* s);

}  // namespace cair
