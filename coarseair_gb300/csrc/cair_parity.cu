// Parity build of the surface evaluation (built with -fmad=false): the three-atom surfaces evaluated
// with the reference's order of operations where this library departs from it for speed -- no
// fused multiply-adds, CUDA's exp instead of the table-driven fexp, the forward-mode PIP gradient
// (EvdMdR / EvdPdr order) instead of the adjoint sweep.  Tests compare it with the production
// kernels against the oracle: what the parity build still misses at 1e-12 is the surfaces' own
// conditioning, not this library's reordering.
#define CAIR_MODEL_TU
#define CAIR_PARITY_MATH
#define CAIR_PIP_FORWARD
#include "cair_kernels.cuh"
#include "cair_launch.h"

namespace cair {

template <int MODEL>
__global__ void __launch_bounds__(128) k_pes_parity(DevSys S, int64_t n, const double* __restrict__ Rin,
                                                    const double* __restrict__ Qin, double* __restrict__ V,
                                                    double* __restrict__ dVdR, double* __restrict__ dVdQ) {
  using T = Traits<MODEL>;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const DevPes& P = S.pes[0];
    double R[T::NP], Ri[T::NP], Q[3 * T::NA], v, g[T::NP], m[T::NV];
#pragma unroll
    for (int i = 0; i < T::NP; ++i) {
      R[i] = Rin[T::NP * k + i];
      Ri[i] = 1.0 / R[i];
    }
#pragma unroll
    for (int i = 0; i < 3 * T::NA; ++i) Q[i] = Qin[3 * T::NA * k + i];
    pes<MODEL, true>(S, P, R, Ri, Q, v, g, m);
    V[k] = v;
#pragma unroll
    for (int i = 0; i < T::NP; ++i) dVdR[T::NP * k + i] = g[i];
#pragma unroll
    for (int i = 0; i < T::NV; ++i) dVdQ[T::NV * k + i] = m[i];
  }
}

int parity_pes_launch(const DevSys& S, int grid, cudaStream_t st, int64_t n, const double* R, const double* Q,
                      double* V, double* dVdR, double* dVdQ) {
  switch (S.pes[0].model) {
    case CAIR_PES_O3_UMN: k_pes_parity<CAIR_PES_O3_UMN><<<grid, 128, 0, st>>>(S, n, R, Q, V, dVdR, dVdQ); break;
    case CAIR_PES_N3_UMN: k_pes_parity<CAIR_PES_N3_UMN><<<grid, 128, 0, st>>>(S, n, R, Q, V, dVdR, dVdQ); break;
    case CAIR_PES_O3_NN: k_pes_parity<CAIR_PES_O3_NN><<<grid, 128, 0, st>>>(S, n, R, Q, V, dVdR, dVdQ); break;
    case CAIR_PES_O3_BNN: k_pes_parity<CAIR_PES_O3_BNN><<<grid, 128, 0, st>>>(S, n, R, Q, V, dVdR, dVdQ); break;
    default: return CAIR_EUNSUPPORTED;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : CAIR_ECUDA;
}

}  // namespace cair
