// Kernels of the density-matrix noise (add_onedot_noise / add_twodot_noise,
// density.C:92-421): random wavefunctions from the shared counter-based
// generator, per-range norms and normalisation, and the trace-scaled update
// of the density matrix.  Every reduction has a fixed order.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace bgpu {
namespace dev {

// x[e] = noise_uniform(seed, quantum, e) for e < n
cudaError_t launch_noise_fill(double* x, int64_t n, uint64_t seed, int quantum, cudaStream_t s);
// out[r] = sum of x[e]^2 over e in [ranges[r].x, ranges[r].y)
cudaError_t launch_range_norm2(const double* x, const longlong2* ranges, int nranges, double* out, cudaStream_t s);
// x[e] *= 1 / sqrt(nrm[r]) over range r (0 when nrm[r] <= 1e-15)
cudaError_t launch_range_normalise(double* x, const longlong2* ranges, int nranges, const double* nrm, cudaStream_t s);
// *out = sum over sectors of the trace of the n_q x n_q blocks at off[q]
cudaError_t launch_block_trace(const double* m, const int64_t* off, const int* dims, int nq, double* out,
                               cudaStream_t s);
// rho += amp / *tr * N when *tr > 1 (n elements)
cudaError_t launch_noise_update(double* rho, const double* N, int64_t n, const double* tr, double amp, cudaStream_t s);

}  // namespace dev
}  // namespace bgpu
