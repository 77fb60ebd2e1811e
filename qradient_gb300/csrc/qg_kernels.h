// Launchers of the sweep kernels (qg_sweep.cu), used by the C ABI (qg_capi.cu).
#pragma once
#include <cuda_runtime.h>

#include "qg_internal.cuh"

namespace qg {

// Record a failure message for qg_last_error() and return the status.
int set_last_error(int status, const char* msg);

// Resident CTAs per SM of a sweep kernel with this descriptor's shared memory
// (pipe: the double-buffered forward kernel).
template <typename R>
int sweep_ctas_per_sm(const SweepDesc& d, bool bwd, bool uncompute, bool pipe = false);

// pipe: use the double-buffered forward kernel for sweeps that load their input.
// pdl: launch as a programmatic dependent of the previous launch in the stream,
// which must be a sweep or observable launch (their kernels trigger early and
// wait for the previous grid before touching its outputs).
template <typename R>
cudaError_t launch_sweep_fwd(const SweepDesc& d, const SweepPtrs<R>& p, int grid, cudaStream_t st, bool pipe = false,
                             bool pdl = false);

template <typename R>
cudaError_t launch_sweep_bwd(const SweepDesc& d, const SweepPtrs<R>& p, bool uncompute, int grid, cudaStream_t st,
                             bool pdl = false);

template <typename R>
cudaError_t launch_observable(const ObsDesc& d, const typename C2T<R>::T* psi, typename C2T<R>::T* lam,
                              const int32_t* cost_i, const double* cost_d, double* partials, int G, int grid,
                              cudaStream_t st, bool pdl = false);

template <typename R>
cudaError_t launch_cost_reduce(int n, const typename C2T<R>::T* lam, const typename C2T<R>::T* psi, int start_plus,
                               int cost, double w0, const int32_t* cost_i, const double* cost_d, double* partials,
                               int slot, int G, cudaStream_t st);

cudaError_t launch_finalize(const double* partials, int G, int kind, int n, int nparam, int eslot, int neslots,
                            double* expec, double* grad, cudaStream_t st);

}  // namespace qg
