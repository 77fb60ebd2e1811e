// Batched persistent kernel (qg_batched.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qgrad.h"
#include "qg_extra.h"

namespace qg {

using BatchJob = qg_batch_job;
using BatchTerm = qg_term;

// threads per CTA: 512 (16 warps).  Measured with 1024 (complex64: 64
// registers a thread, 240 bytes spilled) the n = 14 jobs ran at 60.4k against
// 82.9k circuits/s, the n = 12 ones at 279k against 397k.
constexpr int BATCH_THREADS = 512;
constexpr int BATCH_TABLE = 1024;   // phase-table entries (Z rotations or the QAOA cost)

template <typename R>
struct BatchC;
template <>
struct BatchC<double> {
  using T = double2;
  static constexpr int EPT = 8;     // 2^12 / 512 amplitudes per thread (single CTA)
  static constexpr int MMAX = 12;
};
template <>
struct BatchC<float> {
  using T = float2;
  static constexpr int EPT = 16;    // 2^13 / 512
  static constexpr int MMAX = 13;
};

cudaError_t launch_batched(int dtype_double, int cluster, const BatchJob* jobs, int njobs, int* counter, int mmax,
                           cudaStream_t st, int* grid_out);

}  // namespace qg
