// Cost tables and the sampler (qg_extra.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace qg {

constexpr int SAMPLE_CHUNK = 4096;

struct IntTerm {
  int32_t b0, b1;  // bit positions (b1 < 0 for a Z term)
  int32_t c;       // integer coefficient
  int32_t pad;
};

struct RealTerm {
  int32_t b0, b1;
  double w;
};

// Term lists travel as kernel parameters (no device allocation).
constexpr int MAX_COST_TERMS = 600;
struct IntTermList {
  int32_t nterms;
  int32_t pad;
  IntTerm t[MAX_COST_TERMS];
};
struct RealTermList {
  int32_t nterms;
  int32_t pad;
  RealTerm t[MAX_COST_TERMS];
};

cudaError_t launch_int_cost(int n, const IntTermList& terms, int32_t* table, int grid, cudaStream_t st);
cudaError_t launch_real_cost(int n, const RealTermList& terms, double* table, int grid, cudaStream_t st);

template <typename C>
cudaError_t launch_sample(int n, const C* psi, int64_t nshots, uint64_t seed, uint64_t offset, double* ws,
                          int64_t* out, cudaStream_t st);

}  // namespace qg
