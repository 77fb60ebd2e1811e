// Per-term Pauli expectations and projector shots: the finite-shot estimator
// of qradient (Observable.load_projectors, observable.py:82-104, and
// ParametrizedCircuit.sample_expec_val / sample_component_expec_val,
// base.py:22-46).
//
// For a Pauli term P with eigenvalues +-1, the reference's projector onto the
// +1 eigenspace (Projector, observable.py:126-177) gives
// p = ||Pi_+ psi||^2 = (1 + <P>) / 2; each shot is +w with probability p and
// -w otherwise, and the estimate is the shot mean, summed over the terms.
// Here <P> comes from one reduction over the state per term (deterministic:
// fixed-order block partials), and the shots from Philox4x32-10.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qgrad.h"
#include "qg_kernels.h"
#include "qg_philox.cuh"
#include "qg_shots.h"

namespace qg {

namespace {

constexpr int kThreads = 256;

template <typename C>
__device__ __forceinline__ void load2(const C* p, int64_t i, double& re, double& im) {
  const C v = p[i];
  re = (double)v.x;
  im = (double)v.y;
}

__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  __syncthreads();
  return s;
}

// partials[k * G + block] for the terms of one chunk (k relative to the chunk)
template <typename C>
__global__ void __launch_bounds__(kThreads) pauli_expect_kernel(const C* __restrict__ psi, int n,
                                                                const PauliChunk chunk, double* __restrict__ partials,
                                                                int G) {
  __shared__ double red[kThreads / 32];
  const int64_t N = (int64_t)1 << n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int k = 0; k < chunk.count; ++k) {
    const PauliTerm tm = chunk.term[k];
    double acc = 0.0;
    if (tm.kind == QG_PAULI_Z || tm.kind == QG_PAULI_ZZ) {
      // sum_x |psi_x|^2 s(x), s = -1 on odd parity of the term's bits
      const int64_t mask = ((int64_t)1 << tm.b0) | (tm.kind == QG_PAULI_ZZ ? ((int64_t)1 << tm.b1) : 0);
      for (int64_t x = t0; x < N; x += stride) {
        double re, im;
        load2(psi, x, re, im);
        const double pr = fma(re, re, im * im);
        acc += (__popcll(x & mask) & 1) ? -pr : pr;
      }
    } else {
      // 2 Re / 2 Im of sum over pairs (x0 with bit b clear, x1 = x0 | bit b)
      // of conj(psi_x0) psi_x1: <X> and <Y>
      const int b = tm.b0;
      const int64_t lo = ((int64_t)1 << b) - 1;
      for (int64_t i = t0; i < N / 2; i += stride) {
        const int64_t x0 = ((i & ~lo) << 1) | (i & lo);
        double r0, i0, r1, i1;
        load2(psi, x0, r0, i0);
        load2(psi, x0 | ((int64_t)1 << b), r1, i1);
        acc += tm.kind == QG_PAULI_X ? fma(r0, r1, i0 * i1) : fma(r0, i1, -i0 * r1);
      }
      acc *= 2.0;
    }
    const double s = block_sum(acc, red);
    if (threadIdx.x == 0) partials[(int64_t)k * G + blockIdx.x] = s;
  }
}

// out[k] = sum over blocks of partials[k][.], in block order
__global__ void pauli_finalize_kernel(const double* __restrict__ partials, int G, int count, double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  double s = 0.0;
  for (int g = 0; g < G; ++g) s += partials[(int64_t)k * G + g];
  out[k] = s;
}

// One block per row: thread j handles terms j, j + blockDim.x, ...  Shot s
// of term k in row r uses Philox counter {ctr, ctr >> 32, s / 2, 0} with
// ctr = offset + r * nterms + k, and uniform (s & 1) of that call.
__global__ void projector_shots_kernel(int nterms, const double* __restrict__ expec,
                                       const double* __restrict__ weights, int shots, uint64_t seed, uint64_t offset,
                                       double* __restrict__ term_est, double* __restrict__ total) {
  __shared__ double contrib[1024];
  const int r = blockIdx.x;
  for (int k = threadIdx.x; k < nterms; k += blockDim.x) {
    const double e = expec[(int64_t)r * nterms + k];
    double p = 0.5 * (1.0 + e);
    p = p < 0.0 ? 0.0 : (p > 1.0 ? 1.0 : p);
    const uint64_t ctr = offset + (uint64_t)r * (uint64_t)nterms + (uint64_t)k;
    int plus = 0;
    for (int s = 0; s < shots; s += 2) {
      uint32_t c[4] = {(uint32_t)ctr, (uint32_t)(ctr >> 32), (uint32_t)(s >> 1), 0u};
      philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
      plus += u01_from(c[0], c[1]) < p;
      if (s + 1 < shots) plus += u01_from(c[2], c[3]) < p;
    }
    const double w = weights[k];
    // mean of `plus` samples of +w and (shots - plus) of -w
    const double est = w * (double)(2 * plus - shots) / (double)shots;
    if (term_est) term_est[(int64_t)r * nterms + k] = est;
    if (k < 1024) contrib[k] = est;
  }
  __syncthreads();
  if (threadIdx.x == 0 && total) {
    double s = 0.0;
    for (int k = 0; k < nterms && k < 1024; ++k) s += contrib[k];
    total[r] = s;
  }
}

}  // namespace

size_t pauli_workspace_bytes(int nterms) { return (size_t)(nterms > 0 ? nterms : 1) * PAULI_BLOCKS * sizeof(double); }

template <typename C>
cudaError_t launch_pauli_expectations(int n, const C* psi, int nterms, const PauliTerm* terms, double* ws,
                                      double* out, cudaStream_t st) {
  const int64_t N = (int64_t)1 << n;
  int G = (int)((N / 2 + kThreads - 1) / kThreads);
  G = G < 1 ? 1 : (G > PAULI_BLOCKS ? PAULI_BLOCKS : G);
  for (int k0 = 0; k0 < nterms; k0 += PAULI_CHUNK) {
    PauliChunk ch;
    ch.count = nterms - k0 < PAULI_CHUNK ? nterms - k0 : PAULI_CHUNK;
    for (int k = 0; k < ch.count; ++k) ch.term[k] = terms[k0 + k];
    pauli_expect_kernel<C><<<G, kThreads, 0, st>>>(psi, n, ch, ws, G);
    pauli_finalize_kernel<<<(ch.count + 127) / 128, 128, 0, st>>>(ws, G, ch.count, out + k0);
  }
  return cudaGetLastError();
}

template cudaError_t launch_pauli_expectations<double2>(int, const double2*, int, const PauliTerm*, double*, double*,
                                                        cudaStream_t);
template cudaError_t launch_pauli_expectations<float2>(int, const float2*, int, const PauliTerm*, double*, double*,
                                                       cudaStream_t);

}  // namespace qg

extern "C" int qg_projector_shots(int nrows, int nterms, const double* expec_dev, const double* weights_dev,
                                  int shots, uint64_t seed, uint64_t offset, double* term_est_dev, double* total_dev,
                                  qg_stream stream) {
  if (nrows < 0 || nterms < 0) return qg::set_last_error(QG_ERR_INVALID, "qg_projector_shots: negative size");
  if (nterms > 1024) return qg::set_last_error(QG_ERR_UNSUPPORTED, "qg_projector_shots: more than 1024 terms");
  if (shots < 1) return qg::set_last_error(QG_ERR_INVALID, "qg_projector_shots: shot_num must be at least 1");
  if (nrows == 0) return QG_OK;
  if ((nterms > 0 && (!expec_dev || !weights_dev)) || (!term_est_dev && !total_dev))
    return qg::set_last_error(QG_ERR_INVALID, "qg_projector_shots: null array");
  qg::projector_shots_kernel<<<nrows, 256, 0, (cudaStream_t)stream>>>(nterms, expec_dev, weights_dev, shots, seed,
                                                                      offset, term_est_dev, total_dev);
  if (cudaGetLastError() != cudaSuccess)
    return qg::set_last_error(QG_ERR_CUDA, "qg_projector_shots: launch failed");
  return QG_OK;
}
