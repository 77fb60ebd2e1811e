// Optimiser steps on the device: the parameter updates of
// qradient/optimization.py, run next to grad_run so that a training loop
// keeps parameters, gradients, moments and histories in HBM.
//
// Every update is written with explicitly rounded operations (__dmul_rn,
// __dadd_rn, ...), which the compiler never contracts into fused
// multiply-adds.  Each operation is therefore the single IEEE-754 double
// operation numpy performs for the same Python expression, in the same
// order, and the updated parameters are bit-identical to the reference's for
// the same gradients.  sqrt and division are IEEE round-to-nearest in CUDA.
#include <cuda_runtime.h>

#include <math.h>

#include "../../include/qgrad.h"
#include "qg_kernels.h"

namespace {

constexpr int kThreads = 256;

int grid_for(int np) { return (np + kThreads - 1) / kThreads; }

// Adam (optimization.py:161-167).  c1 = 1 - beta1**iter and
// c2 = 1 - beta2**iter are computed on the host with the C library's pow,
// as Python's float ** does.
__global__ void adam_kernel(double* __restrict__ p, const double* __restrict__ g, double* __restrict__ m,
                            double* __restrict__ v, int np, double lr, double b1, double omb1, double b2,
                            double omb2, double eps, double c1, double c2, double* __restrict__ hist) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const double gi = g[i];
  // m = beta1 * m + (1 - beta1) * gradient
  const double mi = __dadd_rn(__dmul_rn(b1, m[i]), __dmul_rn(omb1, gi));
  // v = beta2 * v + (1 - beta2) * gradient**2   (numpy squares by one multiply)
  const double vi = __dadd_rn(__dmul_rn(b2, v[i]), __dmul_rn(omb2, __dmul_rn(gi, gi)));
  m[i] = mi;
  v[i] = vi;
  const double mh = __ddiv_rn(mi, c1);
  const double vh = __ddiv_rn(vi, c2);
  // parameters -= step_size * m_hat / (sqrt(v_hat) + eps)
  const double upd = __ddiv_rn(__dmul_rn(lr, mh), __dadd_rn(__dsqrt_rn(vh), eps));
  const double pi = __dsub_rn(p[i], upd);
  p[i] = pi;
  if (hist) hist[i] = pi;
}

// GradientDescent and the update of RateDecayOnPlateau
// (optimization.py:175, :194): parameters -= step_size * gradient.
__global__ void gd_kernel(double* __restrict__ p, const double* __restrict__ g, int np, double lr,
                          double* __restrict__ hist) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const double pi = __dsub_rn(p[i], __dmul_rn(lr, g[i]));
  p[i] = pi;
  if (hist) hist[i] = pi;
}

// RateDecayOnPlateau (optimization.py:184-194) with its state on the device:
// state[0] best cost, state[1] plateau counter, state[2] step size.  The new
// cost is read from device memory (the expectation value grad_run wrote), so
// no value returns to the host.  One block: thread 0 updates the state, then
// the block applies the step size to every parameter.
__global__ void plateau_kernel(double* __restrict__ p, const double* __restrict__ g, int np,
                               const double* __restrict__ new_cost, double* __restrict__ state, double plateau_length,
                               double decay_rate, double* __restrict__ hist) {
  __shared__ double lr;
  if (threadIdx.x == 0) {
    const double c = *new_cost;
    double best = state[0], counter = state[1], step = state[2];
    if (c > best) {  // false for NaN, as in Python
      counter = counter + 1.0;
      if (counter >= plateau_length) {
        step = __dmul_rn(step, decay_rate);
        counter = 0.0;
      }
    } else {
      best = c;
      counter = 0.0;
    }
    state[0] = best;
    state[1] = counter;
    state[2] = step;
    lr = step;
  }
  __syncthreads();
  const double s = lr;
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const double pi = __dsub_rn(p[i], __dmul_rn(s, g[i]));
    p[i] = pi;
    if (hist) hist[i] = pi;
  }
}

int cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return QG_OK;
  return qg::set_last_error(QG_ERR_CUDA, what);
}

}  // namespace

extern "C" int qg_adam_step(double* p, const double* g, double* m, double* v, int np, int iter, double lr, double b1,
                            double b2, double eps, double* hist, qg_stream stream) {
  if (np < 0 || iter < 1) return qg::set_last_error(QG_ERR_INVALID, "qg_adam_step: nparams < 0 or iter < 1");
  if (np == 0) return QG_OK;
  if (!p || !g || !m || !v) return qg::set_last_error(QG_ERR_INVALID, "qg_adam_step: null array");
  const double c1 = 1.0 - pow(b1, (double)iter);
  const double c2 = 1.0 - pow(b2, (double)iter);
  adam_kernel<<<grid_for(np), kThreads, 0, (cudaStream_t)stream>>>(p, g, m, v, np, lr, b1, 1.0 - b1, b2, 1.0 - b2,
                                                                     eps, c1, c2, hist);
  return cuda_status(cudaGetLastError(), "qg_adam_step: launch failed");
}

extern "C" int qg_gd_step(double* p, const double* g, int np, double lr, double* hist, qg_stream stream) {
  if (np < 0) return qg::set_last_error(QG_ERR_INVALID, "qg_gd_step: nparams < 0");
  if (np == 0) return QG_OK;
  if (!p || !g) return qg::set_last_error(QG_ERR_INVALID, "qg_gd_step: null array");
  gd_kernel<<<grid_for(np), kThreads, 0, (cudaStream_t)stream>>>(p, g, np, lr, hist);
  return cuda_status(cudaGetLastError(), "qg_gd_step: launch failed");
}

extern "C" int qg_plateau_step(double* p, const double* g, int np, const double* new_cost, double* state,
                               int plateau_length, double decay_rate, double* hist, qg_stream stream) {
  if (np < 0) return qg::set_last_error(QG_ERR_INVALID, "qg_plateau_step: nparams < 0");
  if (!p || !g || !new_cost || !state) return qg::set_last_error(QG_ERR_INVALID, "qg_plateau_step: null array");
  plateau_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(p, g, np, new_cost, state, (double)plateau_length,
                                                       decay_rate, hist);
  return cuda_status(cudaGetLastError(), "qg_plateau_step: launch failed");
}
