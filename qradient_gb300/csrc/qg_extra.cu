// Cost tables and the shot sampler.
#include <stdint.h>

#include "qg_extra.h"
#include "qg_philox.cuh"

namespace qg {

// ------------------------------------------------------------ cost tables
//
// Integer diagonal m(x) = sum_k c_k s_k(x) over Z / ZZ terms with integer
// coefficients c_k, s_k(x) = +1 when the term's bits have even parity (z = +1
// for bit 0), state.py:273-292.  For MaxCut every c_k = 1.

__global__ void int_cost_kernel(int n, const __grid_constant__ IntTermList L, int32_t* table) {
  const int64_t N = (int64_t)1 << n;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < N; x += (int64_t)gridDim.x * blockDim.x) {
    int32_t m = 0;
    for (int k = 0; k < L.nterms; ++k) {
      const IntTerm tk = L.t[k];
      int s = (int)((x >> tk.b0) & 1);
      if (tk.b1 >= 0) s ^= (int)((x >> tk.b1) & 1);
      m += s ? -tk.c : tk.c;
    }
    table[x] = m;
  }
}

// Real diagonal C(x) = sum_k w_k s_k(x) for weights without a common integer base.
__global__ void real_cost_kernel(int n, const __grid_constant__ RealTermList L, double* table) {
  const int64_t N = (int64_t)1 << n;
  for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < N; x += (int64_t)gridDim.x * blockDim.x) {
    double c = 0.0;
    for (int k = 0; k < L.nterms; ++k) {
      const RealTerm tk = L.t[k];
      int s = (int)((x >> tk.b0) & 1);
      if (tk.b1 >= 0) s ^= (int)((x >> tk.b1) & 1);
      c += s ? -tk.w : tk.w;
    }
    table[x] = c;
  }
}

cudaError_t launch_int_cost(int n, const IntTermList& terms, int32_t* table, int grid, cudaStream_t st) {
  int_cost_kernel<<<grid, 256, 0, st>>>(n, terms, table);
  return cudaGetLastError();
}

cudaError_t launch_real_cost(int n, const RealTermList& terms, double* table, int grid, cudaStream_t st) {
  real_cost_kernel<<<grid, 256, 0, st>>>(n, terms, table);
  return cudaGetLastError();
}

// ------------------------------------------------------------ sampler
//
// Inverse-CDF sampling of basis states from |psi|^2 (qaoa.py:196-198 draws
// with scipy.stats.rv_discrete).  Chunk sums, one exclusive scan over the
// chunk sums, then one thread per shot: binary search over the chunks and a
// linear walk inside the chunk.  Uniforms come from Philox4x32-10 (Salmon,
// Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11),
// counter = shot index + offset, key = seed.

template <typename C>
__global__ void chunk_sum_kernel(const C* psi, int64_t N, double* sums) {
  __shared__ double red[32];
  const int64_t b0 = (int64_t)blockIdx.x * SAMPLE_CHUNK;
  double acc = 0.0;
  for (int i = threadIdx.x; i < SAMPLE_CHUNK; i += blockDim.x) {
    const int64_t x = b0 + i;
    if (x < N) {
      const C v = psi[x];
      acc = fma((double)v.x, (double)v.x, fma((double)v.y, (double)v.y, acc));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    sums[blockIdx.x] = s;
  }
}

// Exclusive scan of nb chunk sums by one block (sequential per thread
// segment, then a scan of segment totals); prefix[nb] = total.
__global__ void scan_kernel(const double* sums, int64_t nb, double* prefix) {
  __shared__ double seg[1024];
  const int T = blockDim.x;
  const int64_t per = (nb + T - 1) / T;
  const int64_t lo = threadIdx.x * per, hi = lo + per < nb ? lo + per : nb;
  double s = 0.0;
  for (int64_t i = lo; i < hi; ++i) s += sums[i];
  seg[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double run = 0.0;
    for (int i = 0; i < T; ++i) {
      const double v = seg[i];
      seg[i] = run;
      run += v;
    }
    prefix[nb] = run;
  }
  __syncthreads();
  double run = seg[threadIdx.x];
  for (int64_t i = lo; i < hi; ++i) {
    prefix[i] = run;
    run += sums[i];
  }
}

template <typename C>
__global__ void draw_kernel(const C* psi, int64_t N, const double* prefix, int64_t nb, int64_t nshots, uint64_t seed,
                            uint64_t offset, int64_t* out) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nshots) return;
  const uint64_t ctr = (uint64_t)s + offset;
  uint32_t c[4] = {(uint32_t)ctr, (uint32_t)(ctr >> 32), 0u, 0u};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const double total = prefix[nb];
  const double u = u01_from(c[0], c[1]) * total;
  // last chunk with prefix <= u
  int64_t lo = 0, hi = nb - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= u)
      lo = mid;
    else
      hi = mid - 1;
  }
  // skip empty chunks at the end of the range (rounding)
  while (lo > 0 && prefix[lo + 1] - prefix[lo] <= 0.0) --lo;
  double run = prefix[lo];
  const int64_t x0 = lo * SAMPLE_CHUNK;
  int64_t pick = -1, last_nz = -1;
  for (int64_t i = 0; i < SAMPLE_CHUNK && x0 + i < N; ++i) {
    const C v = psi[x0 + i];
    const double pr = fma((double)v.x, (double)v.x, (double)v.y * (double)v.y);
    if (pr > 0.0) last_nz = x0 + i;
    run += pr;
    if (run > u && pr > 0.0) {
      pick = x0 + i;
      break;
    }
  }
  out[s] = pick >= 0 ? pick : (last_nz >= 0 ? last_nz : x0);
}

template <typename C>
cudaError_t launch_sample(int n, const C* psi, int64_t nshots, uint64_t seed, uint64_t offset, double* ws,
                          int64_t* out, cudaStream_t st) {
  const int64_t N = (int64_t)1 << n;
  const int64_t nb = (N + SAMPLE_CHUNK - 1) / SAMPLE_CHUNK;
  double* sums = ws;
  double* prefix = ws + nb;
  chunk_sum_kernel<C><<<(unsigned)nb, 256, 0, st>>>(psi, N, sums);
  scan_kernel<<<1, 1024, 0, st>>>(sums, nb, prefix);
  if (nshots > 0)
    draw_kernel<C><<<(unsigned)((nshots + 127) / 128), 128, 0, st>>>(psi, N, prefix, nb, nshots, seed, offset, out);
  return cudaGetLastError();
}

template cudaError_t launch_sample<double2>(int, const double2*, int64_t, uint64_t, uint64_t, double*, int64_t*,
                                            cudaStream_t);
template cudaError_t launch_sample<float2>(int, const float2*, int64_t, uint64_t, uint64_t, double*, int64_t*,
                                           cudaStream_t);

}  // namespace qg
