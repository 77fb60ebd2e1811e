// Batched persistent kernel: many small circuits (different parameters,
// qubit counts, depths, McClean or QAOA) in one launch.
//
// Each job is a whole run or adjoint grad_run (mc_clean.py:27-78,
// qaoa.py:23-70) executed with psi and lambda resident in shared memory:
// no state ever goes to HBM.  A CTA holds the whole state when it fits
// (complex64 n <= 13, complex128 n <= 12); a 2-CTA cluster holds one state
// split by its top bit (qubit 0) at the next size (complex64 n = 14,
// complex128 n = 13) and a 4-CTA cluster, split by its top two bits, at the
// one after (complex64 n = 15, complex128 n = 14).  The only cross-CTA
// operations (rotations, reductions and X/Y observable terms on the split
// qubits) read the partner CTA's shared memory (distributed shared memory)
// between cluster barriers.  The CNOT ladder never targets qubit 0; its
// CNOT(0, 1) permutes the 4-CTA blocks, which the CTAs follow by relabelling.
//
// Clusters (or CTAs) take jobs from a device counter until the queue is
// empty (persistent grid, one launch per precision and cluster size; the
// launch is CUDA-graph capturable).  The gradient uses the uncompute form of
// the adjoint sweep (psi is rotated back instead of read from a history).
#include <cooperative_groups.h>
#include <stdint.h>

#include "qg_batched.h"

namespace cg = cooperative_groups;

namespace qg {

namespace {

constexpr int BZMAX = 10;     // Z rotations merged per table (2^BZMAX = BATCH_TABLE entries)
constexpr int BMAXQ = 26;
constexpr int BTERMS = 64;    // observable weights staged in shared memory

__device__ __forceinline__ double2 cmulb(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cmulb(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 tocf(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ double2 tocf(double x, double y) { return make_double2(x, y); }
__device__ __forceinline__ void sincosT(double a, double* s, double* c) { sincos(a, s, c); }
__device__ __forceinline__ void sincosT(float a, float* s, float* c) { sincosf(a, s, c); }

// XOR swizzle of the low index bits with the next ones: 8 (complex128) or 16
// (complex64) amplitudes per 128-byte row, so tasks that stride over the low
// bits still spread over all banks
__device__ __forceinline__ int swb(int e, bool dbl) { return dbl ? e ^ ((e >> 3) & 7) : e ^ ((e >> 4) & 15); }
__device__ __forceinline__ int ins0(int p, int j) { return ((p >> j) << (j + 1)) | (p & ((1 << j) - 1)); }

// index arithmetic of the batched kernel is 32-bit: its jobs have at most 26
// qubits.  The periodic ladder adds CNOT(n-1, 0) to the odd pairs: bit n-1
// flips when bit 0 is set (wrap = 1, wshift = n - 1; wrap = 0 for the open
// ladder).  It targets the top bit, so periodic jobs run in one CTA only.
__device__ __forceinline__ uint32_t lad_fwd(uint32_t x, uint32_t odd, uint32_t even, uint32_t wrap, int wshift) {
  x ^= ((x & odd) >> 1) ^ ((x & wrap) << wshift);
  x ^= (x & even) >> 1;
  return x;
}
__device__ __forceinline__ uint32_t lad_inv(uint32_t x, uint32_t odd, uint32_t even, uint32_t wrap, int wshift) {
  x ^= (x & even) >> 1;
  x ^= ((x & odd) >> 1) ^ ((x & wrap) << wshift);
  return x;
}

// Scaled form of a rotation by theta, in the precision T of the job's
// coefficients (double for complex128, float for complex64: a double
// instruction holds the FP64 pipe for 16 cycles per warp).
template <typename T>
__device__ __forceinline__ T rform(T theta, int* form, T* kappa) {
  T s, c;
  sincosT((T)0.5 * theta, &s, &c);
  if (fabs(c) >= fabs(s)) {
    *form = 0;
    *kappa = c;
    return s / c;
  }
  *form = 1;
  *kappa = s;
  return c / s;
}

// scaled-form rotation of the pair (a: bit 0, b: bit 1); SG = +1 / -1 at compile time
template <int SG, typename C, typename R>
__device__ __forceinline__ void rotp(C& a, C& b, int axis, int form, R u) {
  const C a0 = a, b0 = b;
  const R s1 = SG > 0 ? (R)1 : (R)-1;
  if (axis == 0) {
    if (form == 0) {
      const R us = SG > 0 ? u : -u;
      a.x = fma(us, b0.y, a0.x);
      a.y = fma(-us, b0.x, a0.y);
      b.x = fma(us, a0.y, b0.x);
      b.y = fma(-us, a0.x, b0.y);
    } else {
      a.x = fma(u, a0.x, SG > 0 ? b0.y : -b0.y);
      a.y = fma(u, a0.y, SG > 0 ? -b0.x : b0.x);
      b.x = fma(u, b0.x, SG > 0 ? a0.y : -a0.y);
      b.y = fma(u, b0.y, SG > 0 ? -a0.x : a0.x);
    }
  } else {
    if (form == 0) {
      const R us = SG > 0 ? u : -u;
      a.x = fma(-us, b0.x, a0.x);
      a.y = fma(-us, b0.y, a0.y);
      b.x = fma(us, a0.x, b0.x);
      b.y = fma(us, a0.y, b0.y);
    } else {
      a.x = fma(u, a0.x, SG > 0 ? -b0.x : b0.x);
      a.y = fma(u, a0.y, SG > 0 ? -b0.y : b0.y);
      b.x = fma(u, b0.x, SG > 0 ? a0.x : -a0.x);
      b.y = fma(u, b0.y, SG > 0 ? a0.y : -a0.y);
    }
  }
  (void)s1;
}

template <int SG, int AXIS, int FORM, typename C, typename R>
__device__ __forceinline__ void rotp_t(C& a, C& b, R u) {
  rotp<SG, C, R>(a, b, AXIS, FORM, u);
}

template <int SG, int AXIS, int FORM, int I, int G, typename C, typename R>
__device__ __forceinline__ void rotb(C* el, R u) {
#pragma unroll
  for (int c = 0; c < (1 << G); ++c)
    if (!((c >> I) & 1)) rotp_t<SG, AXIS, FORM, C, R>(el[c], el[c | (1 << I)], u);
}

// warp-uniform dispatch around whole unrolled blocks (no predicated variants)
template <int SG, int I, int G, typename C, typename R>
__device__ __forceinline__ void rotb_any(C* el, int axis, int form, R u) {
  if (axis == 0) {
    if (form == 0)
      rotb<SG, 0, 0, I, G>(el, u);
    else
      rotb<SG, 0, 1, I, G>(el, u);
  } else {
    if (form == 0)
      rotb<SG, 1, 0, I, G>(el, u);
    else
      rotb<SG, 1, 1, I, G>(el, u);
  }
}

// reduction term of one pair for Im<lam|P|psi>: X: Im(conj la qb) + Im(conj lb qa);
// Y: -Re(conj la qb) + Re(conj lb qa)
template <typename C, typename R>
__device__ __forceinline__ R redp(const C& la, const C& lb, const C& qa, const C& qb, int axis) {
  if (axis == 0) return fma(la.x, qb.y, -la.y * qb.x) + fma(lb.x, qa.y, -lb.y * qa.x);
  return -fma(la.x, qb.x, la.y * qb.y) + fma(lb.x, qa.x, lb.y * qa.y);
}

template <typename R>
__device__ __forceinline__ R wsum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// G rotations on ascending local bits bits[0..G-1], each thread owning the
// 2^G amplitudes of one task (all other bits fixed) in registers.
template <typename C, typename R, int G, int NT, bool DBL, int SG>
__device__ __forceinline__ void rot_group(C* v, C* v2, int M, const int* bits, const int* axis, const int* form,
                                          const R* u) {
  const int ntask = M >> G;
  int b[G];
  int ax[G], fm[G];
  R uu[G];
#pragma unroll
  for (int i = 0; i < G; ++i) {
    b[i] = bits[i];
    ax[i] = axis[i];
    fm[i] = form[i];
    uu[i] = (R)u[i];
  }
  // the swizzle is GF(2)-linear: a task's indices are its swizzled base
  // XOR the swizzled group bits
  int sbit[G];
#pragma unroll
  for (int i = 0; i < G; ++i) sbit[i] = swb(1 << b[i], DBL);
  for (int tk = threadIdx.x; tk < ntask; tk += NT) {
    int base = tk;
#pragma unroll
    for (int i = 0; i < G; ++i) base = ins0(base, b[i]);
    const int sb = swb(base, DBL);
    int idx[1 << G];
#pragma unroll
    for (int c = 0; c < (1 << G); ++c) {
      int x = sb;
#pragma unroll
      for (int i = 0; i < G; ++i)
        if ((c >> i) & 1) x ^= sbit[i];
      idx[c] = x;
    }
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
      C* w = pass ? v2 : v;
      if (w == nullptr) break;
      C el[1 << G];
#pragma unroll
      for (int c = 0; c < (1 << G); ++c) el[c] = w[idx[c]];
      rotb_any<SG, 0, G>(el, ax[0], fm[0], uu[0]);
      if (G > 1) rotb_any<SG, (G > 1 ? 1 : 0), G>(el, ax[G > 1 ? 1 : 0], fm[G > 1 ? 1 : 0], uu[G > 1 ? 1 : 0]);
      if (G > 2) rotb_any<SG, (G > 2 ? 2 : 0), G>(el, ax[G > 2 ? 2 : 0], fm[G > 2 ? 2 : 0], uu[G > 2 ? 2 : 0]);
#pragma unroll
      for (int c = 0; c < (1 << G); ++c) w[idx[c]] = el[c];
    }
  }
}

// Gradient reductions of G rotations on ascending bits from one pass over
// the 2^G-amplitude tasks (lambda and psi in registers); the warp sums land
// in out[0..G-1] (this warp's reduction slots).
template <typename C, typename R, int G, int NT, bool DBL>
__device__ __forceinline__ void red_group(const C* lam, const C* psi, int M, const int* bits, const int* axis,
                                          R* out) {
  int b[G], ax[G];
  R acc[G];
#pragma unroll
  for (int i = 0; i < G; ++i) {
    b[i] = bits[i];
    ax[i] = axis[i];
    acc[i] = (R)0;
  }
  const int ntask = M >> G;
  int sbit[G];
#pragma unroll
  for (int i = 0; i < G; ++i) sbit[i] = swb(1 << b[i], DBL);
  for (int tk = threadIdx.x; tk < ntask; tk += NT) {
    int base = tk;
#pragma unroll
    for (int i = 0; i < G; ++i) base = ins0(base, b[i]);
    const int sb = swb(base, DBL);
    C la[1 << G], qa[1 << G];
#pragma unroll
    for (int c = 0; c < (1 << G); ++c) {
      int x = sb;
#pragma unroll
      for (int i = 0; i < G; ++i)
        if ((c >> i) & 1) x ^= sbit[i];
      la[c] = lam[x];
      qa[c] = psi[x];
    }
#pragma unroll
    for (int i = 0; i < G; ++i) {
      // warp-uniform branch around the whole unrolled block
      if (ax[i] == 0) {
#pragma unroll
        for (int c = 0; c < (1 << G); ++c)
          if (!((c >> i) & 1)) acc[i] += redp<C, R>(la[c], la[c | (1 << i)], qa[c], qa[c | (1 << i)], 0);
      } else {
#pragma unroll
        for (int c = 0; c < (1 << G); ++c)
          if (!((c >> i) & 1)) acc[i] += redp<C, R>(la[c], la[c | (1 << i)], qa[c], qa[c | (1 << i)], 1);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < G; ++i) {
    const R v = wsum(acc[i]);
    if ((threadIdx.x & 31) == 0) out[i] = v;
  }
}

// Backward: the gradient reductions of G rotations and their inverses on
// lambda and psi in one pass.  The rotations of a layer commute with each
// other's Paulis and with their own, so Im<lam|P|psi> is the same before and
// after any of them is applied to both states; a group's sums are taken
// from the loaded amplitudes, then both states are rotated back and stored.
// The scaled forms divide each state by the rotation's kappa, so sums taken
// after earlier groups carry 1 / prod(kappa^2) of those groups: `scale`
// (that product) restores them.
template <typename C, typename R, int G, int NT, bool DBL>
__device__ __forceinline__ void rotred_group(C* lam, C* psi, int M, const int* bits, const int* axis, const int* form,
                                             const R* u, R scale, R* out) {
  int b[G], ax[G], fm[G];
  R uu[G], acc[G];
#pragma unroll
  for (int i = 0; i < G; ++i) {
    b[i] = bits[i];
    ax[i] = axis[i];
    fm[i] = form[i];
    uu[i] = u[i];
    acc[i] = (R)0;
  }
  int sbit[G];
#pragma unroll
  for (int i = 0; i < G; ++i) sbit[i] = swb(1 << b[i], DBL);
  const int ntask = M >> G;
  for (int tk = threadIdx.x; tk < ntask; tk += NT) {
    int base = tk;
#pragma unroll
    for (int i = 0; i < G; ++i) base = ins0(base, b[i]);
    const int sb = swb(base, DBL);
    int idx[1 << G];
#pragma unroll
    for (int c = 0; c < (1 << G); ++c) {
      int x = sb;
#pragma unroll
      for (int i = 0; i < G; ++i)
        if ((c >> i) & 1) x ^= sbit[i];
      idx[c] = x;
    }
    C la[1 << G], qa[1 << G];
#pragma unroll
    for (int c = 0; c < (1 << G); ++c) {
      la[c] = lam[idx[c]];
      qa[c] = psi[idx[c]];
    }
#pragma unroll
    for (int i = 0; i < G; ++i) {
      if (ax[i] == 0) {
#pragma unroll
        for (int c = 0; c < (1 << G); ++c)
          if (!((c >> i) & 1)) acc[i] += redp<C, R>(la[c], la[c | (1 << i)], qa[c], qa[c | (1 << i)], 0);
      } else {
#pragma unroll
        for (int c = 0; c < (1 << G); ++c)
          if (!((c >> i) & 1)) acc[i] += redp<C, R>(la[c], la[c | (1 << i)], qa[c], qa[c | (1 << i)], 1);
      }
    }
    rotb_any<-1, 0, G>(la, ax[0], fm[0], uu[0]);
    rotb_any<-1, 0, G>(qa, ax[0], fm[0], uu[0]);
    if (G > 1) {
      rotb_any<-1, (G > 1 ? 1 : 0), G>(la, ax[G > 1 ? 1 : 0], fm[G > 1 ? 1 : 0], uu[G > 1 ? 1 : 0]);
      rotb_any<-1, (G > 1 ? 1 : 0), G>(qa, ax[G > 1 ? 1 : 0], fm[G > 1 ? 1 : 0], uu[G > 1 ? 1 : 0]);
    }
    if (G > 2) {
      rotb_any<-1, (G > 2 ? 2 : 0), G>(la, ax[G > 2 ? 2 : 0], fm[G > 2 ? 2 : 0], uu[G > 2 ? 2 : 0]);
      rotb_any<-1, (G > 2 ? 2 : 0), G>(qa, ax[G > 2 ? 2 : 0], fm[G > 2 ? 2 : 0], uu[G > 2 ? 2 : 0]);
    }
#pragma unroll
    for (int c = 0; c < (1 << G); ++c) {
      lam[idx[c]] = la[c];
      psi[idx[c]] = qa[c];
    }
  }
#pragma unroll
  for (int i = 0; i < G; ++i) {
    const R v = wsum(acc[i]);
    if ((threadIdx.x & 31) == 0) out[i] = v * scale;
  }
}

// T: precision of the per-layer coefficients and partial sums (R)
template <typename T>
struct BShared {
  int job;
  int nxy, nz, ncross;       // gates of the current layer
  int xbit[BMAXQ];           // local bits of the X/Y rotations (cross rotation excluded)
  int xaxis[BMAXQ];
  int xslot[BMAXQ];          // output index
  T xu[BMAXQ];
  T xk[BMAXQ];               // scale factor kappa of each X/Y rotation (scaled form = rotation / kappa)
  int xform[BMAXQ];
  int caxis[2], cform[2], cslot[2], cbit[2];  // rotations on the cluster-split top bits (cbit: rank bit)
  T cu[2];
  int zbit[BMAXQ];           // global bits of the Z rotations
  int zslot[BMAXQ];
  T zs[BMAXQ], zc[BMAXQ];
  T K;
  int zpk[32];               // Z-table index bits of the element-loop step k (e = tid + NT k)
  int zpkf[32];              // the same for the ladder image lad_fwd(top | NT k) (backward fusion)
  T startP[BMAXQ + 1];
  T tw[64];                  // observable weights of the current job
  T red[32][BMAXQ + 4];
};

}  // namespace

template <typename R, int CS, int NT>
__global__ void __launch_bounds__(NT, 1) batched_kernel(const BatchJob* __restrict__ jobs, int njobs, int* counter,
                                                      int mmax) {
  using C = typename BatchC<R>::T;
  constexpr bool DBL = sizeof(R) == 8;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ BShared<R> S;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int Mmax = 1 << mmax;
  // three state buffers: psi, lambda and a scratch that permutations and
  // top-bit rotations write into before the roles are swapped
  C* const buf0 = (C*)smem;
  C* ztab = buf0 + 3 * Mmax;          // BATCH_TABLE entries: Z-rotation phases or QAOA cost phases
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = CS > 1 ? (int)cluster.block_rank() : 0;
  constexpr int LGCS = CS == 4 ? 2 : CS == 2 ? 1 : 0;
  C* psi = buf0;
  C* lam = buf0 + Mmax;
  C* scr = buf0 + 2 * Mmax;
  // The state is split by its top LGCS bits: this CTA holds the block whose
  // top bits are its logical rank.  With 4 CTAs the CNOT ladder's CNOT(0, 1)
  // (control and target both top bits) permutes whole blocks: h(t) = t ^
  // (t >> 1 & 1) in both directions, an involution.  Instead of moving the
  // blocks, every CTA relabels (hflip): logical rank h(rank) while hflip is
  // set, and the CTA holding logical block l is h(l).  2-CTA clusters keep
  // the identity (the ladder never targets qubit 0).
  int hflip = 0;
  auto hmap = [](int t) { return t ^ ((t >> 1) & 1); };
  auto phys = [&](int l) { return CS == 4 && hflip ? hmap(l) : l; };
  // the buffer with the same role (same offset) in the CTA holding logical block l
  auto rmt = [&](C* v, int l) -> C* { return CS > 1 ? cluster.map_shared_rank(v, phys(l)) : v; };
  auto csync = [&]() {
    if (CS > 1)
      cluster.sync();
    else
      __syncthreads();
  };

  for (;;) {
    if (tid == 0 && rank == 0) {
      const int j = atomicAdd(counter, 1);
      S.job = j;
      for (int r = 1; r < CS; ++r) *cluster.map_shared_rank(&S.job, r) = j;
    }
    csync();
    const int jid = S.job;
    if (jid >= njobs) break;
    const BatchJob J = jobs[jid];
    psi = buf0;
    lam = buf0 + Mmax;
    scr = buf0 + 2 * Mmax;
    const int n = J.n;
    const int m = n - LGCS;
    if (m < (CS > 1 ? 2 : 1) || m > mmax || J.layers < 0) {
      // a job this launch cannot hold (its block would overrun the shared
      // memory sized for mmax, or leave a cluster's CTA fewer than 2 bits):
      // NaN outputs, no state touched; the decision is the same in every CTA
      if (tid == 0 && rank == 0) {
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
        if (J.expec) *J.expec = nan;
        if (J.grad && J.layers >= 0)
          for (int i = 0, np = J.kind == 0 ? J.layers * n : 2 * J.layers; i < np; ++i) J.grad[i] = nan;
      }
      csync();  // every thread has read S.job before the next fetch rewrites it
      continue;
    }
    const int M = 1 << m;
    hflip = 0;
    int lrank = rank;  // logical rank: the top bits of this CTA's block
    uint32_t top = (uint32_t)lrank << m;
    // the open CNOT ladder's block permutation (4-CTA jobs), before a gather
    auto relabel = [&]() {
      if (CS == 4) {
        hflip ^= 1;
        lrank = hmap(lrank);
        top = (uint32_t)lrank << m;
      }
    };
    const bool grad = J.grad != nullptr;
    const int L = J.layers;
    uint32_t lodd = 0, leven = 0;
    const uint32_t lwrap = J.entangler == 3 ? 1u : 0u;
    const int lws = n - 1;
    for (int q = 0; q + 1 < n; ++q) {
      const uint32_t b = 1u << (n - 1 - q);
      if (q & 1)
        lodd |= b;
      else
        leven |= b;
    }
    if (tid <= n) {
      // Ry(pi/4)^n |0>: amplitude cos(pi/8)^(n-k) sin(pi/8)^k, one k per thread
      double s8, c8;
      sincospi(0.125, &s8, &c8);
      const int k = tid;
      double q = 1.0;
      for (int i = 0; i < n - k; ++i) q *= c8;
      for (int i = 0; i < k; ++i) q *= s8;
      S.startP[k] = (R)q;
    }
    if (tid == 0 && rank == 0 && CS > 1) {
      if (J.expec) *J.expec = 0.0;
      if (grad) {
        const int np = J.kind == 0 ? L * n : 2 * L;
        for (int i = 0; i < np; ++i) J.grad[i] = 0.0;
      }
      if (J.term_expec)
        for (int k = 0; k < J.nterms; ++k) J.term_expec[k] = 0.0;
    }
    __syncthreads();
    for (int k = tid; k < J.nterms && k < BTERMS; k += NT) S.tw[k] = J.terms[k].w;
    // start state
    const R plus = (R)exp2(-0.5 * n);
    for (int e = tid; e < M; e += NT) {
      const uint32_t x = top | (uint32_t)e;
      C v;
      v.x = J.kind == 0 ? (R)S.startP[__popc(x)] : plus;
      v.y = (R)0;
      psi[swb(e, DBL)] = v;
    }
    __syncthreads();

    // ---- helpers bound to this job
    // warp 0 keeps the next layer's angle and axis in registers: the loads
    // are issued one layer ahead, so a layer setup does not wait on memory
    // while the other warps wait at its barrier
    int pf_layer = -1, pf_axis = 0;
    double pf_th = 0.0;
    auto prefetch = [&](int i) {
      pf_layer = i;
      if (i >= 0 && i < L && lane < n) {
        pf_axis = J.kind == 0 ? (int)J.axes[i * n + lane] : 0;
        pf_th = J.kind == 0 ? J.params[i * n + lane] : J.params[2 * i];
      }
    };
    // layer setup: rotations of layer i into S (forward coefficients); the
    // next layer to be set up is i + step
    auto setup_layer = [&](int i, int step) {
      // warp 0, lane q = qubit q: coefficients in parallel; the X/Y and Z
      // lists are compacted in ascending bit order (descending q) with
      // ballots, and K is a shuffle product over the warp
      if (warp == 0) {
        const unsigned full = 0xffffffffu;
        const int q = lane;
        const bool valid = q < n;
        if (pf_layer != i) prefetch(i);
        const int axis = valid ? pf_axis : 0;
        const R th = valid ? (R)pf_th : (R)0;
        prefetch(i + step);
        const int b = n - 1 - q;
        const int slot = J.kind == 0 ? i * n + q : 2 * i;
        const bool isz = valid && axis == 2;
        const bool iscross = valid && !isz && CS > 1 && b >= m;
        const bool isxy = valid && !isz && !iscross;
        int f = 0;
        R k = (R)1, u = (R)0, zs = (R)0, zc = (R)1;
        if (isxy || iscross) u = rform<R>(th, &f, &k);
        if (isz) sincosT((R)0.5 * th, &zs, &zc);
        const unsigned mxy = __ballot_sync(full, isxy), mz = __ballot_sync(full, isz);
        const unsigned above = q == 31 ? 0u : (full << (q + 1));
        if (isxy) {
          const int idx = __popc(mxy & above);
          S.xbit[idx] = b;
          S.xaxis[idx] = axis;
          S.xslot[idx] = slot;
          S.xu[idx] = u;
          S.xk[idx] = k;
          S.xform[idx] = f;
        }
        if (isz) {
          const int idx = __popc(mz & above);
          S.zbit[idx] = b;
          S.zslot[idx] = slot;
          S.zs[idx] = zs;
          S.zc[idx] = zc;
        }
        const unsigned mc = __ballot_sync(full, iscross);
        if (iscross) {
          const int idx = __popc(mc & above);
          S.caxis[idx] = axis;
          S.cslot[idx] = slot;
          S.cu[idx] = u;
          S.cform[idx] = f;
          S.cbit[idx] = b - m;
        }
        R kk = (isxy || iscross) ? k : (R)1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) kk *= __shfl_xor_sync(full, kk, o);
        if (lane == 0) {
          S.K = kk;
          S.nxy = __popc(mxy);
          S.nz = __popc(mz);
          S.ncross = __popc(mc);
        }
      }
      __syncthreads();
    };
    // diagonal of layer i (Z table * K; QAOA cost phase * K); conj for the inverse.
    // The Z table is built by doubling: 2^nz complex multiplies in all.
    auto build_diag = [&](int i, bool inv) {
      const int nzt = S.nz < BZMAX ? S.nz : BZMAX;
      if (J.kind == 0 && !DBL) {
        // complex64: every entry as its own product (nzt float multiplies),
        // one barrier instead of one per Z rotation
        for (int pp = tid; pp < (1 << nzt); pp += NT) {
          C v = tocf(S.K, (R)0);
          for (int j = 0; j < nzt; ++j) {
            // exp(-i theta/2) on bit 0, exp(+i theta/2) on bit 1 (state.py:168-170); conjugated inverse
            const bool one = (pp >> j) & 1;
            const R sg = (one != inv) ? (R)1 : (R)-1;
            v = cmulb(v, tocf(S.zc[j], sg * S.zs[j]));
          }
          ztab[pp] = v;
        }
      } else if (J.kind == 0) {
        // complex128: doubling, 2^nzt complex multiplies in all
        if (tid == 0) ztab[0] = tocf(S.K, (R)0);
        __syncthreads();
        for (int j = 0; j < nzt; ++j) {
          const int h = 1 << j;
          const C e0 = tocf(S.zc[j], inv ? S.zs[j] : -S.zs[j]);
          const C e1 = tocf(S.zc[j], inv ? -S.zs[j] : S.zs[j]);
          for (int pp = tid; pp < h; pp += NT) {
            const C v = ztab[pp];
            ztab[pp + h] = cmulb(v, e1);
            ztab[pp] = cmulb(v, e0);
          }
          __syncthreads();
        }
      } else {
        const R g = (R)(J.params[2 * i + 1] * J.cost_w0);
        const int MA = J.cost_maxabs;
        for (int k = tid; k <= 2 * MA; k += NT) {
          R s, c;
          sincosT(g * (R)(k - MA), &s, &c);
          ztab[k] = tocf(S.K * c, S.K * (inv ? s : -s));
        }
      }
      // Z-table index bits of the element-loop steps (e = tid + NT k)
      if (J.kind == 0 && tid < (M + NT - 1) / NT) {
        int pat = 0, patf = 0;
        const uint32_t xk = top | (uint32_t)(tid * NT);
        const uint32_t xf = lad_fwd(xk, lodd, leven, lwrap, lws);
        for (int j = 0; j < nzt; ++j) {
          pat |= (int)((xk >> S.zbit[j]) & 1) << j;
          patf |= (int)((xf >> S.zbit[j]) & 1) << j;
        }
        S.zpk[tid] = pat;
        S.zpkf[tid] = patf;
      }
      __syncthreads();
    };
    auto cost_m = [&](uint32_t x) {
      int mm = 0;
      for (int k = 0; k < J.cost_nterms; ++k) {
        const qg_cost_term t = J.cost[k];
        int s = (int)((x >> t.b0) & 1);
        if (t.b1 >= 0) s ^= (int)((x >> t.b1) & 1);
        mm += s ? -t.c : t.c;
      }
      return mm;
    };
    // per-element diagonal multiply on buffer v (table built by build_diag)
    auto apply_diag = [&](C* v, bool inv) {
      const int nzt = S.nz < BZMAX ? S.nz : BZMAX;
      // the pattern of e = tid + NT k is this thread's bits OR the step's
      // (disjoint bit ranges; the top bit is in the step part)
      int ptid = 0;
      if (J.kind == 0)
        for (int j = 0; j < nzt; ++j) ptid |= (int)(((uint32_t)tid >> S.zbit[j]) & 1) << j;
      for (int e = tid, k = 0; e < M; e += NT, ++k) {
        const uint32_t x = top | (uint32_t)e;
        C a = v[swb(e, DBL)];
        if (J.kind == 0) {
          a = cmulb(a, ztab[ptid | S.zpk[k]]);
          for (int j = BZMAX; j < S.nz; ++j) {
            const bool one = (x >> S.zbit[j]) & 1;
            const R sgn = (one != inv) ? (R)1 : (R)-1;
            a = cmulb(a, tocf(S.zc[j], sgn * S.zs[j]));
          }
        } else {
          a = cmulb(a, ztab[cost_m(x) + J.cost_maxabs]);
        }
        v[swb(e, DBL)] = a;
      }
      __syncthreads();
    };
    // entangler on buffer v: (E v)[y] = v[A^{-1} y] (inverse: v[A y]), gathered
    // into the scratch buffer whose role then swaps with v; CZ: sign in place
    auto entangle = [&](C*& v, bool inv) {
      if (J.entangler == 2) {
        for (int e = tid; e < M; e += NT) {
          const uint32_t x = top | (uint32_t)e;
          if (__popc(x & (x >> 1)) & 1) {
            C a = v[swb(e, DBL)];
            a.x = -a.x;
            a.y = -a.y;
            v[swb(e, DBL)] = a;
          }
        }
        __syncthreads();
        return;
      }
      for (int e = tid; e < M; e += NT) {
        const uint32_t x = top | (uint32_t)e;
        const uint32_t src = inv ? lad_fwd(x, lodd, leven, lwrap, lws) : lad_inv(x, lodd, leven, lwrap, lws);
        scr[swb(e, DBL)] = v[swb((int)(src & (uint32_t)(M - 1)), DBL)];
      }
      __syncthreads();
      C* t = v;
      v = scr;
      scr = t;
    };
    // X/Y rotations of the layer in groups of up to 3 bits per shared-memory pass
    // rotation on the top bit (2-CTA clusters): the partner amplitude lives
    // in the other CTA; new values go to the scratch buffer, which then
    // becomes the rotated buffer
    auto rotate_cross = [&](C*& v, C*& v2, bool inverse) {
      const int nc = CS > 1 ? S.ncross : 0;
      for (int c = 0; c < nc; ++c) {
        const int cb = S.cbit[c];
        const bool low = ((lrank >> cb) & 1) == 0;  // this block holds the bit-0 half
        for (int pass = 0; pass < (v2 ? 2 : 1); ++pass) {
          C*& w = pass ? v2 : v;
          cluster.sync();
          const C* rw = rmt(w, lrank ^ (1 << cb));
          for (int e = tid; e < M; e += NT) {
            const C own = w[swb(e, DBL)];
            const C rem = rw[swb(e, DBL)];
            C x0 = low ? own : rem, x1 = low ? rem : own;
            if (inverse)
              rotp<-1, C, R>(x0, x1, S.caxis[c], S.cform[c], (R)S.cu[c]);
            else
              rotp<1, C, R>(x0, x1, S.caxis[c], S.cform[c], (R)S.cu[c]);
            scr[swb(e, DBL)] = low ? x0 : x1;
          }
          cluster.sync();
          C* t = w;
          w = scr;
          scr = t;
        }
      }
    };
    auto rotate = [&](C*& v, C* v2in, bool inverse) {
      C* v2 = v2in;
      const int nxy = S.nxy;
      for (int g0 = 0; g0 < nxy; g0 += 3) {
        const int g = nxy - g0 < 3 ? nxy - g0 : 3;
        if (!inverse) {
          if (g == 3)
            rot_group<C, R, 3, NT, DBL, 1>(v, v2, M, S.xbit + g0, S.xaxis + g0, S.xform + g0, S.xu + g0);
          else if (g == 2)
            rot_group<C, R, 2, NT, DBL, 1>(v, v2, M, S.xbit + g0, S.xaxis + g0, S.xform + g0, S.xu + g0);
          else
            rot_group<C, R, 1, NT, DBL, 1>(v, v2, M, S.xbit + g0, S.xaxis + g0, S.xform + g0, S.xu + g0);
        } else {
          if (g == 3)
            rot_group<C, R, 3, NT, DBL, -1>(v, v2, M, S.xbit + g0, S.xaxis + g0, S.xform + g0, S.xu + g0);
          else if (g == 2)
            rot_group<C, R, 2, NT, DBL, -1>(v, v2, M, S.xbit + g0, S.xaxis + g0, S.xform + g0, S.xu + g0);
          else
            rot_group<C, R, 1, NT, DBL, -1>(v, v2, M, S.xbit + g0, S.xaxis + g0, S.xform + g0, S.xu + g0);
        }
        __syncthreads();
      }
      rotate_cross(v, v2, inverse);
      return v2;
    };

    // block-sum of one value into the job's output (with 2 CTAs: two atomic
    // adds onto 0, whose result does not depend on their order)
    auto emit1 = [&](R val, int slot, double factor) {
      const R v = wsum(val);
      if (lane == 0) S.red[warp][0] = v;
      __syncthreads();
      if (tid == 0) {
        R tot = (R)0;
        for (int w = 0; w < NT / 32; ++w) tot += S.red[w][0];
        const double out = factor * (double)tot;
        if (CS > 1)
          atomicAdd(&J.grad[slot], out);
        else
          J.grad[slot] = out;
      }
      __syncthreads();
    };

    // McClean layers with the entangler before the rotations: the ladder
    // and the layer's diagonal in one pass.  Forward v <- D (E v):
    // new[x] = D[x] v[A^{-1} x]; backward v <- E^{-1} (D^{-1} v):
    // new[x] = D^{-1}[A x] v[A x].  The table index of A x is linear in x,
    // so it splits into a per-thread and a per-step part like the plain one.
    const bool fuse = J.kind == 0 && J.entangler != 0 && J.placement == 0;
    auto entangle_diag = [&](C*& v, bool inv) {
      const int nzt = S.nz;  // callers fuse only when every Z rotation is in the table
      int ptid = 0;
      const uint32_t tsrc = (inv && (J.entangler == 1 || J.entangler == 3)) ? lad_fwd((uint32_t)tid, lodd, leven, lwrap, lws) : (uint32_t)tid;
      for (int j = 0; j < nzt; ++j) ptid |= (int)((tsrc >> S.zbit[j]) & 1) << j;
      if (J.entangler == 2) {
        // CZ: a sign, its own inverse, in place
        for (int e = tid, k = 0; e < M; e += NT, ++k) {
          const uint32_t x = top | (uint32_t)e;
          C a = cmulb(v[swb(e, DBL)], ztab[ptid | S.zpk[k]]);
          if (__popc(x & (x >> 1)) & 1) {
            a.x = -a.x;
            a.y = -a.y;
          }
          v[swb(e, DBL)] = a;
        }
        __syncthreads();
        return;
      }
      for (int e = tid, k = 0; e < M; e += NT, ++k) {
        const uint32_t x = top | (uint32_t)e;
        const uint32_t src = inv ? lad_fwd(x, lodd, leven, lwrap, lws) : lad_inv(x, lodd, leven, lwrap, lws);
        const int pat = inv ? (ptid ^ S.zpkf[k]) : (ptid | S.zpk[k]);
        scr[swb(e, DBL)] = cmulb(v[swb((int)(src & (uint32_t)(M - 1)), DBL)], ztab[pat]);
      }
      __syncthreads();
      C* t = v;
      v = scr;
      scr = t;
    };

    // ---- forward (relabel: the CNOT ladder's block permutation, before
    // anything that reads the new block's index)
    const bool ladder = J.kind == 0 && J.entangler == 1;
    for (int i = 0; i < L; ++i) {
      setup_layer(i, 1);
      if (fuse && S.nz <= BZMAX) {
        if (ladder) relabel();
        build_diag(i, false);
        entangle_diag(psi, false);
      } else {
        if (fuse) {
          if (ladder) relabel();
          entangle(psi, false);
        }
        build_diag(i, false);
        apply_diag(psi, false);
      }
      // (no cluster barrier here: the only cross-CTA reads of a layer,
      // rotate_cross's, sit between barriers of their own)
      rotate(psi, nullptr, false);
      if (J.kind == 0 && J.entangler != 0 && J.placement == 1) {
        if (ladder) relabel();
        entangle(psi, false);
      }
    }
    if (CS > 1) cluster.sync();

    // ---- observable: lam = O psi and E = Re<psi|lam>
    {
      R eacc = (R)0;
      const bool costonly = J.kind == 1 && grad;
      for (int e = tid; e < M; e += NT) {
        const uint32_t x = top | (uint32_t)e;
        const C v = psi[swb(e, DBL)];
        R lx = (R)0, ly = (R)0;
        if (costonly) {
          const R d = (R)J.cost_w0 * (R)cost_m(x);
          lx = d * v.x;
          ly = d * v.y;
        } else {
          for (int k = 0; k < J.nterms; ++k) {
            const BatchTerm t = J.terms[k];
            const uint32_t b0 = 1u << (n - 1 - t.q0);
            const R tw = k < BTERMS ? (R)S.tw[k] : (R)t.w;
            if (t.kind >= 2) {
              bool s = (x & b0) != 0;
              if (t.kind == 3) s ^= (x & (1u << (n - 1 - t.q1))) != 0;
              const R w = s ? -tw : tw;
              lx = fma(w, v.x, lx);
              ly = fma(w, v.y, ly);
            } else {
              const uint32_t xp = x ^ b0;
              C u;
              if ((xp >> m) != (x >> m))
                u = rmt(psi, (int)(xp >> m))[swb((int)(xp & (uint32_t)(M - 1)), DBL)];
              else
                u = psi[swb((int)(xp & (uint32_t)(M - 1)), DBL)];
              const R w = tw;
              if (t.kind == 0) {
                lx = fma(w, u.x, lx);
                ly = fma(w, u.y, ly);
              } else {
                const R sgn = (x & b0) ? (R)1 : (R)-1;
                lx = fma(-sgn * w, u.y, lx);
                ly = fma(sgn * w, u.x, ly);
              }
            }
          }
        }
        eacc = fma(v.x, lx, fma(v.y, ly, eacc));
        if (grad) {
          C o;
          o.x = lx;
          o.y = ly;
          lam[swb(e, DBL)] = o;
        }
      }
      const R v = wsum(eacc);
      if (lane == 0) S.red[warp][0] = v;
      __syncthreads();
      if (tid == 0) {
        R tot = (R)0;
        for (int w = 0; w < NT / 32; ++w) tot += S.red[w][0];
        if (CS > 1)
          atomicAdd(J.expec, (double)tot);
        else
          *J.expec = (double)tot;
      }
      __syncthreads();
    }
    // ---- optional: <P_k> of every observable term on the final state (the
    // per-term expectations the projector-shot estimators draw from,
    // observable.py:82-177, base.py:22-46)
    if (J.term_expec) {
      for (int k = 0; k < J.nterms; ++k) {
        const BatchTerm t = J.terms[k];
        const uint32_t b0 = 1u << (n - 1 - t.q0);
        R acc = (R)0;
        for (int e = tid; e < M; e += NT) {
          const uint32_t x = top | (uint32_t)e;
          const C v = psi[swb(e, DBL)];
          if (t.kind >= 2) {
            bool sg = (x & b0) != 0;
            if (t.kind == 3) sg ^= (x & (1u << (n - 1 - t.q1))) != 0;
            const R p2 = fma(v.x, v.x, v.y * v.y);
            acc += sg ? -p2 : p2;
          } else {
            const uint32_t xp = x ^ b0;
            const C u = (xp >> m) != (x >> m) ? rmt(psi, (int)(xp >> m))[swb((int)(xp & (uint32_t)(M - 1)), DBL)]
                                              : psi[swb((int)(xp & (uint32_t)(M - 1)), DBL)];
            if (t.kind == 0) {
              acc += fma(v.x, u.x, v.y * u.y);  // Re(conj(v) u)
            } else {
              // (Y psi)_x = -i psi_partner (bit 0) or +i psi_partner (bit 1)
              const R sgn = (x & b0) ? (R)1 : (R)-1;
              acc += sgn * fma(-v.x, u.y, v.y * u.x);  // Re(conj(v) i u) * sgn
            }
          }
        }
        const R v = wsum(acc);
        if (lane == 0) S.red[warp][0] = v;
        __syncthreads();
        if (tid == 0) {
          R tot = (R)0;
          for (int w = 0; w < NT / 32; ++w) tot += S.red[w][0];
          if (CS > 1)
            atomicAdd(&J.term_expec[k], (double)tot);
          else
            J.term_expec[k] = (double)tot;
        }
        __syncthreads();
      }
    }
    if (CS > 1) cluster.sync();

    // ---- backward (uncompute form)
    if (grad) {
      for (int i = L - 1; i >= 0; --i) {
        setup_layer(i, -1);
        if (J.kind == 0 && J.entangler != 0 && J.placement == 1) {
          if (ladder) relabel();
          entangle(psi, true);
          entangle(lam, true);
        }
        // gradient reductions of the X/Y rotations on local bits fused with
        // their inverses on lam and psi; per-warp sums in S.red[warp][k].
        // The remaining sums (top bit, Z) are invariant under these
        // rotations and are taken afterwards.
        const int nxy = S.nxy;
        R sc = (R)1;  // prod kappa^2 of the rotations already applied
        if (DBL) {
          // complex128: separate reduction passes at the layer's end point;
          // the fused form needs more than the 128 registers a thread has here
          for (int g0 = 0; g0 < nxy; g0 += 3) {
            const int g = nxy - g0 < 3 ? nxy - g0 : 3;
            if (g == 3)
              red_group<C, R, 3, NT, DBL>(lam, psi, M, S.xbit + g0, S.xaxis + g0, &S.red[warp][g0]);
            else if (g == 2)
              red_group<C, R, 2, NT, DBL>(lam, psi, M, S.xbit + g0, S.xaxis + g0, &S.red[warp][g0]);
            else
              red_group<C, R, 1, NT, DBL>(lam, psi, M, S.xbit + g0, S.xaxis + g0, &S.red[warp][g0]);
          }
        }
        for (int g0 = 0; !DBL && g0 < nxy; g0 += 3) {
          const int g = nxy - g0 < 3 ? nxy - g0 : 3;
          if (g == 3)
            rotred_group<C, R, 3, NT, DBL>(lam, psi, M, S.xbit + g0, S.xaxis + g0, S.xform + g0, S.xu + g0, sc,
                                           &S.red[warp][g0]);
          else if (g == 2)
            rotred_group<C, R, 2, NT, DBL>(lam, psi, M, S.xbit + g0, S.xaxis + g0, S.xform + g0, S.xu + g0, sc,
                                           &S.red[warp][g0]);
          else
            rotred_group<C, R, 1, NT, DBL>(lam, psi, M, S.xbit + g0, S.xaxis + g0, S.xform + g0, S.xu + g0, sc,
                                           &S.red[warp][g0]);
          for (int i = g0; i < g0 + g; ++i) sc *= S.xk[i] * S.xk[i];
          __syncthreads();
        }
        int ns = nxy;
        const int ncr = CS > 1 ? S.ncross : 0;
        if (ncr) cluster.sync();  // the partners' psi has its local rotations applied
        for (int c = 0; c < ncr; ++c) {
          const int cb = S.cbit[c];
          const bool low = ((lrank >> cb) & 1) == 0;  // this block holds the bit-0 half (a)
          const C* rq = rmt(psi, lrank ^ (1 << cb));
          R a = (R)0;
          for (int e = tid; e < M; e += NT) {
            const C l = lam[swb(e, DBL)];
            const C qr = rq[swb(e, DBL)];
            if (S.caxis[c] == 0)
              a += fma(l.x, qr.y, -l.y * qr.x);
            else
              a += low ? -fma(l.x, qr.x, l.y * qr.y) : fma(l.x, qr.x, l.y * qr.y);
          }
          a = wsum(a);
          if (lane == 0) S.red[warp][ns] = a * sc;
          ++ns;
        }
        // Z rotations: sum_x s_j(x) Im(conj lam psi) = T - 2 U_j.  With
        // e = tid + NT k, a Z bit below log2(NT) is fixed per thread, a bit
        // above it is a bit of k (at most 4 of them), the top bit is the rank.
        const int nz = S.nz;
        if (nz > 0) {
          constexpr int LGNT = NT == 512 ? 9 : (NT == 256 ? 8 : 10);
          R T = (R)0;
          R Uk[4] = {(R)0, (R)0, (R)0, (R)0};
          for (int e = tid, k = 0; e < M; e += NT, ++k) {
            const C l = lam[swb(e, DBL)], q = psi[swb(e, DBL)];
            const R w = fma(l.x, q.y, -l.y * q.x);
            T += w;
#pragma unroll
            for (int i = 0; i < 4; ++i)
              if ((k >> i) & 1) Uk[i] += w;
          }
          for (int j = 0; j < nz; ++j) {
            const int b = S.zbit[j];
            R U;
            if (b < LGNT)
              U = ((tid >> b) & 1) ? T : (R)0;
            else if (b < m)
              U = (b - LGNT == 0) ? Uk[0] : (b - LGNT == 1) ? Uk[1] : (b - LGNT == 2) ? Uk[2] : Uk[3];
            else
              U = ((lrank >> (b - m)) & 1) ? T : (R)0;  // a top bit: fixed per block
            R val = wsum(T - (R)2 * U);
            if (lane == 0) S.red[warp][ns + j] = val * sc;
          }
          ns += nz;
        }
        __syncthreads();
        if (J.kind == 0) {
          if (tid < ns) {
            R tot = (R)0;
            for (int w = 0; w < NT / 32; ++w) tot += S.red[w][tid];
            const int slot = tid < nxy ? S.xslot[tid] : tid < nxy + ncr ? S.cslot[tid - nxy] : S.zslot[tid - nxy - ncr];
            if (CS > 1)
              atomicAdd(&J.grad[slot], (double)tot);
            else
              J.grad[slot] = (double)tot;
          }
        } else if (tid == 0) {
          // beta: the sum over all n X rotations of the layer
          R tot = (R)0;
          for (int k = 0; k < ns; ++k)
            for (int w = 0; w < NT / 32; ++w) tot += S.red[w][k];
          if (CS > 1)
            atomicAdd(&J.grad[2 * i], (double)tot);
          else
            J.grad[2 * i] = (double)tot;
        }
        __syncthreads();
        // complex128 rotates psi here before rotate_cross's first barrier:
        // the partners may still read it for their cross reductions
        if (CS > 1 && DBL && ncr) cluster.sync();
        // inverse rotations on lam and psi
        if (DBL)
          psi = rotate(lam, psi, true);
        else
          rotate_cross(lam, psi, true);
        const bool fz = fuse && S.nz <= BZMAX;
        if (fz && ladder) relabel();  // the fused table reads the new block's index
        build_diag(i, true);
        if (fz) {
          entangle_diag(lam, true);
          entangle_diag(psi, true);
          continue;
        }
        apply_diag(lam, true);
        apply_diag(psi, true);
        if (J.kind == 1) {
          // gamma at the point before the cost phase (qaoa.py:65-68), where
          // lambda and psi carry no scale factor
          R gsum = (R)0;
          for (int e = tid; e < M; e += NT) {
            const uint32_t x = top | (uint32_t)e;
            const C l = lam[swb(e, DBL)], q = psi[swb(e, DBL)];
            gsum = fma((R)J.cost_w0 * (R)cost_m(x), fma(l.x, q.y, -l.y * q.x), gsum);
          }
          emit1(gsum, 2 * i + 1, 2.0);
        }
        if (J.kind == 0 && J.entangler != 0 && J.placement == 0) {
          if (ladder) relabel();
          entangle(psi, true);
          entangle(lam, true);
        }
        // (no end-of-layer cluster barrier: every cross-CTA read of the
        // layer ended at rotate_cross's last barrier, and the next layer's
        // first cross read (its reductions) waits at a barrier of its own)
      }
    }
    csync();
  }
}

template <typename R, int CS, int NT>
static cudaError_t launch_one(const BatchJob* jobs, int njobs, int* counter, int mmax, cudaStream_t st,
                              int* grid_out) {
  using C = typename BatchC<R>::T;
  const size_t smem = (size_t)(3 * (1 << mmax) + BATCH_TABLE) * sizeof(C);
  auto kern = batched_kernel<R, CS, NT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, NT, smem);
  if (e != cudaSuccess) return e;
  if (per < 1) return cudaErrorInvalidConfiguration;
  int units = sms * per / CS;                 // clusters (or CTAs) resident at once
  if (units > njobs) units = njobs;
  if (units < 1) units = 1;
  *grid_out = units;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(units * CS);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (CS > 1) {
    // clusters co-resident at once (a cluster's CTAs share one GPC, which
    // can leave SMs over); the job queue needs no co-residency, so this
    // only avoids launching clusters that would wait for others to exit
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, kern, &cfg) == cudaSuccess && nc > 0 && nc < units) {
      units = nc;
      *grid_out = units;
      cfg.gridDim = dim3(units * CS);
    }
    cudaGetLastError();
  }
  e = cudaLaunchKernelEx(&cfg, kern, jobs, njobs, counter, mmax);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t launch_batched(int dtype_double, int cluster, const BatchJob* jobs, int njobs, int* counter, int mmax,
                           cudaStream_t st, int* grid_out) {
  if (dtype_double) {
    if (cluster == 4) return launch_one<double, 4, BATCH_THREADS>(jobs, njobs, counter, mmax, st, grid_out);
    if (cluster == 2) return launch_one<double, 2, BATCH_THREADS>(jobs, njobs, counter, mmax, st, grid_out);
    return launch_one<double, 1, BATCH_THREADS>(jobs, njobs, counter, mmax, st, grid_out);
  }
  if (cluster == 4) return launch_one<float, 4, BATCH_THREADS>(jobs, njobs, counter, mmax, st, grid_out);
  if (cluster == 2) return launch_one<float, 2, BATCH_THREADS>(jobs, njobs, counter, mmax, st, grid_out);
  return launch_one<float, 1, BATCH_THREADS>(jobs, njobs, counter, mmax, st, grid_out);
}

}  // namespace qg
