// Device helpers of the sweep kernels (qg_sweep.cu): launch with
// programmatic dependence, the CNOT
// ladder as a GF(2)-linear index map, scaled-form rotations and their
// gradient pair terms, the per-CTA setup (rotation forms, phase and cost
// tables, tile bases) and the per-amplitude diagonal.
//
// Reference mapping (qradient, pure numpy):
//   rotations          physical_components/state.py:90-97, 142-149, 168-175
//   CNOT ladder        physical_components/state.py:209-251
#pragma once
#include <utility>

#include "qg_internal.cuh"

namespace qg {

// default tile bits (the sizes the shared-memory sweep kernels are also
// instantiated for with the tile size fixed at compile time)
constexpr int kTileC64 = 12, kTileC128 = 11;
template <typename R>
constexpr int kTileFixed = sizeof(R) == 4 ? kTileC64 : kTileC128;

// Programmatic dependent launch.  The sweep and observable kernels let the
// next launch start at once (pdl_trigger) and, after their setup (which
// reads only the angles and the descriptor), wait for the previous grid's
// completion and memory (pdl_wait) before their first access to a state,
// the cost tables or the partial sums.  Launched with the attribute after
// one of these kernels, a kernel's CTAs take the SMs the previous grid's
// finished CTAs free and run their setup while it drains.  Without the
// attribute both instructions return at once.  The wait is the hardware's:
// it ends when the previous grid has completed.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
static inline cudaError_t launch_pdl(void (*kern)(KArgs...), int grid, size_t smem, cudaStream_t st, bool pdl,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(NTHREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ double angle_of(const AngleRef& a, const double* params) {
  return a.param >= 0 ? (double)a.sign * params[a.param] : a.fixed;
}

// Reference CNOT ladder as a basis permutation: CNOT(q, q+1) flips bit
// (n-2-q) when bit (n-1-q) is set, i.e. x ^= (x & bit_c) >> 1.  The odd-pair
// CNOTs act first, then the even pairs (state.py:235-241).  The pairs of one
// parity are disjoint, so each parity is one masked shift-xor.  The periodic
// ladder (state.py:218-219, even n) adds CNOT(n-1, 0) to the odd pairs: bit
// n-1 flips when bit 0 is set, x ^= (x & wrap) << (n - 1).
struct LadderMasks {
  uint64_t odd, even, wrap;
  int wshift;
};

__device__ __forceinline__ LadderMasks ladder_masks(int n, bool periodic) {
  LadderMasks m{0, 0, periodic ? 1ull : 0ull, n - 1};
  for (int q = 0; q + 1 < n; ++q) {
    const uint64_t b = 1ull << (n - 1 - q);
    if (q & 1)
      m.odd |= b;
    else
      m.even |= b;
  }
  return m;
}

// A(x): ladder |x> = |A(x)>
__device__ __forceinline__ uint64_t ladder_fwd(uint64_t x, const LadderMasks& m) {
  x ^= ((x & m.odd) >> 1) ^ ((x & m.wrap) << m.wshift);
  x ^= (x & m.even) >> 1;
  return x;
}
// A^{-1}(x)
__device__ __forceinline__ uint64_t ladder_inv(uint64_t x, const LadderMasks& m) {
  x ^= (x & m.even) >> 1;
  x ^= ((x & m.odd) >> 1) ^ ((x & m.wrap) << m.wshift);
  return x;
}

// CZ on all neighbouring qubit pairs: (-1)^{popcount(x & (x >> 1))}
__device__ __forceinline__ bool cz_negative(uint64_t x) { return __popcll(x & (x >> 1)) & 1; }

// Shared-memory swizzle: XOR the low 3 (complex128) or 4 (complex64) bits of
// an element index with the next 3 / 4 bits, so that the 8 or 16 elements a
// quarter / half warp touches land in distinct banks also when the threads
// stride over the low bits (gate groups on bits 0..2).
template <typename R>
__device__ __forceinline__ int sw(int e);
template <>
__device__ __forceinline__ int sw<double>(int e) {
  return e ^ ((e >> 3) & 7);
}
template <>
__device__ __forceinline__ int sw<float>(int e) {
  return e ^ ((e >> 4) & 15);
}

__device__ __forceinline__ int insert0(int p, int j) { return ((p >> j) << (j + 1)) | (p & ((1 << j) - 1)); }

// complex multiply / real scale in the state's own precision
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cscale(double2 a, double k) { return make_double2(a.x * k, a.y * k); }
__device__ __forceinline__ float2 cscale(float2 a, float k) { return make_float2(a.x * k, a.y * k); }

template <typename C>
__device__ __forceinline__ C to_c(double2 v);
template <>
__device__ __forceinline__ double2 to_c<double2>(double2 v) {
  return v;
}
template <>
__device__ __forceinline__ float2 to_c<float2>(double2 v) {
  return make_float2((float)v.x, (float)v.y);
}

template <typename C>
__device__ __forceinline__ C cneg(C a) {
  a.x = -a.x;
  a.y = -a.y;
  return a;
}

template <typename R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Scaled-form choice for a rotation angle theta (see qg_internal.cuh):
// returns the multiplier u and sets form (0: [[1, .u],[.u, 1]], 1: [[u, .],[., u]])
// and the scale factor kappa.
__device__ __forceinline__ double rot_form(double theta, int* form, double* kappa) {
  double s, c;
  sincos(0.5 * theta, &s, &c);
  if (fabs(c) >= fabs(s)) {
    *form = 0;
    *kappa = c;
    return s / c;
  }
  *form = 1;
  *kappa = s;
  return c / s;
}

// Apply one X/Y rotation (scaled form) to the pair (a, b) = (bit 0, bit 1).
// SG = +1 applies R(theta), SG = -1 applies R(-theta): a compile-time sign,
// folded into the FMAs' operand negations.  Axis and form are compile-time
// too: in unrolled register code a runtime branch would be if-converted and
// all four variants issued under predication.
template <int SG, int AXIS, int FORM, typename C, typename R>
__device__ __forceinline__ void rot_pair_t(C& a, C& b, R u) {
  const C a0 = a, b0 = b;
  const R us = SG > 0 ? u : -u;
  if (AXIS == AX_X) {
    if (FORM == 0) {
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
  } else if constexpr (sizeof(R) == 4) {
    // complex64 Y forms act componentwise on (x, y): one paired FP32 FMA
    // (FFMA2) per amplitude instead of two
    const float2 a2 = *reinterpret_cast<const float2*>(&a0), b2 = *reinterpret_cast<const float2*>(&b0);
    float2 ra, rb;
    if (FORM == 0) {
      ra = __ffma2_rn(make_float2(-us, -us), b2, a2);
      rb = __ffma2_rn(make_float2(us, us), a2, b2);
    } else {
      const float2 uu = make_float2(u, u);
      ra = __ffma2_rn(uu, a2, SG > 0 ? make_float2(-b2.x, -b2.y) : b2);
      rb = __ffma2_rn(uu, b2, SG > 0 ? a2 : make_float2(-a2.x, -a2.y));
    }
    a = *reinterpret_cast<const C*>(&ra);
    b = *reinterpret_cast<const C*>(&rb);
  } else {
    if (FORM == 0) {
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
}

// all pairs of register block el[] that differ in bit I, one rotation type
template <int SG, int AXIS, int FORM, int I, int G, typename C, typename R>
__device__ __forceinline__ void rot_block(C* el, R u) {
#pragma unroll
  for (int c = 0; c < (1 << G); ++c)
    if (!((c >> I) & 1)) rot_pair_t<SG, AXIS, FORM, C, R>(el[c], el[c | (1 << I)], u);
}

template <int SG, int I, int G, typename C, typename R>
__device__ __forceinline__ void rot_block_any(C* el, int axis, int form, R u) {
  // warp-uniform branch around whole unrolled blocks
  if (axis == AX_X) {
    if (form == 0)
      rot_block<SG, AX_X, 0, I, G>(el, u);
    else
      rot_block<SG, AX_X, 1, I, G>(el, u);
  } else {
    if (form == 0)
      rot_block<SG, AX_Y, 0, I, G>(el, u);
    else
      rot_block<SG, AX_Y, 1, I, G>(el, u);
  }
}

// ------------------------------------------------------------ shared setup

// Index into the merged Z-rotation table: bit j = the amplitude's bit at the
// j-th Z rotation.  An index x = base | dep_lo | offhi[k] combines disjoint
// bit sets, so its pattern is the OR of the three parts' patterns (per tile,
// per thread, per element-loop step).
__device__ __forceinline__ int zpattern(uint64_t x, const SweepDesc& d) {
  int pat = 0;
  for (int j = 0; j < d.nz; ++j) pat |= (int)((x >> d.z[j].gbit) & 1) << j;
  return pat;
}


// reduction slots of one CTA: X/Y rotations, U_j of the Z rotations, the
// element total T, the gamma reduction
constexpr int RS_XY = 0, RS_Z = TMAX, RS_T = TMAX + ZMAX, RS_G = TMAX + ZMAX + 1, RS_N = TMAX + ZMAX + 2;

struct SetupShared {
  double u[TMAX];
  double kappa[TMAX];
  double sc[QMAX];     // scale factors of the folded rotations
  double zs[ZMAX], zc[ZMAX];
  double K;  // product of the folded scale factors (diagonal sweeps)
  int form[TMAX];
  int zk[ZMAX];        // Z rotation bit: k bit of the element loop (>= 0), thread bit (-1), outside (-2)
  int zkmask;          // k bits carrying a Z rotation
  int64_t offhi[32];   // deposit(k << 8) for the element loop
  int zpk[32];         // Z-table index bits contributed by offhi[k]
  uint8_t outside[QMAX];
  double startP[QMAX + 1];
  // complex64 kernels keep their per-tile sums and rotation multipliers in
  // float: a double instruction, even on one lane, holds the FP64 pipe
  // (2 lanes per clock) for 16 cycles.  A kernel uses one of the two arrays.
  union {
    double red[NTHREADS / 32][RS_N];
    float redf[NTHREADS / 32][RS_N];
  };
  float uf[TMAX];
  float zsf[ZMAX], zcf[ZMAX];  // float copies of the Z phases (complex64 table)
};

// this warp's partial-sum slot in the kernel's own precision
template <typename R>
__device__ __forceinline__ void red_slot_add(SetupShared& S, int w, int slot, R v) {
  if (sizeof(R) == 4)
    S.redf[w][slot] += (float)v;
  else
    S.red[w][slot] += (double)v;
}
template <typename R>
__device__ __forceinline__ double red_slot(const SetupShared& S, int w, int slot) {
  return sizeof(R) == 4 ? (double)S.redf[w][slot] : S.red[w][slot];
}

// Deposit the low bits of v into the listed bit positions.
__device__ __forceinline__ int64_t deposit(int64_t v, const uint8_t* bits, int nb) {
  int64_t x = 0;
  for (int i = 0; i < nb; ++i)
    if ((v >> i) & 1) x |= (int64_t)1 << bits[i];
  return x;
}

// Element-loop parts in registers (fixed tiles).  With a tile of TB bits the
// element-loop index k has KB = TB - 8 bits, and offhi[k], zpk[k] and ladk[k]
// are GF(2)-linear in k (deposit, the Z-table pattern and the ladder image
// are): each is the XOR of its values at k's single bits, and for offhi,
// whose parts are disjoint, also their sum.  A loop unrolled over k builds
// them from KB registers loaded before the loop instead of one
// shared-memory load per element.
template <typename T, int KB>
struct KParts {
  T v[KB];
  __device__ __forceinline__ explicit KParts(const T* tab) {
#pragma unroll
    for (int i = 0; i < KB; ++i) v[i] = tab[1 << i];
  }
  // k is a compile-time constant in an unrolled loop
  __device__ __forceinline__ T at(int k) const {
    T x = 0;
#pragma unroll
    for (int i = 0; i < KB; ++i)
      if ((k >> i) & 1) x ^= v[i];
    return x;
  }
  __device__ __forceinline__ T sum(int k) const {
    T x = 0;
#pragma unroll
    for (int i = 0; i < KB; ++i)
      if ((k >> i) & 1) x += v[i];
    return x;
  }
};

// The bases of a CTA's tiles (tile ids blockIdx.x, + gridDim.x, ...) in
// turn: deposit(v + g) is deposit(v) plus deposit(g) with the carries passed
// through the tile's own bits, a masked add of three operations per tile
// instead of a loop over the outside bits.
struct TileBases {
  uint64_t next, step, omask;
  __device__ __forceinline__ TileBases(const uint8_t* outside, int nb, int n, const uint8_t* tbits, int t) {
    uint64_t tm = 0;
    for (int i = 0; i < t; ++i) tm |= 1ull << tbits[i];
    omask = ((1ull << n) - 1) & ~tm;
    next = (uint64_t)deposit(blockIdx.x, outside, nb);
    step = (uint64_t)deposit(gridDim.x, outside, nb);
  }
  __device__ __forceinline__ int64_t advance() {
    const uint64_t b = next;
    next = ((next | ~omask) + step) & omask;
    return (int64_t)b;
  }
};

// Common per-CTA setup: gate coefficients, element offsets, outside bits,
// the diagonal phase table (Z rotations * scale) and the integer-cost phase
// table, both stored in the state's precision.
// ladk (complex64 kernels; null for complex128): the CNOT-ladder image of
// offhi[k] (A^-1 forward, A backward), so an element's image is the XOR of
// its parts' images
template <typename C, bool BWD>
__device__ void sweep_setup(const SweepDesc& d, const double* params, SetupShared& S, C* ztab, C* ctab,
                            int64_t* ladk = nullptr) {
  using R = decltype(C{}.x);
  const int tid = threadIdx.x;
  const int t = d.t, n = d.n;
  if (tid < d.nxy) {
    int f;
    double k;
    S.u[tid] = rot_form(angle_of(d.xy[tid].a, params), &f, &k);
    S.uf[tid] = (float)S.u[tid];
    S.form[tid] = f;
    S.kappa[tid] = k;
  }
  if (tid < d.nz) {
    // where the Z rotation's bit lives: tile position >= 8 (a bit of the
    // element-loop index k, zk = position - 8), a bit of the thread index
    // (zk = -1), or outside the tile (zk = -2)
    int zk = -2;
    for (int i = 0; i < t; ++i)
      if (d.bits[i] == d.z[tid].gbit) zk = i >= 8 ? i - 8 : -1;
    S.zk[tid] = zk;
  }
  if (tid == 0) {
    int m = 0;
    for (int j = 0; j < d.nz; ++j) {
      int zk = -2;
      for (int i = 8; i < t; ++i)
        if (d.bits[i] == d.z[j].gbit) zk = i - 8;
      if (zk >= 0) m |= 1 << zk;
    }
    S.zkmask = m;
  }
  for (int i = tid; i < (NTHREADS / 32) * RS_N; i += NTHREADS) (&S.red[0][0])[i] = 0.0;  // clears both views
  if (t > 8) {
    const LadderMasks lm = ladder_masks(n, d.periodic);
    for (int k = tid; k < (1 << (t - 8)); k += NTHREADS) {
      S.offhi[k] = deposit((int64_t)k << 8, d.bits, t);
      S.zpk[k] = zpattern((uint64_t)S.offhi[k], d);
      if (ladk) ladk[k] = (int64_t)(BWD ? ladder_fwd((uint64_t)S.offhi[k], lm) : ladder_inv((uint64_t)S.offhi[k], lm));
    }
  } else if (tid == 0) {
    S.offhi[0] = 0;
    S.zpk[0] = 0;
    if (ladk) ladk[0] = 0;
  }
  if (tid == 0) {
    // bits not in the tile, ascending
    int j = 0, o = 0;
    for (int b = 0; b < n; ++b) {
      if (j < t && d.bits[j] == b)
        ++j;
      else
        S.outside[o++] = (uint8_t)b;
    }
  }
  if (!BWD && d.start == START_MCCLEAN && tid == 0) {
    // Ry(pi/4)|0> = cos(pi/8)|0> + sin(pi/8)|1> on every qubit
    double s8, c8;
    sincospi(0.125, &s8, &c8);
    for (int k = 0; k <= n; ++k) {
      double q = 1.0;
      for (int i = 0; i < n - k; ++i) q *= c8;
      for (int i = 0; i < k; ++i) q *= s8;
      S.startP[k] = q;
    }
  }
  // per-rotation scale factors and Z phases once per CTA, then the table
  if (d.has_diag) {
    for (int i = tid; i < d.nscale; i += NTHREADS) {
      int f;
      double k;
      rot_form(angle_of(d.scale[i], params), &f, &k);
      S.sc[i] = k;
    }
    if (tid < d.nz) {
      sincos(0.5 * angle_of(d.z[tid].a, params), &S.zs[tid], &S.zc[tid]);
      S.zsf[tid] = (float)S.zs[tid];
      S.zcf[tid] = (float)S.zc[tid];
    }
  }
  __syncthreads();
  if (d.has_diag && tid == 0) {
    double K = 1.0;
    for (int i = 0; i < d.nscale; ++i) K *= S.sc[i];
    S.K = K;
  }
  __syncthreads();
  const double K = d.has_diag ? S.K : 1.0;
  const bool fold = d.cost == COST_INT && d.has_diag && d.nz == 0;
  if (d.has_diag && !fold) {
    // exp(-i theta/2) on bit 0, exp(+i theta/2) on bit 1 (state.py:168-170),
    // times the layer scale K; conjugated for the backward sweep
    const int nz = d.nz;
    if (sizeof(R) == 8) {
      // complex128: doubling, 2^nz complex multiplies in all (a product per
      // entry would cost nz times that on the FP64 pipe, in every CTA)
      if (tid == 0) ztab[0] = to_c<C>(make_double2(K, 0.0));
      __syncthreads();
      for (int j = 0; j < nz; ++j) {
        const int h = 1 << j;
        const double zs = BWD ? -S.zs[j] : S.zs[j];
        const C e0 = to_c<C>(make_double2(S.zc[j], -zs)), e1 = to_c<C>(make_double2(S.zc[j], zs));
        for (int pp = tid; pp < h; pp += NTHREADS) {
          const C v = ztab[pp];
          ztab[pp + h] = cmul(v, e1);
          ztab[pp] = cmul(v, e0);
        }
        __syncthreads();
      }
    } else {
      // complex64: a float product per entry, no barriers
      const float Kf = (float)K;
      for (int pat = tid; pat < (1 << nz); pat += NTHREADS) {
        float2 ph = make_float2(Kf, 0.f);
        for (int j = 0; j < nz; ++j) {
          const float zs = ((pat >> j) & 1) ? S.zsf[j] : -S.zsf[j];
          ph = cmul(ph, make_float2(S.zcf[j], BWD ? -zs : zs));
        }
        C v;
        v.x = (R)ph.x;
        v.y = (R)ph.y;
        ztab[pat] = v;
      }
    }
  }
  if (d.cost == COST_INT) {
    // exp(-i gamma w0 m) (times the layer scale when folded)
    const double g = angle_of(d.cost_angle, params) * d.cost_w0;
    const double kf = fold ? K : 1.0;
    const int M = d.cost_maxabs;
    for (int i = tid; i <= 2 * M; i += NTHREADS) {
      double s, c;
      sincos(g * (double)(i - M), &s, &c);
      ctab[i] = to_c<C>(make_double2(kf * c, kf * (BWD ? s : -s)));
    }
  }
  __syncthreads();
}

// Per-amplitude diagonal work of a sweep at index x: the cost phase and the
// merged Z-rotation table (forward tables, or conjugated ones backward).
template <typename C>
__device__ __forceinline__ C apply_diag(C v, uint64_t x, int zpat, const SweepDesc& d, const C* ztab, const C* ctab,
                                        const int32_t* cost_i, const double* cost_d, double gamma, bool fold,
                                        bool bwd) {
  if (d.cost == COST_INT) {
    v = cmul(v, ctab[cost_i[x] + d.cost_maxabs]);
  } else if (d.cost == COST_REAL) {
    double s, c;
    sincos(gamma * cost_d[x], &s, &c);
    v = cmul(v, to_c<C>(make_double2(c, bwd ? s : -s)));
  }
  if (d.has_diag && !fold) {
    if (d.nz)
      v = cmul(v, ztab[zpat]);
    else
      v = cscale(v, ztab[0].x);
  }
  return v;
}

// Warp sums of up to three per-thread values at once (transposed butterfly:
// halves of the values travel at the first two steps), added into this
// warp's slots slot0, slot0+1, slot0+2: 6 adds per lane instead of 15.
template <typename R, int G>
__device__ __forceinline__ void red_add3(SetupShared& S, int slot0, const R* acc) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const R v0 = acc[0], v1 = G > 1 ? acc[1] : (R)0, v2 = G > 2 ? acc[2] : (R)0, v3 = (R)0;
  const bool h16 = lane & 16, h8 = lane & 8;
  R k0 = h16 ? v2 : v0, k1 = h16 ? v3 : v1;
  const R s0 = h16 ? v0 : v2, s1 = h16 ? v1 : v3;
  k0 += __shfl_xor_sync(full, s0, 16);
  k1 += __shfl_xor_sync(full, s1, 16);
  R k = h8 ? k1 : k0;
  const R s = h8 ? k0 : k1;
  k += __shfl_xor_sync(full, s, 8);
  k += __shfl_xor_sync(full, k, 4);
  k += __shfl_xor_sync(full, k, 2);
  k += __shfl_xor_sync(full, k, 1);
  // lanes 0-7: v0, 8-15: v1, 16-23: v2, 24-31: v3
  const int w = threadIdx.x >> 5;
  if (lane == 0) red_slot_add<R>(S, w, slot0, k);
  if (G > 1 && lane == 8) red_slot_add<R>(S, w, slot0 + 1, k);
  if (G > 2 && lane == 16) red_slot_add<R>(S, w, slot0 + 2, k);
}

// add a per-thread value into this warp's reduction slot
template <typename R>
__device__ __forceinline__ void red_add(SetupShared& S, int slot, R v) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) red_slot_add<R>(S, threadIdx.x >> 5, slot, v);
}

// Im<lam|P|psi> pair term: X: Im(conj la qb) + Im(conj lb qa);
// Y: -Re(conj la qb) + Re(conj lb qa)
template <int AXIS, typename C, typename R>
__device__ __forceinline__ R red_pair_t(const C& la, const C& lb, const C& qa, const C& qb, R a) {
  if (AXIS == AX_X) {
    a = fma(la.x, qb.y, a);
    a = fma(-la.y, qb.x, a);
    a = fma(lb.x, qa.y, a);
    a = fma(-lb.y, qa.x, a);
  } else {
    a = fma(-la.x, qb.x, a);
    a = fma(-la.y, qb.y, a);
    a = fma(lb.x, qa.x, a);
    a = fma(lb.y, qa.y, a);
  }
  return a;
}

__device__ __forceinline__ void cp_async_elem(void* dst_smem, const double2* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_elem(void* dst_smem, const float2* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

}  // namespace qg
