// Sweep kernels: forward gate sweeps, adjoint backward sweeps with fused
// gradient reductions, the observable pass, and the gradient finaliser.
//
// Reference mapping (qradient, pure numpy):
//   rotations          physical_components/state.py:90-97, 142-149, 168-175
//   CNOT ladder        physical_components/state.py:209-251
//   observable         physical_components/observable.py:34-73, base.py:17-20
//   McClean grad_run   circuit_logic/mc_clean.py:47-78
//   QAOA grad_run      circuit_logic/qaoa.py:40-70
#include <atomic>
#include <mutex>

#include "qg_internal.cuh"
#include "qg_kernels.h"
#include "qg_sweep_common.cuh"

namespace qg {

// ------------------------------------------------------------ gate groups
//
// The X/Y rotations of a sweep are sorted by local bit.  A group of G of them
// (bits b0 < b1 < b2) is applied with each thread holding the 2^G amplitudes
// of one task (all other tile bits fixed) in registers: one shared-memory
// round trip and one barrier per group instead of per rotation.

template <typename C, typename R, int G, int SG>
__device__ __forceinline__ void apply_group(C* v, C* v2, int tsize, const SweepDesc& d, const SetupShared& S,
                                            int g0) {
  int b[G], ax[G], fm[G];
  R uu[G];
#pragma unroll
  for (int i = 0; i < G; ++i) {
    b[i] = d.xy[g0 + i].lbit;
    ax[i] = d.xy[g0 + i].axis;
    fm[i] = S.form[g0 + i];
    uu[i] = sizeof(R) == 4 ? (R)S.uf[g0 + i] : (R)S.u[g0 + i];
  }
  // complex64: the swizzle is GF(2)-linear, so a task's indices are its
  // swizzled base XOR the swizzled group bits (fewer integer instructions;
  // complex128, bound by the FP64 pipe, keeps the direct form)
  int sbit[sizeof(R) == 4 ? G : 1];
  if constexpr (sizeof(R) == 4) {
#pragma unroll
    for (int i = 0; i < G; ++i) sbit[i] = sw<R>(1 << b[i]);
  }
  const int ntask = tsize >> G;
  for (int tk = threadIdx.x; tk < ntask; tk += NTHREADS) {
    int base = tk;
#pragma unroll
    for (int i = 0; i < G; ++i) base = insert0(base, b[i]);
    int idx[1 << G];
    if constexpr (sizeof(R) == 4) {
      const int sb = sw<R>(base);
#pragma unroll
      for (int c = 0; c < (1 << G); ++c) {
        int x = sb;
#pragma unroll
        for (int i = 0; i < G; ++i)
          if ((c >> i) & 1) x ^= sbit[i];
        idx[c] = x;
      }
    } else {
#pragma unroll
      for (int c = 0; c < (1 << G); ++c) {
        int x = base;
#pragma unroll
        for (int i = 0; i < G; ++i)
          if ((c >> i) & 1) x |= 1 << b[i];
        idx[c] = sw<R>(x);
      }
    }
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
      C* w = pass ? v2 : v;
      if (w == nullptr) break;
      C el[1 << G];
#pragma unroll
      for (int c = 0; c < (1 << G); ++c) el[c] = w[idx[c]];
      rot_block_any<SG, 0, G>(el, ax[0], fm[0], uu[0]);
      if (G > 1) rot_block_any<SG, (G > 1 ? 1 : 0), G>(el, ax[G > 1 ? 1 : 0], fm[G > 1 ? 1 : 0], uu[G > 1 ? 1 : 0]);
      if (G > 2) rot_block_any<SG, (G > 2 ? 2 : 0), G>(el, ax[G > 2 ? 2 : 0], fm[G > 2 ? 2 : 0], uu[G > 2 ? 2 : 0]);
      if (G > 3) rot_block_any<SG, (G > 3 ? 3 : 0), G>(el, ax[G > 3 ? 3 : 0], fm[G > 3 ? 3 : 0], uu[G > 3 ? 3 : 0]);
#pragma unroll
      for (int c = 0; c < (1 << G); ++c) w[idx[c]] = el[c];
    }
  }
}

// Per-thread sums across tiles (ACC): a thread's pair sums of rotation g
// continue in accs[g * NTHREADS + tid] from tile to tile -- loaded into the
// FMA chain and stored back, so no add is spent per tile -- and are summed
// over the CTA's threads once, at its end.  Without ACC each group's sums
// go through a warp reduction per tile (red_add3), whose adds (0.76 per
// amplitude per group of three in complex128) take FP64 pipe slots.

// gradient reductions of a group of G rotations (read-only)
template <typename C, typename R, int G, bool ACC = false>
__device__ __forceinline__ void reduce_group(const C* tl, const C* tp, int tsize, const SweepDesc& d,
                                             SetupShared& S, int g0, R* accs = nullptr) {
  int b[G], ax[G];
  R acc[G];
#pragma unroll
  for (int i = 0; i < G; ++i) {
    b[i] = d.xy[g0 + i].lbit;
    ax[i] = d.xy[g0 + i].axis;
    acc[i] = ACC ? accs[(g0 + i) * NTHREADS + threadIdx.x] : (R)0;
  }
  int sbit[sizeof(R) == 4 ? G : 1];
  if constexpr (sizeof(R) == 4) {
#pragma unroll
    for (int i = 0; i < G; ++i) sbit[i] = sw<R>(1 << b[i]);
  }
  const int ntask = tsize >> G;
  for (int tk = threadIdx.x; tk < ntask; tk += NTHREADS) {
    int base = tk;
#pragma unroll
    for (int i = 0; i < G; ++i) base = insert0(base, b[i]);
    C la[1 << G], qa[1 << G];
    if constexpr (sizeof(R) == 4) {
      const int sb = sw<R>(base);
#pragma unroll
      for (int c = 0; c < (1 << G); ++c) {
        int x = sb;
#pragma unroll
        for (int i = 0; i < G; ++i)
          if ((c >> i) & 1) x ^= sbit[i];
        la[c] = tl[x];
        qa[c] = tp[x];
      }
    } else {
#pragma unroll
      for (int c = 0; c < (1 << G); ++c) {
        int x = base;
#pragma unroll
        for (int i = 0; i < G; ++i)
          if ((c >> i) & 1) x |= 1 << b[i];
        la[c] = tl[sw<R>(x)];
        qa[c] = tp[sw<R>(x)];
      }
    }
#pragma unroll
    for (int i = 0; i < G; ++i) {
      // warp-uniform branch around the whole unrolled block
      if (ax[i] == AX_X) {
#pragma unroll
        for (int c = 0; c < (1 << G); ++c)
          if (!((c >> i) & 1)) acc[i] = red_pair_t<AX_X, C, R>(la[c], la[c | (1 << i)], qa[c], qa[c | (1 << i)], acc[i]);
      } else {
#pragma unroll
        for (int c = 0; c < (1 << G); ++c)
          if (!((c >> i) & 1)) acc[i] = red_pair_t<AX_Y, C, R>(la[c], la[c | (1 << i)], qa[c], qa[c | (1 << i)], acc[i]);
      }
    }
  }
  if constexpr (ACC) {
#pragma unroll
    for (int i = 0; i < G; ++i) accs[(g0 + i) * NTHREADS + threadIdx.x] = acc[i];
  } else {
    red_add3<R, G>(S, RS_XY + g0, acc);
  }
}

// The last gate group of a backward sweep: its gradient reductions and its
// inverse rotations in one pass (each task reads its amplitudes once,
// reduces, rotates lambda -- and psi when PSI -- and writes them back).  The
// reductions of the sweep's other groups must have been taken before: every
// reduction sees lambda and psi before any inverse rotation.
template <typename C, typename R, int G, bool PSI, bool ACC = false>
__device__ __forceinline__ void redrot_group(C* tl, C* tp, int tsize, const SweepDesc& d, SetupShared& S, int g0,
                                             R* accs = nullptr) {
  int b[G], ax[G], fm[G];
  R uu[G], acc[G];
#pragma unroll
  for (int i = 0; i < G; ++i) {
    b[i] = d.xy[g0 + i].lbit;
    ax[i] = d.xy[g0 + i].axis;
    fm[i] = S.form[g0 + i];
    uu[i] = sizeof(R) == 4 ? (R)S.uf[g0 + i] : (R)S.u[g0 + i];
    acc[i] = ACC ? accs[(g0 + i) * NTHREADS + threadIdx.x] : (R)0;
  }
  int sbit[sizeof(R) == 4 ? G : 1];
  if constexpr (sizeof(R) == 4) {
#pragma unroll
    for (int i = 0; i < G; ++i) sbit[i] = sw<R>(1 << b[i]);
  }
  const int ntask = tsize >> G;
  for (int tk = threadIdx.x; tk < ntask; tk += NTHREADS) {
    int base = tk;
#pragma unroll
    for (int i = 0; i < G; ++i) base = insert0(base, b[i]);
    int idx[1 << G];
    if constexpr (sizeof(R) == 4) {
      const int sb = sw<R>(base);
#pragma unroll
      for (int c = 0; c < (1 << G); ++c) {
        int x = sb;
#pragma unroll
        for (int i = 0; i < G; ++i)
          if ((c >> i) & 1) x ^= sbit[i];
        idx[c] = x;
      }
    } else {
#pragma unroll
      for (int c = 0; c < (1 << G); ++c) {
        int x = base;
#pragma unroll
        for (int i = 0; i < G; ++i)
          if ((c >> i) & 1) x |= 1 << b[i];
        idx[c] = sw<R>(x);
      }
    }
    C la[1 << G], qa[1 << G];
#pragma unroll
    for (int c = 0; c < (1 << G); ++c) {
      la[c] = tl[idx[c]];
      qa[c] = tp[idx[c]];
    }
#pragma unroll
    for (int i = 0; i < G; ++i) {
      // warp-uniform branch around the whole unrolled block
      if (ax[i] == AX_X) {
#pragma unroll
        for (int c = 0; c < (1 << G); ++c)
          if (!((c >> i) & 1)) acc[i] = red_pair_t<AX_X, C, R>(la[c], la[c | (1 << i)], qa[c], qa[c | (1 << i)], acc[i]);
      } else {
#pragma unroll
        for (int c = 0; c < (1 << G); ++c)
          if (!((c >> i) & 1)) acc[i] = red_pair_t<AX_Y, C, R>(la[c], la[c | (1 << i)], qa[c], qa[c | (1 << i)], acc[i]);
      }
    }
    rot_block_any<-1, 0, G>(la, ax[0], fm[0], uu[0]);
    if (G > 1) rot_block_any<-1, (G > 1 ? 1 : 0), G>(la, ax[G > 1 ? 1 : 0], fm[G > 1 ? 1 : 0], uu[G > 1 ? 1 : 0]);
    if (G > 2) rot_block_any<-1, (G > 2 ? 2 : 0), G>(la, ax[G > 2 ? 2 : 0], fm[G > 2 ? 2 : 0], uu[G > 2 ? 2 : 0]);
#pragma unroll
    for (int c = 0; c < (1 << G); ++c) tl[idx[c]] = la[c];
    if (PSI) {
      rot_block_any<-1, 0, G>(qa, ax[0], fm[0], uu[0]);
      if (G > 1) rot_block_any<-1, (G > 1 ? 1 : 0), G>(qa, ax[G > 1 ? 1 : 0], fm[G > 1 ? 1 : 0], uu[G > 1 ? 1 : 0]);
      if (G > 2) rot_block_any<-1, (G > 2 ? 2 : 0), G>(qa, ax[G > 2 ? 2 : 0], fm[G > 2 ? 2 : 0], uu[G > 2 ? 2 : 0]);
#pragma unroll
      for (int c = 0; c < (1 << G); ++c) tp[idx[c]] = qa[c];
    }
  }
  if constexpr (ACC) {
#pragma unroll
    for (int i = 0; i < G; ++i) accs[(g0 + i) * NTHREADS + threadIdx.x] = acc[i];
  } else {
    red_add3<R, G>(S, RS_XY + g0, acc);
  }
}

// complex64 forward sweeps: groups of four rotations (16 amplitudes per
// task in registers), one shared-memory round trip fewer per 12 rotations
template <typename C, typename R>
__device__ __forceinline__ void apply_all4(C* v, int tsize, const SweepDesc& d, const SetupShared& S) {
  for (int g0 = 0; g0 < d.nxy; g0 += 4) {
    const int g = d.nxy - g0 < 4 ? d.nxy - g0 : 4;
    if (g == 4)
      apply_group<C, R, 4, 1>(v, nullptr, tsize, d, S, g0);
    else if (g == 3)
      apply_group<C, R, 3, 1>(v, nullptr, tsize, d, S, g0);
    else if (g == 2)
      apply_group<C, R, 2, 1>(v, nullptr, tsize, d, S, g0);
    else
      apply_group<C, R, 1, 1>(v, nullptr, tsize, d, S, g0);
    __syncthreads();
  }
}

template <typename C, typename R, int SG>
__device__ __forceinline__ void apply_all(C* v, C* v2, int tsize, const SweepDesc& d, const SetupShared& S) {
  for (int g0 = 0; g0 < d.nxy; g0 += 3) {
    const int g = d.nxy - g0 < 3 ? d.nxy - g0 : 3;
    if (g == 3)
      apply_group<C, R, 3, SG>(v, v2, tsize, d, S, g0);
    else if (g == 2)
      apply_group<C, R, 2, SG>(v, v2, tsize, d, S, g0);
    else
      apply_group<C, R, 1, SG>(v, v2, tsize, d, S, g0);
    __syncthreads();
  }
}

// ------------------------------------------------------------ forward sweep

template <typename R>
__global__ void __launch_bounds__(NTHREADS) sweep_fwd_kernel(const __grid_constant__ SweepDesc d, SweepPtrs<R> p) {
  using C = typename C2T<R>::T;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ SetupShared S;
  const int t = d.t, n = d.n;
  const int tsize = 1 << t;
  C* tile = (C*)smem;
  C* ztab = tile + tsize;
  C* ctab = ztab + (1 << d.nz);
  __shared__ int64_t ladk[sizeof(R) == 4 ? 32 : 1];  // complex64 only
  sweep_setup<C, false>(d, p.params, S, ztab, ctab, sizeof(R) == 4 ? ladk : nullptr);
  pdl_trigger();
  pdl_wait();

  const int tid = threadIdx.x;
  const LadderMasks lm = ladder_masks(n, d.periodic);
  const int nk = tsize > NTHREADS ? tsize / NTHREADS : 1;
  const bool active = tid < tsize;
  const int64_t dep_lo = active ? deposit(tid, d.bits, t < 8 ? t : 8) : 0;
  const int zpt = zpattern((uint64_t)dep_lo, d);
  // the ladder map is GF(2)-linear: the image of base | dep_lo | offhi[k]
  // is the XOR of the three parts' images
  const uint64_t ldep = ladder_inv((uint64_t)dep_lo, lm);
  const int64_t ntiles = (int64_t)1 << (n - t);
  const R plus = (R)exp2(-0.5 * n);
  const bool fold = d.cost == COST_INT && d.has_diag && d.nz == 0;
  const double gamma = d.cost == COST_REAL ? angle_of(d.cost_angle, p.params) : 0.0;

  for (int64_t tileid = blockIdx.x; tileid < ntiles; tileid += gridDim.x) {
    const int64_t base = deposit(tileid, S.outside, n - t);
    const int zp = zpt | zpattern((uint64_t)base, d);
    const uint64_t lbase = ladder_inv((uint64_t)base, lm) ^ ldep;
    if (active) {
      for (int k = 0; k < nk; ++k) {
        const int e = tid + k * NTHREADS;
        const uint64_t x = (uint64_t)(base | dep_lo | S.offhi[k]);
        // complex64 takes the ladder image from its parts; complex128, bound
        // by the FP64 pipe, computes it (integer work there is free, a
        // shared-memory load is not)
        const uint64_t src =
            d.pre == ENT_CNOT ? (sizeof(R) == 4 ? lbase ^ (uint64_t)ladk[k] : ladder_inv(x, lm)) : x;
        C v;
        if (d.start == START_LOAD) {
          v = p.psi_in[src];
        } else if (d.start == START_MCCLEAN) {
          v.x = (R)S.startP[__popcll(src)];
          v.y = (R)0;
        } else {
          v.x = plus;
          v.y = (R)0;
        }
        if (d.pre == ENT_CZ && cz_negative(x)) v = cneg(v);
        tile[sw<R>(e)] = apply_diag<C>(v, x, zp | S.zpk[k], d, ztab, ctab, p.cost_i, p.cost_d, gamma, fold, false);
      }
    }
    __syncthreads();
    apply_all<C, R, 1>(tile, nullptr, tsize, d, S);
    if (active) {
      for (int k = 0; k < nk; ++k) {
        const int e = tid + k * NTHREADS;
        const uint64_t x = (uint64_t)(base | dep_lo | S.offhi[k]);
        p.psi_out[x] = tile[sw<R>(e)];
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ pipelined forward sweep
//
// The same sweep for an input loaded from memory, with the next tile's loads
// in flight while the current tile is computed: each CTA owns two tile
// buffers; the loads of tile i+1 are issued as asynchronous global->shared
// copies (cp.async, one amplitude each, gathered through the CNOT ladder
// where the sweep starts with it) before tile i's gates run.  The cost phase
// and the CZ sign, which the plain kernel applies on load, run as a pass over
// each thread's own landed elements; a diagonal that commutes with the
// sweep's rotations is applied as the tile is stored.

// TB > 0: an instantiation for tiles of exactly TB bits (the launcher picks
// it when d.t == TB), so that the tile size, the element-loop count and the
// offset between the two tile buffers are compile-time constants: element
// loops unroll and shared-memory offsets become immediates.  TB = 0 takes
// the tile size from the descriptor.
// Three resident CTAs per SM in both precisions (registers capped at 85):
// a complex128 forward sweep with few rotations per amplitude is short of
// FP64 work to overlap its tile loads with, and more CTAs give more.
template <typename R, int TB>
__global__ void __launch_bounds__(NTHREADS, 3) sweep_fwd_pipe_kernel(const __grid_constant__ SweepDesc d,
                                                                  SweepPtrs<R> p) {
  using C = typename C2T<R>::T;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ SetupShared S;
  const int t = TB > 0 ? TB : d.t, n = d.n;
  const int tsize = 1 << t;
  C* buf0 = (C*)smem;
  C* ztab = buf0 + 2 * tsize;
  C* ctab = ztab + (1 << d.nz);
  __shared__ int64_t ladk[sizeof(R) == 4 ? 32 : 1];  // complex64 only
  sweep_setup<C, false>(d, p.params, S, ztab, ctab, sizeof(R) == 4 ? ladk : nullptr);
  pdl_trigger();
  pdl_wait();

  const int tid = threadIdx.x;
  const LadderMasks lm = ladder_masks(n, d.periodic);
  const int nk = tsize > NTHREADS ? tsize / NTHREADS : 1;
  const bool active = tid < tsize;
  const int64_t dep_lo = active ? deposit(tid, d.bits, t < 8 ? t : 8) : 0;
  const int zpt = zpattern((uint64_t)dep_lo, d);
  const int64_t ntiles = (int64_t)1 << (n - t);
  const bool fold = d.cost == COST_INT && d.has_diag && d.nz == 0;
  const double gamma = d.cost == COST_REAL ? angle_of(d.cost_angle, p.params) : 0.0;
  // The cost phase and the CZ sign precede the sweep's rotations and do not
  // commute with them: a pass over the landed tile applies them (with the
  // diagonal).  Otherwise the diagonal (Z rotations on qubits the sweep does
  // not rotate, times the scalar layer scale) commutes with the rotations and
  // is applied as the tile is stored; sweeps with neither skip the pass.
  const bool diag_pass = d.cost != COST_NONE || d.pre == ENT_CZ;
  const bool diag_store = !diag_pass && d.has_diag;

  // Index forms: tile bases by the masked add; an element's shared-memory
  // slot sw(tid + k NTHREADS) = sw(tid) + k NTHREADS (the swizzle mixes bits
  // below 8 only); its global index base | dep_lo | offhi[k] as a per-tile
  // pointer plus offhi[k] (the parts are disjoint).
  TileBases tb(S.outside, n - t, n, d.bits, t);
  const int stid = sw<R>(tid);
  // complex64 fixed tiles: element-loop parts from registers (KParts)
  constexpr bool kRegK = TB > 8 && sizeof(R) == 4;
  constexpr int KB = TB > 8 ? TB - 8 : 1, NK = 1 << KB;

  // copies of one tile into dst: this thread's elements only
  const uint64_t ldep = ladder_inv((uint64_t)dep_lo, lm);  // ladder images are linear: XOR of the parts'
  auto issue = [&](int64_t base, C* dst) {
    if (active) {
      const uint64_t bd = (uint64_t)(base | dep_lo);
      // complex64, limited by its integer and shared-memory instructions,
      // has a loop per case and takes the ladder image from its parts'
      // images; complex128, bound by the FP64 pipe, has one loop that
      // computes the image (measured: a shared-memory load cost more there
      // than the integer work)
      if constexpr (kRegK) {
        if (d.pre == ENT_CNOT) {
          const uint64_t lbase = ladder_inv((uint64_t)base, lm) ^ ldep;
          const KParts<int64_t, KB> L(ladk);
#pragma unroll
          for (int k = 0; k < NK; ++k)
            cp_async_elem(&dst[stid + k * NTHREADS], p.psi_in + (lbase ^ (uint64_t)L.at(k)));
        } else {
          const C* pin = p.psi_in + bd;
          const KParts<int64_t, KB> H(S.offhi);
#pragma unroll
          for (int k = 0; k < NK; ++k) cp_async_elem(&dst[stid + k * NTHREADS], pin + H.sum(k));
        }
      } else if constexpr (sizeof(R) == 4) {
        if (d.pre == ENT_CNOT) {
          const uint64_t lbase = ladder_inv((uint64_t)base, lm) ^ ldep;
          for (int k = 0; k < nk; ++k) cp_async_elem(&dst[stid + k * NTHREADS], p.psi_in + (lbase ^ (uint64_t)ladk[k]));
        } else {
          const C* pin = p.psi_in + bd;
          for (int k = 0; k < nk; ++k) cp_async_elem(&dst[stid + k * NTHREADS], pin + S.offhi[k]);
        }
      } else {
        for (int k = 0; k < nk; ++k) {
          const int64_t oh = S.offhi[k];
          cp_async_elem(&dst[stid + k * NTHREADS],
                        d.pre == ENT_CNOT ? p.psi_in + ladder_inv(bd + (uint64_t)oh, lm) : p.psi_in + bd + oh);
        }
      }
    }
    cp_async_commit();
  };

  int cur = 0;
  int64_t bcur = tb.advance();
  if ((int64_t)blockIdx.x < ntiles) issue(bcur, buf0);
  for (int64_t tileid = blockIdx.x; tileid < ntiles; tileid += gridDim.x) {
    C* tile = buf0 + cur * tsize;
    const int64_t nxt = tileid + gridDim.x;
    const int64_t bnext = tb.advance();
    if (nxt < ntiles)
      issue(bnext, buf0 + (cur ^ 1) * tsize);
    else
      cp_async_commit();  // an empty group keeps the count of pending groups uniform
    cp_async_wait<1>();   // this thread's copies of the current tile have landed
    const int64_t base = bcur;
    const uint64_t bd = (uint64_t)(base | dep_lo);
    const int zp = zpt | zpattern((uint64_t)base, d);
    if (active && diag_pass) {
      for (int k = 0; k < nk; ++k) {
        const int e = stid + k * NTHREADS;
        const uint64_t x = bd + (uint64_t)S.offhi[k];
        C v = tile[e];
        if (d.pre == ENT_CZ && cz_negative(x)) v = cneg(v);
        tile[e] = apply_diag<C>(v, x, zp | S.zpk[k], d, ztab, ctab, p.cost_i, p.cost_d, gamma, fold, false);
      }
    }
    __syncthreads();
    if constexpr (sizeof(R) == 4)
      apply_all4<C, R>(tile, tsize, d, S);
    else
      apply_all<C, R, 1>(tile, nullptr, tsize, d, S);
    if (sizeof(R) == 4 && active && diag_store && d.cost == COST_NONE && d.nz > 0) {
      // complex64, the merged Z table alone: no per-element case tests
      C* out = p.psi_out + bd;
      if constexpr (kRegK) {
        const KParts<int64_t, KB> H(S.offhi);
        const KParts<int, KB> Z(S.zpk);
#pragma unroll
        for (int k = 0; k < NK; ++k) out[H.sum(k)] = cmul(tile[stid + k * NTHREADS], ztab[zp | Z.at(k)]);
      } else {
        for (int k = 0; k < nk; ++k) out[S.offhi[k]] = cmul(tile[stid + k * NTHREADS], ztab[zp | S.zpk[k]]);
      }
    } else if (kRegK && active && !diag_store) {
      C* out = p.psi_out + bd;
      const KParts<int64_t, KB> H(S.offhi);
#pragma unroll
      for (int k = 0; k < NK; ++k) out[H.sum(k)] = tile[stid + k * NTHREADS];
    } else if (active) {
      C* out = p.psi_out + bd;
      if (sizeof(R) == 8 || diag_store) {
        for (int k = 0; k < nk; ++k) {
          const int64_t oh = S.offhi[k];
          const C v = tile[stid + k * NTHREADS];
          out[oh] = diag_store ? apply_diag<C>(v, bd + (uint64_t)oh, zp | S.zpk[k], d, ztab, ctab, p.cost_i,
                                               p.cost_d, gamma, fold, false)
                               : v;
        }
      } else {
        for (int k = 0; k < nk; ++k) out[S.offhi[k]] = tile[stid + k * NTHREADS];
      }
    }
    __syncthreads();  // the buffer is refilled by the copies issued next iteration
    cur ^= 1;
    bcur = bnext;
  }
  cp_async_wait<0>();
}

// ------------------------------------------------------------ backward sweep
//
// Loads lambda and psi at the point after the sweep's gates, accumulates
// Im<lam|P_q|psi> for every rotation of the sweep (the adjoint gradient,
// mc_clean.py:68-77: -2 Re<psi|(-i P/2) lam> = Im<lam|P|psi>), then applies
// the inverse gates to lambda (and to psi when it is uncomputed rather than
// read from the stored history).
//
// Z rotations: S_j = sum_x s_j(x) w_x with w_x = Im(conj(lam_x) psi_x) and
// s_j = +1 on bit 0 is evaluated as T - 2 U_j (T = sum w, U_j = the sum over
// bit j set).  U_j needs a per-element add only when bit j varies inside a
// thread's element loop; otherwise the thread's tile total is added once.

// At least 3 resident CTAs per SM for complex64 (its two tiles take 72 KB
// of shared memory) and 2 for complex128: caps registers at 85 / 128.
template <typename R, bool UNCOMPUTE, int TB>
__global__ void __launch_bounds__(NTHREADS, sizeof(R) == 4 ? 3 : 2) sweep_bwd_kernel(const __grid_constant__ SweepDesc d, SweepPtrs<R> p) {
  using C = typename C2T<R>::T;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ SetupShared S;
  const int t = TB > 0 ? TB : d.t, n = d.n;
  const int tsize = 1 << t;
  C* tl = (C*)smem;
  C* tp = tl + tsize;
  C* ztab = tp + tsize;
  C* ctab = ztab + (1 << d.nz);
  // complex128: per-thread gradient sums kept across tiles in shared memory
  // (reduce_group, ACC); complex64 keeps the per-tile warp reductions (three
  // resident CTAs leave no room for the 13 x 256 sums)
  constexpr bool kAcc = sizeof(R) == 8;
  R* accs = kAcc ? (R*)(ctab + (d.cost == COST_INT ? 2 * d.cost_maxabs + 1 : 0)) : nullptr;
  if constexpr (kAcc) {
    for (int g = 0; g < TMAX; ++g) accs[g * NTHREADS + threadIdx.x] = (R)0;
  }
  __shared__ int64_t ladk[sizeof(R) == 4 ? 32 : 1];  // complex64 only
  sweep_setup<C, true>(d, p.params, S, ztab, ctab, sizeof(R) == 4 ? ladk : nullptr);
  pdl_trigger();
  pdl_wait();

  const int tid = threadIdx.x;
  const LadderMasks lm = ladder_masks(n, d.periodic);
  const int nk = tsize > NTHREADS ? tsize / NTHREADS : 1;
  const bool active = tid < tsize;
  const int64_t dep_lo = active ? deposit(tid, d.bits, t < 8 ? t : 8) : 0;
  const int zpt = zpattern((uint64_t)dep_lo, d);
  const uint64_t ldep = ladder_fwd((uint64_t)dep_lo, lm);  // ladder images are linear: XOR of the parts
  const int64_t ntiles = (int64_t)1 << (n - t);
  const bool fold = d.cost == COST_INT && d.has_diag && d.nz == 0;
  const double gamma = d.cost == COST_REAL ? angle_of(d.cost_angle, p.params) : 0.0;
  const bool need_w = d.nz > 0 || d.gslot >= 0;
  const R w0r = (R)d.cost_w0;
  // Uncomputing psi: the scaled inverse rotations return psi / kappa per
  // rotation, while the forward stored psi with the scale of the forward
  // scaled forms.  Keeping <lam|P|psi> unscaled at every sweep boundary needs
  // psi multiplied by (prod own kappa)^2 (/ K^2 on the diagonal sweep, where
  // the diagonal already multiplies by K).
  R psi_mult = (R)1;
  if (UNCOMPUTE) {
    double own = 1.0;
    for (int g = 0; g < d.nxy; ++g) own *= S.kappa[g];
    double m = own * own;
    if (d.has_diag) m /= S.K * S.K;
    psi_mult = (R)m;
  }

  // Z-rotation sums kept per thread across tiles: the element total T and
  // U per element-loop bit (tile bits 8..t-1); bits inside the thread index
  // are resolved at the end, bits outside the tile per tile.
  R Tacc = (R)0;
  R Uk[5] = {(R)0, (R)0, (R)0, (R)0, (R)0};
  bool any_base = false;
  for (int j = 0; j < d.nz; ++j) any_base |= S.zk[j] == -2;
  // Index forms: tile bases by the masked add; an element's shared-memory
  // slot sw(tid + k NTHREADS) = sw(tid) + k NTHREADS (the swizzle mixes bits
  // below 8 only); its global index base | dep_lo | offhi[k] as a per-tile
  // pointer plus offhi[k] (the parts are disjoint).
  TileBases tb(S.outside, n - t, n, d.bits, t);
  const int stid = sw<R>(tid);
  // The copies of one element of a tile into this thread's slot k: undo the
  // entangler that follows this sweep, (E^{-1} v)[y] = v[A y].  complex64
  // takes the ladder image from its parts' images (fewer integer
  // instructions), complex128 computes it (a shared-memory load costs more
  // there than integer work).
  auto lam_copy = [&](int k, uint64_t bd_, uint64_t lbase_) {
    const int64_t oh = S.offhi[k];
    if (d.lam_undo == ENT_CNOT) {
      const uint64_t ax = sizeof(R) == 4 ? lbase_ ^ (uint64_t)ladk[k] : ladder_fwd(bd_ + (uint64_t)oh, lm);
      cp_async_elem(&tl[stid + k * NTHREADS], p.lam_in + ax);
    } else {
      cp_async_elem(&tl[stid + k * NTHREADS], p.lam_in + bd_ + oh);
    }
  };
  auto psi_copy = [&](int k, uint64_t bd_, uint64_t lbase_) {
    const int64_t oh = S.offhi[k];
    if (d.psi_undo == ENT_CNOT) {
      const uint64_t ax = sizeof(R) == 4 ? lbase_ ^ (uint64_t)ladk[k] : ladder_fwd(bd_ + (uint64_t)oh, lm);
      cp_async_elem(&tp[stid + k * NTHREADS], p.psi_in + ax);
    } else {
      cp_async_elem(&tp[stid + k * NTHREADS], p.psi_in + bd_ + oh);
    }
  };
  // complex64 fixed tiles: the same copies with the element-loop parts from
  // registers (KParts; the loops calling these unroll over k)
  constexpr bool kRegK = TB > 8 && sizeof(R) == 4;
  constexpr int KB = TB > 8 ? TB - 8 : 1, NK = 1 << KB;
  using KP64 = KParts<int64_t, KB>;
  auto lam_copy_r = [&](int k, uint64_t bd_, uint64_t lbase_, const KP64& H, const KP64& L) {
    if (d.lam_undo == ENT_CNOT)
      cp_async_elem(&tl[stid + k * NTHREADS], p.lam_in + (lbase_ ^ (uint64_t)L.at(k)));
    else
      cp_async_elem(&tl[stid + k * NTHREADS], p.lam_in + bd_ + H.sum(k));
  };
  auto psi_copy_r = [&](int k, uint64_t bd_, uint64_t lbase_, const KP64& H, const KP64& L) {
    if (d.psi_undo == ENT_CNOT)
      cp_async_elem(&tp[stid + k * NTHREADS], p.psi_in + (lbase_ ^ (uint64_t)L.at(k)));
    else
      cp_async_elem(&tp[stid + k * NTHREADS], p.psi_in + bd_ + H.sum(k));
  };
  // The next tile's copies go out early, so that their DRAM round trip
  // overlaps the rest of this tile's work: each element's as soon as this
  // thread has stored it (the store pass reads only the thread's own slots,
  // after the last barrier of the cross-thread passes), and in history mode,
  // where psi is only read, psi's already once the last pass that reads psi
  // is done.  A tile's copies touch only that tile (its own elements, or
  // their ladder images in the other buffer of a pair), which no other CTA
  // writes.
  int64_t bnext = tb.advance();
  if (active && (int64_t)blockIdx.x < ntiles) {
    const uint64_t bd0 = (uint64_t)(bnext | dep_lo);
    const uint64_t lb0 = ladder_fwd((uint64_t)bnext, lm) ^ ldep;
    for (int k = 0; k < nk; ++k) {
      lam_copy(k, bd0, lb0);
      psi_copy(k, bd0, lb0);
    }
  }
  cp_async_commit();
  for (int64_t tileid = blockIdx.x; tileid < ntiles; tileid += gridDim.x) {
    const int64_t base = bnext;
    bnext = tb.advance();
    const bool more = tileid + gridDim.x < ntiles;
    const uint64_t bd = (uint64_t)(base | dep_lo);
    const uint64_t bdn = (uint64_t)(bnext | dep_lo);
    const int zp = zpt | zpattern((uint64_t)base, d);
    const uint64_t lbasen = more ? ladder_fwd((uint64_t)bnext, lm) ^ ldep : 0;
    R tT = (R)0, tG = (R)0;
    if (active) {
      // this thread's copies of the tile (issued during the previous tile, all
      // in flight at once) have landed: a load-use loop would wait one
      // memory round trip per element
      cp_async_wait<0>();
      const bool cz_l = d.lam_undo == ENT_CZ, cz_p = d.psi_undo == ENT_CZ;
      if (sizeof(R) == 4 && need_w && !cz_l && !cz_p && d.gslot < 0 && nk >= 4) {
        // complex64, Z sums only: four elements at a time, so that bits 0 and
        // 1 of k are fixed per element and bits 2..4 tested once per four
        // (every U_k is accumulated; those without a Z rotation go unread)
        for (int k0 = 0; k0 < nk; k0 += 4) {
          R w[4];
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const C l = tl[stid + (k0 + c) * NTHREADS];
            const C q = tp[stid + (k0 + c) * NTHREADS];
            w[c] = fma(l.x, q.y, -l.y * q.x);  // Im(conj(l) q)
          }
          const R w13 = w[1] + w[3], w23 = w[2] + w[3];
          const R s4 = (w[0] + w[2]) + w13;
          tT += s4;
          Uk[0] += w13;
          Uk[1] += w23;
          if (k0 & 4) Uk[2] += s4;
          if (k0 & 8) Uk[3] += s4;
          if (k0 & 16) Uk[4] += s4;
        }
      } else if (need_w || cz_l || cz_p) {
        for (int k = 0; k < nk; ++k) {
          const int e = stid + k * NTHREADS;
          const uint64_t x = bd + (uint64_t)S.offhi[k];
          C l = tl[e];
          C q = tp[e];
          const bool neg = (cz_l || cz_p) && cz_negative(x);
          if (cz_l && neg) {
            l = cneg(l);
            tl[e] = l;
          }
          if (cz_p && neg) {
            q = cneg(q);
            tp[e] = q;
          }
          if (need_w) {
            const R w = fma(l.x, q.y, -l.y * q.x);  // Im(conj(l) q)
            tT += w;
#pragma unroll
            for (int i = 0; i < 5; ++i)
              if (((k >> i) & 1) && (S.zkmask >> i) & 1) Uk[i] += w;
            if (d.gslot >= 0) {
              const R cx = d.gcost == COST_INT ? w0r * (R)p.cost_i[x] : (R)p.cost_d[x];
              tG = fma(cx, w, tG);
            }
          }
        }
      }
    }
    if (d.nz > 0) {
      Tacc += tT;
      if (any_base) {
        // Z bits outside the tile: the whole tile's total counts when the bit is set
        const R tot = warp_sum(tT);
        if ((tid & 31) == 0) {
          for (int j = 0; j < d.nz; ++j)
            if (S.zk[j] == -2 && ((base >> d.z[j].gbit) & 1)) red_slot_add<R>(S, tid >> 5, RS_Z + j, tot);
        }
      }
    }
    if (d.gslot >= 0) red_add<R>(S, RS_G, tG);
    __syncthreads();
    // gradient reductions for the X/Y rotations of every group but the last
    // (read-only), then the last group's reductions and inverse rotations in
    // one pass, then the other groups' inverse rotations (they commute, so
    // the group order is free)
    // (complex128 kernels other than the fixed-tile history one keep
    // separate reduction and rotation passes: the fused pass's registers
    // would spill there)
    constexpr bool kFuse = sizeof(R) == 4 || (TB > 0 && !UNCOMPUTE);
    if (!kFuse) {
      for (int g0 = 0; g0 < d.nxy; g0 += 3) {
        const int g = d.nxy - g0 < 3 ? d.nxy - g0 : 3;
        if (g == 3)
          reduce_group<C, R, 3, kAcc>(tl, tp, tsize, d, S, g0, accs);
        else if (g == 2)
          reduce_group<C, R, 2, kAcc>(tl, tp, tsize, d, S, g0, accs);
        else
          reduce_group<C, R, 1, kAcc>(tl, tp, tsize, d, S, g0, accs);
      }
      __syncthreads();
    }
    const int glast = !kFuse ? d.nxy : d.nxy > 0 ? ((d.nxy - 1) / 3) * 3 : 0;
    if (kFuse)
      for (int g0 = 0; g0 < glast; g0 += 3) reduce_group<C, R, 3, kAcc>(tl, tp, tsize, d, S, g0, accs);
    if (kFuse && d.nxy > 0) {
      if (glast > 0) __syncthreads();  // the fused pass rewrites what the reductions above read
      const int g = d.nxy - glast;
      if (g == 3)
        redrot_group<C, R, 3, UNCOMPUTE, kAcc>(tl, tp, tsize, d, S, glast, accs);
      else if (g == 2)
        redrot_group<C, R, 2, UNCOMPUTE, kAcc>(tl, tp, tsize, d, S, glast, accs);
      else
        redrot_group<C, R, 1, UNCOMPUTE, kAcc>(tl, tp, tsize, d, S, glast, accs);
      __syncthreads();
    }
    // history mode: psi is not read again in this tile (every pass above
    // that reads it ended at a barrier): the next tile's psi copies go out now
    if (!UNCOMPUTE && active && more) {
      if constexpr (kRegK) {
        const KP64 H(S.offhi), L(ladk);
#pragma unroll
        for (int k = 0; k < NK; ++k) psi_copy_r(k, bdn, lbasen, H, L);
      } else {
        for (int k = 0; k < nk; ++k) psi_copy(k, bdn, lbasen);
      }
    }
    if (kFuse) {
      for (int g0 = 0; g0 < glast; g0 += 3) {
        apply_group<C, R, 3, -1>(tl, UNCOMPUTE ? tp : nullptr, tsize, d, S, g0);
        __syncthreads();
      }
    } else {
      apply_all<C, R, -1>(tl, UNCOMPUTE ? tp : nullptr, tsize, d, S);
    }
    // (each stored element's slots take the next tile's copies at once: only
    // this thread reads its slots here)
    const bool pf = more;
    if (kRegK && active && !UNCOMPUTE && d.cost == COST_NONE && (!d.has_diag || d.nz > 0)) {
      // the two cases below with the element-loop parts from registers
      C* lout = p.lam_out + bd;
      const KP64 H(S.offhi), L(ladk);
      if (!d.has_diag) {
#pragma unroll
        for (int k = 0; k < NK; ++k) {
          lout[H.sum(k)] = tl[stid + k * NTHREADS];
          if (pf) lam_copy_r(k, bdn, lbasen, H, L);
        }
      } else {
        const KParts<int, KB> Z(S.zpk);
#pragma unroll
        for (int k = 0; k < NK; ++k) {
          lout[H.sum(k)] = cmul(tl[stid + k * NTHREADS], ztab[zp | Z.at(k)]);
          if (pf) lam_copy_r(k, bdn, lbasen, H, L);
        }
      }
    } else if (sizeof(R) == 4 && active && !UNCOMPUTE && !d.has_diag && d.cost == COST_NONE) {
      // nothing diagonal to apply and no psi to write: a plain copy-out
      C* lout = p.lam_out + bd;
      for (int k = 0; k < nk; ++k) {
        lout[S.offhi[k]] = tl[stid + k * NTHREADS];
        if (pf) lam_copy(k, bdn, lbasen);
      }
    } else if (active && !UNCOMPUTE && d.has_diag && d.cost == COST_NONE && d.nz > 0) {
      // the merged Z table alone: no per-element case tests
      C* lout = p.lam_out + bd;
      for (int k = 0; k < nk; ++k) {
        lout[S.offhi[k]] = cmul(tl[stid + k * NTHREADS], ztab[zp | S.zpk[k]]);
        if (pf) lam_copy(k, bdn, lbasen);
      }
    } else if (active) {
      C* lout = p.lam_out + bd;
      C* pout = p.psi_out + bd;
      for (int k = 0; k < nk; ++k) {
        const int e = stid + k * NTHREADS;
        const int64_t oh = S.offhi[k];
        const uint64_t x = bd + (uint64_t)oh;
        const int zpe = zp | S.zpk[k];
        lout[oh] = apply_diag<C>(tl[e], x, zpe, d, ztab, ctab, p.cost_i, p.cost_d, gamma, fold, true);
        if (UNCOMPUTE)
          pout[oh] = cscale(apply_diag<C>(tp[e], x, zpe, d, ztab, ctab, p.cost_i, p.cost_d, gamma, fold, true),
                            psi_mult);
        if (pf) lam_copy(k, bdn, lbasen);
        if (pf && UNCOMPUTE) psi_copy(k, bdn, lbasen);
      }
    }
    cp_async_commit();
    __syncthreads();
  }
  cp_async_wait<0>();

  // X/Y rotations (kAcc): each thread's sums across its tiles into the warp slots
  if constexpr (kAcc) {
    for (int g = 0; g < d.nxy; ++g) {
      const R v = warp_sum(accs[g * NTHREADS + tid]);
      if ((tid & 31) == 0) red_slot_add<R>(S, tid >> 5, RS_XY + g, v);
    }
  }
  // Z rotations: per-thread sums into the warp slots once per CTA
  if (d.nz > 0) {
    for (int j = 0; j < d.nz; ++j) {
      const int zk = S.zk[j];
      R v;
      if (zk >= 0)
        v = Uk[zk < 5 ? zk : 0];
      else if (zk == -1)
        v = (active && ((dep_lo >> d.z[j].gbit) & 1)) ? Tacc : (R)0;  // bit fixed per thread
      else
        continue;  // outside the tile: added per tile
      v = warp_sum(v);
      if ((tid & 31) == 0) red_slot_add<R>(S, tid >> 5, RS_Z + j, v);
    }
    const R tt = warp_sum(Tacc);
    if ((tid & 31) == 0) red_slot_add<R>(S, tid >> 5, RS_T, tt);
  }
  __syncthreads();
  // CTA totals -> partials[slot][blockIdx]
  if (tid < RS_N) {
    int slot = -1;
    double sign = 1.0;
    if (tid < RS_Z) {
      if (tid < d.nxy) slot = d.xy[tid].slot;
    } else if (tid < RS_T) {
      if (tid - RS_Z < d.nz) slot = d.z[tid - RS_Z].slot;
      sign = -2.0;
    } else if (tid == RS_G) {
      slot = d.gslot;
    }
    if (slot >= 0) {
      double s = 0.0, tot = 0.0;
      for (int w = 0; w < NTHREADS / 32; ++w) {
        s += red_slot<R>(S, w, tid);
        tot += red_slot<R>(S, w, RS_T);
      }
      // Z rotations: S_j = T - 2 U_j
      p.partials[(int64_t)slot * p.G + blockIdx.x] = tid >= RS_Z && tid < RS_T ? tot + sign * s : s;
    }
  }
}

// ------------------------------------------------------------ observable
//
// lam = O psi for O = sum of weighted Pauli terms (observable.py:45-73), and
// the partial sums of Re<psi|lam> (base.py:17-20).  X/Y terms need the
// partner amplitude and are taken from the staged tile.
//
// Diagonal terms (Z, ZZ): an element index x = base | dep_lo | offhi[k] has
// three disjoint parts, so a term's sign (-1)^{popc(x & m)} is the sign on
// base | dep_lo (fixed per thread and tile) times the sign on offhi[k]
// (which depends only on the k bits the mask covers).  Per thread and tile
// the terms are summed into b[S], S = the subset of element-loop bits the
// mask covers, and a Walsh-Hadamard transform over those bits gives the
// diagonal of all the thread's elements at once:
//   D(k) = sum_S b[S] (-1)^{popc(S & k)}.
// Per-term work is then per thread and tile, not per element, and integer
// work: the terms of a subset keep the host's order by weight, so the signs
// of a run of equal weights are counted and multiplied once (bit 63 of a
// stored mask marks the last term of a run).  Up to OBS_KBITS element-loop
// bits (16 elements per thread); larger tiles take the per-element loop.

constexpr int OBS_KBITS = 4;
constexpr uint64_t OBS_RUN_END = 1ull << 63;

// Shared-memory layout of the observable kernel after the tile: the thread's
// diagonal values D(k) (one slot per element), then the diagonal terms
// ordered by their k subset (masks, weights) and the subset boundaries.
template <typename R>
struct ObsSmem {
  static size_t bytes(int t, int ndiag) {
    using C = typename C2T<R>::T;
    const size_t tile = ((size_t)1 << t) * sizeof(C);
    const size_t dvals = ((size_t)1 << t) * sizeof(R);
    return tile + dvals + (size_t)ndiag * (sizeof(uint64_t) + sizeof(R)) + ((1 << OBS_KBITS) + 1) * sizeof(int);
  }
};

template <typename R>
__global__ void __launch_bounds__(NTHREADS) observable_kernel(const __grid_constant__ ObsDesc d, const typename C2T<R>::T* psi,
                                                              typename C2T<R>::T* lam, const int32_t* cost_i,
                                                              const double* cost_d, double* partials, int G) {
  using C = typename C2T<R>::T;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int64_t offhi[32];
  __shared__ uint8_t outside[QMAX];
  __shared__ double red[NTHREADS / 32];
  const int t = d.t, n = d.n;
  const int tsize = 1 << t;
  C* tile = (C*)smem;
  R* dval = (R*)(tile + tsize);                   // D(k) of this thread at dval[k * NTHREADS + tid]
  uint64_t* tmask = (uint64_t*)(dval + tsize);    // diagonal terms ordered by k subset
  R* tw = (R*)(tmask + d.ndiag);
  int* tstart = (int*)(tw + d.ndiag);             // subset S: terms [tstart[S], tstart[S + 1])
  const int tid = threadIdx.x;
  const int kb = t > 8 ? t - 8 : 0;               // element-loop bits
  const bool wht = d.ndiag > 0 && d.cost == COST_NONE && kb <= OBS_KBITS;
  if (t > 8) {
    for (int k = tid; k < (1 << (t - 8)); k += NTHREADS) offhi[k] = deposit((int64_t)k << 8, d.bits, t);
  } else if (tid == 0) {
    offhi[0] = 0;
  }
  if (tid == 0) {
    int j = 0, o = 0;
    for (int b = 0; b < n; ++b) {
      if (j < t && d.bits[j] == b)
        ++j;
      else
        outside[o++] = (uint8_t)b;
    }
    if (wht) {
      // counting sort of the diagonal terms by the k bits their mask covers
      int cnt[(1 << OBS_KBITS) + 1] = {0};
      auto subset = [&](const ObsTerm& tm) {
        const uint64_t m = (1ull << tm.b0) | (tm.kind == 3 ? (1ull << tm.b1) : 0ull);
        int sbits = 0;
        for (int i = 0; i < kb; ++i) sbits |= (int)((m >> d.bits[8 + i]) & 1) << i;
        return sbits;
      };
      for (int i = 0; i < d.ndiag; ++i) ++cnt[subset(d.term[i]) + 1];
      for (int sb = 0; sb < (1 << OBS_KBITS); ++sb) cnt[sb + 1] += cnt[sb];
      for (int sb = 0; sb <= (1 << OBS_KBITS); ++sb) tstart[sb] = cnt[sb];
      for (int i = 0; i < d.ndiag; ++i) {
        const ObsTerm& tm = d.term[i];
        const int pos = cnt[subset(tm)]++;
        tmask[pos] = (1ull << tm.b0) | (tm.kind == 3 ? (1ull << tm.b1) : 0ull);
        tw[pos] = sizeof(R) == 4 ? (R)tm.wf : (R)tm.w;
      }
      // the last term of each run of equal weights within a subset
      for (int sb = 0; sb < (1 << OBS_KBITS); ++sb)
        for (int j = tstart[sb]; j < tstart[sb + 1]; ++j)
          if (j + 1 == tstart[sb + 1] || tw[j + 1] != tw[j]) tmask[j] |= OBS_RUN_END;
    }
  }
  __syncthreads();
  pdl_trigger();
  pdl_wait();
  const int nk = tsize > NTHREADS ? tsize / NTHREADS : 1;
  const bool active = tid < tsize;
  const int64_t dep_lo = active ? deposit(tid, d.bits, t < 8 ? t : 8) : 0;
  const int64_t ntiles = (int64_t)1 << (n - t);
  const LadderMasks lm = ladder_masks(n, d.periodic);
  TileBases tb(outside, n - t, n, d.bits, t);
  const int stid = sw<R>(tid);
  double eacc = 0.0;
  const R w0r = (R)d.cost_w0;
  for (int64_t tileid = blockIdx.x; tileid < ntiles; tileid += gridDim.x) {
    const int64_t base = tb.advance();
    const uint64_t bd = (uint64_t)(base | dep_lo);
    if (active) {
      // every load of this thread's elements in flight at once, then one wait
      for (int k = 0; k < nk; ++k) {
        const uint64_t x = bd + (uint64_t)offhi[k];
        cp_async_elem(&tile[stid + k * NTHREADS], psi + (d.pre == ENT_CNOT ? ladder_inv(x, lm) : x));
      }
      cp_async_commit();
      if (wht) {
        // the diagonal of this thread's elements while the loads land
        R b[1 << OBS_KBITS];
#pragma unroll
        for (int sb = 0; sb < (1 << OBS_KBITS); ++sb) {
          R acc = (R)0;
          int cnt = 0;
          for (int j = tstart[sb]; j < tstart[sb + 1]; ++j) {
            const uint64_t m = tmask[j];
            cnt += 1 - 2 * (__popcll(bd & m) & 1);  // bit 63 lies above every index bit
            if (m & OBS_RUN_END) {
              acc = fma(tw[j], (R)cnt, acc);
              cnt = 0;
            }
          }
          b[sb] = acc;
        }
        // butterflies over the kb element-loop bits, on the nk values in use
#pragma unroll
        for (int i = 0; i < OBS_KBITS; ++i)
#pragma unroll
          for (int k = 0; k < (1 << OBS_KBITS); ++k)
            if (!((k >> i) & 1) && i < kb && (k | (1 << i)) < nk) {
              const R u = b[k], v = b[k | (1 << i)];
              b[k] = u + v;
              b[k | (1 << i)] = u - v;
            }
#pragma unroll
        for (int k = 0; k < (1 << OBS_KBITS); ++k)
          if (k < nk) dval[k * NTHREADS + tid] = b[k];
      }
      cp_async_wait<0>();
      if (d.pre == ENT_CZ)
        for (int k = 0; k < nk; ++k) {
          const uint64_t x = bd + (uint64_t)offhi[k];
          if (cz_negative(x)) tile[stid + k * NTHREADS] = cneg(tile[stid + k * NTHREADS]);
        }
    }
    if (d.nxy > 0) __syncthreads();  // X/Y terms read partners other threads loaded
    if (active) {
      R tacc = (R)0;
      for (int k = 0; k < nk; ++k) {
        const int e = tid + k * NTHREADS;
        const uint64_t x = bd + (uint64_t)offhi[k];
        const C v = tile[stid + k * NTHREADS];
        // per-amplitude arithmetic in the state's precision (a double
        // instruction in the complex64 kernel costs 16 cycles of the FP64
        // pipe per warp); the expectation is accumulated in double per tile
        R lx = (R)0, ly = (R)0;
        if (d.cost == COST_INT || d.cost == COST_REAL || d.ndiag > 0) {
          R dv = (R)0;
          if (d.cost == COST_INT) {
            dv = w0r * (R)cost_i[x];
          } else if (d.cost == COST_REAL) {
            dv = (R)cost_d[x];
          } else if (wht) {
            dv = dval[k * NTHREADS + tid];
          } else {
            // integer sign sums per run of equal weights, one multiply per
            // run: the inner loop is integer only, so the compiler cannot
            // predicate the double multiply into every term
            int i = 0;
            while (i < d.ndiag) {
              int cnt = 0;
              bool last;
              R w;
              do {
                const ObsTerm& tm = d.term[i++];
                const uint64_t m = (1ull << tm.b0) | (tm.kind == 3 ? (1ull << tm.b1) : 0ull);
                cnt += 1 - 2 * (__popcll(x & m) & 1);
                last = tm.endgrp;
                w = sizeof(R) == 4 ? (R)tm.wf : (R)tm.w;
              } while (!last && i < d.ndiag);
              dv = fma(w, (R)cnt, dv);
            }
          }
          lx = dv * v.x;
          ly = dv * v.y;
        }
        for (int i = d.ndiag; i < d.ndiag + d.nxy; ++i) {
          const ObsTerm& tm = d.term[i];
          const C u = tile[sw<R>(e ^ (1 << tm.lb0))];
          const R w = sizeof(R) == 4 ? (R)tm.wf : (R)tm.w;
          if (tm.kind == 0) {
            lx = fma(w, u.x, lx);
            ly = fma(w, u.y, ly);
          } else {
            // (Y psi)_x = -i psi_partner (bit 0) or +i psi_partner (bit 1)
            const R sw_ = ((x >> tm.b0) & 1) ? w : -w;
            lx = fma(-sw_, u.y, lx);
            ly = fma(sw_, u.x, ly);
          }
        }
        tacc = fma(v.x, lx, fma(v.y, ly, tacc));
        if (d.store) {
          C o;
          if (d.accumulate) {
            o = lam[x];
            o.x = o.x + lx;
            o.y = o.y + ly;
          } else {
            o.x = lx;
            o.y = ly;
          }
          lam[x] = o;
        }
      }
      eacc += (double)tacc;
    }
    if (d.nxy > 0) __syncthreads();
  }
  const double v = warp_sum(eacc);
  if ((tid & 31) == 0) red[tid >> 5] = v;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < NTHREADS / 32; ++w) s += red[w];
    partials[(int64_t)d.eslot * G + blockIdx.x] = s;
  }
}

// ------------------------------------------------------------ gamma at the start
//
// QAOA: the gamma_0 reduction sits at the start state, which no backward
// sweep loads.  One pass over (lambda, psi_0).
template <typename R>
__global__ void __launch_bounds__(NTHREADS) cost_reduce_kernel(int n, const typename C2T<R>::T* lam,
                                                               const typename C2T<R>::T* psi, int start_plus,
                                                               int cost, double w0, const int32_t* cost_i,
                                                               const double* cost_d, double* partials, int slot,
                                                               int G) {
  __shared__ double red[NTHREADS / 32];
  const int64_t N = (int64_t)1 << n;
  const double plus = exp2(-0.5 * n);
  double acc = 0.0;
  for (int64_t x = (int64_t)blockIdx.x * NTHREADS + threadIdx.x; x < N; x += (int64_t)gridDim.x * NTHREADS) {
    const auto l = lam[x];
    double qx, qy;
    if (start_plus) {
      qx = plus;
      qy = 0.0;
    } else {
      qx = (double)psi[x].x;
      qy = (double)psi[x].y;
    }
    const double w = (double)l.x * qy - (double)l.y * qx;
    const double cx = cost == COST_INT ? w0 * (double)cost_i[x] : cost_d[x];
    acc = fma(cx, w, acc);
  }
  const double v = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < NTHREADS / 32; ++w) s += red[w];
    partials[(int64_t)slot * G + blockIdx.x] = s;
  }
}

// ------------------------------------------------------------ finaliser
//
// grad[p] = factor(p) * sum over the parameter's slots and CTAs, in a fixed
// order (deterministic).  Layout kinds:
//   0 McClean: parameter p <-> slot p
//   1 QAOA:    layer i: beta slots i*(n+1) + q (q < n), gamma slot i*(n+1) + n
//              (factor 2); grad layout [p, 2] with column 0 beta, 1 gamma.
__global__ void finalize_kernel(const double* partials, int G, int kind, int n, int nparam, int eslot, int neslots,
                                double* expec, double* grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && expec) {
    double e = 0.0;
    for (int s = 0; s < neslots; ++s)
      for (int b = 0; b < G; ++b) e += partials[(int64_t)(eslot + s) * G + b];
    *expec = e;
  }
  if (i >= nparam || !grad) return;
  double g = 0.0;
  if (kind == 0) {
    for (int b = 0; b < G; ++b) g += partials[(int64_t)i * G + b];
  } else {
    const int layer = i >> 1;
    if ((i & 1) == 0) {
      for (int q = 0; q < n; ++q)
        for (int b = 0; b < G; ++b) g += partials[(int64_t)(layer * (n + 1) + q) * G + b];
    } else {
      for (int b = 0; b < G; ++b) g += partials[(int64_t)(layer * (n + 1) + n) * G + b];
      g *= 2.0;
    }
  }
  grad[i] = g;
}

// ------------------------------------------------------------ launchers

template <typename R>
static size_t sweep_smem(const SweepDesc& d, bool bwd, bool pipe = false) {
  using C = typename C2T<R>::T;
  size_t s = (size_t)(bwd || pipe ? 2 : 1) * ((size_t)1 << d.t) * sizeof(C);
  s += ((size_t)1 << d.nz) * sizeof(C);
  if (d.cost == COST_INT) s += (size_t)(2 * d.cost_maxabs + 1) * sizeof(C);
  // complex128 backward: the per-thread gradient sums (sweep_bwd_kernel, kAcc)
  if (bwd && sizeof(R) == 8) s += (size_t)TMAX * NTHREADS * sizeof(R);
  return s;
}

// Raise the dynamic shared-memory limit of every kernel of the sweep path
// to what the device allows next to its static shared memory, once per
// device, so that launches need no attribute call.
static cudaError_t set_smem_limit(const void* fn, int optin) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, fn);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)a.sharedSizeBytes);
}

cudaError_t prepare_sweep_kernels() {
  constexpr int kMaxDev = 64;
  static std::atomic<int> ready[kMaxDev];
  static std::mutex mu;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
  if (ready[dev].load(std::memory_order_acquire)) return cudaSuccess;
  std::lock_guard<std::mutex> lock(mu);
  if (ready[dev].load(std::memory_order_relaxed)) return cudaSuccess;
  int optin = 0;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  const void* fns[] = {(const void*)sweep_fwd_kernel<double>,
                       (const void*)sweep_fwd_kernel<float>,
                       (const void*)sweep_fwd_pipe_kernel<double, 0>,
                       (const void*)sweep_fwd_pipe_kernel<float, 0>,
                       (const void*)sweep_fwd_pipe_kernel<float, kTileC64>,
                       (const void*)sweep_fwd_pipe_kernel<double, kTileC128>,
                       (const void*)sweep_bwd_kernel<double, false, 0>,
                       (const void*)sweep_bwd_kernel<double, true, 0>,
                       (const void*)sweep_bwd_kernel<float, false, 0>,
                       (const void*)sweep_bwd_kernel<float, true, 0>,
                       (const void*)sweep_bwd_kernel<float, false, kTileC64>,
                       (const void*)sweep_bwd_kernel<float, true, kTileC64>,
                       (const void*)sweep_bwd_kernel<double, false, kTileC128>,
                       (const void*)sweep_bwd_kernel<double, true, kTileC128>,
                       (const void*)observable_kernel<double>,
                       (const void*)observable_kernel<float>};
  for (const void* fn : fns) {
    e = set_smem_limit(fn, optin);
    if (e != cudaSuccess) return e;
  }
  ready[dev].store(1, std::memory_order_release);
  return cudaSuccess;
}

// The kernel a sweep launches: sweeps over tiles of the default size take
// the instantiation with the tile size fixed at compile time.
template <typename R>
static bool fixed_tile(const SweepDesc& d) {
  return d.t == kTileFixed<R>;
}
template <typename R>
static const void* fwd_pipe_fn(const SweepDesc& d) {
  if (fixed_tile<R>(d)) return (const void*)sweep_fwd_pipe_kernel<R, kTileFixed<R>>;
  return (const void*)sweep_fwd_pipe_kernel<R, 0>;
}
template <typename R>
static const void* bwd_fn(const SweepDesc& d, bool uncompute) {
  if (fixed_tile<R>(d))
    return uncompute ? (const void*)sweep_bwd_kernel<R, true, kTileFixed<R>>
                     : (const void*)sweep_bwd_kernel<R, false, kTileFixed<R>>;
  return uncompute ? (const void*)sweep_bwd_kernel<R, true, 0> : (const void*)sweep_bwd_kernel<R, false, 0>;
}

template <typename R>
int sweep_ctas_per_sm(const SweepDesc& d, bool bwd, bool uncompute, bool pipe) {
  const size_t smem = sweep_smem<R>(d, bwd, pipe && !bwd);
  int blocks = 0;
  cudaError_t e = prepare_sweep_kernels();
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  const void* fn = !bwd && pipe ? fwd_pipe_fn<R>(d) : !bwd ? (const void*)sweep_fwd_kernel<R> : bwd_fn<R>(d, uncompute);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, NTHREADS, smem);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return blocks > 0 ? blocks : 1;
}

template int sweep_ctas_per_sm<double>(const SweepDesc&, bool, bool, bool);
template int sweep_ctas_per_sm<float>(const SweepDesc&, bool, bool, bool);

template <typename R>
cudaError_t launch_sweep_fwd(const SweepDesc& d, const SweepPtrs<R>& p, int grid, cudaStream_t st, bool pipe,
                             bool pdl) {
  cudaError_t e = prepare_sweep_kernels();
  if (e != cudaSuccess) return e;
  if (pipe && d.start == START_LOAD) {
    if (fixed_tile<R>(d))
      return launch_pdl(sweep_fwd_pipe_kernel<R, kTileFixed<R>>, grid, sweep_smem<R>(d, false, true), st, pdl, d, p);
    return launch_pdl(sweep_fwd_pipe_kernel<R, 0>, grid, sweep_smem<R>(d, false, true), st, pdl, d, p);
  }
  return launch_pdl(sweep_fwd_kernel<R>, grid, sweep_smem<R>(d, false), st, pdl, d, p);
}

template <typename R>
cudaError_t launch_sweep_bwd(const SweepDesc& d, const SweepPtrs<R>& p, bool uncompute, int grid, cudaStream_t st,
                             bool pdl) {
  const size_t smem = sweep_smem<R>(d, true);
  cudaError_t e = prepare_sweep_kernels();
  if (e != cudaSuccess) return e;
  if (fixed_tile<R>(d)) {
    if (uncompute) return launch_pdl(sweep_bwd_kernel<R, true, kTileFixed<R>>, grid, smem, st, pdl, d, p);
    return launch_pdl(sweep_bwd_kernel<R, false, kTileFixed<R>>, grid, smem, st, pdl, d, p);
  }
  if (uncompute) return launch_pdl(sweep_bwd_kernel<R, true, 0>, grid, smem, st, pdl, d, p);
  return launch_pdl(sweep_bwd_kernel<R, false, 0>, grid, smem, st, pdl, d, p);
}

template <typename R>
cudaError_t launch_observable(const ObsDesc& d, const typename C2T<R>::T* psi, typename C2T<R>::T* lam,
                              const int32_t* cost_i, const double* cost_d, double* partials, int G, int grid,
                              cudaStream_t st, bool pdl) {
  const size_t smem = ObsSmem<R>::bytes(d.t, d.ndiag);
  cudaError_t e = prepare_sweep_kernels();
  if (e != cudaSuccess) return e;
  return launch_pdl(observable_kernel<R>, grid, smem, st, pdl, d, psi, lam, cost_i, cost_d, partials, G);
}

template <typename R>
cudaError_t launch_cost_reduce(int n, const typename C2T<R>::T* lam, const typename C2T<R>::T* psi, int start_plus,
                               int cost, double w0, const int32_t* cost_i, const double* cost_d, double* partials,
                               int slot, int G, cudaStream_t st) {
  cost_reduce_kernel<R><<<G, NTHREADS, 0, st>>>(n, lam, psi, start_plus, cost, w0, cost_i, cost_d, partials, slot, G);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const double* partials, int G, int kind, int n, int nparam, int eslot, int neslots,
                            double* expec, double* grad, cudaStream_t st) {
  const int threads = 128;
  const int blocks = nparam > 0 ? (nparam + threads - 1) / threads : 1;
  finalize_kernel<<<blocks, threads, 0, st>>>(partials, G, kind, n, nparam, eslot, neslots, expec, grad);
  return cudaGetLastError();
}

template cudaError_t launch_sweep_fwd<double>(const SweepDesc&, const SweepPtrs<double>&, int, cudaStream_t, bool, bool);
template cudaError_t launch_sweep_fwd<float>(const SweepDesc&, const SweepPtrs<float>&, int, cudaStream_t, bool, bool);
template cudaError_t launch_sweep_bwd<double>(const SweepDesc&, const SweepPtrs<double>&, bool, int, cudaStream_t, bool);
template cudaError_t launch_sweep_bwd<float>(const SweepDesc&, const SweepPtrs<float>&, bool, int, cudaStream_t, bool);
template cudaError_t launch_observable<double>(const ObsDesc&, const double2*, double2*, const int32_t*, const double*,
                                               double*, int, int, cudaStream_t, bool);
template cudaError_t launch_observable<float>(const ObsDesc&, const float2*, float2*, const int32_t*, const double*,
                                              double*, int, int, cudaStream_t, bool);
template cudaError_t launch_cost_reduce<double>(int, const double2*, const double2*, int, int, double, const int32_t*,
                                                const double*, double*, int, int, cudaStream_t);
template cudaError_t launch_cost_reduce<float>(int, const float2*, const float2*, int, int, double, const int32_t*,
                                               const double*, double*, int, int, cudaStream_t);

}  // namespace qg
