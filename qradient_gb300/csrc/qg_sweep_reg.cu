// complex64 register-layout sweeps: the forward and adjoint backward sweeps
// over 12-bit tiles (the complex64 default) that rotate only the tile's high
// bits -- the sweeps over the high qubits -- with every amplitude of a tile
// held in registers, 16 per thread, instead of staged in shared memory.
//
// A tile is 4096 amplitudes, local index l = 12 bits (tile bit i is global
// bit d.bits[i]; local bits 0..3 are the state's lowest bits).  A thread
// (lane, warp) of the 256-thread CTA holds 16 of them in one of two layouts:
//   L1: l = lane | warp << 5 | k << 8            in-thread bits 8..11
//   L3: l = (lane & 15) | k << 4 | (lane >> 4) << 8 | warp << 9
//                                                in-thread bits 4..7
// Rotations on in-thread bits need no data movement.  A sweep loads its
// tile from global memory straight into L1 registers (lanes along local bits
// 0..4: coalesced), applies its rotations on bits 8..11, moves to L3 through
// shared memory if it also rotates bits 4..7, and stores from L1 or L3
// (lanes along local bits 0..3: coalesced 128-byte runs).  The sweep over 4
// high bits then costs no shared-memory pass at all and the one over 8 high
// bits one round trip, against a load pass, a store pass and a pass per
// group of rotations in the shared-memory kernels (qg_sweep.cu).
//
// Where they run (measured per sweep at n = 24 on GB300): forward sweeps
// that rotate bits 8..11 only (55 against 59 us), backward sweeps with at
// most one round trip (82 against 94 us; 109 against 119 us).  The sweep
// over the low 12 bits needs two round trips; in this form its unrolled
// per-bit rotation code outgrew the instruction cache and it ran slower
// than the shared-memory kernel, which it keeps.
//
// Arithmetic is that of the shared-memory kernels: the scaled rotation
// forms, the per-sweep diagonal (merged Z table times the layer scale, cost
// phase, CZ sign) at the same point, the CNOT ladder as a gather on load,
// and in the backward sweep Im<lam|P_q|psi> for every rotation of the sweep
// at the sweep's end point (mc_clean.py:68-77, qaoa.py:59-69).  The bits
// 4..7 sums are taken after the bits 8..11 inverse rotations have been
// applied to lambda and psi alike: the rotations of a layer commute with
// each other's Paulis, so the sums are those at the end point, up to the
// factor 1/kappa^2 each unscaled inverse rotation leaves on the product,
// which is multiplied back per CTA.
//
// Reference mapping (qradient, pure numpy):
//   rotations          physical_components/state.py:90-97, 142-149, 168-175
//   CNOT ladder        physical_components/state.py:209-251
//   McClean grad_run   circuit_logic/mc_clean.py:47-78
//   QAOA grad_run      circuit_logic/qaoa.py:40-70
#include "qg_internal.cuh"
#include "qg_kernels.h"
#include "qg_sweep_common.cuh"

namespace qg {

constexpr int RT = 12;        // tile bits
constexpr int RTS = 1 << RT;  // amplitudes per tile
constexpr int RK = 16;        // amplitudes per thread

static_assert(RTS == RK * NTHREADS, "one tile is 16 amplitudes for each of the 256 threads");

// local index of element k of thread (lane, warp) in layout LAY: the thread
// part and the element part occupy disjoint bits
template <int LAY>
struct Lay;
template <>
struct Lay<1> {
  static constexpr int BASE = 8;
  __device__ static __forceinline__ int thr(int lane, int warp) { return lane | (warp << 5); }
  __host__ __device__ static constexpr int kp(int k) { return k << 8; }
};
template <>
struct Lay<3> {
  static constexpr int BASE = 4;
  __device__ static __forceinline__ int thr(int lane, int warp) {
    return (lane & 15) | ((lane >> 4) << 8) | (warp << 9);
  }
  __host__ __device__ static constexpr int kp(int k) { return k << 4; }
};

// the complex64 shared-memory swizzle (sw<float>): GF(2)-linear, so the slot
// of thread part | element part is the XOR of the parts' slots.  In both
// layouts the 16 lanes of a half warp differ in local bits 0..3, which the
// swizzle maps onto 16 distinct 8-byte bank pairs: the 64-bit accesses of a
// round trip are free of bank conflicts.
__host__ __device__ constexpr int swf(int e) { return e ^ ((e >> 4) & 15); }

template <int LAY>
__device__ __forceinline__ void to_smem(float2* buf, const float2* v, int sthr) {
#pragma unroll
  for (int k = 0; k < RK; ++k) buf[sthr ^ swf(Lay<LAY>::kp(k))] = v[k];
}
template <int LAY>
__device__ __forceinline__ void from_smem(const float2* buf, float2* v, int sthr) {
#pragma unroll
  for (int k = 0; k < RK; ++k) v[k] = buf[sthr ^ swf(Lay<LAY>::kp(k))];
}

// Rotation parameters by local bit.
struct RegShared {
  float u[RT];       // scaled-form multiplier
  float kap2[RT];    // kappa^2
  int8_t ax[RT];     // AX_X / AX_Y
  int8_t fm[RT];     // scaled form
  int8_t gate[RT];   // index into d.xy, -1: no rotation on this bit
  int8_t pad[4];
};

// Fill RegShared from the setup (threads 0..11, one bit each; the caller
// synchronises).
__device__ __forceinline__ void reg_setup(const SweepDesc& d, const SetupShared& S, RegShared& R) {
  const int b = threadIdx.x;
  if (b < RT) {
    int g = -1;
    for (int i = 0; i < d.nxy; ++i)
      if (d.xy[i].lbit == b) g = i;
    R.gate[b] = (int8_t)g;
    R.u[b] = g >= 0 ? S.uf[g] : 0.f;
    R.kap2[b] = g >= 0 ? (float)(S.kappa[g] * S.kappa[g]) : 1.f;
    R.ax[b] = g >= 0 ? d.xy[g].axis : 0;
    R.fm[b] = g >= 0 ? (int8_t)S.form[g] : 0;
  }
}

// rotation mask of a sweep by local bit
__host__ __device__ __forceinline__ int rot_mask(const SweepDesc& d) {
  int m = 0;
  for (int i = 0; i < d.nxy; ++i) m |= 1 << d.xy[i].lbit;
  return m;
}

// shared-memory round trips a sweep would need in register layouts: 0
// (rotations on bits 8..11 only), 1 (L1 -> L3: bits 4..7 as well), 2 (bits
// 0..3 as well: a further layout with in-thread bits 0..3)
__host__ __device__ __forceinline__ int reg_transposes(const SweepDesc& d) {
  const int m = rot_mask(d);
  return (m & 0x00f) ? 2 : (m & 0x0f0) ? 1 : 0;
}

// the rotations of one phase (in-thread bits BASE..BASE+3) in registers
template <int SG, int BASE>
__device__ __forceinline__ void rot_phase(float2* v, int mask, const RegShared& R) {
  if (mask & 1) rot_block_any<SG, 0, 4>(v, R.ax[BASE + 0], R.fm[BASE + 0], R.u[BASE + 0]);
  if (mask & 2) rot_block_any<SG, 1, 4>(v, R.ax[BASE + 1], R.fm[BASE + 1], R.u[BASE + 1]);
  if (mask & 4) rot_block_any<SG, 2, 4>(v, R.ax[BASE + 2], R.fm[BASE + 2], R.u[BASE + 2]);
  if (mask & 8) rot_block_any<SG, 3, 4>(v, R.ax[BASE + 3], R.fm[BASE + 3], R.u[BASE + 3]);
}

// Im<lam|P|psi> pair sums of one phase's rotations, into acc[BASE + i]
template <int I>
__device__ __forceinline__ float red_bit(const float2* la, const float2* qa, int axis, float a) {
  if (axis == AX_X) {
#pragma unroll
    for (int c = 0; c < RK; ++c)
      if (!((c >> I) & 1)) a = red_pair_t<AX_X, float2, float>(la[c], la[c | (1 << I)], qa[c], qa[c | (1 << I)], a);
  } else {
#pragma unroll
    for (int c = 0; c < RK; ++c)
      if (!((c >> I) & 1)) a = red_pair_t<AX_Y, float2, float>(la[c], la[c | (1 << I)], qa[c], qa[c | (1 << I)], a);
  }
  return a;
}
template <int BASE>
__device__ __forceinline__ void red_phase(const float2* la, const float2* qa, int mask, const RegShared& R,
                                          float* acc) {
  if (mask & 1) acc[BASE + 0] = red_bit<0>(la, qa, R.ax[BASE + 0], acc[BASE + 0]);
  if (mask & 2) acc[BASE + 1] = red_bit<1>(la, qa, R.ax[BASE + 1], acc[BASE + 1]);
  if (mask & 4) acc[BASE + 2] = red_bit<2>(la, qa, R.ax[BASE + 2], acc[BASE + 2]);
  if (mask & 8) acc[BASE + 3] = red_bit<3>(la, qa, R.ax[BASE + 3], acc[BASE + 3]);
}

// Per-thread index parts of a layout: the global offset of element k is the
// sum of o[i] over its set in-thread bits i (disjoint bits), its Z-table
// pattern the OR of z[i], its ladder image the XOR of lk[i].
struct Parts {
  int64_t o[4];
  int z[4];
};
__device__ __forceinline__ int64_t part_off(const Parts& P, int k) {
  int64_t v = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i)
    if ((k >> i) & 1) v += P.o[i];
  return v;
}
__device__ __forceinline__ int part_z(const Parts& P, int k) {
  int v = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i)
    if ((k >> i) & 1) v |= P.z[i];
  return v;
}
template <int LAY>
__device__ __forceinline__ Parts make_parts(const SweepDesc& d) {
  Parts P;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    P.o[i] = (int64_t)1 << d.bits[Lay<LAY>::BASE + i];
    P.z[i] = zpattern((uint64_t)P.o[i], d);
  }
  return P;
}

// ------------------------------------------------------------ forward

// Sweeps rotating bits 8..11 only: load, rotate and store in L1 registers.
// Three CTAs of 256 threads per SM.
__global__ void __launch_bounds__(NTHREADS, 3) sweep_fwd_reg_kernel(const __grid_constant__ SweepDesc d,
                                                                    SweepPtrs<float> p) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ SetupShared S;
  __shared__ RegShared R;
  __shared__ int64_t ladk[32];
  float2* ztab = (float2*)smem;
  float2* ctab = ztab + (1 << d.nz);
  sweep_setup<float2, false>(d, p.params, S, ztab, ctab, ladk);
  reg_setup(d, S, R);
  __syncthreads();
  pdl_trigger();
  pdl_wait();

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = d.n;
  const LadderMasks lm = ladder_masks(n, d.periodic);
  const int64_t ntiles = (int64_t)1 << (n - RT);
  const bool fold = d.cost == COST_INT && d.has_diag && d.nz == 0;
  const double gamma = d.cost == COST_REAL ? angle_of(d.cost_angle, p.params) : 0.0;
  const bool diag_pass = d.cost != COST_NONE || d.pre == ENT_CZ;
  const bool diag_store = !diag_pass && d.has_diag;
  const int m1 = (rot_mask(d) >> 8) & 15;

  const Parts P1 = make_parts<1>(d);
  const int64_t t1 = deposit(Lay<1>::thr(lane, warp), d.bits, RT);
  const int z1 = zpattern((uint64_t)t1, d);
  int64_t lk[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) lk[i] = (int64_t)ladder_inv((uint64_t)P1.o[i], lm);
  const uint64_t lt1 = ladder_inv((uint64_t)t1, lm);
  TileBases tb(S.outside, n - RT, n, d.bits, RT);

  for (int64_t tileid = blockIdx.x; tileid < ntiles; tileid += gridDim.x) {
    const int64_t base = tb.advance();
    const uint64_t bd = (uint64_t)(base | t1);
    const int zb = zpattern((uint64_t)base, d) | z1;
    float2 v[RK];
    // load in L1, gathered through the CNOT ladder when the sweep starts with it
    if (d.pre == ENT_CNOT) {
      const int64_t lb = (int64_t)(ladder_inv((uint64_t)base, lm) ^ lt1);
#pragma unroll
      for (int k = 0; k < RK; ++k) {
        int64_t s = lb;
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if ((k >> i) & 1) s ^= lk[i];
        v[k] = p.psi_in[s];
      }
    } else {
      const float2* pin = p.psi_in + bd;
#pragma unroll
      for (int k = 0; k < RK; ++k) v[k] = pin[part_off(P1, k)];
    }
    if (diag_pass) {
#pragma unroll
      for (int k = 0; k < RK; ++k) {
        const uint64_t x = bd + (uint64_t)part_off(P1, k);
        float2 e = v[k];
        if (d.pre == ENT_CZ && cz_negative(x)) e = cneg(e);
        v[k] = apply_diag<float2>(e, x, zb | part_z(P1, k), d, ztab, ctab, p.cost_i, p.cost_d, gamma, fold, false);
      }
    }
    rot_phase<1, 8>(v, m1, R);
    // store from L1, with the diagonal when it commutes with the rotations
    float2* out = p.psi_out + bd;
#pragma unroll
    for (int k = 0; k < RK; ++k) {
      const int64_t off = part_off(P1, k);
      float2 e = v[k];
      if (diag_store) {
        const int zp = zb | part_z(P1, k);
        if (d.cost == COST_NONE && d.nz > 0)
          e = cmul(e, ztab[zp]);
        else
          e = apply_diag<float2>(e, bd + (uint64_t)off, zp, d, ztab, ctab, p.cost_i, p.cost_d, gamma, fold, false);
      }
      out[off] = e;
    }
  }
}

// ------------------------------------------------------------ backward

// NT: 0 (rotations on bits 8..11 only) or 1 (bits 4..7 as well: one round
// trip L1 -> L3).  Two CTAs of 256 threads per SM (lambda and psi, 32
// registers each, plus the per-thread sums).  When NT = 1 the two tile
// buffers hold lambda and psi for the round trip; a barrier before it orders
// it after the previous tile's reads.
template <bool UNCOMPUTE, int NT>
__global__ void __launch_bounds__(NTHREADS, 2) sweep_bwd_reg_kernel(const __grid_constant__ SweepDesc d,
                                                                    SweepPtrs<float> p) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ SetupShared S;
  __shared__ RegShared R;
  __shared__ int64_t ladk[32];
  float2* bl = (float2*)smem;
  float2* bp = bl + RTS;
  float2* ztab = bl + (NT > 0 ? 2 * RTS : 0);
  float2* ctab = ztab + (1 << d.nz);
  sweep_setup<float2, true>(d, p.params, S, ztab, ctab, ladk);
  reg_setup(d, S, R);
  __syncthreads();
  pdl_trigger();
  pdl_wait();

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n = d.n;
  const LadderMasks lm = ladder_masks(n, d.periodic);
  const int64_t ntiles = (int64_t)1 << (n - RT);
  const bool fold = d.cost == COST_INT && d.has_diag && d.nz == 0;
  const double gamma = d.cost == COST_REAL ? angle_of(d.cost_angle, p.params) : 0.0;
  const bool need_w = d.nz > 0 || d.gslot >= 0;
  const float w0r = (float)d.cost_w0;
  const int mk = rot_mask(d);
  const int m1 = (mk >> 8) & 15, m3 = (mk >> 4) & 15;
  // psi is inverse-rotated by the bits 8..11 rotations when the bits 4..7
  // sums are taken against it, or when it is uncomputed
  const bool psi1 = UNCOMPUTE || m3;
  // uncomputed psi: see sweep_bwd_kernel (qg_sweep.cu)
  float psi_mult = 1.f;
  if (UNCOMPUTE) {
    double own = 1.0;
    for (int g = 0; g < d.nxy; ++g) own *= S.kappa[g];
    double m = own * own;
    if (d.has_diag) m /= S.K * S.K;
    psi_mult = (float)m;
  }

  const Parts P1 = make_parts<1>(d);
  const int64_t t1 = deposit(Lay<1>::thr(lane, warp), d.bits, RT);
  const int z1 = zpattern((uint64_t)t1, d);
  int64_t lk[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) lk[i] = (int64_t)ladder_fwd((uint64_t)P1.o[i], lm);
  const uint64_t lt1 = ladder_fwd((uint64_t)t1, lm);
  const Parts P3 = make_parts<3>(d);
  const int64_t t3 = deposit(Lay<3>::thr(lane, warp), d.bits, RT);
  const int z3 = zpattern((uint64_t)t3, d);
  const int s1 = swf(Lay<1>::thr(lane, warp)), s3 = swf(Lay<3>::thr(lane, warp));
  TileBases tb(S.outside, n - RT, n, d.bits, RT);

  float acc[RT];
#pragma unroll
  for (int b = 0; b < RT; ++b) acc[b] = 0.f;
  float Tacc = 0.f, Gacc = 0.f;
  float Uk[4] = {0.f, 0.f, 0.f, 0.f};
  bool any_base = false;
  for (int j = 0; j < d.nz; ++j) any_base |= S.zk[j] == -2;

  bool first = true;
  for (int64_t tileid = blockIdx.x; tileid < ntiles; tileid += gridDim.x) {
    const int64_t base = tb.advance();
    const uint64_t bd = (uint64_t)(base | t1);
    const int zb = zpattern((uint64_t)base, d);
    float2 la[RK], qa[RK];
    // load lambda and psi in L1, each gathered through the CNOT ladder when
    // the entangler that follows this sweep is undone on it
    if (d.lam_undo == ENT_CNOT || d.psi_undo == ENT_CNOT) {
      const int64_t lb = (int64_t)(ladder_fwd((uint64_t)base, lm) ^ lt1);
#pragma unroll
      for (int k = 0; k < RK; ++k) {
        int64_t s = lb;
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if ((k >> i) & 1) s ^= lk[i];
        const int64_t x = (int64_t)bd + part_off(P1, k);
        la[k] = p.lam_in[d.lam_undo == ENT_CNOT ? s : x];
        qa[k] = p.psi_in[d.psi_undo == ENT_CNOT ? s : x];
      }
    } else {
      const float2* lin = p.lam_in + bd;
      const float2* pin = p.psi_in + bd;
#pragma unroll
      for (int k = 0; k < RK; ++k) {
        la[k] = lin[part_off(P1, k)];
        qa[k] = pin[part_off(P1, k)];
      }
    }
    if (d.lam_undo == ENT_CZ || d.psi_undo == ENT_CZ) {
#pragma unroll
      for (int k = 0; k < RK; ++k)
        if (cz_negative(bd + (uint64_t)part_off(P1, k))) {
          if (d.lam_undo == ENT_CZ) la[k] = cneg(la[k]);
          if (d.psi_undo == ENT_CZ) qa[k] = cneg(qa[k]);
        }
    }
    // Z-rotation sums (w = Im(conj(lam) psi), S_j = T - 2 U_j) and the QAOA
    // gamma sum at the load point
    if (need_w) {
      float tT = 0.f, tG = 0.f;
#pragma unroll
      for (int k = 0; k < RK; ++k) {
        const float w = fmaf(la[k].x, qa[k].y, -la[k].y * qa[k].x);
        tT += w;
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if ((k >> i) & 1) Uk[i] += w;
        if (d.gslot >= 0) {
          const uint64_t x = bd + (uint64_t)part_off(P1, k);
          const float cx = d.gcost == COST_INT ? w0r * (float)p.cost_i[x] : (float)p.cost_d[x];
          tG = fmaf(cx, w, tG);
        }
      }
      Tacc += tT;
      Gacc += tG;
      if (d.nz > 0 && any_base) {
        // Z bits outside the tile: the whole tile's total counts when the bit is set
        const float tot = warp_sum(tT);
        if (lane == 0)
          for (int j = 0; j < d.nz; ++j)
            if (S.zk[j] == -2 && ((base >> d.z[j].gbit) & 1)) S.redf[warp][RS_Z + j] += tot;
      }
    }
    red_phase<8>(la, qa, m1, R, acc);
    rot_phase<-1, 8>(la, m1, R);
    if (psi1) rot_phase<-1, 8>(qa, m1, R);
    if (NT == 1) {
      if (!first) __syncthreads();
      to_smem<1>(bl, la, s1);
      if (psi1) to_smem<1>(bp, qa, s1);
      __syncthreads();
      from_smem<3>(bl, la, s3);
      if (psi1) from_smem<3>(bp, qa, s3);
    }
    if (NT > 0) {
      red_phase<4>(la, qa, m3, R, acc);
      rot_phase<-1, 4>(la, m3, R);
      if (UNCOMPUTE) rot_phase<-1, 4>(qa, m3, R);
    }
    first = false;
    // store lambda (and the uncomputed psi) from L1 or L3 with the inverse diagonal
    const int64_t bo = base | (NT > 0 ? t3 : t1);
    const int zo = zb | (NT > 0 ? z3 : z1);
    float2* lout = p.lam_out + bo;
    float2* pout = UNCOMPUTE ? p.psi_out + bo : nullptr;
#pragma unroll
    for (int k = 0; k < RK; ++k) {
      const int64_t off = NT > 0 ? part_off(P3, k) : part_off(P1, k);
      const int zp = zo | (NT > 0 ? part_z(P3, k) : part_z(P1, k));
      const uint64_t x = (uint64_t)(bo + off);
      float2 l = la[k];
      if (d.has_diag || d.cost != COST_NONE) {
        if (d.cost == COST_NONE && d.nz > 0)
          l = cmul(l, ztab[zp]);
        else
          l = apply_diag<float2>(l, x, zp, d, ztab, ctab, p.cost_i, p.cost_d, gamma, fold, true);
      }
      lout[off] = l;
      if (UNCOMPUTE)
        pout[off] = cscale(apply_diag<float2>(qa[k], x, zp, d, ztab, ctab, p.cost_i, p.cost_d, gamma, fold, true),
                           psi_mult);
    }
  }

  // per-thread sums into the warp slots once per CTA; the bits 4..7 sums
  // carry 1/kappa^2 of every bits 8..11 rotation already applied to lambda
  // and psi
  float k1 = 1.f;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if ((m1 >> i) & 1) k1 *= R.kap2[8 + i];
  }
#pragma unroll
  for (int b = 4; b < RT; ++b) {
    const int g = R.gate[b];
    if (g < 0) continue;
    const float sc = b >= 8 ? 1.f : k1;
    const float v = warp_sum(acc[b] * sc);
    if (lane == 0) S.redf[warp][RS_XY + g] += v;
  }
  if (d.nz > 0) {
    for (int j = 0; j < d.nz; ++j) {
      const int zk = S.zk[j];
      float v;
      if (zk >= 0)
        v = Uk[zk & 3];
      else if (zk == -1)
        v = ((t1 >> d.z[j].gbit) & 1) ? Tacc : 0.f;  // bit fixed per thread
      else
        continue;  // outside the tile: added per tile
      v = warp_sum(v);
      if (lane == 0) S.redf[warp][RS_Z + j] += v;
    }
    const float tt = warp_sum(Tacc);
    if (lane == 0) S.redf[warp][RS_T] += tt;
  }
  if (d.gslot >= 0) {
    const float gg = warp_sum(Gacc);
    if (lane == 0) S.redf[warp][RS_G] += gg;
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
        s += (double)S.redf[w][tid];
        tot += (double)S.redf[w][RS_T];
      }
      // Z rotations: S_j = T - 2 U_j
      p.partials[(int64_t)slot * p.G + blockIdx.x] = tid >= RS_Z && tid < RS_T ? tot + sign * s : s;
    }
  }
}

// ------------------------------------------------------------ launchers

// Measured per sweep at n=24 (ncu, GB300): the register layout wins where a
// sweep needs few round trips -- forward sweeps with none (55 against
// 59 us), backward sweeps with at most one (82 against 94 us, 109 against
// 119 us).  With two round trips (the 12 rotations of the low-bit sweep)
// its unrolled per-bit rotation code outgrows the instruction cache and
// issue-bound, and the shared-memory kernels (qg_sweep.cu) are faster.
bool reg_sweep_applies(const SweepDesc& d, bool bwd) {
  if (d.t != RT) return false;
  const int nt = reg_transposes(d);
  return bwd ? nt <= 1 : (d.start == START_LOAD && nt == 0);
}

int sweep_occupancy_class(const SweepDesc& d) { return d.t == RT ? reg_transposes(d) : 0; }


// dynamic shared memory: the two round-trip buffers (backward sweeps that
// rotate bits 4..7), the Z table and the cost table
size_t reg_sweep_smem(const SweepDesc& d, bool bwd) {
  size_t s = (bwd && reg_transposes(d) > 0 ? 2 : 0) * (size_t)RTS * sizeof(float2);
  s += ((size_t)1 << d.nz) * sizeof(float2);
  if (d.cost == COST_INT) s += (size_t)(2 * d.cost_maxabs + 1) * sizeof(float2);
  return s;
}

const void* reg_sweep_fn(const SweepDesc& d, bool bwd, bool uncompute) {
  const int nt = reg_transposes(d);
  if (!bwd) return (const void*)sweep_fwd_reg_kernel;
  if (uncompute) return nt == 1 ? (const void*)sweep_bwd_reg_kernel<true, 1> : (const void*)sweep_bwd_reg_kernel<true, 0>;
  return nt == 1 ? (const void*)sweep_bwd_reg_kernel<false, 1> : (const void*)sweep_bwd_reg_kernel<false, 0>;
}

cudaError_t prepare_reg_sweep_kernels(int optin) {
  const void* fns[] = {(const void*)sweep_fwd_reg_kernel, (const void*)sweep_bwd_reg_kernel<false, 0>,
                       (const void*)sweep_bwd_reg_kernel<false, 1>, (const void*)sweep_bwd_reg_kernel<true, 0>,
                       (const void*)sweep_bwd_reg_kernel<true, 1>};
  for (const void* fn : fns) {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, fn);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)a.sharedSizeBytes);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_reg_sweep_fwd(const SweepDesc& d, const SweepPtrs<float>& p, int grid, cudaStream_t st, bool pdl) {
  return launch_pdl(sweep_fwd_reg_kernel, grid, reg_sweep_smem(d, false), st, pdl, d, p);
}

cudaError_t launch_reg_sweep_bwd(const SweepDesc& d, const SweepPtrs<float>& p, bool uncompute, int grid,
                                 cudaStream_t st, bool pdl) {
  const size_t smem = reg_sweep_smem(d, true);
  const int nt = reg_transposes(d);
  if (uncompute) {
    if (nt == 1) return launch_pdl(sweep_bwd_reg_kernel<true, 1>, grid, smem, st, pdl, d, p);
    return launch_pdl(sweep_bwd_reg_kernel<true, 0>, grid, smem, st, pdl, d, p);
  }
  if (nt == 1) return launch_pdl(sweep_bwd_reg_kernel<false, 1>, grid, smem, st, pdl, d, p);
  return launch_pdl(sweep_bwd_reg_kernel<false, 0>, grid, smem, st, pdl, d, p);
}

}  // namespace qg
