// C ABI (include/qgrad.h): circuit plans, workspace layout and the
// forward / adjoint drivers of McClean and QAOA circuits.
//
// Driver structure (history mode, McClean.grad_run, mc_clean.py:47-78):
//   forward:  H[k] = sweep_k(H[k-1])                       (one pass per sweep)
//   E, lam:   lam = O H[last], E = Re<H[last]|lam>         (observable pass)
//   backward: for k = last .. first parameterised sweep:
//               grads of sweep k's rotations from (lam, H[k]), lam <- sweep_k^{-1} lam
//   finalize: grad[p] = sum of the per-CTA partial sums (fixed order)
// Uncompute mode keeps one psi and uncomputes it alongside lam.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cstdlib>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/qgrad.h"
#include "qg_batched.h"
#include "qg_extra.h"
#include "qg_internal.cuh"
#include "qg_kernels.h"
#include "qg_shots.h"

using namespace qg;

namespace {

thread_local std::string g_last_error;

int fail(int status, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

#define QG_CUDA(call)                                                                              \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return fail(QG_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                       __FILE__, __LINE__);                                        \
  } while (0)

struct Term {
  int kind, q0, q1;
  double w;
};

}  // namespace

struct qg_circuit {
  int kind;  // 0 McClean, 1 QAOA
  int n, L;
  std::vector<int8_t> axes;  // McClean [L*n]
  int entangler = QG_ENT_NONE, placement = QG_PLACE_BEFORE;
  std::vector<Term> terms;
  // QAOA classical cost from the Z / ZZ terms
  int cost_kind = COST_NONE;
  double cost_w0 = 1.0;
  int cost_maxabs = 0;
  // tuning per dtype (0 = default): tile bits of a sweep (how many qubits
  // one shared-memory pass fuses) and resident CTAs per SM
  int tune_tile_bits[2] = {0, 0};
  int tune_ctas[2] = {0, 0};
  int tune_flags[2] = {0, 0};  // QG_TUNE_* bits
  // plans (sweep program, workspace layout, observable launches) built on
  // first use per (device, dtype, op, start state) and reused: the host
  // work of a call is then the launches alone
  mutable std::mutex plan_mu;
  mutable std::vector<std::pair<int, std::shared_ptr<const void>>> plans;
  IntTermList* iterms = nullptr;
  RealTermList* rterms = nullptr;
  ~qg_circuit() {
    delete iterms;
    delete rterms;
  }
};

namespace {

int env_int(const char* name, int def) {
  const char* v = getenv(name);
  return v && *v ? atoi(v) : def;
}

struct Layout {
  int t;                                  // tile bits
  std::vector<std::vector<int>> tiles;    // tile bits of each sweep of a layer (canonical: A, B1, ...)
  std::vector<std::vector<int>> active;   // bits whose rotations each sweep applies
};

// Tile plan of one layer: A = bits [0, t); then sweeps over the remaining
// high bits, each padded with the lowest bits (coalesced 128-byte runs).
// Largest tile whose backward sweep (two tiles plus the phase table) fits
// the 227 KB of shared memory a CTA may use.
int max_tile_bits(int dtype) { return dtype == QG_C128 ? TMAX - 1 : TMAX; }

// Forward sweeps that load their input use the double-buffered kernel?
bool fwd_pipelined(const qg_circuit* c, int dtype) {
  const int f = c->tune_flags[dtype == QG_C64 ? 1 : 0];
  if (f & QG_TUNE_FWD_PIPELINED) return true;
  if (f & QG_TUNE_FWD_PLAIN) return false;
  // default on: measured 2.7% (complex128) and 5.5% (complex64) faster
  // per McClean n=24 L=50 grad_run than the single-buffered forward sweeps
  return env_int(dtype == QG_C128 ? "QG_FWD_PIPE_C128" : "QG_FWD_PIPE_C64", 1) != 0;
}

// Sweeps per layer of a layout with t tile bits, c of them kept low in the
// high-bit sweeps for coalescing.
int sweeps_per_layer(int n, int t, int c) { return n <= t ? 1 : 1 + (n - t + (t - c) - 1) / (t - c); }

// Default tile bits: 11 (complex128) / 12 (complex64), the fastest at
// n = 24.  complex128 takes 12 where that saves a sweep per layer (n = 20,
// 21, 28-30): measured 1.032 -> 1.353 circuits/s at n = 28, L = 10 (4 -> 3
// sweeps) and 68.6 -> 69.6 at n = 20, L = 50 (3 -> 2).
int default_tile_bits(int dtype, int n) {
  if (dtype == QG_C128) {
    const int t = env_int("QG_TILE_BITS_C128", 0);
    if (t > 0) return t;
    // (from n = 20 on, where a state spans hundreds of tiles either way)
    return n >= 20 && sweeps_per_layer(n, 12, 3) < sweeps_per_layer(n, 11, 3) ? 12 : 11;
  }
  return env_int("QG_TILE_BITS_C64", 12);
}

// Sweeps per layer with tA tile bits in sweep A and tB in the high-bit sweeps.
int sweeps_per_layer2(int n, int tA, int tB, int c) {
  return n <= tA ? 1 : 1 + (n - tA + (tB - c) - 1) / (tB - c);
}

Layout make_layout(int n, int dtype, int tile_bits) {
  Layout lay;
  int t = tile_bits > 0 ? tile_bits : default_tile_bits(dtype, n);
  const int c = dtype == QG_C128 ? 3 : 4;
  t = std::max(c + 2, std::min(t, max_tile_bits(dtype)));
  // complex128 default with 12-bit tiles: the high-bit sweeps take 11 bits
  // (the compile-time-size kernel, two CTAs per SM) where that costs no
  // sweep per layer (n = 20 and 28); sweep A keeps its 12 bits
  int tb = t;
  if (tile_bits <= 0 && dtype == QG_C128 && t == 12 && env_int("QG_TILE_BITS_C128", 0) == 0 &&
      sweeps_per_layer2(n, 12, 11, c) <= sweeps_per_layer(n, 12, c))
    tb = 11;
  if (n <= t) {
    lay.t = n;
    std::vector<int> all;
    for (int b = 0; b < n; ++b) all.push_back(b);
    lay.tiles.push_back(all);
    lay.active.push_back(all);
    return lay;
  }
  lay.t = t;
  std::vector<int> a;
  for (int b = 0; b < t; ++b) a.push_back(b);
  lay.tiles.push_back(a);
  lay.active.push_back(a);
  int next = t;
  while (next < n) {
    const int k = std::min(tb - c, n - next);
    std::vector<int> bits, act;
    for (int b = 0; b < tb - k; ++b) bits.push_back(b);
    for (int i = 0; i < k; ++i) {
      bits.push_back(next + i);
      act.push_back(next + i);
    }
    next += k;
    lay.tiles.push_back(bits);
    lay.active.push_back(act);
  }
  return lay;
}

int local_of(const std::vector<int>& bits, int b) {
  for (size_t i = 0; i < bits.size(); ++i)
    if (bits[i] == b) return (int)i;
  return -1;
}

AngleRef angle_param(int p, float sign = 1.f) {
  AngleRef a;
  a.param = p;
  a.sign = sign;
  a.fixed = 0.0;
  return a;
}
AngleRef angle_fixed(double v) {
  AngleRef a;
  a.param = -1;
  a.sign = 1.f;
  a.fixed = v;
  return a;
}

SweepDesc blank_sweep(int n, const std::vector<int>& bits) {
  SweepDesc d;
  memset(&d, 0, sizeof d);
  d.n = n;
  d.t = (int)bits.size();
  for (size_t i = 0; i < bits.size(); ++i) d.bits[i] = (uint8_t)bits[i];
  d.gslot = -1;
  for (int i = 0; i < TMAX; ++i) d.xy[i].slot = -1;
  for (int i = 0; i < ZMAX; ++i) d.z[i].slot = -1;
  return d;
}

// One layer of single-qubit rotations (axis[q], angle[q], slot[q]) as
// sweeps, in execution order.  The layer's Z rotations and the scale
// factors of all its X/Y rotations go into one diagonal (ZMAX Z rotations
// per sweep); `ent` is placed before or after the rotations in sweep A.
struct LayerGate {
  int axis;
  AngleRef a;
  int slot;
};

int build_layer(int n, const Layout& lay, const std::vector<LayerGate>& g, int8_t pre, std::vector<SweepDesc>& out) {
  const int ns = (int)lay.tiles.size();
  std::vector<SweepDesc> sw;
  for (int s = 0; s < ns; ++s) sw.push_back(blank_sweep(n, lay.tiles[s]));
  std::vector<int> zq;
  for (int q = 0; q < n; ++q) {
    const int b = n - 1 - q;
    if (g[q].axis == AX_Z) {
      zq.push_back(q);
      continue;
    }
    int s = 0;
    while (s < ns && local_of(lay.active[s], b) < 0) ++s;
    if (s == ns) return fail(QG_ERR_INVALID, "internal: bit %d not covered", b);
    SweepDesc& d = sw[s];
    XYGate& x = d.xy[d.nxy++];
    x.axis = (int8_t)g[q].axis;
    x.lbit = (int8_t)local_of(lay.tiles[s], b);
    x.slot = g[q].slot;
    x.a = g[q].a;
    SweepDesc& d0 = sw[0];
    if (d0.nscale >= QMAX) return fail(QG_ERR_UNSUPPORTED, "too many qubits");
    d0.scale[d0.nscale++] = g[q].a;
    d0.has_diag = 1;
  }
  // Z rotations: chunks of ZMAX into sweeps 0, 1, ...; further chunks get
  // their own diagonal-only sweeps over tile A (Z rotations commute with the
  // other rotations of the layer)
  std::vector<SweepDesc> extra;
  for (size_t i = 0; i < zq.size(); ++i) {
    const int s = (int)(i / ZMAX);
    if (s >= ns + (int)extra.size()) extra.push_back(blank_sweep(n, lay.tiles[0]));
    SweepDesc& d = s < ns ? sw[s] : extra[s - ns];
    const int q = zq[i];
    ZGate& z = d.z[d.nz++];
    z.gbit = (int8_t)(n - 1 - q);
    z.slot = g[q].slot;
    z.a = g[q].a;
    d.has_diag = 1;
  }
  // the rotations of a sweep commute: order them by local bit for the gate groups
  for (auto& d : sw)
    std::sort(d.xy, d.xy + d.nxy, [](const XYGate& a, const XYGate& b) { return a.lbit < b.lbit; });
  sw[0].pre = pre;  // entangler preceding this layer's rotations, gathered on load
  for (auto& d : sw) out.push_back(d);
  for (auto& d : extra) out.push_back(d);
  return QG_OK;
}

struct Program {
  Layout lay;
  std::vector<SweepDesc> sweeps;
  int8_t obs_pre = ENT_NONE;  // entangler between the last sweep and the observable
  int8_t periodic = 0;        // the CNOT ladder is the periodic one
  int first_param = 0;   // first sweep with gradient slots
  int nslots = 0;        // gradient slots (before the expectation slots)
  int grad_kind = 0;     // finalize layout
  int nparams = 0;
};

int build_program(const qg_circuit* c, int dtype, bool with_ini, Program& P) {
  const int n = c->n;
  P.lay = make_layout(n, dtype, c->tune_tile_bits[dtype == QG_C64 ? 1 : 0]);
  P.sweeps.clear();
  if (c->kind == 0) {
    P.nparams = c->L * n;
    P.nslots = P.nparams;
    P.grad_kind = 0;
    if (with_ini) {
      // Ry(pi/4) on every qubit of the caller's state (mc_clean.py:55-56)
      std::vector<LayerGate> g(n);
      for (int q = 0; q < n; ++q) g[q] = LayerGate{AX_Y, angle_fixed(0.78539816339744830962), -1};
      int st = build_layer(n, P.lay, g, ENT_NONE, P.sweeps);
      if (st) return st;
    }
    P.first_param = (int)P.sweeps.size();
    const int8_t e = (c->entangler == QG_ENT_CNOT_LADDER || c->entangler == QG_ENT_CNOT_LADDER_PERIODIC) ? ENT_CNOT
                     : c->entangler == QG_ENT_CZ_LADDER                                          ? ENT_CZ
                                                                                                 : ENT_NONE;
    for (int i = 0; i < c->L; ++i) {
      std::vector<LayerGate> g(n);
      for (int q = 0; q < n; ++q) g[q] = LayerGate{c->axes[i * n + q], angle_param(i * n + q), i * n + q};
      // placement before: E R per layer (mc_clean.py:58-62); after: R E, i.e.
      // E in front of every later layer and once more before the observable
      const int8_t pre = c->placement == QG_PLACE_BEFORE ? e : (i > 0 ? e : ENT_NONE);
      int st = build_layer(n, P.lay, g, pre, P.sweeps);
      if (st) return st;
    }
    if (c->placement == QG_PLACE_AFTER && c->L > 0) P.obs_pre = e;
  } else {
    const int p = c->L;
    P.nparams = 2 * p;
    P.nslots = p * (n + 1);
    P.grad_kind = 1;
    P.first_param = 0;
    for (int i = 0; i < p; ++i) {
      std::vector<LayerGate> g(n);
      for (int q = 0; q < n; ++q) g[q] = LayerGate{AX_X, angle_param(2 * i), i * (n + 1) + q};
      const size_t s0 = P.sweeps.size();
      int st = build_layer(n, P.lay, g, ENT_NONE, P.sweeps);
      if (st) return st;
      SweepDesc& a = P.sweeps[s0];
      a.cost = (int8_t)c->cost_kind;
      a.cost_angle = angle_param(2 * i + 1);
      a.cost_maxabs = c->cost_maxabs;
      a.cost_w0 = c->cost_w0;
      // gamma_{i+1} reduction at the end of layer i (qaoa.py:65-68, moved to
      // the equivalent point before the cost phase of layer i+1)
      if (i + 1 < p) {
        SweepDesc& last = P.sweeps.back();
        last.gslot = (i + 1) * (n + 1) + n;
        last.gcost = (int8_t)c->cost_kind;
        last.cost_w0 = c->cost_w0;
      }
    }
  }
  if (P.sweeps.empty()) {
    // no layers: one empty sweep materialises the start state
    P.sweeps.push_back(blank_sweep(n, P.lay.tiles[0]));
    P.first_param = 1;
  }
  P.periodic = c->kind == 0 && c->entangler == QG_ENT_CNOT_LADDER_PERIODIC;
  for (auto& d : P.sweeps) {
    d.start = START_LOAD;
    d.periodic = P.periodic;
  }
  if (!with_ini) P.sweeps[0].start = c->kind == 0 ? START_MCCLEAN : START_PLUS;
  return QG_OK;
}

int sm_count() {
  static int sms = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                   cudaSuccess)
      sms = 0;
  });
  return sms > 0 ? sms : 1;
}

inline size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

// ------------------------------------------------------------ launch timing
struct Profiler {
  bool on = false;
  std::vector<cudaEvent_t> pool[3];
  size_t used[3] = {0, 0, 0};
  cudaEvent_t get(int cls) {
    auto& p = pool[cls];
    if (used[cls] == p.size()) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
      p.push_back(e);
    }
    return p[used[cls]++];
  }
};
thread_local Profiler g_prof;

struct ProfScope {
  int cls;
  cudaStream_t st;
  ProfScope(int c, cudaStream_t s) : cls(c), st(s) {
    if (g_prof.on) {
      cudaEvent_t e = g_prof.get(cls);
      if (e) cudaEventRecord(e, st);
    }
  }
  ~ProfScope() {
    if (g_prof.on) {
      cudaEvent_t e = g_prof.get(cls);
      if (e) cudaEventRecord(e, st);
    }
  }
};

struct WsLayout {
  size_t partials = 0, lam = 0, psi = 0, cost = 0, total = 0;
  size_t state_bytes = 0;
  int nstates_psi = 0;
  int nstates_lam = 0;
  bool pingpong = false;  // a CNOT-ladder gather needs distinct in / out buffers
  int G = 1, grid_fwd = 1;
  int neslots = 1;
  bool fwd_pipe = false;  // double-buffered forward sweeps
  // per-sweep grids from each sweep's own occupancy (its phase table sets
  // its shared memory); backward grids never exceed G, the width of the
  // partial-sum rows (entries of blocks a sweep does not launch stay zero)
  std::vector<int> grid_fwd_k, grid_bwd_k;
};

int obs_sweeps_needed(const qg_circuit* c, const Layout& lay, bool grad) {
  if (c->kind == 1 && grad) return 1;  // lam = C psi
  int extra = 0;
  std::vector<int> need(lay.tiles.size(), 0);
  for (const auto& tm : c->terms) {
    if (tm.kind == QG_PAULI_X || tm.kind == QG_PAULI_Y) {
      const int b = c->n - 1 - tm.q0;
      if (local_of(lay.tiles[0], b) >= 0) continue;
      for (size_t s = 1; s < lay.tiles.size(); ++s)
        if (local_of(lay.active[s], b) >= 0) need[s] = 1;
    }
  }
  for (size_t s = 1; s < need.size(); ++s) extra += need[s];
  return 1 + extra;
}

WsLayout ws_layout(const qg_circuit* c, int dtype, int op, const Program& P) {
  WsLayout w;
  const int n = c->n;
  const size_t esz = dtype == QG_C128 ? 16 : 8;
  w.state_bytes = ((size_t)1 << n) * esz;
  const int64_t ntiles = (int64_t)1 << (n - P.lay.t);
  const int sms = sm_count();
  // resident CTAs per SM of the largest (shared-memory-wise) sweep
  SweepDesc big = P.sweeps[0];
  for (const auto& d : P.sweeps)
    if (d.nz > big.nz || (d.cost == COST_INT && big.cost != COST_INT)) big = d;
  const bool unc = op == QG_OP_GRAD_UNCOMPUTE;
  int per_bwd = dtype == QG_C128 ? sweep_ctas_per_sm<double>(big, true, unc) : sweep_ctas_per_sm<float>(big, true, unc);
  const bool pipe = fwd_pipelined(c, dtype);
  w.fwd_pipe = pipe;
  int per_fwd = dtype == QG_C128 ? sweep_ctas_per_sm<double>(big, false, false, pipe)
                                 : sweep_ctas_per_sm<float>(big, false, false, pipe);
  const int tuned = c->tune_ctas[dtype == QG_C64 ? 1 : 0];
  if (tuned > 0) {
    // never above what fits: the kernels assume every CTA of the grid is resident
    per_bwd = std::min(per_bwd, tuned);
    per_fwd = std::min(per_fwd, tuned);
  } else {
    per_bwd = env_int("QG_CTAS_PER_SM", per_bwd);
  }
  w.G = (int)std::min<int64_t>(ntiles, (int64_t)sms * per_bwd);
  w.grid_fwd = (int)std::min<int64_t>(ntiles, (int64_t)sms * per_fwd);
  {
    // occupancy per distinct shared-memory footprint (phase-table size, cost table)
    std::vector<std::pair<int64_t, std::pair<int, int>>> memo;
    for (const auto& d : P.sweeps) {
      const int64_t key = ((int64_t)d.t << 40) | ((int64_t)d.nz << 32) | ((int64_t)(d.cost == COST_INT ? 1 : 0) << 31) |
                          d.cost_maxabs;
      int pf = -1, pb = -1;
      for (const auto& mm : memo)
        if (mm.first == key) {
          pf = mm.second.first;
          pb = mm.second.second;
        }
      if (pf < 0) {
        pf = dtype == QG_C128 ? sweep_ctas_per_sm<double>(d, false, false, pipe)
                              : sweep_ctas_per_sm<float>(d, false, false, pipe);
        pb = dtype == QG_C128 ? sweep_ctas_per_sm<double>(d, true, unc) : sweep_ctas_per_sm<float>(d, true, unc);
        if (tuned > 0) {
          pf = std::min(pf, tuned);
          pb = std::min(pb, tuned);
        } else {
          pb = env_int("QG_CTAS_PER_SM", pb);
        }
        memo.push_back({key, {pf, pb}});
      }
      const int64_t nt = (int64_t)1 << (n - d.t);  // this sweep's tiles (high-bit sweeps may be smaller)
      w.grid_fwd_k.push_back((int)std::min<int64_t>(nt, (int64_t)sms * pf));
      w.grid_bwd_k.push_back((int)std::min<int64_t>(nt, (int64_t)sms * pb));
    }
    for (int g : w.grid_bwd_k) w.G = std::max(w.G, g);
  }
  w.neslots = obs_sweeps_needed(c, P.lay, op != QG_OP_RUN);
  const int m = (int)P.sweeps.size();
  w.pingpong = P.obs_pre == ENT_CNOT;
  for (const auto& d : P.sweeps) w.pingpong = w.pingpong || d.pre == ENT_CNOT;
  const int two = w.pingpong ? 2 : 1;
  if (op == QG_OP_GRAD_HISTORY)
    w.nstates_psi = m;
  else
    w.nstates_psi = two;
  w.nstates_lam = op == QG_OP_RUN ? 0 : two;
  size_t off = 0;
  w.partials = off;
  off += align_up((size_t)(P.nslots + w.neslots) * w.G * sizeof(double));
  w.lam = off;
  off += align_up((size_t)w.nstates_lam * w.state_bytes);
  w.psi = off;
  off += align_up((size_t)w.nstates_psi * w.state_bytes);
  w.cost = off;
  if (c->kind == 1) {
    if (c->cost_kind == COST_INT)
      off += align_up(((size_t)1 << n) * sizeof(int32_t));
    else if (c->cost_kind == COST_REAL)
      off += align_up(((size_t)1 << n) * sizeof(double));
  }
  w.total = off;
  return w;
}

int check_circuit(const qg_circuit* c) {
  if (!c) return fail(QG_ERR_INVALID, "null circuit");
  return QG_OK;
}

std::vector<ObsDesc> build_obs(const qg_circuit* c, const Program& P, bool grad, bool store,
                               const std::vector<Term>* terms);

struct Plan {
  Program P;
  WsLayout W;
  std::vector<ObsDesc> obs;  // observable launches (lam stored for gradient ops)
};

// The cached plan of (current device, dtype, op, with_ini); built on first use.
int get_plan(const qg_circuit* c, int dtype, int op, bool with_ini, std::shared_ptr<const Plan>& out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    dev = 0;
  }
  const int key = ((dev * 2 + dtype) * 4 + op) * 2 + (with_ini ? 1 : 0);
  {
    std::lock_guard<std::mutex> lock(c->plan_mu);
    for (const auto& kv : c->plans)
      if (kv.first == key) {
        out = std::static_pointer_cast<const Plan>(kv.second);
        return QG_OK;
      }
  }
  auto plan = std::make_shared<Plan>();
  if (int s = build_program(c, dtype, with_ini, plan->P)) return s;
  plan->W = ws_layout(c, dtype, op, plan->P);
  plan->obs = build_obs(c, plan->P, op != QG_OP_RUN, op != QG_OP_RUN, nullptr);
  std::lock_guard<std::mutex> lock(c->plan_mu);
  c->plans.emplace_back(key, plan);
  out = plan;
  return QG_OK;
}

void clear_plans(const qg_circuit* c) {
  std::lock_guard<std::mutex> lock(c->plan_mu);
  c->plans.clear();
}

int build_cost(const qg_circuit* c, char* ws, const WsLayout& W, cudaStream_t st) {
  if (c->kind != 1) return QG_OK;
  const int grid = sm_count() * 8;
  if (c->cost_kind == COST_INT) {
    QG_CUDA(launch_int_cost(c->n, *c->iterms, (int32_t*)(ws + W.cost), grid, st));
  } else if (c->cost_kind == COST_REAL) {
    QG_CUDA(launch_real_cost(c->n, *c->rterms, (double*)(ws + W.cost), grid, st));
  }
  return QG_OK;
}

// Observable passes: lam = O psi (store) and the expectation partial sums.
// `terms` replaces the circuit's observable (the sampled component of
// grad_run_with_component_sampling); null means the circuit's own terms.
// Built on the host once per plan; launched by run_observable.
std::vector<ObsDesc> build_obs(const qg_circuit* c, const Program& P, bool grad, bool store,
                               const std::vector<Term>* terms) {
  const int n = c->n;
  std::vector<ObsDesc> out;
  const Layout& lay = P.lay;
  const int eslot0 = P.nslots;
  auto fresh = [&](int s) {
    out.emplace_back();
    ObsDesc* d = &out.back();
    memset(d, 0, sizeof *d);
    d->n = n;
    d->t = (int)lay.tiles[s].size();
    for (size_t i = 0; i < lay.tiles[s].size(); ++i) d->bits[i] = (uint8_t)lay.tiles[s][i];
    d->store = store;
    d->pre = P.obs_pre;
    d->periodic = P.periodic;
    return d;
  };
  if (c->kind == 1 && grad) {
    // lam = C psi with the classical cost (qaoa.py:56-57)
    ObsDesc* d = fresh(0);
    d->cost = (int8_t)c->cost_kind;
    d->cost_w0 = c->cost_w0;
    d->eslot = eslot0;
    return out;
  }
  // diagonal terms sorted by weight, then X/Y terms of tile A
  std::vector<Term> diag, xy;
  for (const auto& tm : terms ? *terms : c->terms) (tm.kind >= QG_PAULI_Z ? diag : xy).push_back(tm);
  std::stable_sort(diag.begin(), diag.end(), [](const Term& a, const Term& b) { return a.w < b.w; });
  int es = 0;
  for (size_t s = 0; s < lay.tiles.size(); ++s) {
    ObsDesc* d = fresh((int)s);
    int k = 0;
    if (s == 0) {
      for (const auto& tm : diag) {
        ObsTerm& o = d->term[k++];
        o.kind = (int8_t)tm.kind;
        o.b0 = (int8_t)(n - 1 - tm.q0);
        o.b1 = (int8_t)(tm.kind == QG_PAULI_ZZ ? n - 1 - tm.q1 : 0);
        o.w = tm.w;
        o.wf = (float)tm.w;
      }
      d->ndiag = k;
      // weight runs (the terms are sorted by weight): the kernel sums the
      // signs of a run in integers and multiplies by the weight once
      for (int i = 0; i < k; ++i) d->term[i].endgrp = (int8_t)(i + 1 == k || d->term[i + 1].w != d->term[i].w);
    }
    int nxy = 0;
    for (const auto& tm : xy) {
      const int b = n - 1 - tm.q0;
      const bool mine = s == 0 ? local_of(lay.tiles[0], b) >= 0
                               : (local_of(lay.tiles[0], b) < 0 && local_of(lay.active[s], b) >= 0);
      if (!mine) continue;
      ObsTerm& o = d->term[k++];
      o.kind = (int8_t)tm.kind;
      o.b0 = (int8_t)b;
      o.lb0 = (int8_t)local_of(lay.tiles[s], b);
      o.w = tm.w;
        o.wf = (float)tm.w;
      ++nxy;
    }
    d->nxy = nxy;
    if (s > 0 && nxy == 0) {
      out.pop_back();
      continue;
    }
    d->accumulate = s > 0;
    d->eslot = eslot0 + es++;
  }
  return out;
}

template <typename R>
// after_sweep: the previous launch in the stream is a sweep or observable
// launch, so the first pass may start as its programmatic dependent.
int run_observable(const std::vector<ObsDesc>& obs, const WsLayout& W, const typename C2T<R>::T* psi,
                   typename C2T<R>::T* lam, char* ws, cudaStream_t st, bool after_sweep) {
  double* partials = (double*)(ws + W.partials);
  const int32_t* ci = (const int32_t*)(ws + W.cost);
  const double* cd = (const double*)(ws + W.cost);
  bool pdl = after_sweep;
  for (const ObsDesc& d : obs) {
    ProfScope ps(2, st);
    QG_CUDA(launch_observable<R>(d, psi, lam, ci, cd, partials, W.G, W.G, st, pdl));
    pdl = true;
  }
  return QG_OK;
}

template <typename R>
int forward(const qg_circuit* c, const Program& P, const WsLayout& W, const double* params, const void* ini,
            bool history, char* ws, cudaStream_t st, const typename C2T<R>::T** final_state) {
  using C = typename C2T<R>::T;
  SweepPtrs<R> p;
  memset(&p, 0, sizeof p);
  p.params = params;
  p.cost_i = (const int32_t*)(ws + W.cost);
  p.cost_d = (const double*)(ws + W.cost);
  p.partials = (double*)(ws + W.partials);
  p.G = W.G;
  const size_t N = (size_t)1 << c->n;
  C* buf[2] = {(C*)(ws + W.psi), W.pingpong && !history ? (C*)(ws + W.psi) + N : nullptr};
  int cur = 0;
  const int m = (int)P.sweeps.size();
  const C* in = (const C*)ini;
  for (int k = 0; k < m; ++k) {
    C* out;
    if (history) {
      out = buf[0] + (size_t)k * N;
    } else {
      // in place, except that a ladder gather reads other tiles: write the other buffer
      if (P.sweeps[k].pre == ENT_CNOT && in == buf[cur]) cur ^= 1;
      out = buf[cur];
    }
    p.psi_in = in;
    p.psi_out = out;
    ProfScope ps(0, st);
    // every sweep but the first follows a sweep launch: programmatic dependent
    QG_CUDA(launch_sweep_fwd<R>(P.sweeps[k], p, W.grid_fwd_k[k], st, W.fwd_pipe, k > 0));
    in = out;
  }
  *final_state = in;
  return QG_OK;
}

template <typename R>
int do_run(const qg_circuit* c, const double* params, const void* ini, char* ws, size_t wsb, double* expec,
           void* state_out, cudaStream_t st, int dtype) {
  using C = typename C2T<R>::T;
  std::shared_ptr<const Plan> plan;
  int s = get_plan(c, dtype, QG_OP_RUN, ini != nullptr, plan);
  if (s) return s;
  const Program& P = plan->P;
  const WsLayout& W = plan->W;
  if (wsb < W.total) return fail(QG_ERR_WORKSPACE, "workspace %zu bytes < %zu needed", wsb, W.total);
  s = build_cost(c, ws, W, st);
  if (s) return s;
  const C* fin = nullptr;
  s = forward<R>(c, P, W, params, ini, false, ws, st, &fin);
  if (s) return s;
  s = run_observable<R>(plan->obs, W, fin, nullptr, ws, st, !P.sweeps.empty());
  if (s) return s;
  QG_CUDA(launch_finalize((double*)(ws + W.partials), W.G, 0, c->n, 0, P.nslots, W.neslots, expec, nullptr, st));
  if (state_out) QG_CUDA(cudaMemcpyAsync(state_out, fin, W.state_bytes, cudaMemcpyDeviceToDevice, st));
  return QG_OK;
}

// component >= 0: the gradient of the single observable term `component`
// (weight included), with E still the full expectation value.
template <typename R>
int do_grad(const qg_circuit* c, int op, const double* params, const void* ini, char* ws, size_t wsb, double* expec,
            double* grad, cudaStream_t st, int dtype, int component = -1) {
  using C = typename C2T<R>::T;
  std::shared_ptr<const Plan> plan;
  int s = get_plan(c, dtype, op, ini != nullptr, plan);
  if (s) return s;
  const Program& P = plan->P;
  const WsLayout& W = plan->W;
  if (wsb < W.total) return fail(QG_ERR_WORKSPACE, "workspace %zu bytes < %zu needed", wsb, W.total);
  const bool history = op == QG_OP_GRAD_HISTORY;
  QG_CUDA(cudaMemsetAsync(ws + W.partials, 0, (size_t)(P.nslots + W.neslots) * W.G * sizeof(double), st));
  s = build_cost(c, ws, W, st);
  if (s) return s;
  const C* fin = nullptr;
  s = forward<R>(c, P, W, params, ini, history, ws, st, &fin);
  if (s) return s;
  const size_t N = (size_t)1 << c->n;
  C* lbuf[2] = {(C*)(ws + W.lam), W.pingpong ? (C*)(ws + W.lam) + N : nullptr};
  C* pbuf[2] = {(C*)(ws + W.psi), W.pingpong && !history ? (C*)(ws + W.psi) + N : nullptr};
  int lc = 0, pc = 0;
  if (!history) pc = fin == pbuf[1] ? 1 : 0;
  if (component >= 0) {
    // lam = w_k P_k psi (mc_clean.py:103-105); its expectation slots are then
    // overwritten by the full-observable pass, which writes at least the
    // same slots, so E stays <psi|O|psi> (mc_clean.py:99-100)
    const std::vector<Term> one(1, c->terms[component]);
    s = run_observable<R>(build_obs(c, P, true, true, &one), W, fin, lbuf[lc], ws, st, !P.sweeps.empty());
    if (s) return s;
    s = run_observable<R>(build_obs(c, P, false, false, nullptr), W, fin, nullptr, ws, st, true);
  } else {
    s = run_observable<R>(plan->obs, W, fin, lbuf[lc], ws, st, !P.sweeps.empty());
  }
  if (s) return s;
  SweepPtrs<R> p;
  memset(&p, 0, sizeof p);
  p.params = params;
  p.cost_i = (const int32_t*)(ws + W.cost);
  p.cost_d = (const double*)(ws + W.cost);
  p.partials = (double*)(ws + W.partials);
  p.G = W.G;
  C* psi0 = (C*)(ws + W.psi);
  const int m = (int)P.sweeps.size();
  for (int k = m - 1; k >= P.first_param; --k) {
    SweepDesc d = P.sweeps[k];
    // undo, on load, the entangler the forward applied right after sweep k
    d.lam_undo = k + 1 < m ? P.sweeps[k + 1].pre : P.obs_pre;
    d.psi_undo = history ? ENT_NONE : (k + 1 < m ? P.sweeps[k + 1].pre : ENT_NONE);
    p.lam_in = lbuf[lc];
    if (d.lam_undo == ENT_CNOT) lc ^= 1;
    p.lam_out = lbuf[lc];
    if (history) {
      p.psi_in = psi0 + (size_t)k * N;
      p.psi_out = nullptr;
    } else {
      p.psi_in = pbuf[pc];
      if (d.psi_undo == ENT_CNOT) pc ^= 1;
      p.psi_out = pbuf[pc];
    }
    ProfScope ps(1, st);
    // follows the observable pass or the previous backward sweep
    QG_CUDA(launch_sweep_bwd<R>(d, p, !history, W.grid_bwd_k[k], st, true));
  }
  C* lam = lbuf[lc];
  if (c->kind == 1 && c->L > 0) {
    // gamma_0 at the start state (qaoa.py:65-68 for i = 0)
    const C* psi_start = history ? (const C*)ini : (ini ? pbuf[pc] : nullptr);
    QG_CUDA(launch_cost_reduce<R>(c->n, lam, psi_start, psi_start == nullptr, c->cost_kind, c->cost_w0,
                                  p.cost_i, p.cost_d, p.partials, 0 * (c->n + 1) + c->n, W.G, st));
  }
  QG_CUDA(launch_finalize(p.partials, W.G, P.grad_kind, c->n, P.nparams, P.nslots, W.neslots, expec, grad, st));
  return QG_OK;
}

int parse_terms(int n, int nterms, const int32_t* kind, const int32_t* q0, const int32_t* q1, const double* w,
                std::vector<Term>& out) {
  if (nterms < 0) return fail(QG_ERR_INVALID, "negative term count");
  if (nterms > 0 && (!kind || !q0 || !w)) return fail(QG_ERR_INVALID, "null term arrays");
  for (int k = 0; k < nterms; ++k) {
    Term t{kind[k], q0[k], q1 ? q1[k] : q0[k], w[k]};
    if (t.kind < 0 || t.kind > 3) return fail(QG_ERR_INVALID, "term %d: unknown kind %d", k, t.kind);
    if (t.q0 < 0 || t.q0 >= n) return fail(QG_ERR_INVALID, "term %d: qubit %d out of range", k, t.q0);
    if (t.kind == QG_PAULI_ZZ && (t.q1 <= t.q0 || t.q1 >= n))
      return fail(QG_ERR_INVALID, "term %d: zz needs q0 < q1 < n (upper triangle, observable.py:57-64)", k);
    if (!std::isfinite(t.w)) return fail(QG_ERR_INVALID, "term %d: non-finite weight", k);
    out.push_back(t);
  }
  if ((int)out.size() > OBS_MAX_TERMS) return fail(QG_ERR_UNSUPPORTED, "more than %d observable terms", OBS_MAX_TERMS);
  return QG_OK;
}

}  // namespace

namespace qg {
int set_last_error(int status, const char* msg) { return fail(status, "%s", msg); }
}  // namespace qg

extern "C" {

int qg_version(void) { return 1; }

const char* qg_status_string(int s) {
  switch (s) {
    case QG_OK:
      return "ok";
    case QG_ERR_INVALID:
      return "invalid argument";
    case QG_ERR_CUDA:
      return "CUDA error";
    case QG_ERR_WORKSPACE:
      return "workspace too small";
    case QG_ERR_UNSUPPORTED:
      return "unsupported";
    case QG_ERR_HOST_MEMORY:
      return "host memory";
  }
  return "unknown status";
}

const char* qg_last_error(void) { return g_last_error.c_str(); }

int qg_profile_enable(int on) {
  g_prof.on = on != 0;
  for (int c = 0; c < 3; ++c) g_prof.used[c] = 0;
  return QG_OK;
}

int qg_profile_collect(int cls, double* total_ms, int* launches) {
  if (cls < 0 || cls > 2 || !total_ms || !launches) return fail(QG_ERR_INVALID, "bad profile query");
  const size_t used = g_prof.used[cls];
  double ms = 0.0;
  for (size_t i = 0; i + 1 < used; i += 2) {
    QG_CUDA(cudaEventSynchronize(g_prof.pool[cls][i + 1]));
    float f = 0.f;
    QG_CUDA(cudaEventElapsedTime(&f, g_prof.pool[cls][i], g_prof.pool[cls][i + 1]));
    ms += f;
  }
  *total_ms = ms;
  *launches = (int)(used / 2);
  return QG_OK;
}

int qg_mcclean_create(int n, int layers, const int32_t* axes, int entangler, int placement, int nterms,
                      const int32_t* kind, const int32_t* q0, const int32_t* q1, const double* w, qg_circuit** out) {
  if (!out) return fail(QG_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (n < 1 || n > QMAX) return fail(QG_ERR_UNSUPPORTED, "qubit number %d outside 1..%d", n, QMAX);
  if (layers < 0) return fail(QG_ERR_INVALID, "negative layer number");
  if (layers > 0 && !axes) return fail(QG_ERR_INVALID, "null axes");
  if (entangler < 0 || entangler > 3) return fail(QG_ERR_INVALID, "unknown entangler %d", entangler);
  if (entangler == QG_ENT_CNOT_LADDER_PERIODIC && n % 2)
    return fail(QG_ERR_INVALID,
                "CNOT gates in a ladder structure with periodic boundaries are ambiguous for uneven number of "
                "qubits.");  // state.py:210-214
  if (placement < 0 || placement > 1) return fail(QG_ERR_INVALID, "unknown placement %d", placement);
  qg_circuit* c = new (std::nothrow) qg_circuit;
  if (!c) return fail(QG_ERR_HOST_MEMORY, "host allocation failed");
  c->kind = 0;
  c->n = n;
  c->L = layers;
  c->entangler = entangler;
  c->placement = placement;
  c->axes.resize((size_t)layers * n);
  for (size_t k = 0; k < c->axes.size(); ++k) {
    if (axes[k] < 0 || axes[k] > 2) {
      delete c;
      return fail(QG_ERR_INVALID, "Invalid axis %d", axes[k]);  // mc_clean.py:391-392
    }
    c->axes[k] = (int8_t)axes[k];
  }
  int s = parse_terms(n, nterms, kind, q0, q1, w, c->terms);
  if (s) {
    delete c;
    return s;
  }
  *out = c;
  return QG_OK;
}

int qg_qaoa_create(int n, int layers, int nterms, const int32_t* kind, const int32_t* q0, const int32_t* q1,
                   const double* w, qg_circuit** out) {
  if (!out) return fail(QG_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (n < 1 || n > QMAX) return fail(QG_ERR_UNSUPPORTED, "qubit number %d outside 1..%d", n, QMAX);
  if (layers < 0) return fail(QG_ERR_INVALID, "negative layer number");
  qg_circuit* c = new (std::nothrow) qg_circuit;
  if (!c) return fail(QG_ERR_HOST_MEMORY, "host allocation failed");
  c->kind = 1;
  c->n = n;
  c->L = layers;
  int s = parse_terms(n, nterms, kind, q0, q1, w, c->terms);
  if (s) {
    delete c;
    return s;
  }
  // classical cost from the Z / ZZ terms (state.py:261-297)
  std::vector<Term> diag;
  for (const auto& t : c->terms)
    if (t.kind >= QG_PAULI_Z) diag.push_back(t);
  if ((int)diag.size() > MAX_COST_TERMS) {
    delete c;
    return fail(QG_ERR_UNSUPPORTED, "more than %d cost terms", MAX_COST_TERMS);
  }
  // integer form C = w0 * m(x) when every weight is an integer multiple of the smallest one
  double w0 = 0.0;
  for (const auto& t : diag)
    if (t.w != 0.0 && (w0 == 0.0 || fabs(t.w) < w0)) w0 = fabs(t.w);
  bool integral = w0 > 0.0;
  long maxabs = 0;
  std::vector<int> coef;
  for (const auto& t : diag) {
    const double r = t.w / w0;
    const double k = nearbyint(r);
    if (!(fabs(r - k) == 0.0 && k * w0 == t.w && fabs(k) <= 1 << 20)) integral = false;
    coef.push_back((int)k);
    maxabs += labs((long)k);
  }
  if (diag.empty()) {
    integral = true;
    w0 = 1.0;
  }
  if (integral && maxabs <= (MAX_COST_TAB - 1) / 2) {
    c->cost_kind = COST_INT;
    c->cost_w0 = w0;
    c->cost_maxabs = (int)maxabs;
    c->iterms = new (std::nothrow) IntTermList;
    if (!c->iterms) {
      delete c;
      return fail(QG_ERR_HOST_MEMORY, "host allocation failed");
    }
    memset(c->iterms, 0, sizeof(IntTermList));
    c->iterms->nterms = (int)diag.size();
    for (size_t k = 0; k < diag.size(); ++k) {
      c->iterms->t[k].b0 = n - 1 - diag[k].q0;
      c->iterms->t[k].b1 = diag[k].kind == QG_PAULI_ZZ ? n - 1 - diag[k].q1 : -1;
      c->iterms->t[k].c = coef[k];
    }
  } else {
    c->cost_kind = COST_REAL;
    c->rterms = new (std::nothrow) RealTermList;
    if (!c->rterms) {
      delete c;
      return fail(QG_ERR_HOST_MEMORY, "host allocation failed");
    }
    memset(c->rterms, 0, sizeof(RealTermList));
    c->rterms->nterms = (int)diag.size();
    for (size_t k = 0; k < diag.size(); ++k) {
      c->rterms->t[k].b0 = n - 1 - diag[k].q0;
      c->rterms->t[k].b1 = diag[k].kind == QG_PAULI_ZZ ? n - 1 - diag[k].q1 : -1;
      c->rterms->t[k].w = diag[k].w;
    }
  }
  *out = c;
  return QG_OK;
}

void qg_destroy(qg_circuit* c) { delete c; }

int qg_num_params(const qg_circuit* c, int* np) {
  if (int s = check_circuit(c)) return s;
  if (!np) return fail(QG_ERR_INVALID, "null output");
  *np = c->kind == 0 ? c->L * c->n : 2 * c->L;
  return QG_OK;
}

int qg_workspace_size(const qg_circuit* c, int dtype, int op, size_t* bytes) {
  if (int s = check_circuit(c)) return s;
  if (!bytes) return fail(QG_ERR_INVALID, "null output");
  if (dtype != QG_C128 && dtype != QG_C64) return fail(QG_ERR_INVALID, "unknown dtype %d", dtype);
  if (op < QG_OP_RUN || op > QG_OP_GRAD_UNCOMPUTE) return fail(QG_ERR_INVALID, "unknown op %d", op);
  // the start state adds a fixed Ry layer (McClean) when given; size for the larger case
  std::shared_ptr<const Plan> plan;
  if (int s = get_plan(c, dtype, op, c->kind == 0, plan)) return s;
  *bytes = plan->W.total;
  return QG_OK;
}

int qg_run(const qg_circuit* c, int dtype, const double* params, const void* ini, void* ws, size_t wsb, double* expec,
           void* state_out, qg_stream stream) {
  if (int s = check_circuit(c)) return s;
  int np = 0;
  qg_num_params(c, &np);
  if (np > 0 && !params) return fail(QG_ERR_INVALID, "null params");
  if (!ws || !expec) return fail(QG_ERR_INVALID, "null workspace or output");
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == QG_C128) return do_run<double>(c, params, ini, (char*)ws, wsb, expec, state_out, st, dtype);
  if (dtype == QG_C64) return do_run<float>(c, params, ini, (char*)ws, wsb, expec, state_out, st, dtype);
  return fail(QG_ERR_INVALID, "unknown dtype %d", dtype);
}

int qg_grad(const qg_circuit* c, int dtype, int op, const double* params, const void* ini, void* ws, size_t wsb,
            double* expec, double* grad, qg_stream stream) {
  if (int s = check_circuit(c)) return s;
  int np = 0;
  qg_num_params(c, &np);
  if (np > 0 && (!params || !grad)) return fail(QG_ERR_INVALID, "null params or grad");
  if (!ws || !expec) return fail(QG_ERR_INVALID, "null workspace or output");
  if (op != QG_OP_GRAD_HISTORY && op != QG_OP_GRAD_UNCOMPUTE) return fail(QG_ERR_INVALID, "unknown grad op %d", op);
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == QG_C128) return do_grad<double>(c, op, params, ini, (char*)ws, wsb, expec, grad, st, dtype);
  if (dtype == QG_C64) return do_grad<float>(c, op, params, ini, (char*)ws, wsb, expec, grad, st, dtype);
  return fail(QG_ERR_INVALID, "unknown dtype %d", dtype);
}

int qg_grad_component(const qg_circuit* c, int dtype, int op, const double* params, const void* ini, int component,
                      void* ws, size_t wsb, double* expec, double* grad, qg_stream stream) {
  if (int s = check_circuit(c)) return s;
  if (c->kind != 0) return fail(QG_ERR_INVALID, "component sampling is defined for McClean circuits");
  if (component < 0 || component >= (int)c->terms.size())
    return fail(QG_ERR_INVALID, "component %d outside 0..%d", component, (int)c->terms.size() - 1);
  int np = 0;
  qg_num_params(c, &np);
  if (np > 0 && (!params || !grad)) return fail(QG_ERR_INVALID, "null params or grad");
  if (!ws || !expec) return fail(QG_ERR_INVALID, "null workspace or output");
  if (op != QG_OP_GRAD_HISTORY && op != QG_OP_GRAD_UNCOMPUTE) return fail(QG_ERR_INVALID, "unknown grad op %d", op);
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == QG_C128)
    return do_grad<double>(c, op, params, ini, (char*)ws, wsb, expec, grad, st, dtype, component);
  if (dtype == QG_C64) return do_grad<float>(c, op, params, ini, (char*)ws, wsb, expec, grad, st, dtype, component);
  return fail(QG_ERR_INVALID, "unknown dtype %d", dtype);
}

int qg_maxcut_table(int n, int nedges, const int32_t* edges, int32_t* table, qg_stream stream) {
  if (n < 1 || n > QMAX) return fail(QG_ERR_UNSUPPORTED, "qubit number %d outside 1..%d", n, QMAX);
  if (nedges < 0 || nedges > MAX_COST_TERMS) return fail(QG_ERR_UNSUPPORTED, "edge count %d", nedges);
  if ((nedges > 0 && !edges) || !table) return fail(QG_ERR_INVALID, "null pointer");
  IntTermList* L = new (std::nothrow) IntTermList;
  if (!L) return fail(QG_ERR_HOST_MEMORY, "host allocation failed");
  std::unique_ptr<IntTermList> guard(L);
  memset(L, 0, sizeof *L);
  L->nterms = nedges;
  for (int e = 0; e < nedges; ++e) {
    const int i = edges[2 * e], j = edges[2 * e + 1];
    if (i < 0 || i >= n || j < 0 || j >= n || i == j) return fail(QG_ERR_INVALID, "bad edge (%d, %d)", i, j);
    L->t[e].b0 = n - 1 - i;
    L->t[e].b1 = n - 1 - j;
    L->t[e].c = 1;
  }
  QG_CUDA(launch_int_cost(n, *L, table, sm_count() * 8, (cudaStream_t)stream));
  return QG_OK;
}

int qg_sample_workspace_size(int n, size_t* bytes) {
  if (n < 1 || n > QMAX) return fail(QG_ERR_UNSUPPORTED, "qubit number %d outside 1..%d", n, QMAX);
  if (!bytes) return fail(QG_ERR_INVALID, "null output");
  const int64_t N = (int64_t)1 << n;
  const int64_t nb = (N + SAMPLE_CHUNK - 1) / SAMPLE_CHUNK;
  *bytes = (size_t)(2 * nb + 1) * sizeof(double);
  return QG_OK;
}

int qg_sample(int n, int dtype, const void* state, int64_t nshots, uint64_t seed, uint64_t offset, void* ws,
              size_t wsb, int64_t* out, qg_stream stream) {
  size_t need = 0;
  if (int s = qg_sample_workspace_size(n, &need)) return s;
  if (!state || !ws || (nshots > 0 && !out)) return fail(QG_ERR_INVALID, "null pointer");
  if (nshots < 0) return fail(QG_ERR_INVALID, "negative shot number");
  if (wsb < need) return fail(QG_ERR_WORKSPACE, "workspace %zu bytes < %zu needed", wsb, need);
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == QG_C128)
    QG_CUDA(launch_sample<double2>(n, (const double2*)state, nshots, seed, offset, (double*)ws, out, st));
  else if (dtype == QG_C64)
    QG_CUDA(launch_sample<float2>(n, (const float2*)state, nshots, seed, offset, (double*)ws, out, st));
  else
    return fail(QG_ERR_INVALID, "unknown dtype %d", dtype);
  return QG_OK;
}

int qg_set_tuning(qg_circuit* c, int dtype, int tile_bits, int ctas_per_sm, int flags) {
  if (int s = check_circuit(c)) return s;
  if (dtype != QG_C128 && dtype != QG_C64) return fail(QG_ERR_INVALID, "unknown dtype %d", dtype);
  const int tmin = dtype == QG_C128 ? 5 : 6;
  if (tile_bits != 0 && (tile_bits < tmin || tile_bits > max_tile_bits(dtype)))
    return fail(QG_ERR_INVALID, "tile_bits %d outside %d..%d (0: default)", tile_bits, tmin, max_tile_bits(dtype));
  if (ctas_per_sm < 0 || ctas_per_sm > 64) return fail(QG_ERR_INVALID, "ctas_per_sm %d outside 0..64", ctas_per_sm);
  if (flags & ~(QG_TUNE_FWD_PIPELINED | QG_TUNE_FWD_PLAIN) ||
      (flags & QG_TUNE_FWD_PIPELINED && flags & QG_TUNE_FWD_PLAIN))
    return fail(QG_ERR_INVALID, "bad tuning flags 0x%x", flags);
  c->tune_tile_bits[dtype] = tile_bits;
  c->tune_ctas[dtype] = ctas_per_sm;
  c->tune_flags[dtype] = flags;
  clear_plans(c);
  return QG_OK;
}

int qg_get_tuning(const qg_circuit* c, int dtype, int* tile_bits, int* ctas_per_sm, int* flags) {
  if (int s = check_circuit(c)) return s;
  if (dtype != QG_C128 && dtype != QG_C64) return fail(QG_ERR_INVALID, "unknown dtype %d", dtype);
  if (!tile_bits || !ctas_per_sm) return fail(QG_ERR_INVALID, "null output");
  std::shared_ptr<const Plan> plan;
  if (int s = get_plan(c, dtype, QG_OP_GRAD_HISTORY, false, plan)) return s;
  const WsLayout& W = plan->W;
  *tile_bits = plan->P.lay.t;
  const int sms = sm_count();
  *ctas_per_sm = sms > 0 ? (W.G + sms - 1) / sms : W.G;
  if (flags) *flags = W.fwd_pipe ? QG_TUNE_FWD_PIPELINED : QG_TUNE_FWD_PLAIN;
  return QG_OK;
}

int qg_pauli_workspace_size(const qg_circuit* c, size_t* bytes) {
  if (int s = check_circuit(c)) return s;
  if (!bytes) return fail(QG_ERR_INVALID, "null output");
  *bytes = pauli_workspace_bytes((int)c->terms.size());
  return QG_OK;
}

int qg_pauli_expectations(const qg_circuit* c, int dtype, const void* state, void* ws, size_t wsb, double* out,
                          qg_stream stream) {
  if (int s = check_circuit(c)) return s;
  const int K = (int)c->terms.size();
  if (K == 0) return QG_OK;
  if (!state || !ws || !out) return fail(QG_ERR_INVALID, "null pointer");
  const size_t need = pauli_workspace_bytes(K);
  if (wsb < need) return fail(QG_ERR_WORKSPACE, "workspace %zu bytes < %zu needed", wsb, need);
  std::vector<PauliTerm> t(K);
  for (int k = 0; k < K; ++k) {
    const Term& tm = c->terms[k];
    t[k].kind = (int8_t)tm.kind;
    t[k].b0 = (int8_t)(c->n - 1 - tm.q0);
    t[k].b1 = (int8_t)(tm.kind == QG_PAULI_ZZ ? c->n - 1 - tm.q1 : 0);
    t[k].pad = 0;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == QG_C128)
    QG_CUDA(launch_pauli_expectations<double2>(c->n, (const double2*)state, K, t.data(), (double*)ws, out, st));
  else if (dtype == QG_C64)
    QG_CUDA(launch_pauli_expectations<float2>(c->n, (const float2*)state, K, t.data(), (double*)ws, out, st));
  else
    return fail(QG_ERR_INVALID, "unknown dtype %d", dtype);
  return QG_OK;
}

int qg_qaoa_cost_terms(int n, int nterms, const int32_t* kind, const int32_t* q0, const int32_t* q1,
                       const double* w, int max_out, qg_cost_term* out, int* nout, double* w0_out, int* maxabs_out) {
  if (!nout || !w0_out || !maxabs_out || (max_out > 0 && !out)) return fail(QG_ERR_INVALID, "null output");
  std::vector<Term> terms;
  if (int st = parse_terms(n, nterms, kind, q0, q1, w, terms)) return st;
  std::vector<Term> diag;
  for (const auto& t : terms)
    if (t.kind >= QG_PAULI_Z) diag.push_back(t);
  double w0 = 0.0;
  for (const auto& t : diag)
    if (t.w != 0.0 && (w0 == 0.0 || fabs(t.w) < w0)) w0 = fabs(t.w);
  if (diag.empty()) w0 = 1.0;
  long maxabs = 0;
  int k = 0;
  for (const auto& t : diag) {
    const double r = t.w / w0;
    const double c = nearbyint(r);
    if (!(fabs(r - c) == 0.0 && c * w0 == t.w && fabs(c) <= 1 << 20))
      return fail(QG_ERR_UNSUPPORTED, "cost weights have no common integer base");
    if (k >= max_out) return fail(QG_ERR_UNSUPPORTED, "more than %d cost terms", max_out);
    out[k].b0 = n - 1 - t.q0;
    out[k].b1 = t.kind == QG_PAULI_ZZ ? n - 1 - t.q1 : -1;
    out[k].c = (int32_t)c;
    out[k].pad = 0;
    maxabs += labs((long)c);
    ++k;
  }
  *nout = k;
  *w0_out = w0;
  *maxabs_out = (int)maxabs;
  return QG_OK;
}

int qg_batch_workspace_size(size_t* bytes) {
  if (!bytes) return fail(QG_ERR_INVALID, "null output");
  *bytes = 256;
  return QG_OK;
}

int qg_batch_launch(int dtype, const qg_batch_job* jobs, int njobs, int max_qubits, int cluster, void* ws,
                    size_t wsb, qg_stream stream) {
  if (njobs < 0) return fail(QG_ERR_INVALID, "negative job count");
  if (njobs == 0) return QG_OK;
  if (!jobs || !ws) return fail(QG_ERR_INVALID, "null pointer");
  if (wsb < 256) return fail(QG_ERR_WORKSPACE, "workspace %zu bytes < 256 needed", wsb);
  if (dtype != QG_C128 && dtype != QG_C64) return fail(QG_ERR_INVALID, "unknown dtype %d", dtype);
  if (cluster != 1 && cluster != 2 && cluster != 4) return fail(QG_ERR_INVALID, "cluster must be 1, 2 or 4");
  const int mlimit = dtype == QG_C128 ? BatchC<double>::MMAX : BatchC<float>::MMAX;
  const int lg = cluster == 4 ? 2 : cluster - 1;  // top bits split across the cluster
  const int m = max_qubits - lg;
  if (max_qubits < 1 || m > mlimit)
    return fail(QG_ERR_UNSUPPORTED, "batched jobs need n <= %d (cluster %d)", mlimit + lg, cluster);
  cudaStream_t st = (cudaStream_t)stream;
  QG_CUDA(cudaMemsetAsync(ws, 0, sizeof(int), st));
  int grid = 0;
  QG_CUDA(launch_batched(dtype == QG_C128, cluster, jobs, njobs, (int*)ws, m < 1 ? 1 : m, st, &grid));
  return QG_OK;
}

}  // extern "C"
