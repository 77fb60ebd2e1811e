// Internal definitions shared by the qgrad CUDA translation units.
//
// A circuit is executed as a sequence of *sweeps*.  A sweep owns a set of t
// "tile bits" of the basis index; the state is cut into 2^(n-t) tiles of 2^t
// amplitudes (all combinations of the tile bits for one assignment of the
// other bits).  One CTA stages a tile in shared memory, applies every X/Y
// rotation of the sweep whose qubit lies on a tile bit, and writes it back, so
// a layer of n single-qubit rotations costs one pass per sweep instead of one
// per gate.  Diagonal work (Z rotations, CZ signs, the QAOA cost phase, the
// gate scale factors) is applied per amplitude while the tile streams in.
//
// Qubit q of the reference is bit (n-1-q) of the basis index
// (qradient/physical_components/state.py:84-88).
//
// Rotation arithmetic.  R_P(theta) = cos(theta/2) 1 - i sin(theta/2) P is
// applied in one of two scaled forms so that each output component costs one
// FMA:  c * [[1, -i t], [-i t, 1]] with t = tan(theta/2) when |cos| >= |sin|,
// otherwise s * [[u, -i], [-i, u]] with u = cot(theta/2).  The scalar factor
// (c or s) of every X/Y rotation of a layer is multiplied into that layer's
// single per-amplitude diagonal multiply (the merged Z-rotation phase table or
// a plain real scale), so a layer costs 2 FMA per amplitude per X/Y rotation
// plus one complex (or real) multiply per amplitude.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace qg {

constexpr int TMAX = 13;           // max tile bits per sweep
constexpr int NTHREADS = 256;      // threads per sweep CTA
constexpr int ZMAX = 10;           // Z rotations merged into one phase table
constexpr int QMAX = 34;           // max qubits
constexpr int MAX_COST_TAB = 4097; // entries of the integer cost-phase table

enum Axis : int8_t { AX_X = 0, AX_Y = 1, AX_Z = 2 };

// Entangler.  The CNOT ladder permutes amplitudes across tiles, so it is
// only ever applied as a gather while a sweep loads its input (from a buffer
// other than the one it writes); the CZ ladder is a sign and works in place.
enum Ent : int8_t {
  ENT_NONE = 0,
  ENT_CNOT = 1,  // reference CNOT ladder, state.py:209-251 (odd pairs, then even pairs; open or,
                 // with the descriptor's periodic flag, periodic)
  ENT_CZ = 2,    // CZ on neighbours (q, q+1)
};

enum Start : int8_t {
  START_LOAD = 0,     // read the input buffer
  START_MCCLEAN = 1,  // Ry(pi/4)^n |0..0> (mc_clean.py:48-56), evaluated per amplitude
  START_PLUS = 2,     // |+>^n, 2^(-n/2) everywhere (state.py:68-69)
};

enum CostKind : int8_t {
  COST_NONE = 0,
  COST_INT = 1,   // C(x) = w0 * m(x), m from an int32 table; phase from a (2M+1)-entry table
  COST_REAL = 2,  // C(x) from a double table; phase by sincos per amplitude
};

// An angle: params[param] * sign, or `fixed` when param < 0.
struct AngleRef {
  int32_t param;
  float sign;
  double fixed;
};

struct XYGate {
  int8_t axis;  // AX_X or AX_Y
  int8_t lbit;  // local tile bit
  int16_t pad;
  int32_t slot;  // reduction slot (backward), -1 if none
  AngleRef a;
};

struct ZGate {
  int8_t gbit;  // global bit
  int8_t pad[3];
  int32_t slot;
  AngleRef a;
};

struct SweepDesc {
  int32_t n;    // qubits
  int32_t t;    // tile bits
  int32_t nxy;  // X/Y rotations applied in this sweep
  int32_t nz;   // Z rotations merged into this sweep's diagonal (<= ZMAX)
  XYGate xy[TMAX];
  ZGate z[ZMAX];
  int32_t nscale;          // X/Y rotations whose scale factor is folded into this sweep's diagonal
  AngleRef scale[QMAX];
  uint8_t bits[TMAX];      // global bit positions of the tile bits, ascending
  int8_t has_diag;         // apply the diagonal (phase table * scale) in this sweep
  int8_t pre;              // forward: Ent applied to the input as it is loaded (before the gates)
  int8_t lam_undo;         // backward: Ent undone on lambda as it is loaded
  int8_t start;            // Start kind of the forward input
  int8_t cost;             // CostKind: QAOA exp(-i gamma C), applied before the gates
  int8_t psi_undo;         // backward: Ent undone on psi as it is loaded (uncompute mode)
  int8_t gcost;            // CostKind of the gslot reduction
  int8_t periodic;         // the CNOT ladder is the periodic one (CNOT(n-1, 0) joins the odd pairs)
  AngleRef cost_angle;     // gamma
  int32_t cost_maxabs;     // |m| <= cost_maxabs (COST_INT)
  int32_t gslot;           // backward: slot of Im<lam|C|psi> at the load point, -1 if none
  double cost_w0;          // C(x) = w0 * m(x) (COST_INT)
  double pad2;
};

// Observable: sum of weighted X_q, Y_q, Z_q, Z_i Z_j terms (observable.py:45-73).
// Diagonal terms (Z, ZZ) are listed first, grouped by equal weight, so a run
// of equal weights costs integer sign counting and one multiply.
constexpr int OBS_MAX_TERMS = 400;
struct ObsTerm {
  int8_t kind;    // 0 X, 1 Y, 2 Z, 3 ZZ
  int8_t b0, b1;  // global bit positions
  int8_t lb0;     // local tile bit of b0 (X/Y terms)
  int8_t endgrp;  // diagonal terms: the last of a run of equal weights
  int8_t pad[3];
  float wf;       // w in single precision (complex64 observable)
  double w;
};

struct ObsDesc {
  int32_t n, t;
  uint8_t bits[TMAX];
  int8_t accumulate;   // 0: lam = O_part psi; 1: lam += O_part psi
  int8_t store;        // write lam
  int8_t cost;         // diagonal from the QAOA cost (CostKind) instead of the diagonal terms
  int8_t pre;          // Ent applied to psi as it is loaded (entangler after the last layer)
  int8_t periodic;     // ENT_CNOT is the periodic ladder
  int8_t pad0[2];
  int32_t ndiag;       // diagonal terms (first)
  int32_t nxy;         // X/Y terms handled here (after the diagonal ones)
  int32_t eslot;       // slot of the expectation partial sums
  int32_t pad;
  double cost_w0;
  ObsTerm term[OBS_MAX_TERMS];
};

template <typename R>
struct C2T;
template <>
struct C2T<double> {
  using T = double2;
};
template <>
struct C2T<float> {
  using T = float2;
};

// Buffers used by one sweep launch.
template <typename R>
struct SweepPtrs {
  using C = typename C2T<R>::T;
  const C* psi_in;   // forward input / backward psi (history point or uncompute state)
  C* psi_out;        // forward output / backward uncomputed psi (uncompute mode)
  const C* lam_in;   // backward lambda in
  C* lam_out;        // backward lambda out (may alias lam_in: tiles are disjoint)
  const double* params;   // device parameters
  const int32_t* cost_i;  // int cost table (COST_INT)
  const double* cost_d;   // real cost table (COST_REAL)
  double* partials;       // [slot][G]
  int32_t G;              // grid size used for partial indexing
};

}  // namespace qg
