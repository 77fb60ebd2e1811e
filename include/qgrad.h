/*
 * qgrad: C ABI of the GB300-native statevector run / adjoint grad_run path
 * of qradient's McClean and QAOA circuits.
 *
 * The reference (frederikwilde/qradient) is pure Python; it has no FFI.  Its
 * drop-in boundary is the circuit_logic class API, and every entry point here
 * is what a Python (ctypes) binding of that API calls:
 *
 *   qg_mcclean_create  <- McClean.__init__       qradient/circuit_logic/mc_clean.py:9-25
 *                         (+ Observable matrix   qradient/physical_components/observable.py:34-73)
 *   qg_qaoa_create     <- Qaoa.__init__          qradient/circuit_logic/qaoa.py:9-21
 *   qg_run             <- McClean.run_expec_val  qradient/circuit_logic/mc_clean.py:27-45
 *                         Qaoa.run_expec_val     qradient/circuit_logic/qaoa.py:23-38
 *   qg_grad            <- McClean.grad_run       qradient/circuit_logic/mc_clean.py:47-78
 *                         Qaoa.grad_run          qradient/circuit_logic/qaoa.py:40-70
 *   qg_maxcut_table    <- State.load_classical_ham (its diagonal)
 *                                                qradient/physical_components/state.py:261-297
 *   qg_sample          <- Qaoa.__sample          qradient/circuit_logic/qaoa.py:196-198
 *
 * Conventions
 *   - Qubit q is bit (n-1-q) of the basis index (state.py:84-88).
 *   - States are interleaved complex arrays: complex128 (QG_C128) or
 *     complex64 (QG_C64), 2^n elements.
 *   - Every pointer argument of qg_run / qg_grad / qg_sample /
 *     qg_maxcut_table named *_dev is device memory; the caller owns all device
 *     buffers.  The library allocates no device memory: scratch lives in the
 *     caller's workspace, sized by qg_workspace_size.
 *   - Calls are ordered on the given stream; a circuit handle is immutable
 *     after creation and may be used from several threads on distinct streams
 *     and workspaces.  Inside one call, each sweep launch after the first is
 *     a programmatic dependent of the previous one (its setup overlaps that
 *     sweep's tail; it touches no state before that sweep completes); the
 *     call's first launch is ordered after earlier work as usual.
 *   - Errors are returned as status codes (never traps); qg_last_error()
 *     gives a message for the calling thread.
 */
#ifndef QGRAD_H
#define QGRAD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qg_circuit qg_circuit;
typedef struct CUstream_st* qg_stream; /* cudaStream_t */

enum qg_status {
  QG_OK = 0,
  QG_ERR_INVALID = 1,     /* bad argument; the reference raises ValueError here */
  QG_ERR_CUDA = 2,        /* a CUDA call failed; see qg_last_error() */
  QG_ERR_WORKSPACE = 3,   /* workspace too small */
  QG_ERR_UNSUPPORTED = 4, /* valid request outside this build's limits */
  QG_ERR_HOST_MEMORY = 5
};

enum qg_dtype { QG_C128 = 0, QG_C64 = 1 };

/* Entangler of a McClean layer.  QG_ENT_CNOT_LADDER is the reference's
 * ladder (state.py:209-251): CNOT(q, q+1) on odd q, then on even q.
 * QG_ENT_CNOT_LADDER_PERIODIC is its periodic form (load_cnot_ladder(
 * periodic=True), state.py:209-241): CNOT(n-1, 0) joins the odd pairs; even n
 * only (QG_ERR_INVALID otherwise, where the reference raises ValueError). */
enum qg_entangler {
  QG_ENT_NONE = 0,
  QG_ENT_CNOT_LADDER = 1,
  QG_ENT_CZ_LADDER = 2,
  QG_ENT_CNOT_LADDER_PERIODIC = 3
};
/* Where the entangler sits in a layer.  The reference applies it before the
 * rotations (mc_clean.py:58-62). */
enum qg_placement { QG_PLACE_BEFORE = 0, QG_PLACE_AFTER = 1 };

enum qg_pauli { QG_PAULI_X = 0, QG_PAULI_Y = 1, QG_PAULI_Z = 2, QG_PAULI_ZZ = 3 };

/* qg_grad strategies: keep every intermediate state (fewest operations,
 * memory ~ (sweeps + 2) states) or uncompute psi backwards (3 states). */
enum qg_op { QG_OP_RUN = 0, QG_OP_GRAD_HISTORY = 1, QG_OP_GRAD_UNCOMPUTE = 2 };

/* McClean.__init__ (mc_clean.py:9-25) with the observable dict flattened to
 * terms (observable.py:12-17): term k is kind[k] in qg_pauli on qubit q0[k]
 * (and q1[k] > q0[k] for ZZ) with weight w[k].  axes is host int32 [L*n]
 * with values 0 (X), 1 (Y), 2 (Z) (mc_clean.py:383-392).  Angles are passed
 * per call.  All arrays are host memory. */
int qg_mcclean_create(int n, int layers, const int32_t* axes, int entangler, int placement, int nterms,
                      const int32_t* kind, const int32_t* q0, const int32_t* q1, const double* w, qg_circuit** out);

/* Qaoa.__init__ (qaoa.py:9-21): the observable's Z and ZZ terms form the
 * classical cost C (state.py:261-297); X and Y terms only enter qg_run's
 * expectation value, as in the reference (base.py:17-20). */
int qg_qaoa_create(int n, int layers, int nterms, const int32_t* kind, const int32_t* q0, const int32_t* q1,
                   const double* w, qg_circuit** out);

void qg_destroy(qg_circuit* c);

/* Number of parameters: McClean L*n (angles [L, n] row-major); QAOA 2p
 * (params [p, 2] row-major: column 0 beta, column 1 gamma, the grad layout
 * of qaoa.py:46). */
int qg_num_params(const qg_circuit* c, int* nparams);

/* Device workspace bytes for an operation (qg_op) at a dtype. */
int qg_workspace_size(const qg_circuit* c, int dtype, int op, size_t* bytes);

/* Forward run and exact expectation value <psi|O|psi> (run_expec_val with
 * exact_expec_val=True).  params_dev: double [nparams].  ini_state_dev:
 * optional start state (NULL: |0..0> for McClean, |+..+> for QAOA); McClean
 * still applies its Ry(pi/4) layer to it (mc_clean.py:29-36).  expec_dev:
 * one double.  state_out_dev: optional, receives the final state. */
int qg_run(const qg_circuit* c, int dtype, const double* params_dev, const void* ini_state_dev, void* workspace_dev,
           size_t workspace_bytes, double* expec_dev, void* state_out_dev, qg_stream stream);

/* Adjoint gradient (grad_run): expec_dev receives E, grad_dev the nparams
 * derivatives.  op is QG_OP_GRAD_HISTORY or QG_OP_GRAD_UNCOMPUTE. */
int qg_grad(const qg_circuit* c, int dtype, int op, const double* params_dev, const void* ini_state_dev,
            void* workspace_dev, size_t workspace_bytes, double* expec_dev, double* grad_dev, qg_stream stream);

/* Component-sampled adjoint gradient (McClean.grad_run_with_component_sampling,
 * mc_clean.py:80-115): expec_dev receives the full E = <psi|O|psi>, grad_dev
 * the gradient of <psi|w_k P_k|psi> for the single observable term
 * `component` (0-based, in the order the terms were given to
 * qg_mcclean_create).  The caller draws `component`; the reference draws it
 * with numpy.random.choice over the normalised weights (mc_clean.py:102).
 * Same workspace as qg_grad. */
int qg_grad_component(const qg_circuit* c, int dtype, int op, const double* params_dev, const void* ini_state_dev,
                      int component, void* workspace_dev, size_t workspace_bytes, double* expec_dev,
                      double* grad_dev, qg_stream stream);

/* Integer MaxCut / ZZ cost table: table_dev[x] = sum over edges (i, j) of
 * z_i z_j with z = +1 for bit 0 (state.py:280-292 with unit weights).
 * edges: host int32 [nedges, 2]. */
int qg_maxcut_table(int n, int nedges, const int32_t* edges, int32_t* table_dev, qg_stream stream);

/* Draw nshots basis indices from |psi|^2 (Qaoa.__sample, qaoa.py:196-198)
 * with a counter-based Philox4x32-10 stream (seed, offset).  Returns indices
 * in out_dev (int64 [nshots]).  Needs qg_sample_workspace_size bytes. */
int qg_sample_workspace_size(int n, size_t* bytes);
int qg_sample(int n, int dtype, const void* state_dev, int64_t nshots, uint64_t seed, uint64_t offset,
              void* workspace_dev, size_t workspace_bytes, int64_t* out_dev, qg_stream stream);

/* ---- Tuning (no reference counterpart).  A sweep stages 2^tile_bits
 * amplitudes in shared memory and applies every rotation on those bits in
 * one pass (the fusion depth); ctas_per_sm sets the persistent grid (block
 * shape across the SMs, capped at what fits).  0 restores the default
 * (tile_bits 11 for complex128, 12 for complex64; complex128 takes 12 for
 * the first sweep of a layer where that saves a sweep per layer, with 11
 * for the others where that costs none; ctas_per_sm from the
 * occupancy query).  A non-zero tile_bits applies to every sweep.
 * tile_bits: 5..12 for complex128, 6..13 for
 * complex64 (the backward sweep holds two tiles in shared memory); tiles
 * larger than the state use the whole state.  Call before launches that use the handle, not while
 * another thread uses it; the workspace size may change with the setting.
 * flags: QG_TUNE_FWD_PIPELINED or QG_TUNE_FWD_PLAIN choose the forward
 * sweep kernel (0: the default, pipelined).
 * qg_get_tuning reports the effective values (tile bits of a layer's first
 * sweep after clamping to n, CTAs per SM of the backward sweeps, the
 * forward kernel flag).  The autotuner of
 * qradient_gb300/tuning.py picks them by timing. */
enum {
  QG_TUNE_FWD_PIPELINED = 1, /* forward sweeps prefetch the next tile (double-buffered) */
  QG_TUNE_FWD_PLAIN = 2      /* forward sweeps load, compute, store (single buffer) */
};
int qg_set_tuning(qg_circuit* c, int dtype, int tile_bits, int ctas_per_sm, int flags);
int qg_get_tuning(const qg_circuit* c, int dtype, int* tile_bits, int* ctas_per_sm, int* flags);

/* ---- Finite-shot estimates (the projector estimator of
 * ParametrizedCircuit.sample_expec_val / sample_component_expec_val,
 * base.py:22-46, with the projectors of observable.py:82-177).
 *
 * qg_pauli_expectations: out_dev[k] = <psi|P_k|psi> (unweighted, real) for
 *   every observable term of circuit c, in the order given at creation,
 *   for a device state of 2^n amplitudes at `dtype`.  Deterministic.
 *   Workspace: qg_pauli_workspace_size bytes.
 * qg_projector_shots: for each row r and term k, draws `shots` outcomes of
 *   the term's +1/-1 projective measurement, +w_k with probability
 *   p = (1 + <P_k>) / 2 (the reference's ||Pi_+ psi||^2) and -w_k otherwise,
 *   and writes their mean to term_est_dev[r][k] (optional) and the sum over
 *   terms to total_dev[r] (optional): the reference's
 *   sample_expec_val(shots) per row.  expec_dev [nrows][nterms] holds the
 *   <P_k>, weights_dev [nterms] the w_k.  Uniforms come from
 *   Philox4x32-10 with key `seed` and counter {offset + r*nterms + k,
 *   shot / 2}; the reference draws with scipy.stats.rv_discrete instead, so
 *   parity is statistical.  nterms <= 1024. */
int qg_pauli_workspace_size(const qg_circuit* c, size_t* bytes);
int qg_pauli_expectations(const qg_circuit* c, int dtype, const void* state_dev, void* workspace_dev,
                          size_t workspace_bytes, double* out_dev, qg_stream stream);
int qg_projector_shots(int nrows, int nterms, const double* expec_dev, const double* weights_dev, int shots,
                       uint64_t seed, uint64_t offset, double* term_est_dev, double* total_dev, qg_stream stream);

/* ---- Optimiser steps on the device.  No reference counterpart as C
 * functions: they are the parameter updates of qradient/optimization.py
 * (Adam :151-167, GradientDescent :169-175, RateDecayOnPlateau :177-194),
 * run on the stream of qg_grad so a training loop never copies parameters,
 * gradients or costs to the host.  Arrays are device float64 of length
 * nparams; params are updated in place; history_row_dev (optional, may be
 * NULL) receives a copy of the updated parameters (the param_history row of
 * McCleanOpt.step / QaoaOpt.step, optimization.py:90,129).  Every operation
 * is one IEEE-754 double operation in numpy's order (no fused multiply-add),
 * so results are bit-identical to the reference's for equal gradients.
 *
 * qg_adam_step: iter is the step count including this step (1 first);
 *   m_dev, v_dev are the first and second moments (zero before step 1).
 * qg_gd_step: step_size is the already-decayed rate
 *   (decay_function(step_size, iter) of optimization.py:175).
 * qg_plateau_step: new_cost_dev points at the step's cost (the expectation
 *   value qg_grad wrote); state_dev holds 3 doubles {best cost, plateau
 *   counter, step size}, initialised to {1e10, 0, step_size} as at
 *   optimization.py:180-183. */
int qg_adam_step(double* params_dev, const double* grad_dev, double* m_dev, double* v_dev, int nparams, int iter,
                 double step_size, double beta1, double beta2, double eps, double* history_row_dev, qg_stream stream);
int qg_gd_step(double* params_dev, const double* grad_dev, int nparams, double step_size, double* history_row_dev,
               qg_stream stream);
int qg_plateau_step(double* params_dev, const double* grad_dev, int nparams, const double* new_cost_dev,
                    double* state_dev, int plateau_length, double decay_rate, double* history_row_dev,
                    qg_stream stream);

/* ---- Batched persistent execution (no reference counterpart: the
 * reference runs one circuit per Python call).  Many small circuits, each
 * a whole run or grad_run with psi and lambda resident in shared memory,
 * in one launch (CUDA-graph capturable).  Limits: complex64 n <= 15,
 * complex128 n <= 14, L <= 4096, and for QAOA an integer cost with
 * |m| <= 511. */
typedef struct qg_term {
  int32_t kind, q0, q1, pad; /* qg_pauli, qubits (q1 for ZZ) */
  double w;
} qg_term;

typedef struct qg_cost_term {
  int32_t b0, b1, c, pad; /* bit positions (b1 < 0: Z term) and integer coefficient */
} qg_cost_term;

/* One job; every pointer is device memory. */
typedef struct qg_batch_job {
  int32_t kind;        /* 0 McClean, 1 QAOA */
  int32_t n, layers;
  int32_t entangler;   /* McClean: qg_entangler (QG_ENT_CNOT_LADDER_PERIODIC only in jobs one
                          CTA holds: complex64 n <= 13, complex128 n <= 12) */
  int32_t placement;   /* McClean: qg_placement */
  int32_t nterms;      /* observable terms */
  const qg_term* terms;
  const int8_t* axes;  /* McClean [layers * n] */
  const double* params;/* McClean [layers * n]; QAOA [layers, 2] */
  double* expec;       /* out: one double */
  double* grad;        /* out: nparams doubles, or NULL for a run */
  int32_t cost_nterms; /* QAOA cost C = cost_w0 * sum c_k s_k(x) */
  int32_t cost_maxabs;
  double cost_w0;
  const qg_cost_term* cost;
  double* term_expec;  /* out, optional (NULL: none): <P_k> of every observable term on the final
                          state, nterms doubles -- what the projector-shot estimators draw from */
} qg_batch_job;

/* QAOA integer cost of a term list (host): fills up to max_out cost terms,
 * *w0 and *maxabs; QG_ERR_UNSUPPORTED when the weights have no common
 * integer base. */
int qg_qaoa_cost_terms(int n, int nterms, const int32_t* kind, const int32_t* q0, const int32_t* q1,
                       const double* w, int max_out, qg_cost_term* out, int* nout, double* w0, int* maxabs);

/* Workspace bytes for one batched launch. */
int qg_batch_workspace_size(size_t* bytes);

/* Run njobs jobs (jobs_dev: device array) in persistent launches.  All jobs
 * must share dtype; max_qubits bounds their n (sets the shared-memory size).
 * cluster: CTAs per job, 1, 2 or 4 (the state split by its top 0, 1 or 2
 * bits): one CTA holds complex64 n <= 13 / complex128 n <= 12, two one
 * qubit more, four two more.  A job whose n exceeds max_qubits, or leaves a
 * cluster's CTA fewer than 2 qubits, gets NaN outputs.  4-CTA jobs add their partial sums with atomic
 * adds in arrival order (their outputs can vary in the last bit). */
int qg_batch_launch(int dtype, const qg_batch_job* jobs_dev, int njobs, int max_qubits, int cluster,
                    void* workspace_dev, size_t workspace_bytes, qg_stream stream);

/* ---- Allocation-free gradient (no counterpart in the reference).
 * For callers that cannot allocate device memory where they need a
 * gradient: plug-ins whose host process owns every device allocation
 * through its own pool, and real-time loops that forbid allocation (which
 * may synchronise the device) after start-up.  Same inputs and outputs as
 * qg_grad in uncompute mode, but the scratch is a library-owned static
 * device array of QG_NOALLOC_SCRATCH_BYTES that every GPU loading the
 * library's device code holds until exit.  Circuits whose uncompute
 * workspace exceeds it get QG_ERR_UNSUPPORTED.  The first call on a device
 * looks up the array's address (with that device current) and caches it; a
 * context reset (cudaDeviceReset) invalidates the cached address, so the
 * entry point must not be used after one.  Calls share the array and it
 * keeps the previous call's contents: calls that overlap on the GPU race,
 * so order them (one stream). */
#define QG_NOALLOC_SCRATCH_BYTES ((size_t)16 << 20)
int qg_grad_noalloc(const qg_circuit* c, int dtype, const double* params_dev, const void* ini_state_dev,
                    double* expec_dev, double* grad_dev, qg_stream stream);

/* Launch timing for roofline reporting.  While enabled, the library records
 * a CUDA event pair (on the launching stream) around every sweep launch of
 * the calling thread; qg_profile_collect waits for them and returns the
 * summed device time and launch count of one kernel class
 * (0: forward sweeps, 1: backward sweeps, 2: observable passes) since the
 * last qg_profile_enable(1). */
int qg_profile_enable(int on);
int qg_profile_collect(int kernel_class, double* total_ms, int* launches);

const char* qg_status_string(int status);
/* Message of the last failed call on this thread. */
const char* qg_last_error(void);
int qg_version(void);

#ifdef __cplusplus
}
#endif

#endif /* QGRAD_H */
