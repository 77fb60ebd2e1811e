/*
 * CPU restatement of qradient's statevector run / adjoint grad_run path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it to check or
 * time the reference's algorithm.  Nothing in the qradient_gb300 product path
 * links or calls it.
 *
 * It restates, gate by gate, the arithmetic of the reference package
 * (pure numpy/scipy):
 *   - qradient/physical_components/state.py:90-97   xrot / dxrot
 *   - qradient/physical_components/state.py:142-149 yrot / dyrot
 *   - qradient/physical_components/state.py:168-175 zrot / dzrot
 *   - qradient/physical_components/state.py:209-251 CNOT ladder (odd pairs,
 *     then even pairs; stacking 1 is the inverse), open or periodic
 *   - qradient/physical_components/state.py:261-301,319-321 classical
 *     Hamiltonian, exp(-i g C), (-i C)
 *   - qradient/physical_components/state.py:107-123 x_summed = 1/2 sum(-iX)
 *   - qradient/physical_components/observable.py:34-73 Pauli-sum matrix
 *   - qradient/circuit_logic/base.py:17-20 expec_val
 *   - qradient/circuit_logic/mc_clean.py:27-78 run_expec_val / grad_run
 *   - qradient/circuit_logic/qaoa.py:23-70 run_expec_val / grad_run
 * with the same history-storing adjoint sweep (L+1 stored states; per
 * parameter the rot + drot of the reference applied per amplitude and summed
 * against the stored state in one pass), parallelised over amplitudes with
 * OpenMP.  An uncompute mode (psi taken backwards instead of stored) serves
 * the sizes whose L+1 host states do not fit.
 *
 * Index convention: qubit q is bit (n-1-q) of the basis index
 * (kron(id(2^q), op, id(2^(n-q-1))), state.py:84-88).  States are
 * interleaved complex128 (re, im) arrays of length 2^n.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex cplx;

static const double QGO_PI = 3.14159265358979323846;

enum { QGO_OK = 0, QGO_EINVAL = 1, QGO_ENOMEM = 2 };
enum { QGO_X = 0, QGO_Y = 1, QGO_Z = 2, QGO_ZZ = 3 };
enum { QGO_ENT_NONE = 0, QGO_ENT_CNOT = 1, QGO_ENT_CZ = 2, QGO_ENT_CNOT_PERIODIC = 3 };

static inline int64_t bitpos(int n, int q) { return (int64_t)(n - 1 - q); }

/* v <- sin(t/2) * (-i P_q) v + cos(t/2) * v for P in {X, Y}
 * (state.py:90-92, 142-144).  (-iX)|a,b> pairs: (-iX v)_a = -i v_b;
 * (-iY v): Y = [[0,-i],[i,0]] so (-iY v)_0 = -v_1, (-iY v)_1 = v_0. */
static void rot_xy(cplx* v, int n, int q, int axis, double angle) {
  const double s = sin(0.5 * angle), c = cos(0.5 * angle);
  const int64_t half = (int64_t)1 << (n - 1);
  const int64_t stride = (int64_t)1 << bitpos(n, q);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < half; k++) {
    const int64_t a = ((k & ~(stride - 1)) << 1) | (k & (stride - 1));
    const int64_t b = a | stride;
    const cplx va = v[a], vb = v[b];
    cplx pa, pb;
    if (axis == QGO_X) {
      pa = -I * vb;
      pb = -I * va;
    } else {
      pa = -vb;
      pb = va;
    }
    v[a] = s * pa + c * va;
    v[b] = s * pb + c * vb;
  }
}

/* derivative: v <- 1/2 cos(t/2) (-iP) v - 1/2 sin(t/2) v (state.py:94-97, 146-149) */
static void drot_xy(cplx* v, int n, int q, int axis, double angle) {
  const double s = sin(0.5 * angle), c = cos(0.5 * angle);
  const int64_t half = (int64_t)1 << (n - 1);
  const int64_t stride = (int64_t)1 << bitpos(n, q);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < half; k++) {
    const int64_t a = ((k & ~(stride - 1)) << 1) | (k & (stride - 1));
    const int64_t b = a | stride;
    const cplx va = v[a], vb = v[b];
    cplx pa, pb;
    if (axis == QGO_X) {
      pa = -I * vb;
      pb = -I * va;
    } else {
      pa = -vb;
      pb = va;
    }
    v[a] = 0.5 * c * pa - 0.5 * s * va;
    v[b] = 0.5 * c * pb - 0.5 * s * vb;
  }
}

/* v <- e^{-it/2} mask0 v + e^{it/2} mask1 v (state.py:168-170) */
static void rot_z(cplx* v, int n, int q, double angle) {
  const cplx e0 = cexp(-0.5 * I * angle), e1 = cexp(0.5 * I * angle);
  const int64_t N = (int64_t)1 << n;
  const int64_t bp = bitpos(n, q);
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < N; x++) v[x] *= ((x >> bp) & 1) ? e1 : e0;
}

/* state.py:172-175 */
static void drot_z(cplx* v, int n, int q, double angle) {
  const cplx e0 = -0.5 * I * cexp(-0.5 * I * angle), e1 = 0.5 * I * cexp(0.5 * I * angle);
  const int64_t N = (int64_t)1 << n;
  const int64_t bp = bitpos(n, q);
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < N; x++) v[x] *= ((x >> bp) & 1) ? e1 : e0;
}

static void rot(cplx* v, int n, int q, int axis, double angle) {
  if (axis == QGO_Z)
    rot_z(v, n, q, angle);
  else
    rot_xy(v, n, q, axis, angle);
}

static void drot(cplx* v, int n, int q, int axis, double angle) {
  if (axis == QGO_Z)
    drot_z(v, n, q, angle);
  else
    drot_xy(v, n, q, axis, angle);
}

/* Basis permutation of the reference CNOT ladder (state.py:229-241): the
 * matrix product puts the odd-pair CNOTs (1,2),(3,4),... rightmost, so they
 * act first, then the even pairs (0,1),(2,3),...  CNOT(c, t) flips bit t when
 * bit c is set.  The periodic ladder (state.py:218-219,231-232, even n) adds
 * CNOT(n-1, 0) to the odd pairs.  Returns A(x) with ladder|x> = |A(x)>;
 * stacking 1 applies the inverse (even pairs first, then odd pairs). */
static int64_t ladder_map(int64_t x, int n, int inverse, int periodic) {
  for (int pass = 0; pass < 2; pass++) {
    const int first = inverse ? (pass == 0 ? 0 : 1) : (pass == 0 ? 1 : 0);
    for (int c = first; c + 1 < n; c += 2) {
      const int64_t cb = bitpos(n, c), tb = bitpos(n, c + 1);
      if ((x >> cb) & 1) x ^= (int64_t)1 << tb;
    }
    if (periodic && first == 1 && n >= 2) {
      const int64_t cb = bitpos(n, n - 1), tb = bitpos(n, 0);
      if ((x >> cb) & 1) x ^= (int64_t)1 << tb;
    }
  }
  return x;
}

static int entangle(cplx* v, cplx* scratch, int n, int kind, int inverse) {
  const int64_t N = (int64_t)1 << n;
  if (kind == QGO_ENT_NONE) return QGO_OK;
  if (kind == QGO_ENT_CZ) {
    /* CZ on neighbours (q, q+1): sign (-1)^{sum_q z_q z_{q+1}}; self-inverse */
#pragma omp parallel for schedule(static)
    for (int64_t x = 0; x < N; x++) {
      int par = __builtin_popcountll((uint64_t)(x & (x >> 1))) & 1;
      if (par) v[x] = -v[x];
    }
    return QGO_OK;
  }
  if (kind != QGO_ENT_CNOT && kind != QGO_ENT_CNOT_PERIODIC) return QGO_EINVAL;
  const int periodic = kind == QGO_ENT_CNOT_PERIODIC;
  if (periodic && (n % 2)) return QGO_EINVAL; /* ambiguous for odd n (state.py:210-214) */
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < N; x++) scratch[ladder_map(x, n, inverse, periodic)] = v[x];
  memcpy(v, scratch, sizeof(cplx) * (size_t)N);
  return QGO_OK;
}

/* out <- O v for O = sum of weighted X_q, Y_q, Z_q, Z_i Z_j terms
 * (observable.py:45-73). */
static void apply_observable(const cplx* v, cplx* out, int n, int nterms, const int* kind, const int* q0,
                             const int* q1, const double* w) {
  const int64_t N = (int64_t)1 << n;
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < N; x++) {
    cplx acc = 0;
    for (int t = 0; t < nterms; t++) {
      const int64_t b0 = (int64_t)1 << bitpos(n, q0[t]);
      switch (kind[t]) {
        case QGO_X:
          acc += w[t] * v[x ^ b0];
          break;
        case QGO_Y: /* (Y v)_x = -i v_{x^b} if bit 0 else +i v_{x^b} */
          acc += w[t] * ((x & b0) ? I * v[x ^ b0] : -I * v[x ^ b0]);
          break;
        case QGO_Z:
          acc += w[t] * ((x & b0) ? -v[x] : v[x]);
          break;
        case QGO_ZZ: {
          const int64_t b1 = (int64_t)1 << bitpos(n, q1[t]);
          const int s = (((x & b0) != 0) ^ ((x & b1) != 0));
          acc += w[t] * (s ? -v[x] : v[x]);
          break;
        }
      }
    }
    out[x] = acc;
  }
}

/* Sums below run in blocks of QGO_BLOCK elements: each block is summed on
 * its own, then the block sums are added, as BLAS dot products accumulate in
 * several partial sums (numpy's vdot, base.py:17-20 and mc_clean.py:66,74).
 * A single running sum over 2^30 elements would lose about 1e-11 of
 * absolute accuracy. */
#define QGO_BLOCK 4096

static double re_vdot(const cplx* a, const cplx* b, int64_t N) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t x0 = 0; x0 < N; x0 += QGO_BLOCK) {
    const int64_t x1 = x0 + QGO_BLOCK < N ? x0 + QGO_BLOCK : N;
    double bs = 0;
    for (int64_t x = x0; x < x1; x++) bs += creal(conj(a[x]) * b[x]);
    s += bs;
  }
  return s;
}

/* Start state: |0..0> (state.py:65-67) or a caller state, then Ry(pi/4) on
 * every qubit (mc_clean.py:48-56). */
static void mcclean_start(cplx* v, int n, const double* ini) {
  const int64_t N = (int64_t)1 << n;
  if (ini) {
    memcpy(v, ini, sizeof(cplx) * (size_t)N);
  } else {
    memset(v, 0, sizeof(cplx) * (size_t)N);
    v[0] = 1.0;
  }
  for (int q = 0; q < n; q++) rot_xy(v, n, q, QGO_Y, QGO_PI / 4.0);
}

static int check_mcclean(int n, int L, const int* axes, int entangler) {
  if (n < 1 || n > 34 || L < 0) return QGO_EINVAL;
  if (entangler < 0 || entangler > 3 || (entangler == QGO_ENT_CNOT_PERIODIC && (n % 2))) return QGO_EINVAL;
  for (int64_t k = 0; k < (int64_t)L * n; k++)
    if (axes[k] < 0 || axes[k] > 2) return QGO_EINVAL; /* mc_clean.py:391-392 */
  return QGO_OK;
}

/* McClean.run_expec_val (mc_clean.py:27-45) with exact expectation value.
 * placement 0: entangler before the rotations of each layer (reference);
 * placement 1: after. */
int qgo_mcclean_run(int n, int L, const int* axes, const double* angles, int entangler, int placement, int nterms,
                    const int* kind, const int* q0, const int* q1, const double* w, const double* ini, double* E,
                    double* final_state) {
  int st = check_mcclean(n, L, axes, entangler);
  if (st) return st;
  const int64_t N = (int64_t)1 << n;
  cplx* v = (cplx*)malloc(sizeof(cplx) * (size_t)N);
  cplx* t = (cplx*)malloc(sizeof(cplx) * (size_t)N);
  if (!v || !t) {
    free(v);
    free(t);
    return QGO_ENOMEM;
  }
  mcclean_start(v, n, ini);
  for (int i = 0; i < L; i++) {
    if (placement == 0) entangle(v, t, n, entangler, 0);
    for (int q = 0; q < n; q++) rot(v, n, q, axes[i * n + q], angles[i * n + q]);
    if (placement == 1) entangle(v, t, n, entangler, 0);
  }
  apply_observable(v, t, n, nterms, kind, q0, q1, w);
  *E = re_vdot(v, t, N);
  if (final_state) memcpy(final_state, v, sizeof(cplx) * (size_t)N);
  free(v);
  free(t);
  return QGO_OK;
}

/* One gradient entry of McClean.grad_run (mc_clean.py:72-75): the
 * reference applies __rot(i, q) and __drot(i, q, -1) to a copy of lambda
 * and takes -2 Re <hist|copy>.  Here the same two gate updates run per
 * amplitude pair (X/Y, state.py:90-97, 142-149) or per amplitude (Z,
 * state.py:168-175) in registers, each element receiving exactly the
 * operations of the two full-vector passes, and the products with conj(hist)
 * are summed in the same pass: no copy of lambda and no write. */
static double grad_entry(const cplx* h, const cplx* v, int n, int q, int axis, double angle) {
  double s = 0;
  if (axis == QGO_Z) {
    const cplx r0 = cexp(-0.5 * I * angle), r1 = cexp(0.5 * I * angle);  /* zrot(angle) */
    const cplx d0 = -0.5 * I * cexp(-0.5 * I * -angle), d1 = 0.5 * I * cexp(0.5 * I * -angle);  /* dzrot(-angle) */
    const int64_t N = (int64_t)1 << n;
    const int64_t bp = bitpos(n, q);
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t x0 = 0; x0 < N; x0 += QGO_BLOCK) {
      const int64_t x1 = x0 + QGO_BLOCK < N ? x0 + QGO_BLOCK : N;
      double bs = 0;
      for (int64_t x = x0; x < x1; x++) {
        const int one = (int)((x >> bp) & 1);
        const cplx r = v[x] * (one ? r1 : r0);
        const cplx d = r * (one ? d1 : d0);
        bs += creal(conj(h[x]) * d);
      }
      s += bs;
    }
    return -2.0 * s;
  }
  const double rs = sin(0.5 * angle), rc = cos(0.5 * angle);       /* rot(angle) */
  const double ds = sin(0.5 * -angle), dc = cos(0.5 * -angle);     /* drot(-angle) */
  const int64_t half = (int64_t)1 << (n - 1);
  const int64_t stride = (int64_t)1 << bitpos(n, q);
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t k0 = 0; k0 < half; k0 += QGO_BLOCK) {
    const int64_t k1 = k0 + QGO_BLOCK < half ? k0 + QGO_BLOCK : half;
    double bs = 0;
    for (int64_t k = k0; k < k1; k++) {
      const int64_t a = ((k & ~(stride - 1)) << 1) | (k & (stride - 1));
      const int64_t b = a | stride;
      const cplx va = v[a], vb = v[b];
      cplx pa, pb;
      if (axis == QGO_X) {
        pa = -I * vb;
        pb = -I * va;
      } else {
        pa = -vb;
        pb = va;
      }
      const cplx ra = rs * pa + rc * va, rb = rs * pb + rc * vb;
      if (axis == QGO_X) {
        pa = -I * rb;
        pb = -I * ra;
      } else {
        pa = -rb;
        pb = ra;
      }
      const cplx da = 0.5 * dc * pa - 0.5 * ds * ra, db = 0.5 * dc * pb - 0.5 * ds * rb;
      bs += creal(conj(h[a]) * da) + creal(conj(h[b]) * db);
    }
    s += bs;
  }
  return -2.0 * s;
}

/* McClean.grad_run (mc_clean.py:47-78).  Forward: store the state before
 * each layer's rotations; E = Re <psi|O psi>.  Backward, per layer: undo the
 * rotations on lambda, then for every qubit grad = -2 Re <hist|drot rot lam>
 * (grad_entry), then the inverse ladder.
 * mode 0 keeps the reference's history of L+1 states (mc_clean.py:22,60);
 * mode 1 (for sizes where L+1 host states do not fit) keeps one psi and
 * uncomputes it alongside lambda: the inverse rotations and inverse ladder
 * take psi back to the state the history would hold, up to rounding
 * (about L n ulps). */
static int mcclean_grad_impl(int n, int L, const int* axes, const double* angles, int entangler, int placement,
                             int nterms, const int* kind, const int* q0, const int* q1, const double* w,
                             const double* ini, double* E, double* grad, int uncompute) {
  int st = check_mcclean(n, L, axes, entangler);
  if (st) return st;
  const int64_t N = (int64_t)1 << n;
  const size_t nh = uncompute ? 1 : (size_t)(L + 1);
  cplx* hist = (cplx*)malloc(sizeof(cplx) * (size_t)N * nh);
  cplx* v = (cplx*)malloc(sizeof(cplx) * (size_t)N);
  cplx* scr = (cplx*)malloc(sizeof(cplx) * (size_t)N);
  if (!hist || !v || !scr) {
    free(hist);
    free(v);
    free(scr);
    return QGO_ENOMEM;
  }
  cplx* psi = hist; /* uncompute mode: the one psi */
  mcclean_start(v, n, ini);
  for (int i = 0; i < L; i++) {
    if (placement == 0) entangle(v, scr, n, entangler, 0);
    if (!uncompute) memcpy(hist + (size_t)i * N, v, sizeof(cplx) * (size_t)N);
    for (int q = 0; q < n; q++) rot(v, n, q, axes[i * n + q], angles[i * n + q]);
    if (placement == 1) entangle(v, scr, n, entangler, 0);
  }
  cplx* last = uncompute ? psi : hist + (size_t)L * N;
  memcpy(last, v, sizeof(cplx) * (size_t)N);
  apply_observable(last, v, n, nterms, kind, q0, q1, w);
  *E = re_vdot(last, v, N);
  for (int i = L - 1; i >= 0; i--) {
    if (placement == 1) {
      entangle(v, scr, n, entangler, 1);
      if (uncompute) entangle(psi, scr, n, entangler, 1);
    }
    for (int q = 0; q < n; q++) rot(v, n, q, axes[i * n + q], -angles[i * n + q]);
    if (uncompute)
      for (int q = 0; q < n; q++) rot(psi, n, q, axes[i * n + q], -angles[i * n + q]);
    const cplx* h = uncompute ? psi : hist + (size_t)i * N;
    for (int q = 0; q < n; q++) grad[i * n + q] = grad_entry(h, v, n, q, axes[i * n + q], angles[i * n + q]);
    if (placement == 0) {
      entangle(v, scr, n, entangler, 1);
      if (uncompute) entangle(psi, scr, n, entangler, 1);
    }
  }
  free(hist);
  free(v);
  free(scr);
  return QGO_OK;
}

int qgo_mcclean_grad(int n, int L, const int* axes, const double* angles, int entangler, int placement, int nterms,
                     const int* kind, const int* q0, const int* q1, const double* w, const double* ini, double* E,
                     double* grad) {
  return mcclean_grad_impl(n, L, axes, angles, entangler, placement, nterms, kind, q0, q1, w, ini, E, grad, 0);
}

int qgo_mcclean_grad_uncompute(int n, int L, const int* axes, const double* angles, int entangler, int placement,
                               int nterms, const int* kind, const int* q0, const int* q1, const double* w,
                               const double* ini, double* E, double* grad) {
  return mcclean_grad_impl(n, L, axes, angles, entangler, placement, nterms, kind, q0, q1, w, ini, E, grad, 1);
}

/* Classical (diagonal) Hamiltonian from the z and zz terms
 * (state.py:261-297): C(x) = sum w_q z_q + sum w_ij z_i z_j, z = +1 for bit 0.
 * X/Y terms are ignored, as there. */
static void classical_ham(double* C, int n, int nterms, const int* kind, const int* q0, const int* q1,
                          const double* w) {
  const int64_t N = (int64_t)1 << n;
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < N; x++) {
    double c = 0;
    for (int t = 0; t < nterms; t++) {
      const int64_t b0 = (int64_t)1 << bitpos(n, q0[t]);
      if (kind[t] == QGO_Z) {
        c += (x & b0) ? -w[t] : w[t];
      } else if (kind[t] == QGO_ZZ) {
        const int64_t b1 = (int64_t)1 << bitpos(n, q1[t]);
        c += (((x & b0) != 0) ^ ((x & b1) != 0)) ? -w[t] : w[t];
      }
    }
    C[x] = c;
  }
}

/* Integer MaxCut table: C(x) = sum_{(i,j)} z_i z_j for unit-weight edges. */
int qgo_maxcut_table(int n, int nedges, const int* edges, int32_t* table) {
  if (n < 1 || n > 34) return QGO_EINVAL;
  const int64_t N = (int64_t)1 << n;
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < N; x++) {
    int32_t c = 0;
    for (int e = 0; e < nedges; e++) {
      const int bi = (int)((x >> bitpos(n, edges[2 * e])) & 1);
      const int bj = (int)((x >> bitpos(n, edges[2 * e + 1])) & 1);
      c += (bi ^ bj) ? -1 : 1;
    }
    table[x] = c;
  }
  return QGO_OK;
}

static void exp_ham(cplx* v, const double* C, int64_t N, double angle) {
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < N; x++) v[x] *= cexp(-I * angle * C[x]);
}

static void qaoa_start(cplx* v, int n, const double* ini) {
  const int64_t N = (int64_t)1 << n;
  if (ini) {
    memcpy(v, ini, sizeof(cplx) * (size_t)N);
  } else {
    const double a = pow(2.0, -0.5 * n); /* state.py:68-69 */
    for (int64_t x = 0; x < N; x++) v[x] = a;
  }
}

/* Qaoa.run_expec_val (qaoa.py:23-38): exp(-i g C) then Rx(beta) on every
 * qubit per layer; exact expectation of the full observable (base.py:17-20). */
int qgo_qaoa_run(int n, int p, const double* betas, const double* gammas, int nterms, const int* kind, const int* q0,
                 const int* q1, const double* w, const double* ini, double* E, double* final_state) {
  if (n < 1 || n > 34 || p < 0) return QGO_EINVAL;
  const int64_t N = (int64_t)1 << n;
  cplx* v = (cplx*)malloc(sizeof(cplx) * (size_t)N);
  cplx* t = (cplx*)malloc(sizeof(cplx) * (size_t)N);
  double* C = (double*)malloc(sizeof(double) * (size_t)N);
  if (!v || !t || !C) {
    free(v);
    free(t);
    free(C);
    return QGO_ENOMEM;
  }
  classical_ham(C, n, nterms, kind, q0, q1, w);
  qaoa_start(v, n, ini);
  for (int i = 0; i < p; i++) {
    exp_ham(v, C, N, gammas[i]);
    for (int q = 0; q < n; q++) rot_xy(v, n, q, QGO_X, betas[i]);
  }
  apply_observable(v, t, n, nterms, kind, q0, q1, w);
  *E = re_vdot(v, t, N);
  if (final_state) memcpy(final_state, v, sizeof(cplx) * (size_t)N);
  free(v);
  free(t);
  free(C);
  return QGO_OK;
}

/* grad[i, 0] of Qaoa.grad_run (qaoa.py:60-64): -2 Re <h| x_summed lam> with
 * x_summed = 1/2 sum_q (-i X_q) (state.py:107-123), evaluated per amplitude
 * and summed in the same pass (no copy of lambda). */
static double grad_beta(const cplx* h, const cplx* v, int n) {
  const int64_t N = (int64_t)1 << n;
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t x0 = 0; x0 < N; x0 += QGO_BLOCK) {
    const int64_t x1 = x0 + QGO_BLOCK < N ? x0 + QGO_BLOCK : N;
    double bs = 0;
    for (int64_t x = x0; x < x1; x++) {
      cplx acc = 0;
      for (int q = 0; q < n; q++) acc += 0.5 * (-I) * v[x ^ ((int64_t)1 << bitpos(n, q))];
      bs += creal(conj(h[x]) * acc);
    }
    s += bs;
  }
  return -2.0 * s;
}

/* grad[i, 1] (qaoa.py:65-69): -2 Re <h| (-i C) lam> (state.py:319-321). */
static double grad_gamma(const cplx* h, const cplx* v, const double* C, int64_t N) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t x0 = 0; x0 < N; x0 += QGO_BLOCK) {
    const int64_t x1 = x0 + QGO_BLOCK < N ? x0 + QGO_BLOCK : N;
    double bs = 0;
    for (int64_t x = x0; x < x1; x++) bs += creal(conj(h[x]) * (v[x] * (-I * C[x])));
    s += bs;
  }
  return -2.0 * s;
}

/* Qaoa.grad_run (qaoa.py:40-70).  grad[i,0] is d/d beta_i, grad[i,1] is
 * d/d gamma_i; E uses the classical Hamiltonian (qaoa.py:56-57).  mode 0
 * keeps the reference's history of 2p+1 states; mode 1 uncomputes psi
 * alongside lambda (inverse mixer, inverse cost phase). */
static int qaoa_grad_impl(int n, int p, const double* betas, const double* gammas, int nterms, const int* kind,
                          const int* q0, const int* q1, const double* w, const double* ini, double* E, double* grad,
                          int uncompute) {
  if (n < 1 || n > 34 || p < 0) return QGO_EINVAL;
  const int64_t N = (int64_t)1 << n;
  const size_t nh = uncompute ? 1 : (size_t)(2 * p + 1);
  cplx* hist = (cplx*)malloc(sizeof(cplx) * (size_t)N * nh);
  cplx* v = (cplx*)malloc(sizeof(cplx) * (size_t)N);
  double* C = (double*)malloc(sizeof(double) * (size_t)N);
  if (!hist || !v || !C) {
    free(hist);
    free(v);
    free(C);
    return QGO_ENOMEM;
  }
  cplx* psi = hist;
  classical_ham(C, n, nterms, kind, q0, q1, w);
  qaoa_start(v, n, ini);
  for (int i = 0; i < p; i++) {
    if (!uncompute) memcpy(hist + (size_t)(2 * i) * N, v, sizeof(cplx) * (size_t)N);
    exp_ham(v, C, N, gammas[i]);
    if (!uncompute) memcpy(hist + (size_t)(2 * i + 1) * N, v, sizeof(cplx) * (size_t)N);
    for (int q = 0; q < n; q++) rot_xy(v, n, q, QGO_X, betas[i]);
  }
  cplx* last = uncompute ? psi : hist + (size_t)(2 * p) * N;
  memcpy(last, v, sizeof(cplx) * (size_t)N);
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < N; x++) v[x] *= C[x];
  *E = re_vdot(last, v, N);
  for (int i = p - 1; i >= 0; i--) {
    for (int q = 0; q < n; q++) rot_xy(v, n, q, QGO_X, -betas[i]);
    if (uncompute)
      for (int q = 0; q < n; q++) rot_xy(psi, n, q, QGO_X, -betas[i]);
    grad[2 * i + 0] = grad_beta(uncompute ? psi : hist + (size_t)(2 * i + 1) * N, v, n);
    exp_ham(v, C, N, -gammas[i]);
    if (uncompute) exp_ham(psi, C, N, -gammas[i]);
    grad[2 * i + 1] = grad_gamma(uncompute ? psi : hist + (size_t)(2 * i) * N, v, C, N);
  }
  free(hist);
  free(v);
  free(C);
  return QGO_OK;
}

int qgo_qaoa_grad(int n, int p, const double* betas, const double* gammas, int nterms, const int* kind,
                  const int* q0, const int* q1, const double* w, const double* ini, double* E, double* grad) {
  return qaoa_grad_impl(n, p, betas, gammas, nterms, kind, q0, q1, w, ini, E, grad, 0);
}

int qgo_qaoa_grad_uncompute(int n, int p, const double* betas, const double* gammas, int nterms, const int* kind,
                            const int* q0, const int* q1, const double* w, const double* ini, double* E,
                            double* grad) {
  return qaoa_grad_impl(n, p, betas, gammas, nterms, kind, q0, q1, w, ini, E, grad, 1);
}

/* Entangler alone, for tests of the ladder permutation. */
int qgo_entangle(int n, int kind, int inverse, double* state) {
  const int64_t N = (int64_t)1 << n;
  cplx* scr = (cplx*)malloc(sizeof(cplx) * (size_t)N);
  if (!scr) return QGO_ENOMEM;
  int st = entangle((cplx*)state, scr, n, kind, inverse);
  free(scr);
  return st;
}

int qgo_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
