/*
 * qcs_oracle.c -- CPU FP64 oracle (test infrastructure only; see the header).
 *
 * Compile with -std=c89 -O2 -ffp-contract=off: the reference is built the
 * same way, and contraction into FMA would change the last bit of results.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "qcs_oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  double re;
  double im;
} oc;

struct orc_state {
  int n;
  long size;
  int mode;
  oc *vec;     /* live state (reference: state->vector) */
  oc *scratch; /* second buffer (reference: state->scratch_vector) */
};

/* Complex helpers: src/complex.c:23-57 (c_add, c_mul) and :88-99
 * (c_norm_sq, c_magnitude), same operation order. */
static oc oc_add(oc a, oc b) {
  oc r;
  r.re = a.re + b.re;
  r.im = a.im + b.im;
  return r;
}

static oc oc_mul(oc a, oc b) {
  oc r;
  r.re = (a.re * b.re) - (a.im * b.im);
  r.im = (a.re * b.im) + (a.im * b.re);
  return r;
}

static double oc_norm_sq(oc a) { return (a.re * a.re) + (a.im * a.im); }

static oc oc_make(double re, double im) {
  oc r;
  r.re = re;
  r.im = im;
  return r;
}

static void swap_buffers(orc_state *s) {
  oc *t = s->vec;
  s->vec = s->scratch;
  s->scratch = t;
}

/* q_state_init (src/q_state.c:32-101): both buffers zeroed, vector[0] = 1. */
orc_state *orc_create(int num_qubits, int mode) {
  orc_state *s;
  long size;
  if (num_qubits <= 0 || num_qubits > 40)
    return NULL;
  size = 1L << num_qubits;
  s = (orc_state *)malloc(sizeof(orc_state));
  if (!s)
    return NULL;
  s->n = num_qubits;
  s->size = size;
  s->mode = mode;
  s->vec = (oc *)calloc((size_t)size, sizeof(oc));
  s->scratch = (oc *)calloc((size_t)size, sizeof(oc));
  if (!s->vec || !s->scratch) {
    free(s->vec);
    free(s->scratch);
    free(s);
    return NULL;
  }
  s->vec[0].re = 1.0;
  return s;
}

void orc_destroy(orc_state *s) {
  if (!s)
    return;
  free(s->vec);
  free(s->scratch);
  free(s);
}

int orc_num_qubits(const orc_state *s) { return s->n; }

/* Threads of the OpenMP sweeps (timing of the CPU baseline: 1 = the
 * reference's sequential mode, all cores = its OpenMP mode); returns the
 * previous setting, 1 without OpenMP. */
int orc_set_threads(int threads) {
#ifdef _OPENMP
  int prev = omp_get_max_threads();
  if (threads > 0)
    omp_set_num_threads(threads);
  return prev;
#else
  (void)threads;
  return 1;
#endif
}
long orc_size(const orc_state *s) { return s->size; }
int orc_mode(const orc_state *s) { return s->mode; }

/* q_state_set_basis (src/q_state.c:122-132): zeroes the live buffer only. */
void orc_set_basis(orc_state *s, long index) {
  long i;
  if (index < 0 || index >= s->size)
    return;
  for (i = 0; i < s->size; i++)
    s->vec[i] = oc_make(0.0, 0.0);
  s->vec[index] = oc_make(1.0, 0.0);
}

void orc_read(const orc_state *s, long first, long count, double *out) {
  long i;
  for (i = 0; i < count; i++) {
    out[2 * i] = s->vec[first + i].re;
    out[2 * i + 1] = s->vec[first + i].im;
  }
}

void orc_write(orc_state *s, long first, long count, const double *in) {
  long i;
  for (i = 0; i < count; i++) {
    s->vec[first + i].re = in[2 * i];
    s->vec[first + i].im = in[2 * i + 1];
  }
}

/* Gate matrices, row-major {U00,U01,U10,U11} as (re,im) pairs:
 * src/q_gates.c:362-491 (I, X, H, CP, Y, Z, P, RX, RY, RZ). */
void orc_gate_matrix(int kind, double angle, double out[8]) {
  double h;
  double ch;
  double sh;
  memset(out, 0, 8 * sizeof(double));
  switch (kind) {
  case ORC_GATE_I:
    out[0] = 1.0;
    out[6] = 1.0;
    break;
  case ORC_GATE_X:
  case ORC_GATE_CNOT:
    out[2] = 1.0;
    out[4] = 1.0;
    break;
  case ORC_GATE_H:
    h = 1.0 / sqrt(2.0);
    out[0] = h;
    out[2] = h;
    out[4] = h;
    out[6] = -h;
    break;
  case ORC_GATE_Y:
    out[3] = -1.0;
    out[5] = 1.0;
    break;
  case ORC_GATE_Z:
    out[0] = 1.0;
    out[6] = -1.0;
    break;
  case ORC_GATE_P:
  case ORC_GATE_CPHASE:
    out[0] = 1.0;
    out[6] = cos(angle);
    out[7] = sin(angle);
    break;
  case ORC_GATE_RX:
    ch = cos(angle / 2.0);
    sh = sin(angle / 2.0);
    out[0] = ch;
    out[3] = -sh;
    out[5] = -sh;
    out[6] = ch;
    break;
  case ORC_GATE_RY:
    ch = cos(angle / 2.0);
    sh = sin(angle / 2.0);
    out[0] = ch;
    out[2] = -sh;
    out[4] = sh;
    out[6] = ch;
    break;
  case ORC_GATE_RZ:
    ch = cos(angle / 2.0);
    sh = sin(angle / 2.0);
    out[0] = ch;
    out[1] = -sh;
    out[6] = ch;
    out[7] = sh;
    break;
  default:
    out[0] = 1.0;
    out[6] = 1.0;
    break;
  }
}

static void load_matrix(const double m[8], oc g[4]) {
  int i;
  for (i = 0; i < 4; i++)
    g[i] = oc_make(m[2 * i], m[2 * i + 1]);
}

/* q_apply_1q_gate, sequential branch (src/q_gates.c:131-148). Physical mode
 * sweeps in place; compat mode writes the scratch buffer and swaps, so the
 * previous state stays behind in scratch exactly as in the reference. */
int orc_apply_1q(orc_state *s, const double m[8], int target) {
  long step;
  long np;
  long p;
  oc g[4];
  oc *dst;
  oc *src;
  if (target < 0 || target >= s->n)
    return -1;
  load_matrix(m, g);
  step = 1L << target;
  np = s->size / 2;
  src = s->vec;
  dst = (s->mode == ORC_COMPAT) ? s->scratch : s->vec;
  /* pair p -> (lo, lo + step): the reference's block/offset double loop
   * (src/q_gates.c:133-143) flattened; pairs are independent, so the sweep
   * may run on several threads without changing a bit. */
#pragma omp parallel for schedule(static)
  for (p = 0; p < np; p++) {
    long lo = ((p >> target) << (target + 1)) | (p & (step - 1));
    oc v0 = src[lo];
    oc v1 = src[lo + step];
    dst[lo] = oc_add(oc_mul(g[0], v0), oc_mul(g[1], v1));
    dst[lo + step] = oc_add(oc_mul(g[2], v0), oc_mul(g[3], v1));
  }
  if (s->mode == ORC_COMPAT)
    swap_buffers(s);
  return 0;
}

/* q_apply_2q_gate, sequential branch (src/q_gates.c:277-297).
 * Compat: the ascending loop first writes both members of each control=1
 * pair and later overwrites the target=1 member with its old value, so the
 * net effect is (U00 v0 + U01 v1, v1) on control=1 pairs and a copy
 * elsewhere.  Physical: the unitary controlled-U on control=1 pairs.
 * Sums (norms, means, probabilities) below stay sequential: their order
 * fixes the last bit. */
int orc_apply_controlled(orc_state *s, const double m[8], int control,
                         int target) {
  long cb;
  long tb;
  long np;
  long p;
  oc g[4];
  oc *src;
  oc *dst;
  int compat;
  if (control < 0 || target < 0 || control >= s->n || target >= s->n ||
      control == target)
    return -1;
  load_matrix(m, g);
  cb = 1L << control;
  tb = 1L << target;
  np = s->size / 2;
  compat = s->mode == ORC_COMPAT;
  src = s->vec;
  dst = compat ? s->scratch : s->vec;
  /* Per target pair (lo, hi = lo | tb); the sequential loop's final values
   * of both members are written at once, so pairs are independent. */
#pragma omp parallel for schedule(static)
  for (p = 0; p < np; p++) {
    long lo = ((p >> target) << (target + 1)) | (p & (tb - 1));
    long hi = lo | tb;
    oc v0 = src[lo];
    oc v1 = src[hi];
    if (lo & cb) {
      dst[lo] = oc_add(oc_mul(g[0], v0), oc_mul(g[1], v1));
      dst[hi] = compat ? v1 : oc_add(oc_mul(g[2], v0), oc_mul(g[3], v1));
    } else if (compat) {
      dst[lo] = v0;
      dst[hi] = v1;
    }
  }
  if (compat)
    swap_buffers(s);
  return 0;
}

/* One named gate, as the qc_<gate> wrappers of src/qcs.c:159-228,431-437,
 * 485-516 build and apply it. */
int orc_apply_gate(orc_state *s, int kind, int target, int control,
                   double angle) {
  double m[8];
  orc_gate_matrix(kind, angle, m);
  if (kind == ORC_GATE_CNOT || kind == ORC_GATE_CPHASE)
    return orc_apply_controlled(s, m, control, target);
  return orc_apply_1q(s, m, target);
}

int orc_run_gates(orc_state *s, int count, const int *kinds,
                  const int *targets, const int *controls,
                  const double *angles) {
  int i;
  int rc;
  for (i = 0; i < count; i++) {
    rc = orc_apply_gate(s, kinds[i], targets[i], controls[i], angles[i]);
    if (rc != 0)
      return rc;
  }
  return 0;
}

int orc_run_ops(orc_state *s, int count, const int *kinds, const int *targets,
                const int *controls, const double *angles,
                const long *indices) {
  int i;
  int rc;
  for (i = 0; i < count; i++) {
    if (kinds[i] == ORC_OP_PHASE_FLIP)
      rc = orc_phase_flip(s, indices[i]);
    else if (kinds[i] == ORC_OP_DIFFUSION)
      rc = orc_diffusion(s);
    else
      rc = orc_apply_gate(s, kinds[i], targets[i], controls[i], angles[i]);
    if (rc != 0)
      return rc;
  }
  return 0;
}

/* Dense 2^k x 2^k block on an ordered qubit list (bit j of the block index
 * is qubit qubits[j]); u is row-major (re,im).  The reference has no fused
 * path; its dense N x N apply (src/q_matrix.c:59-96) is the closest
 * ancestor.  Physical semantics, in place. */
int orc_apply_block(orc_state *s, int k, const int *qubits, const double *u) {
  long kk;
  long mask = 0;
  long base;
  long a;
  long b;
  long *off;
  oc *vin;
  oc *vout;
  int j;
  if (k < 1 || k > 12 || k > s->n)
    return -1;
  for (j = 0; j < k; j++) {
    if (qubits[j] < 0 || qubits[j] >= s->n || (mask & (1L << qubits[j])))
      return -1;
    mask |= 1L << qubits[j];
  }
  kk = 1L << k;
  off = (long *)malloc((size_t)kk * sizeof(long));
  vin = (oc *)malloc((size_t)kk * sizeof(oc));
  vout = (oc *)malloc((size_t)kk * sizeof(oc));
  if (!off || !vin || !vout) {
    free(off);
    free(vin);
    free(vout);
    return -1;
  }
  for (a = 0; a < kk; a++) {
    off[a] = 0;
    for (j = 0; j < k; j++)
      if ((a >> j) & 1)
        off[a] |= 1L << qubits[j];
  }
  for (base = 0; base < s->size; base++) {
    if (base & mask)
      continue;
    for (a = 0; a < kk; a++)
      vin[a] = s->vec[base | off[a]];
    for (a = 0; a < kk; a++) {
      oc acc = oc_make(0.0, 0.0);
      for (b = 0; b < kk; b++) {
        oc g = oc_make(u[2 * (a * kk + b)], u[2 * (a * kk + b) + 1]);
        acc = oc_add(acc, oc_mul(g, vin[b]));
      }
      vout[a] = acc;
    }
    for (a = 0; a < kk; a++)
      s->vec[base | off[a]] = vout[a];
  }
  free(off);
  free(vin);
  free(vout);
  return 0;
}

/* q_apply_phase_flip (src/q_gates.c:305-317).  Compat swaps first, so the
 * live buffer becomes the stale previous state with one entry replaced by
 * the negated current amplitude. */
int orc_phase_flip(orc_state *s, long index) {
  if (index < 0 || index >= s->size)
    return -1;
  if (s->mode == ORC_COMPAT) {
    swap_buffers(s);
    s->vec[index].re = -s->scratch[index].re;
    s->vec[index].im = -s->scratch[index].im;
  } else {
    s->vec[index].re = -s->vec[index].re;
    s->vec[index].im = -s->vec[index].im;
  }
  return 0;
}

/* q_apply_diffusion (src/q_gates.c:323-356).  Compat divides the summed
 * amplitude by its magnitude (when above 1e-10) and writes 2m - psi into the
 * swapped-in buffer; physical uses the true mean sum/N, in place. */
int orc_diffusion(orc_state *s) {
  long i;
  oc mean = oc_make(0.0, 0.0);
  oc two;
  for (i = 0; i < s->size; i++)
    mean = oc_add(mean, s->vec[i]);
  if (s->mode == ORC_COMPAT) {
    double mag = sqrt(oc_norm_sq(mean));
    if (mag > 1e-10) {
      mean.re /= mag;
      mean.im /= mag;
    }
    two = oc_make(2.0 * mean.re, 2.0 * mean.im);
    swap_buffers(s);
#pragma omp parallel for schedule(static)
    for (i = 0; i < s->size; i++) {
      s->vec[i].re = two.re - s->scratch[i].re;
      s->vec[i].im = two.im - s->scratch[i].im;
    }
  } else {
    mean.re /= (double)s->size;
    mean.im /= (double)s->size;
    two = oc_make(2.0 * mean.re, 2.0 * mean.im);
#pragma omp parallel for schedule(static)
    for (i = 0; i < s->size; i++) {
      s->vec[i].re = two.re - s->vec[i].re;
      s->vec[i].im = two.im - s->vec[i].im;
    }
  }
  return 0;
}

double orc_norm_sq(const orc_state *s) {
  long i;
  double t = 0.0;
  for (i = 0; i < s->size; i++)
    t += oc_norm_sq(s->vec[i]);
  return t;
}

/* q_state_normalize, sequential branch (src/q_utils.c:44-119 at :105-118):
 * rescale only when the norm^2 is above 1e-12 and not exactly 1. */
void orc_normalize(orc_state *s) {
  long i;
  double total = orc_norm_sq(s);
  if (total > 1e-12 && total != 1.0) {
    double inv = 1.0 / sqrt(total);
#pragma omp parallel for schedule(static)
    for (i = 0; i < s->size; i++) {
      s->vec[i].re *= inv;
      s->vec[i].im *= inv;
    }
  }
}

/* First loop of qc_measure (src/qcs.c:253-259). */
double orc_prob_zero(const orc_state *s, int qubit) {
  long i;
  double p0 = 0.0;
  for (i = 0; i < s->size; i++) {
    if ((i & (1L << qubit)) == 0) {
      double re = s->vec[i].re;
      double im = s->vec[i].im;
      p0 += (re * re) + (im * im);
    }
  }
  return p0;
}

/* qc_measure (src/qcs.c:237-284) with the caller's rand()/RAND_MAX value:
 * outcome 0 when random_val <= p0, the other half zeroed, then normalised. */
int orc_measure(orc_state *s, int qubit, double random_val) {
  long i;
  double p0;
  int outcome;
  if (qubit < 0 || qubit >= s->n)
    return 0;
  p0 = orc_prob_zero(s, qubit);
  outcome = (random_val <= p0) ? 0 : 1;
  for (i = 0; i < s->size; i++) {
    int bit = (i & (1L << qubit)) != 0;
    if (bit != outcome) {
      s->vec[i].re = 0.0;
      s->vec[i].im = 0.0;
    }
  }
  orc_normalize(s);
  return outcome;
}

/* qc_get_probability (src/qcs.c:391-395). */
double orc_probability(const orc_state *s, long index) {
  if (index < 0 || index >= s->size)
    return 0.0;
  return oc_norm_sq(s->vec[index]);
}

/* qc_find_most_likely_state (src/qcs.c:464-478): first strict maximum,
 * starting from (0, 0.0). */
long orc_argmax(const orc_state *s) {
  long i;
  long best = 0;
  double bp = 0.0;
  for (i = 0; i < s->size; i++) {
    double p = oc_norm_sq(s->vec[i]);
    if (p > bp) {
      bp = p;
      best = i;
    }
  }
  return best;
}

/* Sampling loop of qc_run_shots (src/qcs.c:589-605): per shot, the first
 * index whose running FP64 sum exceeds the draw (strict <); -1 when the draw
 * is not below the total (the reference then counts nothing). */
void orc_sample(const orc_state *s, const double *random_vals, int shots,
                long *out_index) {
  int k;
  long i;
  double *p = (double *)malloc((size_t)s->size * sizeof(double));
  if (!p)
    return;
  for (i = 0; i < s->size; i++)
    p[i] = orc_probability(s, i);
  for (k = 0; k < shots; k++) {
    double cum = 0.0;
    out_index[k] = -1;
    for (i = 0; i < s->size; i++) {
      cum += p[i];
      if (random_vals[k] < cum) {
        out_index[k] = i;
        break;
      }
    }
  }
  free(p);
}

/* <Z_q> = sum over i of (+1 if bit q of i is 0 else -1) |psi_i|^2.  Not in
 * the reference; the variational-batch workload returns it per instance. */
double orc_expect_z(const orc_state *s, int qubit) {
  long i;
  double t = 0.0;
  for (i = 0; i < s->size; i++) {
    double p = oc_norm_sq(s->vec[i]);
    if (i & (1L << qubit))
      t -= p;
    else
      t += p;
  }
  return t;
}

/* q_grover_iterations (src/q_utils.c:126-134).  The reference forms
 * (double)(1 << n), which overflows int for n >= 31; ldexp gives the same
 * value wherever the reference is defined. */
int orc_grover_iterations(int num_qubits) {
  double pi = 3.14159265358979323846;
  double n = ldexp(1.0, num_qubits);
  return (int)floor((pi / 4.0) * sqrt(n));
}

/* qc_quantum_fourier_transform (src/qcs.c:443-457): H(i), then
 * CPHASE(control j, target i, pi / 2^(j-i)) for j > i; no final swaps.
 * ldexp replaces the reference's (1 << (j-i)), equal for j-i <= 30. */
void orc_qft(orc_state *s) {
  double pi = 3.14159265358979323846;
  int i;
  int j;
  for (i = 0; i < s->n; i++) {
    orc_apply_gate(s, ORC_GATE_H, i, -1, 0.0);
    for (j = i + 1; j < s->n; j++) {
      double angle = pi / ldexp(1.0, j - i);
      orc_apply_gate(s, ORC_GATE_CPHASE, i, j, angle);
    }
  }
}

/* qc_grover_search (src/qcs.c:402-419): H on every qubit, then
 * `iterations` x (phase flip, diffusion).  iterations < 0 selects the
 * reference's count q_grover_iterations(n). */
void orc_grover(orc_state *s, long solution, int iterations) {
  int q;
  int i;
  if (iterations < 0)
    iterations = orc_grover_iterations(s->n);
  for (q = 0; q < s->n; q++)
    orc_apply_gate(s, ORC_GATE_H, q, -1, 0.0);
  for (i = 0; i < iterations; i++) {
    orc_phase_flip(s, solution);
    orc_diffusion(s);
  }
}
