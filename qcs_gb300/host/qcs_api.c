/*
 * qcs_api.c -- the public QCS API (include/qcs.h) on the GB300 backend.
 *
 * C89 host code over the C ABI of include/qcs_cuda.h: the circuit keeps the
 * reference's gate history and printing (src/qcs.c:13-23, :132-152,
 * :308-383, :650-698), while every touch of the state vector goes to the
 * device.  Argument errors print the reference's messages and leave the
 * state alone, exactly as src/q_gates.c:32-36 and :165-170 do; a gate is
 * recorded in the history even when its arguments were rejected (the
 * reference calls qc_add_gate unconditionally).
 *
 * With a fusion width k >= 2 gates are queued and applied, fused, at the
 * next point where the state is observed (measure, probability, argmax,
 * shots, print, Grover, basis reset); results are the same up to rounding.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/qcs.h"
#include "../../include/qcs_cuda.h"
#include "../../include/qcs_ext.h"

struct t_q_circuit {
  int num_qubits;
  int num_gates;
  qcs_cuda_state *state;
  char **gate_history;
  int *target_qubits;
  int *control_qubits;
  double *parameters;
  int history_size;
  int history_capacity;
  int fusion_k;
  qcs_cuda_op *pending;
  int num_pending;
  int pending_capacity;
};

static void report(const char *what, int rc) {
  fprintf(stderr, "Error: %s failed: %s (%s)\n", what, qcs_cuda_strerror(rc),
          qcs_cuda_last_error());
}

static int env_int(const char *name, int dflt) {
  const char *v = getenv(name);
  if (!v || !*v)
    return dflt;
  return atoi(v);
}

static int env_precision(void) {
  const char *v = getenv("QCS_CUDA_PRECISION");
  if (v && (strcmp(v, "c128") == 0 || strcmp(v, "complex128") == 0))
    return QCS_CUDA_C128;
  return QCS_CUDA_C64;
}

static int env_semantics(void) {
  const char *v = getenv("QCS_CUDA_SEMANTICS");
  if (v && strcmp(v, "reference") == 0)
    return QCS_CUDA_REFERENCE;
  return QCS_CUDA_PHYSICAL;
}

t_q_circuit *qc_create_ex(int num_qubits, int precision, int semantics,
                          int fusion_k) {
  t_q_circuit *c;
  int rc;
  if (num_qubits <= 0) {
    fprintf(stderr, "Error: Number of qubits must be positive.\n");
    return NULL;
  }
  c = (t_q_circuit *)calloc(1, sizeof(t_q_circuit));
  if (!c)
    return NULL;
  c->num_qubits = num_qubits;
  c->history_capacity = 100;
  c->fusion_k = (semantics == QCS_CUDA_REFERENCE) ? 0 : fusion_k;
  rc = qcs_cuda_state_create(num_qubits, precision, semantics, &c->state);
  c->gate_history = (char **)malloc(c->history_capacity * sizeof(char *));
  c->target_qubits = (int *)malloc(c->history_capacity * sizeof(int));
  c->control_qubits = (int *)malloc(c->history_capacity * sizeof(int));
  c->parameters = (double *)malloc(c->history_capacity * sizeof(double));
  if (rc != QCS_CUDA_OK || !c->gate_history || !c->target_qubits ||
      !c->control_qubits || !c->parameters) {
    if (rc != QCS_CUDA_OK)
      report("qc_create", rc);
    qc_destroy(c);
    return NULL;
  }
  return c;
}

t_q_circuit *qc_create(int num_qubits) {
  return qc_create_ex(num_qubits, env_precision(), env_semantics(),
                      env_int("QCS_CUDA_FUSION", 0));
}

void qc_destroy(t_q_circuit *circuit) {
  int i;
  if (!circuit)
    return;
  if (circuit->state)
    qcs_cuda_state_destroy(circuit->state);
  if (circuit->gate_history) {
    for (i = 0; i < circuit->history_size; i++)
      free(circuit->gate_history[i]);
    free(circuit->gate_history);
  }
  free(circuit->target_qubits);
  free(circuit->control_qubits);
  free(circuit->parameters);
  free(circuit->pending);
  free(circuit);
}

/* ---- gate history (src/qcs.c:109-152) --------------------------------- */

static char *dup_name(const char *s) {
  size_t n = strlen(s) + 1;
  char *d = (char *)malloc(n);
  if (d)
    memcpy(d, s, n);
  return d;
}

static void add_gate(t_q_circuit *c, const char *name, int target, int control,
                     double param) {
  if (c->history_size >= c->history_capacity) {
    int cap = c->history_capacity * 2;
    char **h = (char **)realloc(c->gate_history, cap * sizeof(char *));
    int *t = (int *)realloc(c->target_qubits, cap * sizeof(int));
    int *k = (int *)realloc(c->control_qubits, cap * sizeof(int));
    double *p = (double *)realloc(c->parameters, cap * sizeof(double));
    if (h)
      c->gate_history = h;
    if (t)
      c->target_qubits = t;
    if (k)
      c->control_qubits = k;
    if (p)
      c->parameters = p;
    if (!h || !t || !k || !p)
      return;
    c->history_capacity = cap;
  }
  c->gate_history[c->history_size] = dup_name(name);
  c->target_qubits[c->history_size] = target;
  c->control_qubits[c->history_size] = control;
  c->parameters[c->history_size] = param;
  c->history_size++;
  c->num_gates++;
}

/* ---- the device queue --------------------------------------------------- */

void qc_flush(t_q_circuit *c) {
  qcs_cuda_run_options opt;
  int rc;
  if (!c || !c->state || c->num_pending == 0)
    return;
  opt.fusion_k = c->fusion_k;
  opt.fusion_engine = QCS_FUSE_AUTO;
  opt.partitioner = QCS_PARTITION_GREEDY;
  opt.flags = 0;
  rc = qcs_cuda_run(c->state, c->pending, c->num_pending, &opt);
  c->num_pending = 0;
  if (rc != QCS_CUDA_OK)
    report("gate application", rc);
}

static void submit(t_q_circuit *c, int kind, int target, int control,
                   double angle, long long index) {
  qcs_cuda_op *o;
  int rc;
  if (c->fusion_k < 2) {
    qcs_cuda_op op;
    memset(&op, 0, sizeof(op));
    op.kind = kind;
    op.target = target;
    op.control = control;
    op.angle = angle;
    op.index = index;
    rc = qcs_cuda_run(c->state, &op, 1, NULL);
    if (rc != QCS_CUDA_OK)
      report("gate application", rc);
    return;
  }
  if (c->num_pending >= c->pending_capacity) {
    int cap = c->pending_capacity ? 2 * c->pending_capacity : 256;
    qcs_cuda_op *p =
        (qcs_cuda_op *)realloc(c->pending, cap * sizeof(qcs_cuda_op));
    if (!p) {
      qc_flush(c);
      p = c->pending;
      if (!p)
        return;
    } else {
      c->pending = p;
      c->pending_capacity = cap;
    }
  }
  o = &c->pending[c->num_pending++];
  memset(o, 0, sizeof(*o));
  o->kind = kind;
  o->target = target;
  o->control = control;
  o->angle = angle;
  o->index = index;
  if (c->num_pending >= 4096)
    qc_flush(c);
}

static int valid_1q(t_q_circuit *c, int q) {
  if (!c || !c->state || q < 0 || q >= c->num_qubits) {
    fprintf(stderr, "Error: Invalid arguments for 1-qubit gate application.\n");
    return 0;
  }
  return 1;
}

static int valid_2q(t_q_circuit *c, int ctl, int tgt) {
  if (!c || !c->state || ctl < 0 || tgt < 0 || ctl >= c->num_qubits ||
      tgt >= c->num_qubits || ctl == tgt) {
    fprintf(stderr, "Error: Invalid arguments for 2-qubit gate application.\n");
    return 0;
  }
  return 1;
}

static void gate1(t_q_circuit *c, int kind, const char *name, int q, double a) {
  if (valid_1q(c, q))
    submit(c, kind, q, -1, a, 0);
  add_gate(c, name, q, -1, a);
}

void qc_h(t_q_circuit *c, int q) { gate1(c, QCS_GATE_H, "H", q, 0.0); }
void qc_x(t_q_circuit *c, int q) { gate1(c, QCS_GATE_X, "X", q, 0.0); }
void qc_y(t_q_circuit *c, int q) { gate1(c, QCS_GATE_Y, "Y", q, 0.0); }
void qc_z(t_q_circuit *c, int q) { gate1(c, QCS_GATE_Z, "Z", q, 0.0); }
void qc_phase(t_q_circuit *c, int q, double a) { gate1(c, QCS_GATE_P, "P", q, a); }
void qc_rx(t_q_circuit *c, int q, double a) { gate1(c, QCS_GATE_RX, "RX", q, a); }
void qc_ry(t_q_circuit *c, int q, double a) { gate1(c, QCS_GATE_RY, "RY", q, a); }
void qc_rz(t_q_circuit *c, int q, double a) { gate1(c, QCS_GATE_RZ, "RZ", q, a); }

void qc_cnot(t_q_circuit *c, int control, int target) {
  if (valid_2q(c, control, target))
    submit(c, QCS_GATE_CNOT, target, control, 0.0, 0);
  add_gate(c, "CNOT", target, control, 0.0);
}

void qc_cphase(t_q_circuit *c, int control, int target, double angle) {
  if (valid_2q(c, control, target))
    submit(c, QCS_GATE_CPHASE, target, control, angle, 0);
  add_gate(c, "CPHASE", target, control, angle);
}

void qc_barrier(t_q_circuit *c) { add_gate(c, "BARRIER", -1, -1, 0.0); }

/* ---- measurement and read-out ------------------------------------------ */

/* qc_measure (src/qcs.c:237-284): one rand() draw per call, outcome 0 when
 * rand()/RAND_MAX <= P(0). */
int qc_measure(t_q_circuit *c, int qubit) {
  double r;
  int outcome = 0;
  int rc;
  if (c == NULL || c->state == NULL || qubit < 0 || qubit >= c->num_qubits)
    return 0;
  qc_flush(c);
  r = rand() / (double)RAND_MAX;
  rc = qcs_cuda_measure(c->state, qubit, r, &outcome);
  if (rc != QCS_CUDA_OK) {
    report("qc_measure", rc);
    return 0;
  }
  return outcome;
}

void qc_measure_all(t_q_circuit *c, int *results) {
  int i;
  if (c == NULL || results == NULL)
    return;
  for (i = 0; i < c->num_qubits; i++)
    results[i] = qc_measure(c, i);
  add_gate(c, "MEASURE", -1, -1, 0.0);
}

void qc_reset(t_q_circuit *c, int qubit) {
  if (qc_measure(c, qubit) == 1)
    qc_x(c, qubit);
  add_gate(c, "RESET", qubit, -1, 0.0);
}

void qc_run(t_q_circuit *c) {
  int *results;
  if (!c)
    return;
  results = (int *)malloc(c->num_qubits * sizeof(int));
  if (results) {
    qc_measure_all(c, results);
    free(results);
  }
}

int qc_sample_shots(t_q_circuit *c, int shots, long long *samples) {
  double *draws;
  int s;
  int rc;
  if (!c || !c->state || shots <= 0 || !samples)
    return -1;
  qc_flush(c);
  draws = (double *)malloc(shots * sizeof(double));
  if (!draws)
    return -1;
  for (s = 0; s < shots; s++)
    draws[s] = rand() / (double)RAND_MAX;
  rc = qcs_cuda_sample(c->state, draws, shots, samples);
  free(draws);
  if (rc != QCS_CUDA_OK) {
    report("qc_run_shots", rc);
    return -1;
  }
  return 0;
}

/* qc_run_shots (src/qcs.c:575-607): `results` is a histogram over all 2^n
 * basis states. */
void qc_run_shots(t_q_circuit *c, int shots, int *results) {
  long long *samples;
  long n_states;
  int s;
  if (!c || shots <= 0 || !results || !c->state)
    return;
  n_states = 1L << c->num_qubits;
  samples = (long long *)malloc(shots * sizeof(long long));
  if (!samples)
    return;
  if (qc_sample_shots(c, shots, samples) == 0) {
    memset(results, 0, n_states * sizeof(int));
    for (s = 0; s < shots; s++)
      if (samples[s] >= 0)
        results[samples[s]]++;
  }
  free(samples);
}

long long qc_find_most_likely_state64(t_q_circuit *c) {
  long long idx = 0;
  int rc;
  if (!c || !c->state)
    return 0;
  qc_flush(c);
  rc = qcs_cuda_argmax(c->state, &idx, NULL);
  if (rc != QCS_CUDA_OK) {
    report("qc_find_most_likely_state", rc);
    return 0;
  }
  return idx;
}

int qc_find_most_likely_state(t_q_circuit *c) {
  return (int)qc_find_most_likely_state64(c);
}

double qc_get_probability64(t_q_circuit *c, long long state) {
  double p = 0.0;
  int rc;
  if (!c || !c->state || state < 0 || state >= (1LL << c->num_qubits))
    return 0.0;
  qc_flush(c);
  rc = qcs_cuda_probability(c->state, state, &p);
  if (rc != QCS_CUDA_OK) {
    report("qc_get_probability", rc);
    return 0.0;
  }
  return p;
}

double qc_get_probability(t_q_circuit *c, int state) {
  return qc_get_probability64(c, (long long)state);
}

double qc_expect_z(t_q_circuit *c, int qubit) {
  double z = 0.0;
  int rc;
  if (!c || !c->state)
    return 0.0;
  qc_flush(c);
  rc = qcs_cuda_expect_z(c->state, qubit, &z);
  if (rc != QCS_CUDA_OK)
    report("qc_expect_z", rc);
  return z;
}

void qc_set_basis(t_q_circuit *c, long long index) {
  int rc;
  if (!c || !c->state)
    return;
  c->num_pending = 0; /* the queued gates would act on a discarded state */
  rc = qcs_cuda_set_basis(c->state, index);
  if (rc != QCS_CUDA_OK)
    fprintf(stderr, "Error: Invalid state or basis index\n");
}

qcs_cuda_state *qc_cuda_state(t_q_circuit *c) {
  if (!c)
    return NULL;
  qc_flush(c);
  return c->state;
}

/* ---- printing (src/qcs.c:308-383, src/q_state.c:139-168) --------------- */

static void read_amp(t_q_circuit *c, long long i, double *re, double *im) {
  double a[2] = {0.0, 0.0};
  qcs_cuda_read_amplitudes(c->state, i, 1, a);
  *re = a[0];
  *im = a[1];
}

void qc_print_state(t_q_circuit *c, int solution_index) {
  long long size;
  long long i;
  long long max_print;
  double re;
  double im;
  if (!c || !c->state)
    return;
  qc_flush(c);
  size = 1LL << c->num_qubits;
  max_print = size > 8 ? 4 : size;
  printf("--- Quantum State (%d Qubits) ---\n", c->num_qubits);
  for (i = 0; i < max_print; i++) {
    read_amp(c, i, &re, &im);
    printf("|%lld>: %f + i%f%s\n", i, re, im,
           i == solution_index ? " <-- SOLUTION" : "");
  }
  if (solution_index >= max_print && solution_index < size - 1) {
    read_amp(c, solution_index, &re, &im);
    printf("...\n");
    printf("|%d>: %f + i%f <-- SOLUTION\n", solution_index, re, im);
  }
  if (size > max_print) {
    long long last = size - 1;
    read_amp(c, last, &re, &im);
    printf("...\n");
    printf("|%lld>: %f + i%f%s\n", last, re, im,
           last == solution_index ? " <-- SOLUTION" : "");
  }
  printf("----------------------------------\n");
}

void qc_print_circuit(t_q_circuit *c) {
  int q;
  int g;
  int has_measurement = 0;
  printf("\n╔══════════════════════════════════════════╗\n");
  printf("║              QUANTUM CIRCUIT             ║\n");
  printf("╚══════════════════════════════════════════╝\n");
  printf("Qubits: %d | Gates: %d\n\n", c->num_qubits, c->num_gates);
  for (g = 0; g < c->history_size; g++) {
    if (strcmp(c->gate_history[g], "MEASURE") == 0) {
      has_measurement = 1;
      break;
    }
  }
  for (q = 0; q < c->num_qubits; q++) {
    printf("q%-2d ", q);
    for (g = 0; g < c->history_size; g++) {
      const char *name = c->gate_history[g];
      int target = c->target_qubits[g];
      int control = c->control_qubits[g];
      if (strcmp(name, "H") == 0 && target == q)
        printf("─H─");
      else if (strcmp(name, "X") == 0 && target == q)
        printf("─X─");
      else if (strcmp(name, "CNOT") == 0) {
        if (control == q)
          printf("─∙─");
        else if (target == q)
          printf("─⊕─");
        else
          printf("───");
      } else
        printf("───");
      if (g < c->history_size - 1)
        printf("─");
    }
    if (!has_measurement)
      printf("─M─");
    printf("─┐\n");
  }
  printf("\nGATE SEQUENCE: ");
  for (g = 0; g < c->history_size; g++) {
    const char *name = c->gate_history[g];
    if (strcmp(name, "CNOT") == 0)
      printf("CNOT(%d,%d) ", c->control_qubits[g], c->target_qubits[g]);
    else if (strcmp(name, "MEASURE") == 0)
      printf("MEASURE ");
    else
      printf("%s(%d) ", name, c->target_qubits[g]);
  }
  printf("\n\n");
}

/* ---- algorithms ------------------------------------------------------------ */

/* q_grover_iterations (src/q_utils.c:126-134); ldexp keeps it defined for
 * n >= 31, where the reference's (1 << n) overflows. */
static int grover_iterations(int n) {
  double pi = 3.14159265358979323846;
  return (int)floor((pi / 4.0) * sqrt(ldexp(1.0, n)));
}

/* qc_grover_search (src/qcs.c:402-419). */
void qc_grover_search(t_q_circuit *c, int solution_state) {
  int q;
  int i;
  int iterations;
  if (!c)
    return;
  iterations = grover_iterations(c->num_qubits);
  for (q = 0; q < c->num_qubits; q++)
    qc_h(c, q);
  for (i = 0; i < iterations; i++) {
    if (c->state && solution_state >= 0 &&
        (long long)solution_state < (1LL << c->num_qubits))
      submit(c, QCS_OP_PHASE_FLIP, -1, -1, 0.0, solution_state);
    else
      fprintf(stderr, "Error: Invalid state or index for phase flip.\n");
    add_gate(c, "ORACLE", solution_state, -1, 0.0);
    if (c->state)
      submit(c, QCS_OP_DIFFUSION, -1, -1, 0.0, 0);
    add_gate(c, "DIFFUSION", -1, -1, 0.0);
  }
}

int qc_get_num_qubits(t_q_circuit *c) { return c->num_qubits; }
int qc_get_num_gates(t_q_circuit *c) { return c->num_gates; }

/* qc_quantum_fourier_transform (src/qcs.c:443-457): H, then controlled
 * phases pi/2^(j-i); no final swaps. */
void qc_quantum_fourier_transform(t_q_circuit *c) {
  double pi = 3.14159265358979323846;
  int i;
  int j;
  for (i = 0; i < c->num_qubits; i++) {
    qc_h(c, i);
    for (j = i + 1; j < c->num_qubits; j++)
      qc_cphase(c, j, i, pi / ldexp(1.0, j - i));
  }
}

/* qc_ghz_state (src/qcs.c:521-535). */
void qc_ghz_state(t_q_circuit *c) {
  int i;
  if (c->num_qubits < 2) {
    fprintf(stderr, "Error: GHZ state requires at least 2 qubits.\n");
    return;
  }
  qc_h(c, 0);
  for (i = 0; i < c->num_qubits - 1; i++)
    qc_cnot(c, i, i + 1);
}

/* qc_bernstein_vazirani (src/qcs.c:614-644). */
void qc_bernstein_vazirani(t_q_circuit *c, int hidden_string) {
  int n = c->num_qubits - 1;
  int i;
  if (n <= 0) {
    fprintf(stderr, "Bernstein-Vazirani requires at least 2 qubits (1 input + "
                    "1 ancilla).\n");
    return;
  }
  qc_x(c, n);
  qc_h(c, n);
  for (i = 0; i < n; i++)
    qc_h(c, i);
  qc_barrier(c);
  for (i = 0; i < n; i++)
    if ((hidden_string >> i) & 1)
      qc_cnot(c, i, n);
  qc_barrier(c);
  for (i = 0; i < n; i++)
    qc_h(c, i);
}

/* qc_optimize (src/qcs.c:650-698): cancel adjacent identical self-inverse
 * pairs (H, X, Y, Z on one qubit; CNOT on one control/target) in the
 * history, restarting the scan after every cancellation.  Like the
 * reference it edits the record only; the state is not touched. */
void qc_optimize(t_q_circuit *c) {
  int i = 0;
  int j;
  while (i < c->history_size - 1) {
    const char *a = c->gate_history[i];
    const char *b = c->gate_history[i + 1];
    int t1 = c->target_qubits[i], t2 = c->target_qubits[i + 1];
    int c1 = c->control_qubits[i], c2 = c->control_qubits[i + 1];
    int self_inverse = strcmp(a, "H") == 0 || strcmp(a, "X") == 0 ||
                       strcmp(a, "Y") == 0 || strcmp(a, "Z") == 0;
    int one = t1 == t2 && strcmp(a, b) == 0 && self_inverse;
    int two = strcmp(a, "CNOT") == 0 && strcmp(b, "CNOT") == 0 && t1 == t2 &&
              c1 == c2;
    if (one || two) {
      free(c->gate_history[i]);
      free(c->gate_history[i + 1]);
      for (j = i; j < c->history_size - 2; j++) {
        c->gate_history[j] = c->gate_history[j + 2];
        c->target_qubits[j] = c->target_qubits[j + 2];
        c->control_qubits[j] = c->control_qubits[j + 2];
        c->parameters[j] = c->parameters[j + 2];
      }
      c->history_size -= 2;
      c->num_gates -= 2;
      i = 0;
    } else {
      i++;
    }
  }
}
