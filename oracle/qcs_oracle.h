/*
 * qcs_oracle.h -- CPU FP64 oracle for the QCS state-vector hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library, and only
 * as the checker or the timed CPU baseline.  The product (libqcs_gb300.so)
 * never links it and never falls back to it.
 *
 * It restates, in plain C89 with complex128 arithmetic, the algorithm of the
 * reference's sequential build (SegusFaultise/qcs, src/q_gates.c,
 * src/q_utils.c, src/q_state.c, src/qcs.c) in two modes:
 *
 *   ORC_PHYSICAL  textbook semantics: unitary controlled-U on the
 *                 (control=1) pairs, phase flip in place, diffusion
 *                 2*(sum/N) - psi.
 *   ORC_COMPAT    the reference's observable behaviour, bit for bit:
 *                 out-of-place sweeps with a buffer swap, the controlled sweep
 *                 acting as [[U00,U01],[0,1]] on control=1 pairs
 *                 (src/q_gates.c:279-291), the phase flip that swaps in the
 *                 stale buffer (src/q_gates.c:311-316) and the diffusion that
 *                 divides the mean by its magnitude (src/q_gates.c:334-355).
 *
 * Every floating-point expression keeps the reference's operation order
 * (c_add(c_mul(g0,v0), c_mul(g1,v1)), src/q_gates.c:140-141 and
 * src/complex.c:23-57) and the library is compiled with -ffp-contract=off, so
 * results are bit-identical to the reference's sequential build.
 *
 * Parity pins: tests/test_oracle_pins.py checks this oracle against golden
 * vectors generated from the reference's own sequential build
 * (tests/golden/make_golden.py) and, where oracle/_ref is built, against the
 * reference library directly.
 */
#ifndef QCS_ORACLE_H
#define QCS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_PHYSICAL 0
#define ORC_COMPAT 1

/* Gate kinds: same numbering as QCS_GATE_* in include/qcs_cuda.h. */
#define ORC_GATE_H 0
#define ORC_GATE_X 1
#define ORC_GATE_Y 2
#define ORC_GATE_Z 3
#define ORC_GATE_P 4
#define ORC_GATE_RX 5
#define ORC_GATE_RY 6
#define ORC_GATE_RZ 7
#define ORC_GATE_CNOT 8
#define ORC_GATE_CPHASE 9
#define ORC_GATE_I 10
#define ORC_OP_PHASE_FLIP 20
#define ORC_OP_DIFFUSION 21

typedef struct orc_state orc_state;

orc_state *orc_create(int num_qubits, int mode);
int orc_set_threads(int threads);
void orc_destroy(orc_state *s);
int orc_num_qubits(const orc_state *s);
long orc_size(const orc_state *s);
int orc_mode(const orc_state *s);

void orc_set_basis(orc_state *s, long index);
void orc_read(const orc_state *s, long first, long count, double *out);
void orc_write(orc_state *s, long first, long count, const double *in);

void orc_gate_matrix(int kind, double angle, double out[8]);
int orc_apply_1q(orc_state *s, const double m[8], int target);
int orc_apply_controlled(orc_state *s, const double m[8], int control,
                         int target);
int orc_apply_gate(orc_state *s, int kind, int target, int control,
                   double angle);
int orc_run_gates(orc_state *s, int count, const int *kinds,
                  const int *targets, const int *controls,
                  const double *angles);
/* As orc_run_gates, plus the non-gate operations ORC_OP_PHASE_FLIP (index)
 * and ORC_OP_DIFFUSION. */
int orc_run_ops(orc_state *s, int count, const int *kinds, const int *targets,
                const int *controls, const double *angles,
                const long *indices);
int orc_apply_block(orc_state *s, int k, const int *qubits, const double *u);

int orc_phase_flip(orc_state *s, long index);
int orc_diffusion(orc_state *s);

double orc_norm_sq(const orc_state *s);
void orc_normalize(orc_state *s);
double orc_prob_zero(const orc_state *s, int qubit);
int orc_measure(orc_state *s, int qubit, double random_val);
double orc_probability(const orc_state *s, long index);
long orc_argmax(const orc_state *s);
void orc_sample(const orc_state *s, const double *random_vals, int shots,
                long *out_index);
double orc_expect_z(const orc_state *s, int qubit);

int orc_grover_iterations(int num_qubits);
void orc_qft(orc_state *s);
void orc_grover(orc_state *s, long solution, int iterations);

#ifdef __cplusplus
}
#endif

#endif
