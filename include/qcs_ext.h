/*
 * qcs_ext.h -- additive extensions of the QCS API (GB300 backend).
 *
 * Nothing here changes a declaration of qcs.h.  The reference caps basis
 * indices at int (include/qcs.h:57-66) and returns shot results as a
 * 2^n-entry histogram (src/qcs.c:593); these entry points lift both limits
 * for 31..36-qubit states and expose the backend's knobs.
 */
#ifndef QCS_EXT_H
#define QCS_EXT_H

#include "qcs.h"
#include "qcs_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Controlled phase; the reference defines qc_cphase (src/qcs.c:431) but
 * does not declare it. */
void qc_cphase(t_q_circuit *circuit, int control, int target, double angle);

/* Circuit with explicit precision (QCS_CUDA_C64/C128), semantics
 * (QCS_CUDA_PHYSICAL/REFERENCE) and fusion width (0: one kernel per gate).
 * qc_create reads the same settings from QCS_CUDA_PRECISION ("c64",
 * "c128"), QCS_CUDA_SEMANTICS ("physical", "reference") and QCS_CUDA_FUSION
 * (an integer k) and defaults to c64 / physical / 0. */
t_q_circuit *qc_create_ex(int num_qubits, int precision, int semantics, int fusion_k);

/* 64-bit index forms of qc_get_probability / qc_find_most_likely_state. */
double qc_get_probability64(t_q_circuit *circuit, long long state);
long long qc_find_most_likely_state64(t_q_circuit *circuit);
/* Basis state |index> (the reference's internal q_state_set_basis,
 * src/q_state.c:122-132). */
void qc_set_basis(t_q_circuit *circuit, long long index);
/* Per-sample shots: samples[i] = outcome of shot i (or -1), drawing with
 * rand() like qc_run_shots.  Returns 0 on success. */
int qc_sample_shots(t_q_circuit *circuit, int shots, long long *samples);
/* <Z_qubit>. */
double qc_expect_z(t_q_circuit *circuit, int qubit);
/* Apply the queued gates now (a no-op when fusion is off). */
void qc_flush(t_q_circuit *circuit);
/* The device state behind a circuit (flushes first). */
qcs_cuda_state *qc_cuda_state(t_q_circuit *circuit);

#ifdef __cplusplus
}
#endif

#endif
