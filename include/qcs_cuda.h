/*
 * qcs_cuda.h -- C ABI of the GB300 (sm_103a) state-vector backend of QCS.
 *
 * This is the boundary a QCS_GPU_CUDA build of the reference calls in place
 * of its OpenCL backend (SegusFaultise/qcs src/gpu_complex.c) and of the
 * direct state->vector loops of src/q_gates.c, src/q_utils.c, src/q_state.c
 * and src/qcs.c.  Plain C types only: no CUDA, C++ or torch types appear in
 * any signature.  libqcs_gb300.so exports every function declared here, and
 * also the unchanged public API of include/qcs.h implemented on top of it.
 *
 * Conventions
 *  - Every function returns a status (QCS_CUDA_OK == 0 on success); values
 *    come back through out-pointers.  qcs_cuda_last_error() gives a message
 *    for the last failure on the calling thread.
 *  - A 2x2 gate is 8 doubles: {U00.re, U00.im, U01.re, U01.im, U10.re,
 *    U10.im, U11.re, U11.im}, the memory layout of t_q_matrix.data in the
 *    reference (src/internal.h:55-59, data[r*2+c] of struct t_complex), so
 *    (const double *)gate->data can be passed as is.
 *  - Qubit q is bit q of the basis index (reference convention,
 *    src/q_gates.c:28).  Basis indices are 64-bit.
 *  - Work is queued on the state's own CUDA stream.  Functions that return
 *    a host value synchronise that stream; the others return immediately.
 *  - One state must not be used from two threads at once (the reference is
 *    not reentrant either, src/qcs.c:9-11); distinct states are independent.
 *  - There is no CPU fallback: without a usable GPU, state creation fails
 *    with QCS_CUDA_ENODEV.
 */
#ifndef QCS_CUDA_H
#define QCS_CUDA_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define QCS_CUDA_OK 0
#define QCS_CUDA_EINVAL 1   /* bad argument (qubit, index, size, null)   */
#define QCS_CUDA_ENOMEM 2   /* device or host allocation failed          */
#define QCS_CUDA_ENODEV 3   /* no usable CUDA device                      */
#define QCS_CUDA_ELAUNCH 4  /* a kernel launch or CUDA call failed        */
#define QCS_CUDA_ETIMEOUT 5 /* a bounded device-side wait gave up         */
#define QCS_CUDA_EUNSUP 6   /* valid but unsupported combination          */

/* ---- state precision -------------------------------------------------- */
#define QCS_CUDA_C64 0  /* complex64 amplitudes (8 B), FP32 gate math      */
#define QCS_CUDA_C128 1 /* complex128 amplitudes (16 B), FP64 gate math,
                           same operation order as the reference          */

/* ---- semantics ---------------------------------------------------------*/
#define QCS_CUDA_PHYSICAL 0  /* unitary controlled-U, textbook Grover     */
#define QCS_CUDA_REFERENCE 1 /* the reference's sequential build, bit for
                                bit: out-of-place sweeps with a buffer swap,
                                controlled sweep acting as [[U00,U01],[0,1]]
                                on control=1 pairs (src/q_gates.c:279-291),
                                stale-buffer phase flip (:311-316) and
                                mean/|mean| diffusion (:334-355).  Allocates
                                a second state buffer.                     */

/* ---- gate kinds (struct qcs_cuda_op.kind) ----------------------------- */
#define QCS_GATE_H 0
#define QCS_GATE_X 1
#define QCS_GATE_Y 2
#define QCS_GATE_Z 3
#define QCS_GATE_P 4      /* phase, angle                                  */
#define QCS_GATE_RX 5
#define QCS_GATE_RY 6
#define QCS_GATE_RZ 7
#define QCS_GATE_CNOT 8   /* control, target                               */
#define QCS_GATE_CPHASE 9 /* control, target, angle (qc_cphase)            */
#define QCS_GATE_I 10
#define QCS_OP_PHASE_FLIP 20 /* index                                      */
#define QCS_OP_DIFFUSION 21

/* One operation of a gate list; 32 bytes, naturally aligned. */
typedef struct qcs_cuda_op {
  int kind;
  int target;
  int control; /* -1 when unused */
  int reserved;
  double angle;
  long long index; /* basis index for QCS_OP_PHASE_FLIP */
} qcs_cuda_op;

/* How qcs_cuda_run executes a gate list. */
typedef struct qcs_cuda_run_options {
  int fusion_k;  /* 0 or 1: one kernel per gate; 2..7: greedy fusion into
                    dense blocks of at most fusion_k qubits               */
  int fusion_engine; /* QCS_FUSE_AUTO, QCS_FUSE_SIMT or QCS_FUSE_TENSOR    */
  int partitioner;   /* QCS_PARTITION_GREEDY or QCS_PARTITION_LEARNED     */
  int flags;         /* QCS_RUN_* bits, 0 by default                      */
} qcs_cuda_run_options;

/* A fused run keeps its plan and block matrices with the state, keyed on the
 * exact bytes of the op list and on the options (and, for the learned
 * partitioner, the cost model and its current parameters); running the same
 * list again skips planning.  Any change (one angle) plans afresh.  A plain
 * run (one kernel per op) of a state of at most 26 qubits and at least 16
 * ops is captured into a CUDA graph when the same list runs twice in a row,
 * and replayed from then on (not while profiling).  This bit plans
 * afresh every time, launches kernel by kernel, and leaves what is kept
 * untouched. */
#define QCS_RUN_NO_PLAN_CACHE 1

#define QCS_FUSE_AUTO 0
#define QCS_FUSE_SIMT 1   /* FP32 CUDA-core block kernel (k <= 5)          */
#define QCS_FUSE_TENSOR 2 /* tcgen05 split-BF16x3 block kernels (k <= 7)   */
#define QCS_PARTITION_GREEDY 0
#define QCS_PARTITION_LEARNED 1

typedef struct qcs_cuda_state qcs_cuda_state;

/* ---- library / device --------------------------------------------------*/
const char *qcs_cuda_strerror(int status);
const char *qcs_cuda_last_error(void);
/* Number of visible CUDA devices (0 without a GPU; never fails). */
int qcs_cuda_device_count(int *count);
/* Host-side fault injection for tests: make the next `count` device
 * allocations (what == 1) or kernel launches (what == 2) report failure
 * without touching the GPU.  what == 0 clears it. */
int qcs_cuda_debug_inject(int what, int count);
/* Clock-cycle limit of the bounded device-side waits in kernels launched
 * from now on (the tensor-core pipelines' handoffs and the batched kernel's
 * CTA-group counters): cycles > 0 sets it, cycles == 0 restores the default
 * (about 2 s).  For tests of the timeout path: a wait that runs out raises
 * the device error flag, its CTA leaves its loops and releases what it
 * holds, and the next qcs_cuda_synchronize (or batch run) returns
 * QCS_CUDA_ETIMEOUT.  No counterpart in the reference (it has no device
 * code). */
int qcs_cuda_debug_set_wait_cycles(long long cycles);

/* ---- state lifecycle ---------------------------------------------------
 * Replaces q_state_init / q_state_free (src/q_state.c:32-115) and the
 * OpenCL buffer set-up (src/gpu_complex.c:250-279): the state lives on the
 * device, initialised to |0...0> (and, in REFERENCE semantics, a zeroed
 * second buffer). */
int qcs_cuda_state_create(int num_qubits, int precision, int semantics,
                          qcs_cuda_state **out);
int qcs_cuda_state_destroy(qcs_cuda_state *s);
int qcs_cuda_state_info(const qcs_cuda_state *s, int *num_qubits,
                        int *precision, int *semantics);
/* The state's cudaStream_t, as void*. */
int qcs_cuda_state_stream(qcs_cuda_state *s, void **stream);
/* Bytes moved between host and device for this state since it was created:
 * explicit copies (amplitude reads and writes, results, shot draws and
 * samples, tensor-core block images) and the gate and block matrices carried
 * in kernel parameters.  No reference counterpart (the reference's state is
 * host memory). */
int qcs_cuda_transfer_bytes(qcs_cuda_state *s, long long *h2d, long long *d2h);
/* Device address of the live amplitude buffer (valid until the next call
 * that may swap buffers in REFERENCE semantics). */
int qcs_cuda_state_device_ptr(qcs_cuda_state *s, void **ptr);
int qcs_cuda_synchronize(qcs_cuda_state *s);

/* q_state_set_basis (src/q_state.c:122-132): live buffer := |index>. */
int qcs_cuda_set_basis(qcs_cuda_state *s, long long index);

/* Host copies of amplitudes [first, first+count), (re,im) doubles.
 * read replaces the state->vector reads of q_state_print
 * (src/q_state.c:145-165). */
int qcs_cuda_read_amplitudes(qcs_cuda_state *s, long long first,
                             long long count, double *out);
int qcs_cuda_write_amplitudes(qcs_cuda_state *s, long long first,
                              long long count, const double *in);

/* ---- gates ---------------------------------------------------------------
 * q_apply_1q_gate (src/q_gates.c:25-149; OpenCL q_apply_1q_gate_gpu,
 * src/gpu_complex.c:521). */
int qcs_cuda_apply_1q(qcs_cuda_state *s, const double m[8], int target);
/* q_apply_2q_gate (src/q_gates.c:158-298; OpenCL q_apply_2q_gate_gpu,
 * src/gpu_complex.c:704): the 2x2 gate on `target` where `control` is 1. */
int qcs_cuda_apply_controlled_1q(qcs_cuda_state *s, const double m[8],
                                 int control, int target);
/* One named gate, built as the qc_<gate> wrappers do
 * (src/qcs.c:159-228,431-437,485-516; matrices src/q_gates.c:362-491). */
int qcs_cuda_apply_gate(qcs_cuda_state *s, int kind, int target, int control,
                        double angle);
/* Dense 2^k x 2^k block (k <= 7) on an ordered qubit list: bit j of the
 * block index is qubits[j]; u is row-major (re,im) doubles.  PHYSICAL
 * semantics only.  No reference counterpart: the reference's only dense
 * apply is the unused q_gate_apply (src/q_matrix.c:59-96). */
int qcs_cuda_apply_block(qcs_cuda_state *s, int k, const int *qubits,
                         const double *u, int engine);
/* q_apply_phase_flip (src/q_gates.c:305-317). */
int qcs_cuda_phase_flip(qcs_cuda_state *s, long long index);
/* q_apply_diffusion (src/q_gates.c:323-356). */
int qcs_cuda_diffusion(qcs_cuda_state *s);
/* A whole gate list, optionally fused (options may be NULL: per-gate). */
int qcs_cuda_run(qcs_cuda_state *s, const qcs_cuda_op *ops, int count,
                 const qcs_cuda_run_options *options);

/* Host only (no GPU needed): the execution order qcs_cuda_run would use for
 * ops[0..count) on a num_qubits state with fusion width kmax.  order[j] is
 * the op applied j-th; item[j] numbers the fused block (or single op) it
 * belongs to; *num_items receives the number of items.  Both arrays have
 * `count` entries. */
int qcs_cuda_plan(const qcs_cuda_op *ops, int count, int num_qubits, int kmax,
                  int *order, int *item, int *num_items);

/* ---- measurement support (benchmarks) ----------------------------------
 * Kernel classes for qcs_cuda_profile_read. */
#define QCS_KCLASS_DENSE1Q 0    /* dense 2x2 sweep                        */
#define QCS_KCLASS_DIAG1Q 1     /* diagonal 2x2 on every amplitude (RZ)   */
#define QCS_KCLASS_PHASE_MASK 2 /* phase on amplitudes with bits set      */
#define QCS_KCLASS_CTRL1Q 3     /* controlled 2x2 (control=1 half)        */
#define QCS_KCLASS_BLOCK_SIMT 4 /* fused block, CUDA cores                */
#define QCS_KCLASS_BLOCK_TC 5   /* fused block (k <= 6), tensor cores     */
#define QCS_KCLASS_REDUCE 6     /* norm / probability / sum reductions    */
#define QCS_KCLASS_DIFFUSE 7    /* diffusion update (+ fused sum)         */
#define QCS_KCLASS_COLLAPSE 8   /* measurement collapse, rescale          */
#define QCS_KCLASS_SAMPLE 9     /* shot sampling                          */
#define QCS_KCLASS_OTHER 10     /* set-basis, phase flip, finalisers      */
#define QCS_KCLASS_BLOCK_TC7 11 /* fused 7-qubit block, tensor cores      */
#define QCS_KCLASS_COUNT 12
/* enable != 0: from now on bracket every kernel with CUDA events on the
 * state's stream and accumulate device time and algorithmic bytes per
 * class (counters are cleared); enable == 0 stops recording. */
int qcs_cuda_profile_enable(qcs_cuda_state *s, int enable);
/* Synchronises the stream, then reports class `cls`: launches, total device
 * milliseconds and algorithmic bytes (any pointer may be NULL). */
int qcs_cuda_profile_read(qcs_cuda_state *s, int cls, long long *launches,
                          double *ms, double *bytes);
/* Kernels launched on this state since it was created. */
int qcs_cuda_launch_count(qcs_cuda_state *s, long long *count);

/* CUDA events on the state's stream, for device-side timing: record creates
 * and records one event; elapsed waits for `stop` and returns milliseconds
 * between the two; destroy frees an event. */
int qcs_cuda_event_record(qcs_cuda_state *s, void **event);
int qcs_cuda_event_elapsed(void *start, void *stop, double *ms);
int qcs_cuda_event_destroy(void *event);

/* ---- batched circuits ---------------------------------------------------
 * Many independent circuits (1..26 qubits each) run by one persistent
 * kernel, captured once into a CUDA graph and replayed.  Instance i has
 * num_qubits[i] qubits and the gates ops[op_offsets[i] .. op_offsets[i+1]);
 * the state starts at |0...0>.  Each run returns <Z_0> per instance (FP64
 * accumulation) and `shots` samples per instance drawn from a counter-based
 * generator keyed by (seed, instance, shot).  The reference has no batched
 * form; per circuit this replaces qc_create + gates + the shot loop of
 * qc_run_shots (src/qcs.c:575-607). */
typedef struct qcs_cuda_batch qcs_cuda_batch;
int qcs_cuda_batch_create(int count, const int *num_qubits,
                          const int *op_offsets, const qcs_cuda_op *ops,
                          int shots, unsigned long long seed,
                          qcs_cuda_batch **out);
int qcs_cuda_batch_destroy(qcs_cuda_batch *b);
/* New angles for every op (in op order); the plan and graph are kept. */
int qcs_cuda_batch_set_angles(qcs_cuda_batch *b, const double *angles);
/* One replay.  expect_z0: `count` doubles; samples: count*shots indices
 * (instance-major), may be NULL; ms: device time of the replay. */
int qcs_cuda_batch_run(qcs_cuda_batch *b, double *expect_z0,
                       long long *samples, double *ms);
/* Times every schedule (threads per CTA 256/512/1024, tile 2^12..2^14,
 * 1, 2 or 4 CTAs per SM as fit, largest-first or given order) on this batch, then how
 * widely large instances spread (an instance above split_q qubits is shared
 * by 2^(n - split_q) CTAs, split_q in 17..20 or never), and keeps the
 * fastest; chosen (4 ints) receives threads, tile qubits, CTAs per SM and
 * order. */
int qcs_cuda_batch_autotune(qcs_cuda_batch *b, int repeats, int *chosen);
/* The schedule in force (5 ints): threads, tile qubits, CTAs per SM that
 * actually run, order, split_q. */
int qcs_cuda_batch_schedule(qcs_cuda_batch *b, int *schedule);
/* Instances above split_q qubits (and above the tile) are shared by
 * 2^(n - split_q) CTAs, at most half the grid; 27 never splits. */
int qcs_cuda_batch_split(qcs_cuda_batch *b, int split_q);
/* Algorithmic HBM bytes of one run under the schedule in force: for every
 * instance above the tile (kept in a global slot), one write of its 2^n
 * complex64 amplitudes in the first stage, a read and a write in each later
 * stage, and one read for <Z_0> and the sampling masses; plus the results
 * (8 bytes per instance and 8 per shot).  Instances that fit the tile live
 * in shared memory and move no state bytes. */
int qcs_cuda_batch_traffic(qcs_cuda_batch *b, double *hbm_bytes);
/* Sets one schedule explicitly (split_q is kept). */
int qcs_cuda_batch_config(qcs_cuda_batch *b, int threads, int tile_q,
                          int ctas_per_sm, int order);

/* ---- learned fusion cost model ------------------------------------------
 * An MLP (QCS_COSTMODEL_FEATURES inputs, three hidden layers of 64 ReLU
 * units, one output) that predicts log2 of a plan item's device time in ms.
 * Forward, backward and Adam run on the GPU in this library's own kernels;
 * the host keeps a copy of the weights for planning.  Created where no
 * device is visible, a model serves planning only: get/set_params,
 * predict_host and plan_learned work, training and predict return
 * QCS_CUDA_ENODEV.  No reference counterpart (the reference has no fusion). */
#define QCS_COSTMODEL_FEATURES 20
typedef struct qcs_cuda_costmodel qcs_cuda_costmodel;
int qcs_cuda_costmodel_create(int num_features, unsigned long long seed,
                              qcs_cuda_costmodel **out);
int qcs_cuda_costmodel_destroy(qcs_cuda_costmodel *m);
int qcs_cuda_costmodel_num_params(qcs_cuda_costmodel *m, int *count);
int qcs_cuda_costmodel_get_params(qcs_cuda_costmodel *m, float *out);
int qcs_cuda_costmodel_set_params(qcs_cuda_costmodel *m, const float *in,
                                  int count);
/* Mean squared error over n samples (x: n x F row-major, y: n) and its
 * gradient with respect to every parameter (grad may be NULL). */
int qcs_cuda_costmodel_loss_grad(qcs_cuda_costmodel *m, const float *x,
                                 const float *y, int n, double *loss,
                                 float *grad);
/* Adam, mini-batches of `batch` rows in the given order, `epochs` passes. */
int qcs_cuda_costmodel_train(qcs_cuda_costmodel *m, const float *x,
                             const float *y, int n, int epochs, int batch,
                             float lr, double *final_loss);
int qcs_cuda_costmodel_predict(qcs_cuda_costmodel *m, const float *x, int n,
                               float *out);
int qcs_cuda_costmodel_predict_host(qcs_cuda_costmodel *m, const float *x,
                                    int n, float *out);
/* Features of one plan item (category QCS_CAT_*, state qubits n, item
 * qubits, gate count) into out[QCS_COSTMODEL_FEATURES]. */
#define QCS_CAT_DENSE 0
#define QCS_CAT_DIAG 1
#define QCS_CAT_PHASE 2
#define QCS_CAT_CTRL 3
#define QCS_CAT_CPHASE 4
#define QCS_CAT_SIMT 5
#define QCS_CAT_TC 6
int qcs_cuda_item_features(int category, int n, int k, const int *qubits,
                           int ngates, float *out);
/* Run ops[0..count) on the state with fusion width kmax and `engine`, timing
 * every plan item with CUDA events: features (max x F) and milliseconds
 * (max) of up to `max` items; *written receives how many. */
int qcs_cuda_collect_timings(qcs_cuda_state *s, const qcs_cuda_op *ops,
                             int count, int kmax, int engine, float *features,
                             float *ms, int max, int *written);
/* The model qcs_cuda_run uses when options.partitioner is
 * QCS_PARTITION_LEARNED (NULL detaches it; the greedy plan is then used). */
int qcs_cuda_state_set_costmodel(qcs_cuda_state *s, qcs_cuda_costmodel *m);
/* Host only: the learned plan for a num_qubits state (order/item as in
 * qcs_cuda_plan), the model's predicted ms for it and for the greedy
 * width-kmax plan, and which candidate won: the greedy width k (2..7), plus
 * 100 when the model stopped blocks from growing, plus 200 when ties were
 * broken by lookahead, plus 1000 x the number of that candidate's blocks the
 * model then split into narrower items. */
int qcs_cuda_plan_learned(const qcs_cuda_op *ops, int count, int num_qubits,
                          int kmax, qcs_cuda_costmodel *m, int *order,
                          int *item, int *num_items, double *pred_ms,
                          double *greedy_ms, int *choice);

/* ---- reductions and read-out (FP64 accumulation) ----------------------- */
int qcs_cuda_norm_sq(qcs_cuda_state *s, double *out);
/* q_state_normalize (src/q_utils.c:44-119): rescale when the norm^2 is
 * above 1e-12 and not exactly 1. */
int qcs_cuda_normalize(qcs_cuda_state *s);
/* Probability of reading 0 on `qubit` (first loop of qc_measure,
 * src/qcs.c:253-259). */
int qcs_cuda_prob_zero(qcs_cuda_state *s, int qubit, double *p0);
/* qc_measure (src/qcs.c:237-284) given the caller's rand()/RAND_MAX draw:
 * outcome 0 when random_val <= p0; collapse and renormalise. */
int qcs_cuda_measure(qcs_cuda_state *s, int qubit, double random_val,
                     int *outcome);
/* qc_get_probability (src/qcs.c:391-395), 64-bit index. */
int qcs_cuda_probability(qcs_cuda_state *s, long long index, double *p);
/* qc_find_most_likely_state (src/qcs.c:464-478): first index of the
 * largest |amplitude|^2 (0 for an all-zero state); prob may be NULL. */
int qcs_cuda_argmax(qcs_cuda_state *s, long long *index, double *prob);
/* <Z_qubit> = P(0) - P(1). */
int qcs_cuda_expect_z(qcs_cuda_state *s, int qubit, double *out);
/* Sampling of qc_run_shots (src/qcs.c:584-605): for each draw r in [0,1],
 * the first index whose running FP64 probability sum exceeds r, or -1 when
 * r is not below the total.  out_index has `shots` entries. */
int qcs_cuda_sample(qcs_cuda_state *s, const double *random_vals, int shots,
                    long long *out_index);

/* Shot sampling that allocates no memory (no counterpart in the reference).
 * For callers that cannot call cudaMalloc where they sample: a host
 * application that owns all device memory through its own pool, or a
 * latency-critical loop that must not take cudaMalloc's implicit device
 * synchronisation.
 * Same draws-to-indices rule as qcs_cuda_sample, but every pointer is a
 * device pointer the caller provides: `amplitudes` (count complex64 or
 * complex128 values, precision QCS_CUDA_C64 / QCS_CUDA_C128), `draws`
 * (shots doubles) and `samples` (shots 64-bit indices, -1 when a draw is not
 * below the total).  Work is queued on `stream` (a cudaStream_t, NULL for the
 * default stream); the call does not wait for it.
 * Limit: count must be a power of two no larger than 2^28 amplitudes; the
 * scratch is a fixed array of about 544 KB inside the library, held on every GPU that
 * loads it until the process exits.  The first call on a device looks up
 * that array's device address and should come before any stream capture;
 * a device reset invalidates it (a call whose launch fails looks it up
 * again on the next call).  Calls share the array: two calls that overlap
 * on the GPU race. */
int qcs_cuda_sample_noalloc(const void *amplitudes, long long count,
                            int precision, const double *draws, int shots,
                            long long *samples, void *stream);

#ifdef __cplusplus
}
#endif

#endif
