// common.cuh -- shared definitions of the GB300 state-vector backend.
//
// Layout in HBM: one contiguous array of 2^n amplitudes, complex64
// (float2, 8 B) or complex128 (double2, 16 B), basis index i at offset i.
// REFERENCE semantics add a second buffer of the same size (the reference's
// scratch_vector, src/internal.h:43-48); PHYSICAL semantics sweep in place.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "qcs_cuda.h"

namespace qcs {

typedef long long i64;
typedef unsigned long long u64;

// Per-state device scratch for reductions: one slot per block of the
// reduction grid.  The grid is fixed per device (SM count x blocks per SM)
// so results are deterministic run to run.
constexpr int kReduceThreads = 256;
constexpr int kReduceBlocksPerSM = 4;
constexpr int kSweepThreads = 256;

struct DeviceInfo {
  int device;
  int num_sms;
  int reduce_blocks;  // num_sms * kReduceBlocksPerSM
  int cc_major, cc_minor;
};

struct ReduceSlot {  // one block's partial result
  double a, b, c, d;
};

enum KClass {
  KC_DENSE1Q = QCS_KCLASS_DENSE1Q,
  KC_DIAG1Q = QCS_KCLASS_DIAG1Q,
  KC_PHASE_MASK = QCS_KCLASS_PHASE_MASK,
  KC_CTRL1Q = QCS_KCLASS_CTRL1Q,
  KC_BLOCK_SIMT = QCS_KCLASS_BLOCK_SIMT,
  KC_BLOCK_TC = QCS_KCLASS_BLOCK_TC,
  KC_REDUCE = QCS_KCLASS_REDUCE,
  KC_DIFFUSE = QCS_KCLASS_DIFFUSE,
  KC_COLLAPSE = QCS_KCLASS_COLLAPSE,
  KC_SAMPLE = QCS_KCLASS_SAMPLE,
  KC_OTHER = QCS_KCLASS_OTHER,
  KC_BLOCK_TC7 = QCS_KCLASS_BLOCK_TC7,
  KC_COUNT = QCS_KCLASS_COUNT
};

struct ProfData;  // per-state event bookkeeping (state.cu)
struct TcRing;    // tensor-core engine block-matrix uploads (blocks_tc.cu)
struct PlanCache; // kept fused plan of the last run (blocks.cu)
struct PlainGraph;  // kept plain run as a CUDA graph (blocks.cu)
struct TcResident;  // a tensor-core block with its image on the device (blocks_tc.cu)
// What a tensor-core block also does: take the state through a physical
// diffusion first (the block reads psi, acts on 2m - psi), and/or leave the
// sum of its output amplitudes as the state's cached sum.
struct BlockFuse {
  bool diffuse_in;
  bool sum_out;
};
// Tensor-core blocks kept with a plan (blocks_tc.cu).
int tc_make_resident(qcs_cuda_state *s, int k, const int *qubits, const double *u,
                     bool known_unitary, TcResident **out);
int tc_launch_resident(qcs_cuda_state *s, const TcResident *b, const BlockFuse *fuse);
size_t tc_resident_bytes(const TcResident *b);
void tc_free_resident(TcResident *b);
void plan_cache_free(qcs_cuda_state *s);
void tc_release(TcRing *r);

}  // namespace qcs

struct qcs_cuda_state {
  int n;
  qcs::i64 size;
  int prec;  // QCS_CUDA_C64 / QCS_CUDA_C128
  int sem;   // QCS_CUDA_PHYSICAL / QCS_CUDA_REFERENCE
  void *vec;      // live amplitudes
  void *scratch;  // second buffer (REFERENCE semantics only)
  cudaStream_t stream;
  qcs::DeviceInfo dev;
  // reductions: per-block partials, a final result slot, pinned host mirror
  qcs::ReduceSlot *d_partials;
  double *d_result;    // 8 doubles
  double *h_result;    // pinned, 8 doubles
  // cached sum of amplitudes (complex, FP64) for Grover iterations; valid
  // while sum_valid != 0 (kept on the device in d_result[4..5])
  int sum_valid;
  // sampling scratch (grown on demand)
  double *d_tile_prefix;  // n_tiles + 1 (exclusive prefix, then total)
  qcs::i64 n_tiles;
  double *d_draws;
  qcs::i64 *d_samples;
  int sample_cap;
  double *h_draws;        // pinned staging
  qcs::i64 *h_samples;    // pinned staging
  // measurement support
  long long launches;
  qcs::ProfData *prof;    // non-null while profiling
  qcs::TcRing *tc;        // created on first tensor-core block
  int *d_err;             // device error flag (bounded waits that gave up)
  qcs_cuda_costmodel *cm; // model for QCS_PARTITION_LEARNED (not owned)
  qcs::PlanCache *plans;  // last fused run's plan and block matrices
  qcs::PlainGraph *plain_graph;  // last plain run, captured once repeated
  // bytes moved between host and device on this state's behalf: explicit
  // copies and the matrices carried in kernel parameters
  long long h2d_bytes;
  long long d2h_bytes;
};

namespace qcs {

// ---- status / errors ------------------------------------------------------
int set_error(int status, const char *fmt, ...);
int check_cuda(cudaError_t e, const char *what);
// Host <-> device copies on the state's stream, counted in h2d/d2h_bytes.
int copy_h2d(qcs_cuda_state *s, void *dst, const void *src, size_t bytes, const char *what);
int copy_d2h(qcs_cuda_state *s, void *dst, const void *src, size_t bytes, const char *what);
int check_launch(const char *what);
// Every kernel launch on a state is bracketed by these two calls:
// prof_begin before the launch, launched() after it (checks the launch,
// counts it and, when profiling, records the closing event with the launch's
// algorithmic bytes).
void prof_begin(qcs_cuda_state *s);
int launched(qcs_cuda_state *s, int cls, double bytes, const char *what);
// Host-side fault injection (tests): returns nonzero when the next
// allocation / launch must report failure.
bool inject_alloc_failure();
bool inject_launch_failure();
// Clock-cycle limit of the bounded device-side waits (pipeline handoffs,
// CTA-group counters) of kernels launched from now on: kDefaultWaitCycles
// (~2 s) unless qcs_cuda_debug_set_wait_cycles set another.
constexpr long long kDefaultWaitCycles = 4000000000LL;
long long wait_cycles();
int device_info(int device, DeviceInfo *out);

// ---- complex helpers --------------------------------------------------------
template <typename R> struct CT;
template <> struct CT<float> { typedef float2 C; };
template <> struct CT<double> { typedef double2 C; };

// complex64: plain FP32 expressions (the compiler contracts to FMA).
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  return make_float2(a.x + b.x, a.y + b.y);
}
// complex128: the reference's exact operation order with round-to-nearest
// intrinsics, so no FMA contraction can change a bit (src/complex.c:23-57).
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                      __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) {
  return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y));
}

template <typename C> struct Mat2 { C g[4]; };

template <typename C>
__host__ __device__ inline C make_c(double re, double im);
template <> __host__ __device__ inline float2 make_c<float2>(double re, double im) {
  return make_float2((float)re, (float)im);
}
template <> __host__ __device__ inline double2 make_c<double2>(double re, double im) {
  return make_double2(re, im);
}

template <typename C> inline Mat2<C> to_mat2(const double m[8]) {
  Mat2<C> r;
  for (int i = 0; i < 4; i++) r.g[i] = make_c<C>(m[2 * i], m[2 * i + 1]);
  return r;
}

// Insert a zero bit at position b of x.
__host__ __device__ __forceinline__ i64 insert_zero(i64 x, int b) {
  i64 low = x & ((1LL << b) - 1);
  return ((x >> b) << (b + 1)) | low;
}

inline int grid_for(i64 work, int threads, const DeviceInfo &d, int per_sm) {
  i64 g = (work + threads - 1) / threads;
  i64 cap = (i64)d.num_sms * per_sm;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

// ---- cross-file entry points ------------------------------------------------
void invalidate_sum(qcs_cuda_state *s);
int ensure_sum(qcs_cuda_state *s);                  // readout.cu
int finalize_sum(qcs_cuda_state *s, int nslots);    // readout.cu
int ensure_sample_scratch(qcs_cuda_state *s, int shots);

}  // namespace qcs

#define QCS_CHECK_STATE(s)                                                   \
  do {                                                                       \
    if (!(s)) return qcs::set_error(QCS_CUDA_EINVAL, "null state");          \
  } while (0)
