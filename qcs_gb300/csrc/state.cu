// state.cu -- state lifecycle, errors, host copies.
//
// Replaces q_state_init / q_state_free / q_state_set_basis
// (src/q_state.c:32-132) and the OpenCL buffer management of
// src/gpu_complex.c:250-313.  Each state owns its device buffers and its own
// CUDA stream; there is no process-global device state (the reference keeps
// global OpenCL buffers, src/gpu_complex.c:6-20).
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <vector>

#include "common.cuh"

namespace qcs {

static thread_local char g_last_error[512] = "";
static std::atomic<int> g_inject_alloc{0};
static std::atomic<int> g_inject_launch{0};
static std::atomic<long long> g_wait_cycles{0};  // 0: kDefaultWaitCycles

int set_error(int status, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return status;
}

int check_cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return QCS_CUDA_OK;
  int st = (e == cudaErrorMemoryAllocation) ? QCS_CUDA_ENOMEM
           : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
               ? QCS_CUDA_ENODEV
               : QCS_CUDA_ELAUNCH;
  return set_error(st, "%s: %s", what, cudaGetErrorString(e));
}

int check_launch(const char *what) {
  if (inject_launch_failure()) {
    return set_error(QCS_CUDA_ELAUNCH, "%s: injected launch failure", what);
  }
  return check_cuda(cudaGetLastError(), what);
}

long long wait_cycles() {
  const long long w = g_wait_cycles.load();
  return w > 0 ? w : kDefaultWaitCycles;
}

static bool take_one(std::atomic<int> &c) {
  int v = c.load();
  while (v > 0) {
    if (c.compare_exchange_weak(v, v - 1)) return true;
  }
  return false;
}
bool inject_alloc_failure() { return take_one(g_inject_alloc); }
bool inject_launch_failure() { return take_one(g_inject_launch); }

int device_info(int device, DeviceInfo *out) {
  static DeviceInfo cache[64];
  static bool have[64] = {false};
  if (device < 0 || device >= 64) return set_error(QCS_CUDA_ENODEV, "bad device id");
  if (!have[device]) {
    DeviceInfo d;
    d.device = device;
    int rc = check_cuda(cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, device),
                        "cudaDeviceGetAttribute(SM count)");
    if (rc) return rc;
    cudaDeviceGetAttribute(&d.cc_major, cudaDevAttrComputeCapabilityMajor, device);
    cudaDeviceGetAttribute(&d.cc_minor, cudaDevAttrComputeCapabilityMinor, device);
    d.reduce_blocks = d.num_sms * kReduceBlocksPerSM;
    cache[device] = d;
    have[device] = true;
  }
  *out = cache[device];
  return QCS_CUDA_OK;
}

template <typename C>
__global__ void k_set_one(C *v, i64 index) {
  v[index] = make_c<C>(1.0, 0.0);
}

static int dmalloc(void **p, size_t bytes, const char *what) {
  *p = nullptr;
  if (inject_alloc_failure())
    return set_error(QCS_CUDA_ENOMEM, "%s: injected allocation failure", what);
  return check_cuda(cudaMalloc(p, bytes), what);
}

static size_t amp_bytes(const qcs_cuda_state *s) {
  return s->prec == QCS_CUDA_C128 ? 16 : 8;
}

static int launch_set_one(qcs_cuda_state *s, void *buf, i64 index) {
  prof_begin(s);
  if (s->prec == QCS_CUDA_C128)
    k_set_one<double2><<<1, 1, 0, s->stream>>>((double2 *)buf, index);
  else
    k_set_one<float2><<<1, 1, 0, s->stream>>>((float2 *)buf, index);
  return launched(s, KC_OTHER, (double)amp_bytes(s), "set_basis");
}

void invalidate_sum(qcs_cuda_state *s) { s->sum_valid = 0; }

// ---- per-class device timing -------------------------------------------------
struct ProfData {
  struct Rec {
    int cls;
    double bytes;
    cudaEvent_t a, b;
  };
  std::vector<Rec> pending;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t open = nullptr;
  double ms[KC_COUNT] = {0};
  double bytes[KC_COUNT] = {0};
  long long launches[KC_COUNT] = {0};
};

static cudaEvent_t take_event(ProfData *p) {
  cudaEvent_t e = nullptr;
  if (!p->pool.empty()) {
    e = p->pool.back();
    p->pool.pop_back();
  } else {
    cudaEventCreate(&e);
  }
  return e;
}

static int prof_flush(qcs_cuda_state *s) {
  ProfData *p = s->prof;
  if (!p) return QCS_CUDA_OK;
  int rc = check_cuda(cudaStreamSynchronize(s->stream), "profile sync");
  if (rc) return rc;
  for (auto &r : p->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    p->ms[r.cls] += ms;
    p->bytes[r.cls] += r.bytes;
    p->launches[r.cls] += 1;
    p->pool.push_back(r.a);
    p->pool.push_back(r.b);
  }
  p->pending.clear();
  return QCS_CUDA_OK;
}

static void prof_free(qcs_cuda_state *s) {
  if (!s->prof) return;
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (auto &r : s->prof->pending) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (auto e : s->prof->pool) cudaEventDestroy(e);
  if (s->prof->open) cudaEventDestroy(s->prof->open);
  delete s->prof;
  s->prof = nullptr;
}

void prof_begin(qcs_cuda_state *s) {
  ProfData *p = s->prof;
  if (!p) return;
  if (p->open) p->pool.push_back(p->open);
  p->open = take_event(p);
  cudaEventRecord(p->open, s->stream);
}

int copy_h2d(qcs_cuda_state *s, void *dst, const void *src, size_t bytes, const char *what) {
  s->h2d_bytes += (long long)bytes;
  return check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s->stream), what);
}

int copy_d2h(qcs_cuda_state *s, void *dst, const void *src, size_t bytes, const char *what) {
  s->d2h_bytes += (long long)bytes;
  return check_cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s->stream), what);
}

int launched(qcs_cuda_state *s, int cls, double bytes, const char *what) {
  int rc = check_launch(what);
  s->launches++;
  ProfData *p = s->prof;
  if (p && p->open) {
    cudaEvent_t e = take_event(p);
    cudaEventRecord(e, s->stream);
    p->pending.push_back({cls, bytes, p->open, e});
    p->open = nullptr;
    if (p->pending.size() >= 8192) {
      int r2 = prof_flush(s);
      if (!rc) rc = r2;
    }
  }
  return rc;
}

static void free_state(qcs_cuda_state *s) {
  if (!s) return;
  if (s->stream) cudaStreamSynchronize(s->stream);
  prof_free(s);
  plan_cache_free(s);
  tc_release(s->tc);
  cudaFree(s->d_err);
  cudaFree(s->vec);
  cudaFree(s->scratch);
  cudaFree(s->d_partials);
  cudaFree(s->d_result);
  cudaFree(s->d_tile_prefix);
  cudaFree(s->d_draws);
  cudaFree(s->d_samples);
  if (s->h_result) cudaFreeHost(s->h_result);
  if (s->h_draws) cudaFreeHost(s->h_draws);
  if (s->h_samples) cudaFreeHost(s->h_samples);
  if (s->stream) cudaStreamDestroy(s->stream);
  free(s);
}

int ensure_sample_scratch(qcs_cuda_state *s, int shots) {
  int rc;
  if (!s->d_tile_prefix) {
    i64 tile = s->size < 4096 ? s->size : 4096;
    s->n_tiles = s->size / tile;
    // the tiles' prefixes within their ranges, then the range offsets and
    // the total (at most 8 ranges per SM)
    rc = dmalloc((void **)&s->d_tile_prefix,
                 (size_t)(s->n_tiles + (i64)s->dev.num_sms * 8 + 1) * sizeof(double),
                 "cudaMalloc(tile prefix)");
    if (rc) return rc;
  }
  if (shots > s->sample_cap) {
    int cap = shots < 1024 ? 1024 : shots;
    cudaFree(s->d_draws);
    cudaFree(s->d_samples);
    if (s->h_draws) cudaFreeHost(s->h_draws);
    if (s->h_samples) cudaFreeHost(s->h_samples);
    s->d_draws = nullptr;
    s->d_samples = nullptr;
    s->h_draws = nullptr;
    s->h_samples = nullptr;
    s->sample_cap = 0;
    rc = dmalloc((void **)&s->d_draws, (size_t)cap * sizeof(double), "cudaMalloc(draws)");
    if (rc) return rc;
    rc = dmalloc((void **)&s->d_samples, (size_t)cap * sizeof(i64), "cudaMalloc(samples)");
    if (rc) return rc;
    rc = check_cuda(cudaMallocHost((void **)&s->h_draws, (size_t)cap * sizeof(double)),
                    "cudaMallocHost(draws)");
    if (rc) return rc;
    rc = check_cuda(cudaMallocHost((void **)&s->h_samples, (size_t)cap * sizeof(i64)),
                    "cudaMallocHost(samples)");
    if (rc) return rc;
    s->sample_cap = cap;
  }
  return QCS_CUDA_OK;
}

}  // namespace qcs

using namespace qcs;

extern "C" {

const char *qcs_cuda_strerror(int status) {
  switch (status) {
    case QCS_CUDA_OK: return "ok";
    case QCS_CUDA_EINVAL: return "invalid argument";
    case QCS_CUDA_ENOMEM: return "out of memory";
    case QCS_CUDA_ENODEV: return "no usable CUDA device";
    case QCS_CUDA_ELAUNCH: return "CUDA launch or call failed";
    case QCS_CUDA_ETIMEOUT: return "device-side wait timed out";
    case QCS_CUDA_EUNSUP: return "unsupported";
    default: return "unknown status";
  }
}

const char *qcs_cuda_last_error(void) { return g_last_error; }

int qcs_cuda_device_count(int *count) {
  if (!count) return set_error(QCS_CUDA_EINVAL, "null count");
  int c = 0;
  if (cudaGetDeviceCount(&c) != cudaSuccess) {
    cudaGetLastError();
    c = 0;
  }
  *count = c;
  return QCS_CUDA_OK;
}

int qcs_cuda_debug_set_wait_cycles(long long cycles) {
  if (cycles < 0) return set_error(QCS_CUDA_EINVAL, "negative wait limit");
  g_wait_cycles = cycles;
  return QCS_CUDA_OK;
}

int qcs_cuda_debug_inject(int what, int count) {
  if (what == 0) {
    g_inject_alloc = 0;
    g_inject_launch = 0;
    return QCS_CUDA_OK;
  }
  if (count < 0) return set_error(QCS_CUDA_EINVAL, "negative count");
  if (what == 1) g_inject_alloc = count;
  else if (what == 2) g_inject_launch = count;
  else return set_error(QCS_CUDA_EINVAL, "unknown injection target %d", what);
  return QCS_CUDA_OK;
}

int qcs_cuda_state_create(int num_qubits, int precision, int semantics,
                          qcs_cuda_state **out) {
  if (!out) return set_error(QCS_CUDA_EINVAL, "null out");
  *out = nullptr;
  if (num_qubits < 1 || num_qubits > 36)
    return set_error(QCS_CUDA_EINVAL, "num_qubits %d outside [1, 36]", num_qubits);
  if (precision != QCS_CUDA_C64 && precision != QCS_CUDA_C128)
    return set_error(QCS_CUDA_EINVAL, "unknown precision %d", precision);
  if (semantics != QCS_CUDA_PHYSICAL && semantics != QCS_CUDA_REFERENCE)
    return set_error(QCS_CUDA_EINVAL, "unknown semantics %d", semantics);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(QCS_CUDA_ENODEV, "no CUDA device visible");
  }
  int device = 0;
  int rc = check_cuda(cudaGetDevice(&device), "cudaGetDevice");
  if (rc) return rc;

  qcs_cuda_state *s = (qcs_cuda_state *)calloc(1, sizeof(qcs_cuda_state));
  if (!s) return set_error(QCS_CUDA_ENOMEM, "host allocation of state failed");
  s->n = num_qubits;
  s->size = 1LL << num_qubits;
  s->prec = precision;
  s->sem = semantics;
  rc = device_info(device, &s->dev);
  if (rc) { free_state(s); return rc; }
  size_t bytes = (size_t)s->size * amp_bytes(s);
  rc = dmalloc(&s->vec, bytes, "cudaMalloc(state)");
  if (!rc && semantics == QCS_CUDA_REFERENCE) rc = dmalloc(&s->scratch, bytes, "cudaMalloc(scratch)");
  if (!rc) rc = check_cuda(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking),
                           "cudaStreamCreate");
  if (!rc) rc = dmalloc((void **)&s->d_partials,
                        (size_t)s->dev.reduce_blocks * sizeof(ReduceSlot), "cudaMalloc(partials)");
  if (!rc) rc = dmalloc((void **)&s->d_result, 8 * sizeof(double), "cudaMalloc(result)");
  if (!rc) rc = dmalloc((void **)&s->d_err, sizeof(int), "cudaMalloc(error flag)");
  if (!rc) rc = check_cuda(cudaMemsetAsync(s->d_err, 0, sizeof(int), s->stream), "cudaMemset(err)");
  if (!rc) rc = check_cuda(cudaMallocHost((void **)&s->h_result, 8 * sizeof(double)),
                           "cudaMallocHost(result)");
  if (!rc) rc = check_cuda(cudaMemsetAsync(s->vec, 0, bytes, s->stream), "cudaMemset(state)");
  if (!rc && s->scratch)
    rc = check_cuda(cudaMemsetAsync(s->scratch, 0, bytes, s->stream), "cudaMemset(scratch)");
  if (!rc) rc = check_cuda(cudaMemsetAsync(s->d_result, 0, 8 * sizeof(double), s->stream),
                           "cudaMemset(result)");
  if (!rc) rc = launch_set_one(s, s->vec, 0);
  if (!rc) rc = check_cuda(cudaStreamSynchronize(s->stream), "state init");
  if (rc) { free_state(s); return rc; }
  *out = s;
  return QCS_CUDA_OK;
}

int qcs_cuda_state_destroy(qcs_cuda_state *s) {
  QCS_CHECK_STATE(s);
  free_state(s);
  return QCS_CUDA_OK;
}

int qcs_cuda_state_info(const qcs_cuda_state *s, int *num_qubits, int *precision,
                        int *semantics) {
  QCS_CHECK_STATE(s);
  if (num_qubits) *num_qubits = s->n;
  if (precision) *precision = s->prec;
  if (semantics) *semantics = s->sem;
  return QCS_CUDA_OK;
}

int qcs_cuda_state_stream(qcs_cuda_state *s, void **stream) {
  QCS_CHECK_STATE(s);
  if (!stream) return set_error(QCS_CUDA_EINVAL, "null out");
  *stream = (void *)s->stream;
  return QCS_CUDA_OK;
}

int qcs_cuda_transfer_bytes(qcs_cuda_state *s, long long *h2d, long long *d2h) {
  QCS_CHECK_STATE(s);
  if (h2d) *h2d = s->h2d_bytes;
  if (d2h) *d2h = s->d2h_bytes;
  return QCS_CUDA_OK;
}

int qcs_cuda_state_device_ptr(qcs_cuda_state *s, void **ptr) {
  QCS_CHECK_STATE(s);
  if (!ptr) return set_error(QCS_CUDA_EINVAL, "null out");
  *ptr = s->vec;
  return QCS_CUDA_OK;
}

int qcs_cuda_synchronize(qcs_cuda_state *s) {
  QCS_CHECK_STATE(s);
  int rc = check_cuda(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
  if (rc) return rc;
  int flag = 0;
  s->d2h_bytes += (long long)sizeof(int);
  rc = check_cuda(cudaMemcpy(&flag, s->d_err, sizeof(int), cudaMemcpyDeviceToHost), "error flag");
  if (rc) return rc;
  if (flag) {
    cudaMemset(s->d_err, 0, sizeof(int));
    return set_error(QCS_CUDA_ETIMEOUT, "a bounded device-side wait gave up (site %d)", flag);
  }
  return QCS_CUDA_OK;
}

int qcs_cuda_set_basis(qcs_cuda_state *s, long long index) {
  QCS_CHECK_STATE(s);
  if (index < 0 || index >= s->size)
    return set_error(QCS_CUDA_EINVAL, "basis index %lld outside [0, %lld)", index, s->size);
  int rc = check_cuda(cudaMemsetAsync(s->vec, 0, (size_t)s->size * amp_bytes(s), s->stream),
                      "cudaMemset(state)");
  if (rc) return rc;
  invalidate_sum(s);
  return launch_set_one(s, s->vec, index);
}

// Host copies of complex64 states convert through a bounded host chunk, so
// reading an 8 GiB state never needs an 8 GiB host temporary.  Every copy is
// queued on the state's stream and waited for before returning.
static const i64 kCopyChunk = 1LL << 22;  // amplitudes per chunk

int qcs_cuda_read_amplitudes(qcs_cuda_state *s, long long first, long long count,
                             double *out) {
  QCS_CHECK_STATE(s);
  if (count == 0) return QCS_CUDA_OK;
  if (!out || first < 0 || count < 0 || first + count > s->size)
    return set_error(QCS_CUDA_EINVAL, "amplitude range [%lld, +%lld) outside the state", first,
                     count);
  int rc = check_cuda(cudaStreamSynchronize(s->stream), "sync before read");
  if (rc) return rc;
  if (s->prec == QCS_CUDA_C128) {
    rc = copy_d2h(s, out, (double2 *)s->vec + first, (size_t)count * 16, "cudaMemcpy(read)");
    return rc ? rc : check_cuda(cudaStreamSynchronize(s->stream), "sync after read");
  }
  std::vector<float2> tmp((size_t)(count < kCopyChunk ? count : kCopyChunk));
  for (i64 off = 0; off < count; off += kCopyChunk) {
    i64 m = count - off < kCopyChunk ? count - off : kCopyChunk;
    rc = copy_d2h(s, tmp.data(), (float2 *)s->vec + first + off, (size_t)m * 8,
                  "cudaMemcpy(read)");
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s->stream), "sync after read");
    if (rc) return rc;
    for (i64 i = 0; i < m; i++) {
      out[2 * (off + i)] = tmp[i].x;
      out[2 * (off + i) + 1] = tmp[i].y;
    }
  }
  return QCS_CUDA_OK;
}

int qcs_cuda_write_amplitudes(qcs_cuda_state *s, long long first, long long count,
                              const double *in) {
  QCS_CHECK_STATE(s);
  if (count == 0) return QCS_CUDA_OK;
  if (!in || first < 0 || count < 0 || first + count > s->size)
    return set_error(QCS_CUDA_EINVAL, "amplitude range [%lld, +%lld) outside the state", first,
                     count);
  int rc = check_cuda(cudaStreamSynchronize(s->stream), "sync before write");
  if (rc) return rc;
  invalidate_sum(s);
  if (s->prec == QCS_CUDA_C128) {
    rc = copy_h2d(s, (double2 *)s->vec + first, in, (size_t)count * 16, "cudaMemcpy(write)");
    return rc ? rc : check_cuda(cudaStreamSynchronize(s->stream), "sync after write");
  }
  std::vector<float2> tmp((size_t)(count < kCopyChunk ? count : kCopyChunk));
  for (i64 off = 0; off < count; off += kCopyChunk) {
    i64 m = count - off < kCopyChunk ? count - off : kCopyChunk;
    for (i64 i = 0; i < m; i++)
      tmp[i] = make_float2((float)in[2 * (off + i)], (float)in[2 * (off + i) + 1]);
    rc = copy_h2d(s, (float2 *)s->vec + first + off, tmp.data(), (size_t)m * 8,
                  "cudaMemcpy(write)");
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s->stream), "sync after write");
    if (rc) return rc;
  }
  return QCS_CUDA_OK;
}

int qcs_cuda_profile_enable(qcs_cuda_state *s, int enable) {
  QCS_CHECK_STATE(s);
  int rc = check_cuda(cudaStreamSynchronize(s->stream), "profile sync");
  if (rc) return rc;
  prof_free(s);
  if (enable) s->prof = new ProfData();
  return QCS_CUDA_OK;
}

int qcs_cuda_profile_read(qcs_cuda_state *s, int cls, long long *launches, double *ms,
                          double *bytes) {
  QCS_CHECK_STATE(s);
  if (cls < 0 || cls >= KC_COUNT) return set_error(QCS_CUDA_EINVAL, "bad kernel class %d", cls);
  if (!s->prof) return set_error(QCS_CUDA_EINVAL, "profiling is not enabled");
  int rc = prof_flush(s);
  if (rc) return rc;
  if (launches) *launches = s->prof->launches[cls];
  if (ms) *ms = s->prof->ms[cls];
  if (bytes) *bytes = s->prof->bytes[cls];
  return QCS_CUDA_OK;
}

int qcs_cuda_event_record(qcs_cuda_state *s, void **event) {
  QCS_CHECK_STATE(s);
  if (!event) return set_error(QCS_CUDA_EINVAL, "null out");
  cudaEvent_t e = nullptr;
  int rc = check_cuda(cudaEventCreate(&e), "cudaEventCreate");
  if (!rc) rc = check_cuda(cudaEventRecord(e, s->stream), "cudaEventRecord");
  if (rc) {
    if (e) cudaEventDestroy(e);
    return rc;
  }
  *event = (void *)e;
  return QCS_CUDA_OK;
}

int qcs_cuda_event_elapsed(void *start, void *stop, double *ms) {
  if (!start || !stop || !ms) return set_error(QCS_CUDA_EINVAL, "null event");
  int rc = check_cuda(cudaEventSynchronize((cudaEvent_t)stop), "cudaEventSynchronize");
  if (rc) return rc;
  float f = 0.f;
  rc = check_cuda(cudaEventElapsedTime(&f, (cudaEvent_t)start, (cudaEvent_t)stop),
                  "cudaEventElapsedTime");
  if (!rc) *ms = f;
  return rc;
}

int qcs_cuda_event_destroy(void *event) {
  if (!event) return QCS_CUDA_OK;
  return check_cuda(cudaEventDestroy((cudaEvent_t)event), "cudaEventDestroy");
}

int qcs_cuda_launch_count(qcs_cuda_state *s, long long *count) {
  QCS_CHECK_STATE(s);
  if (!count) return set_error(QCS_CUDA_EINVAL, "null out");
  *count = s->launches;
  return QCS_CUDA_OK;
}

}  // extern "C"
