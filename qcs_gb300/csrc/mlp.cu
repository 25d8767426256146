// mlp.cu -- the fusion cost model's network: forward, backward and Adam on the
// GPU.
//
// Network: F input features -> 64 -> 64 -> 64 (ReLU) -> 1 (linear), FP32,
// trained on squared error of log2(kernel milliseconds).  A CTA takes 64
// samples; the three weight matrices stay in shared memory and every layer is
// a small tiled product (256 threads, 16 outputs each).  The backward pass
// writes each CTA's gradient sum to its own slot and a second kernel adds the
// slots in a fixed order, so gradients are deterministic.  There is nothing
// like it in the reference (its only optimisation is the gate-history
// peephole of qc_optimize, src/qcs.c:650-698).
#include <atomic>
#include <math.h>
#include <string.h>

#include <vector>

#include "common.cuh"
#include "costmodel.h"

namespace qcs {

constexpr int kMlpRows = 64;      // samples per CTA
constexpr int kMlpThreads = 256;

struct MlpShape {
  int F;
  int off_w1, off_b1, off_w2, off_b2, off_w3, off_b3, off_w4, off_b4, count;
  __host__ __device__ MlpShape(int f) : F(f) {
    off_w1 = 0;
    off_b1 = off_w1 + F * kMlpHidden;
    off_w2 = off_b1 + kMlpHidden;
    off_b2 = off_w2 + kMlpHidden * kMlpHidden;
    off_w3 = off_b2 + kMlpHidden;
    off_b3 = off_w3 + kMlpHidden * kMlpHidden;
    off_w4 = off_b3 + kMlpHidden;
    off_b4 = off_w4 + kMlpHidden;
    count = off_b4 + 1;
  }
};

// out[s][j] = act(b[j] + sum_i in[s][i] * w[i][j]) for s < rows, j < 64;
// in is [rows][K] with row stride ld_in.
__device__ __forceinline__ void layer(const float *in, int ld_in, int K, const float *w,
                                      const float *b, float *out, bool relu) {
  for (int e = threadIdx.x; e < kMlpRows * kMlpHidden; e += kMlpThreads) {
    const int s = e / kMlpHidden, j = e % kMlpHidden;
    float acc = b[j];
    for (int i = 0; i < K; i++) acc += in[s * ld_in + i] * w[i * kMlpHidden + j];
    out[e] = relu ? fmaxf(acc, 0.f) : acc;
  }
}

// Forward (and, with y != nullptr, backward) for samples [r0, r0 + 64).
__global__ void __launch_bounds__(kMlpThreads)
    k_mlp(const float *params, int F, const float *X, const float *Y, int n, float inv_n,
          float *grad_slots, double *loss_slots, float *pred) {
  extern __shared__ float sm[];
  const MlpShape S(F);
  float *w = sm;                                  // all parameters
  float *x = w + S.count;                         // [64][F]
  float *h1 = x + kMlpRows * F;                   // [64][64] activations
  float *h2 = h1 + kMlpRows * kMlpHidden;
  float *h3 = h2 + kMlpRows * kMlpHidden;
  float *d = h3 + kMlpRows * kMlpHidden;          // [64] output error
  float *g = d + kMlpRows;                        // [64][64] back-propagated error
  float *g2 = g + kMlpRows * kMlpHidden;
  __shared__ double lsum[kMlpThreads / 32];
  const int r0 = blockIdx.x * kMlpRows;
  const int rows = n - r0 < kMlpRows ? n - r0 : kMlpRows;
  for (int i = threadIdx.x; i < S.count; i += kMlpThreads) w[i] = params[i];
  for (int e = threadIdx.x; e < kMlpRows * F; e += kMlpThreads) {
    const int s = e / F;
    x[e] = s < rows ? X[(size_t)(r0 + s) * F + e % F] : 0.f;
  }
  __syncthreads();
  layer(x, F, F, w + S.off_w1, w + S.off_b1, h1, true);
  __syncthreads();
  layer(h1, kMlpHidden, kMlpHidden, w + S.off_w2, w + S.off_b2, h2, true);
  __syncthreads();
  layer(h2, kMlpHidden, kMlpHidden, w + S.off_w3, w + S.off_b3, h3, true);
  __syncthreads();
  if (threadIdx.x < kMlpRows) {
    const int s = threadIdx.x;
    float o = w[S.off_b4];
    for (int i = 0; i < kMlpHidden; i++) o += h3[s * kMlpHidden + i] * w[S.off_w4 + i];
    if (pred && s < rows) pred[r0 + s] = o;
    // dLoss/dout for loss = (1/n) sum (out - y)^2
    d[s] = (Y && s < rows) ? 2.f * (o - Y[r0 + s]) * inv_n : 0.f;
    double l = (Y && s < rows) ? (double)(o - Y[r0 + s]) * (o - Y[r0 + s]) : 0.0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
    if ((threadIdx.x & 31) == 0) lsum[threadIdx.x >> 5] = l;
  }
  __syncthreads();
  if (!Y) return;
  if (threadIdx.x == 0) loss_slots[blockIdx.x] = lsum[0] + lsum[1];
  float *gs = grad_slots + (size_t)blockIdx.x * S.count;
  // ---- output layer
  for (int i = threadIdx.x; i < kMlpHidden; i += kMlpThreads) {
    float a = 0.f;
    for (int s = 0; s < kMlpRows; s++) a += d[s] * h3[s * kMlpHidden + i];
    gs[S.off_w4 + i] = a;
  }
  if (threadIdx.x == 0) {
    float a = 0.f;
    for (int s = 0; s < kMlpRows; s++) a += d[s];
    gs[S.off_b4] = a;
  }
  for (int e = threadIdx.x; e < kMlpRows * kMlpHidden; e += kMlpThreads) {
    const int s = e / kMlpHidden, i = e % kMlpHidden;
    g[e] = h3[e] > 0.f ? d[s] * w[S.off_w4 + i] : 0.f;  // dL/d(pre-act 3)
  }
  __syncthreads();
  // ---- hidden layers: g holds dL/d(pre-activation) of the layer above
  const float *acts[3] = {x, h1, h2};
  const int widths[3] = {F, kMlpHidden, kMlpHidden};
  const int woff[3] = {S.off_w1, S.off_w2, S.off_w3};
  const int boff[3] = {S.off_b1, S.off_b2, S.off_b3};
  float *cur = g, *nxt = g2;
  for (int L = 2; L >= 0; L--) {
    const float *a = acts[L];
    const int K = widths[L];
    for (int e = threadIdx.x; e < K * kMlpHidden; e += kMlpThreads) {
      const int i = e / kMlpHidden, j = e % kMlpHidden;
      float acc = 0.f;
      for (int s = 0; s < kMlpRows; s++) acc += a[s * K + i] * cur[s * kMlpHidden + j];
      gs[woff[L] + e] = acc;
    }
    for (int j = threadIdx.x; j < kMlpHidden; j += kMlpThreads) {
      float acc = 0.f;
      for (int s = 0; s < kMlpRows; s++) acc += cur[s * kMlpHidden + j];
      gs[boff[L] + j] = acc;
    }
    if (L > 0) {
      const float *wl = w + woff[L];
      for (int e = threadIdx.x; e < kMlpRows * kMlpHidden; e += kMlpThreads) {
        const int s = e / kMlpHidden, i = e % kMlpHidden;
        float acc = 0.f;
        for (int j = 0; j < kMlpHidden; j++) acc += cur[s * kMlpHidden + j] * wl[i * kMlpHidden + j];
        nxt[e] = a[e] > 0.f ? acc : 0.f;
      }
      __syncthreads();
      float *t = cur;
      cur = nxt;
      nxt = t;
    }
  }
}

// Sum the per-CTA slots in a fixed order.
__global__ void k_mlp_reduce(const float *slots, const double *loss_slots, int nslots, int count,
                             float *grad, double *loss) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < count) {
    float a = 0.f;
    for (int k = 0; k < nslots; k++) a += slots[(size_t)k * count + p];
    grad[p] = a;
  }
  if (p == 0) {
    double l = 0.0;
    for (int k = 0; k < nslots; k++) l += loss_slots[k];
    *loss = l;
  }
}

__global__ void k_adam(float *params, const float *grad, float *m, float *v, int count, float lr,
                       float b1, float b2, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= count) return;
  const float gp = grad[p];
  const float mp = b1 * m[p] + (1.f - b1) * gp;
  const float vp = b2 * v[p] + (1.f - b2) * gp * gp;
  m[p] = mp;
  v[p] = vp;
  params[p] -= lr * (mp / c1) / (sqrtf(vp / c2) + 1e-8f);
}

}  // namespace qcs

struct qcs_cuda_costmodel {
  int F;
  int count;
  float *d_params, *d_grad, *d_m, *d_v, *d_slots;
  double *d_loss_slots, *d_loss;
  float *d_x, *d_y, *d_pred;
  int cap_rows;
  int step;
  std::vector<float> host_params;  // mirror for planning on the host
  unsigned long long generation;   // bumped whenever host_params change
  bool host_only;                  // no device: host planning only
  cudaStream_t stream;
};

namespace qcs {

static size_t mlp_smem(int F) {
  MlpShape S(F);
  return sizeof(float) * ((size_t)S.count + kMlpRows * F + 5 * kMlpRows * kMlpHidden + kMlpRows);
}

static int cm_reserve(qcs_cuda_costmodel *m, int rows) {
  if (rows <= m->cap_rows) return QCS_CUDA_OK;
  cudaFree(m->d_x);
  cudaFree(m->d_y);
  cudaFree(m->d_pred);
  cudaFree(m->d_slots);
  cudaFree(m->d_loss_slots);
  const int nblk = (rows + kMlpRows - 1) / kMlpRows;
  int rc = check_cuda(cudaMalloc((void **)&m->d_x, (size_t)rows * m->F * sizeof(float)), "cudaMalloc(mlp)");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&m->d_y, (size_t)rows * sizeof(float)), "cudaMalloc(mlp)");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&m->d_pred, (size_t)rows * sizeof(float)), "cudaMalloc(mlp)");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&m->d_slots, (size_t)nblk * m->count * sizeof(float)), "cudaMalloc(mlp)");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&m->d_loss_slots, (size_t)nblk * sizeof(double)), "cudaMalloc(mlp)");
  if (!rc) m->cap_rows = rows;
  return rc;
}

// Loss (sum of squares) and gradient of the mean loss over rows [0, n) of
// the device arrays d_x/d_y; results stay on the device.
static int cm_grad_device(qcs_cuda_costmodel *m, const float *x, const float *y, int n) {
  const int nblk = (n + kMlpRows - 1) / kMlpRows;
  k_mlp<<<nblk, kMlpThreads, mlp_smem(m->F), m->stream>>>(m->d_params, m->F, x, y, n, 1.f / n,
                                                          m->d_slots, m->d_loss_slots, nullptr);
  int rc = check_launch("cost model backward");
  if (rc) return rc;
  k_mlp_reduce<<<(m->count + 255) / 256, 256, 0, m->stream>>>(m->d_slots, m->d_loss_slots, nblk,
                                                              m->count, m->d_grad, m->d_loss);
  return check_launch("cost model gradient sum");
}

// Generations are unique across models, so a plan kept for a destroyed model
// never matches a new model that happens to reuse its address.
static std::atomic<unsigned long long> g_cm_generation{0};

static int cm_sync_host(qcs_cuda_costmodel *m) {
  m->generation = ++g_cm_generation;
  m->host_params.resize(m->count);
  int rc = check_cuda(cudaMemcpyAsync(m->host_params.data(), m->d_params, m->count * sizeof(float),
                                      cudaMemcpyDeviceToHost, m->stream),
                      "cost model params");
  return rc ? rc : check_cuda(cudaStreamSynchronize(m->stream), "cost model sync");
}

// Host forward pass (used while planning), FP32 like the device: every
// output sums its inputs in index order, as the row-major loops below do
// with the input index outermost.
float costmodel_predict_host(const qcs_cuda_costmodel *m, const float *x) {
  const MlpShape S(m->F);
  const float *w = m->host_params.data();
  float h[kMlpHidden], t[kMlpHidden];
  memcpy(h, w + S.off_b1, sizeof(h));
  for (int i = 0; i < m->F; i++) {
    const float xi = x[i];
    if (xi == 0.f) continue;  // one-hot and flag features are mostly zero
    const float *row = w + S.off_w1 + i * kMlpHidden;
    for (int j = 0; j < kMlpHidden; j++) h[j] += xi * row[j];
  }
  for (int j = 0; j < kMlpHidden; j++) h[j] = h[j] > 0.f ? h[j] : 0.f;
  const int wo[2] = {S.off_w2, S.off_w3}, bo[2] = {S.off_b2, S.off_b3};
  for (int L = 0; L < 2; L++) {
    memcpy(t, w + bo[L], sizeof(t));
    for (int i = 0; i < kMlpHidden; i++) {
      const float hi = h[i];
      if (hi == 0.f) continue;  // ReLU zeros
      const float *row = w + wo[L] + i * kMlpHidden;
      for (int j = 0; j < kMlpHidden; j++) t[j] += hi * row[j];
    }
    for (int j = 0; j < kMlpHidden; j++) h[j] = t[j] > 0.f ? t[j] : 0.f;
  }
  float o = w[S.off_b4];
  for (int i = 0; i < kMlpHidden; i++) o += h[i] * w[S.off_w4 + i];
  return o;
}

unsigned long long costmodel_generation(const qcs_cuda_costmodel *m) { return m->generation; }

bool costmodel_ready(const qcs_cuda_costmodel *m) { return m && !m->host_params.empty(); }
int costmodel_features(const qcs_cuda_costmodel *m) { return m->F; }

}  // namespace qcs

using namespace qcs;

extern "C" {

int qcs_cuda_costmodel_create(int num_features, unsigned long long seed, qcs_cuda_costmodel **out) {
  if (!out || num_features < 1 || num_features > 64)
    return set_error(QCS_CUDA_EINVAL, "cost model: 1..64 features");
  *out = nullptr;
  int ndev = 0;
  const bool host_only = cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0;
  if (host_only) cudaGetLastError();
  qcs_cuda_costmodel *m = new qcs_cuda_costmodel();
  m->F = num_features;
  m->count = MlpShape(num_features).count;
  m->host_only = host_only;
  int rc = QCS_CUDA_OK;
  if (!host_only) {
    rc = check_cuda(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    const size_t pb = (size_t)m->count * sizeof(float);
    if (!rc) rc = check_cuda(cudaMalloc((void **)&m->d_params, pb), "cudaMalloc(mlp)");
    if (!rc) rc = check_cuda(cudaMalloc((void **)&m->d_grad, pb), "cudaMalloc(mlp)");
    if (!rc) rc = check_cuda(cudaMalloc((void **)&m->d_m, pb), "cudaMalloc(mlp)");
    if (!rc) rc = check_cuda(cudaMalloc((void **)&m->d_v, pb), "cudaMalloc(mlp)");
    if (!rc) rc = check_cuda(cudaMalloc((void **)&m->d_loss, sizeof(double)), "cudaMalloc(mlp)");
    if (!rc)
      rc = check_cuda(cudaFuncSetAttribute(k_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)mlp_smem(64)),
                      "cudaFuncSetAttribute(mlp)");
    if (rc) {
      qcs_cuda_costmodel_destroy(m);
      return rc;
    }
  }
  // He initialisation from a splitmix64 stream (host), biases zero
  std::vector<float> p(m->count, 0.f);
  const MlpShape S(num_features);
  unsigned long long st = seed;
  auto unif = [&]() {
    st += 0x9E3779B97F4A7C15ULL;
    unsigned long long z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  auto normal = [&]() {
    double u1 = unif(), u2 = unif();
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
  };
  const int fan[4] = {num_features, kMlpHidden, kMlpHidden, kMlpHidden};
  const int off[4] = {S.off_w1, S.off_w2, S.off_w3, S.off_w4};
  const int cnt[4] = {num_features * kMlpHidden, kMlpHidden * kMlpHidden, kMlpHidden * kMlpHidden,
                      kMlpHidden};
  for (int L = 0; L < 4; L++) {
    const double sd = sqrt(2.0 / fan[L]);
    for (int i = 0; i < cnt[L]; i++) p[off[L] + i] = (float)(sd * normal());
  }
  rc = qcs_cuda_costmodel_set_params(m, p.data(), m->count);
  if (rc) {
    qcs_cuda_costmodel_destroy(m);
    return rc;
  }
  *out = m;
  return QCS_CUDA_OK;
}

int qcs_cuda_costmodel_destroy(qcs_cuda_costmodel *m) {
  if (!m) return set_error(QCS_CUDA_EINVAL, "null model");
  if (m->host_only) {
    delete m;
    return QCS_CUDA_OK;
  }
  if (m->stream) cudaStreamSynchronize(m->stream);
  cudaFree(m->d_params);
  cudaFree(m->d_grad);
  cudaFree(m->d_m);
  cudaFree(m->d_v);
  cudaFree(m->d_loss);
  cudaFree(m->d_x);
  cudaFree(m->d_y);
  cudaFree(m->d_pred);
  cudaFree(m->d_slots);
  cudaFree(m->d_loss_slots);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return QCS_CUDA_OK;
}

int qcs_cuda_costmodel_num_params(qcs_cuda_costmodel *m, int *count) {
  if (!m || !count) return set_error(QCS_CUDA_EINVAL, "null argument");
  *count = m->count;
  return QCS_CUDA_OK;
}

int qcs_cuda_costmodel_get_params(qcs_cuda_costmodel *m, float *out) {
  if (!m || !out) return set_error(QCS_CUDA_EINVAL, "null argument");
  int rc = m->host_only ? QCS_CUDA_OK : cm_sync_host(m);
  if (!rc) memcpy(out, m->host_params.data(), m->count * sizeof(float));
  return rc;
}

int qcs_cuda_costmodel_set_params(qcs_cuda_costmodel *m, const float *in, int count) {
  if (!m || !in || count != m->count) return set_error(QCS_CUDA_EINVAL, "bad parameter vector");
  if (m->host_only) {
    m->host_params.assign(in, in + count);
    m->generation = ++g_cm_generation;
    return QCS_CUDA_OK;
  }
  int rc = check_cuda(cudaMemcpyAsync(m->d_params, in, count * sizeof(float), cudaMemcpyHostToDevice,
                                      m->stream),
                      "cost model params");
  if (!rc) rc = check_cuda(cudaMemsetAsync(m->d_m, 0, count * sizeof(float), m->stream), "adam");
  if (!rc) rc = check_cuda(cudaMemsetAsync(m->d_v, 0, count * sizeof(float), m->stream), "adam");
  m->step = 0;
  return rc ? rc : cm_sync_host(m);
}

int qcs_cuda_costmodel_loss_grad(qcs_cuda_costmodel *m, const float *x, const float *y, int n,
                                 double *loss, float *grad) {
  if (!m || !x || !y || n < 1) return set_error(QCS_CUDA_EINVAL, "bad arguments");
  if (m->host_only) return set_error(QCS_CUDA_ENODEV, "cost model without a device: planning only");
  int rc = cm_reserve(m, n);
  if (!rc) rc = check_cuda(cudaMemcpyAsync(m->d_x, x, (size_t)n * m->F * 4, cudaMemcpyHostToDevice, m->stream), "upload");
  if (!rc) rc = check_cuda(cudaMemcpyAsync(m->d_y, y, (size_t)n * 4, cudaMemcpyHostToDevice, m->stream), "upload");
  if (!rc) rc = cm_grad_device(m, m->d_x, m->d_y, n);
  double l = 0.0;
  if (!rc) rc = check_cuda(cudaMemcpyAsync(&l, m->d_loss, sizeof(double), cudaMemcpyDeviceToHost, m->stream), "loss");
  if (!rc && grad)
    rc = check_cuda(cudaMemcpyAsync(grad, m->d_grad, m->count * sizeof(float), cudaMemcpyDeviceToHost, m->stream), "grad");
  if (!rc) rc = check_cuda(cudaStreamSynchronize(m->stream), "sync");
  if (!rc && loss) *loss = l / n;
  return rc;
}

int qcs_cuda_costmodel_train(qcs_cuda_costmodel *m, const float *x, const float *y, int n,
                             int epochs, int batch, float lr, double *final_loss) {
  if (!m || !x || !y || n < 1 || epochs < 1 || batch < 1) return set_error(QCS_CUDA_EINVAL, "bad arguments");
  if (m->host_only) return set_error(QCS_CUDA_ENODEV, "cost model without a device: planning only");
  if (batch > n) batch = n;
  int rc = cm_reserve(m, n);
  if (!rc) rc = check_cuda(cudaMemcpyAsync(m->d_x, x, (size_t)n * m->F * 4, cudaMemcpyHostToDevice, m->stream), "upload");
  if (!rc) rc = check_cuda(cudaMemcpyAsync(m->d_y, y, (size_t)n * 4, cudaMemcpyHostToDevice, m->stream), "upload");
  const float b1 = 0.9f, b2 = 0.999f;
  for (int e = 0; !rc && e < epochs; e++) {
    for (int r = 0; !rc && r < n; r += batch) {
      const int rows = n - r < batch ? n - r : batch;
      rc = cm_grad_device(m, m->d_x + (size_t)r * m->F, m->d_y + r, rows);
      if (rc) break;
      m->step++;
      const float c1 = 1.f - powf(b1, (float)m->step), c2 = 1.f - powf(b2, (float)m->step);
      k_adam<<<(m->count + 255) / 256, 256, 0, m->stream>>>(m->d_params, m->d_grad, m->d_m, m->d_v,
                                                            m->count, lr, b1, b2, c1, c2);
      rc = check_launch("adam");
    }
  }
  if (!rc && final_loss) rc = qcs_cuda_costmodel_loss_grad(m, x, y, n, final_loss, nullptr);
  if (!rc) rc = cm_sync_host(m);
  return rc;
}

int qcs_cuda_costmodel_predict(qcs_cuda_costmodel *m, const float *x, int n, float *out) {
  if (!m || !x || !out || n < 1) return set_error(QCS_CUDA_EINVAL, "bad arguments");
  if (m->host_only) return set_error(QCS_CUDA_ENODEV, "cost model without a device: planning only");
  int rc = cm_reserve(m, n);
  if (!rc) rc = check_cuda(cudaMemcpyAsync(m->d_x, x, (size_t)n * m->F * 4, cudaMemcpyHostToDevice, m->stream), "upload");
  if (rc) return rc;
  const int nblk = (n + kMlpRows - 1) / kMlpRows;
  k_mlp<<<nblk, kMlpThreads, mlp_smem(m->F), m->stream>>>(m->d_params, m->F, m->d_x, nullptr, n,
                                                          1.f / n, nullptr, nullptr, m->d_pred);
  rc = check_launch("cost model forward");
  if (!rc) rc = check_cuda(cudaMemcpyAsync(out, m->d_pred, (size_t)n * 4, cudaMemcpyDeviceToHost, m->stream), "predict");
  return rc ? rc : check_cuda(cudaStreamSynchronize(m->stream), "sync");
}

int qcs_cuda_costmodel_predict_host(qcs_cuda_costmodel *m, const float *x, int n, float *out) {
  if (!m || !x || !out || n < 1) return set_error(QCS_CUDA_EINVAL, "bad arguments");
  for (int i = 0; i < n; i++) out[i] = costmodel_predict_host(m, x + (size_t)i * m->F);
  return QCS_CUDA_OK;
}

}  // extern "C"
