// noalloc.cu -- shot sampling that allocates no memory at call time.
//
// Who needs it: callers that cannot call cudaMalloc on the path where they
// sample.  Examples are a host application that owns all device memory
// through its own pool and forbids libraries from allocating, and code that
// must not take cudaMalloc's implicit device synchronisation (latency-
// critical serving loops).  qcs_cuda_sample keeps its scratch in per-state
// buffers it allocates on first use; this variant keeps it in one fixed
// array that is part of the library image instead.
//
// The scratch is the per-tile probability prefix of the sampler: one double
// per tile of 4096 amplitudes plus the total.  It lives in a file-scope
// __device__ array sized for kNoAllocMaxTiles tiles (512 KB + 8 B), which
// every GPU that loads the library holds until the process exits.  States
// larger than kNoAllocMaxTiles * 4096 = 2^28 amplitudes are rejected.
//
// Host code cannot use the array's name as a device address, so the device
// address is looked up with cudaGetSymbolAddress once per device, with that
// device current, on the first call made on it.  That first call should come
// before any stream capture that the caller starts.  A device reset
// (cudaDeviceReset) ends the context the address belongs to; a call whose
// launch fails forgets the address, so the next call looks it up again.
//
// Every call writes every prefix entry it later reads, so no entry has to
// start at zero; the array simply keeps the previous call's values.  All
// calls share the one array: two calls whose kernels overlap on the GPU
// (different streams without ordering between them) race on it.
#include <mutex>

#include "common.cuh"

namespace qcs {

constexpr i64 kNoAllocTile = 4096;
constexpr i64 kNoAllocMaxTiles = 65536;

static __device__ __align__(256) double g_noalloc_prefix[kNoAllocMaxTiles + 1];

static std::mutex g_noalloc_mu;
static double *g_noalloc_addr[64];

// Device address of g_noalloc_prefix on the current device (set-up on the
// first call per device).
static int noalloc_scratch(double **out) {
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= 64) return set_error(QCS_CUDA_ENODEV, "device id %d unsupported", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    rc = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_prefix),
                    "cudaGetSymbolAddress(sampling scratch)");
    if (rc) return rc;
    g_noalloc_addr[dev] = (double *)p;
  }
  *out = g_noalloc_addr[dev];
  return QCS_CUDA_OK;
}

template <typename C>
__device__ __forceinline__ double na_prob(C x) {
  return ((double)x.x * (double)x.x) + ((double)x.y * (double)x.y);
}

__device__ __forceinline__ double na_warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// A thread's share of a tile's probability mass, with the same arithmetic
// as qcs_cuda_sample: FP64 for complex128; for complex64 an FP32 partial over
// the thread's amplitudes, added in FP64.
template <typename C>
__device__ __forceinline__ double na_thread_mass(const C *v, i64 first, i64 tile) {
  double a = 0.0;
  for (i64 j = threadIdx.x; j < tile; j += blockDim.x) a += na_prob(v[first + j]);
  return a;
}
template <>
__device__ __forceinline__ double na_thread_mass<float2>(const float2 *v, i64 first, i64 tile) {
  float a = 0.f;
  for (i64 j = threadIdx.x; j < tile; j += blockDim.x) {
    const float2 x = v[first + j];
    a = fmaf(x.x, x.x, fmaf(x.y, x.y, a));
  }
  return (double)a;
}

// Probability mass of each tile into prefix[0..n_tiles).
template <typename C>
__global__ void __launch_bounds__(256)
    k_na_tile_sums(const C *v, i64 tile, i64 n_tiles, double *prefix) {
  __shared__ double part[8];
  for (i64 t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    double a = na_thread_mass<C>(v, t * tile, tile);
    a = na_warp_sum(a);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x < 32) {
      double b = threadIdx.x < 8 ? part[threadIdx.x] : 0.0;
      b = na_warp_sum(b);
      if (threadIdx.x == 0) prefix[t] = b;
    }
    __syncthreads();
  }
}

// In-place exclusive prefix of prefix[0..n), total into prefix[n].
__global__ void __launch_bounds__(1024) k_na_prefix(double *x, i64 n) {
  __shared__ double part[1024];
  const i64 per = (n + blockDim.x - 1) / blockDim.x;
  const i64 b = threadIdx.x * per;
  const i64 e = b + per < n ? b + per : n;
  double s = 0.0;
  for (i64 i = b; i < e; i++) s += x[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double run = 0.0;
    for (int k = 0; k < (int)blockDim.x; k++) {
      double t = part[k];
      part[k] = run;
      run += t;
    }
    x[n] = run;
  }
  __syncthreads();
  double run = part[threadIdx.x];
  for (i64 i = b; i < e; i++) {
    double t = x[i];
    x[i] = run;
    run += t;
  }
}

// One warp per draw: binary search over the tile prefix, then an FP64 warp
// scan of the chosen tile.  First index with r < running sum, or -1.
template <typename C>
__global__ void k_na_sample(const C *v, i64 tile, i64 n_tiles, const double *prefix,
                            const double *draws, int shots, i64 *out) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int s = warp; s < shots; s += nwarps) {
    const double r = draws[s];
    i64 result = -1;
    if (r < prefix[n_tiles]) {
      i64 lo = 0, hi = n_tiles - 1;
      while (lo < hi) {
        i64 mid = (lo + hi) >> 1;
        if (r < prefix[mid + 1]) hi = mid;
        else lo = mid + 1;
      }
      double cum = prefix[lo];
      i64 last_nonzero = lo * tile;
      for (i64 base = lo * tile; base < (lo + 1) * tile && result < 0; base += 32) {
        double p = lane < tile ? na_prob(v[base + lane]) : 0.0;
        double incl = p;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          double y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += y;
        }
        unsigned hit = __ballot_sync(0xffffffffu, lane < tile && r < cum + incl);
        unsigned nz = __ballot_sync(0xffffffffu, lane < tile && p > 0.0);
        if (hit) result = base + __ffs(hit) - 1;
        else if (nz) last_nonzero = base + 31 - __clz(nz);
        cum += __shfl_sync(0xffffffffu, incl, 31);
      }
      if (result < 0) result = last_nonzero;
    }
    if (lane == 0) out[s] = result;
  }
}

// Forgets the current device's scratch address (after a failed launch).
static void noalloc_forget() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  g_noalloc_addr[dev] = nullptr;
}

template <typename C>
static int na_launch(const C *v, i64 count, const double *draws, int shots, i64 *samples,
                     cudaStream_t st, double *prefix) {
  const i64 tile = count < kNoAllocTile ? count : kNoAllocTile;
  const i64 n_tiles = count / tile;
  int dev = 0, sms = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (!rc)
    rc = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                    "cudaDeviceGetAttribute(multiprocessor count)");
  if (rc) return rc;
  const int gt = (int)(n_tiles < (i64)sms * 8 ? n_tiles : (i64)sms * 8);
  k_na_tile_sums<C><<<gt, 256, 0, st>>>(v, tile, n_tiles, prefix);
  rc = check_launch("sample_noalloc tile sums");
  if (rc) return rc;
  k_na_prefix<<<1, 1024, 0, st>>>(prefix, n_tiles);
  rc = check_launch("sample_noalloc prefix");
  if (rc || shots == 0) return rc;
  int blocks = (int)(((i64)shots * 32 + 255) / 256);
  if (blocks > sms * 16) blocks = sms * 16;
  k_na_sample<C><<<blocks, 256, 0, st>>>(v, tile, n_tiles, prefix, draws, shots, samples);
  return check_launch("sample_noalloc");
}

}  // namespace qcs

using namespace qcs;

extern "C" int qcs_cuda_sample_noalloc(const void *amplitudes, long long count, int precision,
                                       const double *draws, int shots, long long *samples,
                                       void *stream) {
  if (!amplitudes) return set_error(QCS_CUDA_EINVAL, "sample_noalloc: null amplitudes");
  if (precision != QCS_CUDA_C64 && precision != QCS_CUDA_C128)
    return set_error(QCS_CUDA_EINVAL, "sample_noalloc: unknown precision %d", precision);
  if (count < 1 || (count & (count - 1)) != 0)
    return set_error(QCS_CUDA_EINVAL, "sample_noalloc: count %lld is not a power of two", count);
  if (count > kNoAllocMaxTiles * kNoAllocTile)
    return set_error(QCS_CUDA_EINVAL,
                     "sample_noalloc: %lld amplitudes exceed its fixed scratch (at most 2^28 "
                     "amplitudes: %lld tiles of %lld)",
                     count, kNoAllocMaxTiles, kNoAllocTile);
  if (shots < 0 || (shots > 0 && (!draws || !samples)))
    return set_error(QCS_CUDA_EINVAL, "sample_noalloc: bad shot arguments");
  double *prefix = nullptr;
  int rc = noalloc_scratch(&prefix);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == QCS_CUDA_C128)
    rc = na_launch<double2>((const double2 *)amplitudes, count, draws, shots, (i64 *)samples,
                            st, prefix);
  else
    rc = na_launch<float2>((const float2 *)amplitudes, count, draws, shots, (i64 *)samples, st,
                           prefix);
  if (rc == QCS_CUDA_ELAUNCH) noalloc_forget();
  return rc;
}
