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
// per tile of 4096 amplitudes, then one per range of tiles (at most
// kNoAllocMaxRanges) and the total.  It lives in a file-scope __device__
// array of kNoAllocMaxTiles + kNoAllocMaxRanges + 1 doubles (about 544 KB),
// which every GPU that loads the library holds until the process exits.
// States larger than kNoAllocMaxTiles * 4096 = 2^28 amplitudes are rejected.
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
#include "sampler.cuh"

namespace qcs {

constexpr i64 kNoAllocTile = kSampleTile;
constexpr i64 kNoAllocMaxTiles = 65536;
constexpr int kNoAllocMaxRanges = 4096;

static __device__ __align__(256) double g_noalloc_prefix[kNoAllocMaxTiles + kNoAllocMaxRanges + 1];

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

// The kernels are those of qcs_cuda_sample (sampler.cuh): the same rule and
// the same arithmetic, so both give the same indices for the same draws.

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
  int G = 1;
  i64 per = 1;
  smp_ranges(n_tiles, sms, kNoAllocMaxRanges, &G, &per);
  double *in = prefix, *boff = prefix + n_tiles;
  k_smp_tile_sums<C><<<G, kSampleThreads, 0, st>>>(v, tile, n_tiles, per, in, boff);
  rc = check_launch("sample_noalloc tile sums");
  if (rc) return rc;
  k_smp_prefix<<<1, 1024, 0, st>>>(boff, G);
  rc = check_launch("sample_noalloc prefix");
  if (rc || shots == 0) return rc;
  int blocks = (int)(((i64)shots * 32 + 255) / 256);
  if (blocks > sms * 16) blocks = sms * 16;
  k_smp_sample<C><<<blocks, 256, 0, st>>>(v, tile, n_tiles, per, in, boff, G, draws, shots,
                                         samples);
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
