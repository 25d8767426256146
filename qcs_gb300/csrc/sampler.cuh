// sampler.cuh -- the kernels of shot sampling (qc_run_shots, src/qcs.c:575-607):
// per-tile probability masses, their exclusive prefix, and one warp per draw.
//
// Scratch layout (doubles): in[0 .. n_tiles) then boff[0 .. G].  The tiles
// are cut into G contiguous ranges of `per` tiles, one per block of the
// tile-sum pass; in[t] is the exclusive prefix of tile t within its range and
// boff[b] the exclusive prefix of the range totals, boff[G] the total mass.
// The prefix of tile t is boff[t / per] + in[t].  Summing within ranges on
// many SMs keeps the FP64 additions off a single SM (GB300's FP64 rate per
// SM is low).
// Shared by qcs_cuda_sample (per-state scratch) and qcs_cuda_sample_noalloc
// (a fixed library array), so that both give the same indices for the same
// draws.  The kernels have internal linkage: each translation unit that
// includes this header has its own copy.
#pragma once

#include "common.cuh"

namespace qcs {
namespace {

constexpr i64 kSampleTile = 4096;    // amplitudes per tile of the prefix
constexpr int kSampleThreads = 256;  // threads of the tile-sum blocks

// The ranges of the tile-sum pass: G blocks of `per` tiles (at most
// max_blocks blocks, 8 per SM).
inline void smp_ranges(i64 n_tiles, int sms, int max_blocks, int *G, i64 *per) {
  i64 g = (i64)sms * 8;
  if (g > max_blocks) g = max_blocks;
  if (g > n_tiles) g = n_tiles;
  if (g < 1) g = 1;
  *per = (n_tiles + g - 1) / g;
  *G = (int)((n_tiles + *per - 1) / *per);
}

__device__ __forceinline__ double smp_warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

template <typename C>
__device__ __forceinline__ double smp_prob(C x) {
  return ((double)x.x * (double)x.x) + ((double)x.y * (double)x.y);
}

// A warp's share of a full tile's probability mass.  complex64: each thread
// issues its 8 float4 loads together (units t, t + 256, ... of the tile's
// 2048 pairs of amplitudes) and sums |a|^2 in FP32 in that order; the warp
// adds its 32 partials by an FP32 tree (five roundings) and returns the sum
// in FP64 -- GB300's FP64 rate would otherwise bound this pass.  complex128:
// 16 double2 loads a thread, FP64 throughout.  Every lane returns the sum.
template <typename C>
__device__ __forceinline__ double smp_full_tile_mass(const C *v, i64 first);
template <>
__device__ __forceinline__ double smp_full_tile_mass<float2>(const float2 *v, i64 first) {
  constexpr int U = (int)(kSampleTile / 2 / kSampleThreads);  // 8
  const float4 *p = reinterpret_cast<const float4 *>(v + first) + threadIdx.x;
  float4 x[U];
#pragma unroll
  for (int k = 0; k < U; k++) x[k] = p[k * kSampleThreads];
  float a = 0.f;
#pragma unroll
  for (int k = 0; k < U; k++) {
    a = fmaf(x[k].x, x[k].x, fmaf(x[k].y, x[k].y, a));
    a = fmaf(x[k].z, x[k].z, fmaf(x[k].w, x[k].w, a));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  return (double)a;
}
template <>
__device__ __forceinline__ double smp_full_tile_mass<double2>(const double2 *v, i64 first) {
  constexpr int U = (int)(kSampleTile / kSampleThreads);  // 16
  const double2 *p = v + first + threadIdx.x;
  double2 x[U];
#pragma unroll
  for (int k = 0; k < U; k++) x[k] = p[k * kSampleThreads];
  double a = 0.0;
#pragma unroll
  for (int k = 0; k < U; k++) a += smp_prob(x[k]);
  return smp_warp_sum(a);
}

// The same for a state smaller than one full tile (its single tile); each
// lane returns its own partial (the caller sums the warp in FP64).
template <typename C>
__device__ __forceinline__ double smp_small_tile_mass(const C *v, i64 tile) {
  double a = 0.0;
  for (i64 j = threadIdx.x; j < tile; j += blockDim.x) a += smp_prob(v[j]);
  return a;
}
template <>
__device__ __forceinline__ double smp_small_tile_mass<float2>(const float2 *v, i64 tile) {
  float a = 0.f;
  for (i64 j = threadIdx.x; j < tile; j += blockDim.x) {
    const float2 x = v[j];
    a = fmaf(x.x, x.x, fmaf(x.y, x.y, a));
  }
  return (double)a;
}

// Tile masses: block b takes tiles [b per, (b + 1) per) one after another
// (FP64 across its threads in a fixed order), writes each tile's exclusive
// prefix within the range to in[t] and the range total to bsum[b].
template <typename C>
__global__ void __launch_bounds__(kSampleThreads)
    k_smp_tile_sums(const C *v, i64 tile, i64 n_tiles, i64 per, double *in, double *bsum) {
  __shared__ double part[kSampleThreads / 32];
  const i64 t0 = (i64)blockIdx.x * per;
  const i64 t1 = t0 + per < n_tiles ? t0 + per : n_tiles;
  double run = 0.0;  // thread 0: the range's running total
  for (i64 t = t0; t < t1; t++) {
    const double a = tile == kSampleTile ? smp_full_tile_mass<C>(v, t * kSampleTile)
                                         : smp_warp_sum(smp_small_tile_mass<C>(v, tile));
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x < 32) {
      double b = threadIdx.x < kSampleThreads / 32 ? part[threadIdx.x] : 0.0;
      b = smp_warp_sum(b);
      if (threadIdx.x == 0) {
        in[t] = run;
        run += b;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) bsum[blockIdx.x] = run;
}

// In-place exclusive prefix of x[0 .. n) in FP64, the total into x[n] (the
// range totals bsum[0 .. G) into the offsets boff[0 .. G]): one
// block of 1024 threads walks x in chunks of 8192 entries with a running
// carry.  Thread t owns the 8 adjacent entries 8t .. 8t+7 of a chunk (moved
// in 16-byte pieces, so a warp reads and writes 2 KB contiguous); the
// block scans the threads' totals (warp shuffles, then the 32 warp totals),
// and each thread adds its entries one after another to its offset.  The
// order of the additions is fixed, so the prefix is deterministic.
__global__ void __launch_bounds__(1024) k_smp_prefix(double *x, i64 n) {
  constexpr int E = 8;
  __shared__ double wtot[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  double carry = 0.0;
  for (i64 c0 = 0; c0 < n; c0 += (i64)blockDim.x * E) {
    const i64 i0 = c0 + (i64)t * E;
    double v[E];
    if (i0 + E <= n) {
      const double2 *p = reinterpret_cast<const double2 *>(x + i0);
#pragma unroll
      for (int k = 0; k < E / 2; k++) {
        const double2 d = p[k];
        v[2 * k] = d.x;
        v[2 * k + 1] = d.y;
      }
    } else {
#pragma unroll
      for (int k = 0; k < E; k++) v[k] = i0 + k < n ? x[i0 + k] : 0.0;
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < E; k++) s += v[k];
    double incl = s;  // inclusive scan of the thread totals within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    double excl = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0) excl = 0.0;
    if (lane == 31) wtot[w] = incl;
    __syncthreads();
    if (w == 0) {  // inclusive scan of the warp totals
      double wt = lane < (int)(blockDim.x >> 5) ? wtot[lane] : 0.0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, wt, o);
        if (lane >= o) wt += y;
      }
      wtot[lane] = wt;
    }
    __syncthreads();
    double run = carry + ((w > 0 ? wtot[w - 1] : 0.0) + excl);
    double out[E];
#pragma unroll
    for (int k = 0; k < E; k++) {
      out[k] = run;
      run += v[k];
    }
    if (i0 + E <= n) {
      double2 *p = reinterpret_cast<double2 *>(x + i0);
#pragma unroll
      for (int k = 0; k < E / 2; k++) p[k] = make_double2(out[2 * k], out[2 * k + 1]);
    } else {
#pragma unroll
      for (int k = 0; k < E; k++)
        if (i0 + k < n) x[i0 + k] = out[k];
    }
    carry += wtot[31];
    __syncthreads();  // wtot is rewritten by the next chunk
  }
  if (t == 0) x[n] = carry;
}

// One warp per draw r: the tile whose inclusive prefix first exceeds r (a
// binary search over the range offsets, then one over the tiles of that
// range), then an FP64 scan of that tile 32 amplitudes at a time (four
// groups' loads in flight together).  Result: the first index with
// r < running sum (strict, as src/qcs.c:600), or -1 when r is not below the
// total.  When r falls in a tile by its total but not by the element scan
// (rounding at the tile's upper edge), the tile's last nonzero index.
template <typename C>
__global__ void k_smp_sample(const C *v, i64 tile, i64 n_tiles, i64 per, const double *in,
                             const double *boff, int G, const double *draws, int shots, i64 *out) {
  constexpr int G4 = 4;  // 32-amplitude groups loaded together
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int s = warp; s < shots; s += nwarps) {
    const double r = draws[s];
    i64 result = -1;
    if (r < boff[G]) {
      int blo = 0, bhi = G - 1;  // the range: smallest b with r < boff[b + 1]
      while (blo < bhi) {
        const int mid = (blo + bhi) >> 1;
        if (r < boff[mid + 1]) bhi = mid;
        else blo = mid + 1;
      }
      const double off = boff[blo], end_off = boff[blo + 1];
      const i64 t0 = (i64)blo * per;
      const i64 t1 = t0 + per < n_tiles ? t0 + per : n_tiles;
      i64 lo = t0, hi = t1 - 1;  // the tile: smallest t with r < prefix(t + 1)
      while (lo < hi) {
        const i64 mid = (lo + hi) >> 1;
        const double next = mid + 1 < t1 ? off + in[mid + 1] : end_off;
        if (r < next) hi = mid;
        else lo = mid + 1;
      }
      double cum = off + in[lo];
      i64 last_nonzero = lo * tile;
      const i64 end = (lo + 1) * tile;
      for (i64 base = lo * tile; base < end && result < 0; base += 32 * G4) {
        double p[G4];
#pragma unroll
        for (int k = 0; k < G4; k++) {
          const i64 i = base + 32 * k + lane;
          p[k] = i < end ? smp_prob(v[i]) : 0.0;
        }
#pragma unroll
        for (int k = 0; k < G4; k++) {
          const i64 gb = base + 32 * k;
          if (result >= 0 || gb >= end) break;  // warp-uniform
          double incl = p[k];
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
          }
          const bool valid = gb + lane < end;
          const unsigned hit = __ballot_sync(0xffffffffu, valid && r < cum + incl);
          const unsigned nz = __ballot_sync(0xffffffffu, valid && p[k] > 0.0);
          if (hit) result = gb + __ffs(hit) - 1;
          else if (nz) last_nonzero = gb + 31 - __clz(nz);
          cum += __shfl_sync(0xffffffffu, incl, 31);
        }
      }
      if (result < 0) result = last_nonzero;
    }
    if (lane == 0) out[s] = result;
  }
}

}  // namespace
}  // namespace qcs
