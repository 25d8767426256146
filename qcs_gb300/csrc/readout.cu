// readout.cu -- FP64-accumulated reductions, measurement, diffusion and shot
// sampling.
//
// Replaces the host loops of q_state_normalize (src/q_utils.c:44-119),
// qc_measure (src/qcs.c:237-284), qc_get_probability (:391-395),
// qc_find_most_likely_state (:464-478), qc_run_shots (:575-607) and
// q_apply_diffusion (src/q_gates.c:323-356).
//
// Precision plan (GB300 has little FP64 throughput): for complex64 states a
// thread forms |a|^2 (or re, im) in FP32 over 8 amplitudes, then adds that
// partial into FP64 accumulators; block and grid combination are FP64.  The
// grid is fixed per device, so every reduction is deterministic.  complex128
// states use FP64 throughout.
#include "common.cuh"
#include "sampler.cuh"

namespace qcs {

enum { OP_NORM = 0, OP_MASK = 1, OP_SUM = 2 };

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Sum four FP64 values over the block; thread 0 writes `out`.
__device__ void block_sum4(double a, double b, double c, double d, ReduceSlot *out) {
  __shared__ double sh[4][kReduceThreads / 32];
  a = warp_sum(a);
  b = warp_sum(b);
  c = warp_sum(c);
  d = warp_sum(d);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = a;
    sh[1][w] = b;
    sh[2][w] = c;
    sh[3][w] = d;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    a = l < nw ? sh[0][l] : 0.0;
    b = l < nw ? sh[1][l] : 0.0;
    c = l < nw ? sh[2][l] : 0.0;
    d = l < nw ? sh[3][l] : 0.0;
    a = warp_sum(a);
    b = warp_sum(b);
    c = warp_sum(c);
    d = warp_sum(d);
    if (l == 0) {
      out->a = a;
      out->b = b;
      out->c = c;
      out->d = d;
    }
  }
}

template <int OP, typename R>
__device__ __forceinline__ void accum(i64 idx, R re, R im, int q, R &pa, R &pb) {
  if (OP == OP_NORM) {
    pa += re * re + im * im;
  } else if (OP == OP_MASK) {
    R p = re * re + im * im;
    if ((idx >> q) & 1) pb += p;
    else pa += p;
  } else {
    pa += re;
    pb += im;
  }
}

// complex64: units of two amplitudes (one 16-byte load), four units per
// step, FP32 within a step, FP64 across steps.
template <int OP>
__global__ void __launch_bounds__(kReduceThreads)
    k_reduce_c64(const float4 *v, i64 units, int q, ReduceSlot *out) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  double A = 0.0, B = 0.0;
  for (i64 u = (i64)blockIdx.x * blockDim.x + threadIdx.x; u < units; u += 4 * nthr) {
    float pa = 0.f, pb = 0.f;
    float4 x[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      i64 uu = u + k * nthr;
      x[k] = uu < units ? v[uu] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      i64 i0 = 2 * (u + k * nthr);
      if (OP == OP_MASK && q > 0) {
        // both amplitudes of the unit share bit q: one selection per unit
        const float p = (x[k].x * x[k].x + x[k].y * x[k].y) + (x[k].z * x[k].z + x[k].w * x[k].w);
        if ((i0 >> q) & 1) pb += p;
        else pa += p;
      } else {
        accum<OP>(i0, x[k].x, x[k].y, q, pa, pb);
        accum<OP>(i0 + 1, x[k].z, x[k].w, q, pa, pb);
      }
    }
    A += (double)pa;
    B += (double)pb;
  }
  block_sum4(A, B, 0.0, 0.0, out + blockIdx.x);
}

template <int OP>
__global__ void __launch_bounds__(kReduceThreads)
    k_reduce_c128(const double2 *v, i64 size, int q, ReduceSlot *out) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  double A = 0.0, B = 0.0;
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < size; i += nthr) {
    double2 x = v[i];
    accum<OP, double>(i, x.x, x.y, q, A, B);
  }
  block_sum4(A, B, 0.0, 0.0, out + blockIdx.x);
}

// One warp combines the per-block partials in a fixed order.
__global__ void k_finalize(const ReduceSlot *p, int nblocks, double *result) {
  double a = 0.0, b = 0.0, c = 0.0, d = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += 32) {
    a += p[i].a;
    b += p[i].b;
    c += p[i].c;
    d += p[i].d;
  }
  a = warp_sum(a);
  b = warp_sum(b);
  c = warp_sum(c);
  d = warp_sum(d);
  if (threadIdx.x == 0) {
    result[0] = a;
    result[1] = b;
    result[2] = c;
    result[3] = d;
  }
}

// Physical diffusion psi := 2*(S/N) - psi, fused with the sum of the new
// amplitudes (the sum is invariant in exact arithmetic; carrying the real
// sum of what was stored keeps a following phase flip's cached sum exact).
__global__ void __launch_bounds__(kReduceThreads)
    k_diffuse_c64(float4 *v, i64 units, const double *S, double inv_n, ReduceSlot *out) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  const float tr = (float)(2.0 * (S[0] * inv_n));
  const float ti = (float)(2.0 * (S[1] * inv_n));
  double A = 0.0, B = 0.0;
  for (i64 u = (i64)blockIdx.x * blockDim.x + threadIdx.x; u < units; u += 4 * nthr) {
    float pa = 0.f, pb = 0.f;
    float4 x[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      i64 uu = u + k * nthr;
      if (uu < units) x[k] = v[uu];
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      i64 uu = u + k * nthr;
      if (uu < units) {
        float4 y = make_float4(tr - x[k].x, ti - x[k].y, tr - x[k].z, ti - x[k].w);
        v[uu] = y;
        pa += y.x + y.z;
        pb += y.y + y.w;
      }
    }
    A += (double)pa;
    B += (double)pb;
  }
  block_sum4(A, B, 0.0, 0.0, out + blockIdx.x);
}

__global__ void __launch_bounds__(kReduceThreads)
    k_diffuse_c128(double2 *v, i64 size, const double *S, double inv_n, ReduceSlot *out) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  const double tr = 2.0 * (S[0] * inv_n);
  const double ti = 2.0 * (S[1] * inv_n);
  double A = 0.0, B = 0.0;
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < size; i += nthr) {
    double2 x = v[i];
    double2 y = make_double2(__dsub_rn(tr, x.x), __dsub_rn(ti, x.y));
    v[i] = y;
    A += y.x;
    B += y.y;
  }
  block_sum4(A, B, 0.0, 0.0, out + blockIdx.x);
}

// The reference's diffusion (src/q_gates.c:334-355): mean := S/|S| when
// |S| > 1e-10, dst := 2*mean - src (dst is the swapped-in buffer).
template <typename C>
__global__ void __launch_bounds__(kSweepThreads)
    k_diffuse_reference(C *dst, const C *src, i64 size, const double *S) {
  double mr = S[0], mi = S[1];
  double mag = sqrt(__dadd_rn(__dmul_rn(mr, mr), __dmul_rn(mi, mi)));
  if (mag > 1e-10) {
    mr /= mag;
    mi /= mag;
  }
  const C two = make_c<C>(2.0 * mr, 2.0 * mi);
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < size; i += nthr) {
    C x = src[i];
    dst[i] = make_c<C>((double)(two.x - x.x), (double)(two.y - x.y));
  }
}

// Collapse after a measurement: amplitudes whose bit q differs from the
// outcome become 0, the others are multiplied by `scale` when do_scale.
// complex64 in units of two amplitudes (one 16-byte access), four units in
// flight per thread: for q >= 1 both amplitudes of a unit share bit q, so
// the discarded half is written without being read, and the kept half is
// read only when it is rescaled; for q = 0 each unit holds one of each.
__global__ void __launch_bounds__(kReduceThreads)
    k_collapse_c64(float4 *v, i64 units, int q, int outcome, float scale, int do_scale) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  for (i64 u = (i64)blockIdx.x * blockDim.x + threadIdx.x; u < units; u += 4 * nthr) {
    float4 x[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const i64 uu = u + k * nthr;
      const bool keep = q == 0 || (int)(((2 * uu) >> q) & 1) == outcome;
      if (uu < units && keep && (q == 0 || do_scale)) x[k] = v[uu];
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const i64 uu = u + k * nthr;
      if (uu >= units) continue;
      if (q == 0) {
        const float s = do_scale ? scale : 1.f;
        v[uu] = outcome == 0 ? make_float4(x[k].x * s, x[k].y * s, 0.f, 0.f)
                             : make_float4(0.f, 0.f, x[k].z * s, x[k].w * s);
      } else if ((int)(((2 * uu) >> q) & 1) == outcome) {
        if (do_scale)
          v[uu] = make_float4(x[k].x * scale, x[k].y * scale, x[k].z * scale, x[k].w * scale);
      } else {
        v[uu] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
  }
}

// complex128: one amplitude (16 bytes) per unit, four in flight per thread.
__global__ void __launch_bounds__(kReduceThreads)
    k_collapse_c128(double2 *v, i64 size, int q, int outcome, double scale, int do_scale) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < size; i += 4 * nthr) {
    double2 x[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const i64 j = i + k * nthr;
      if (j < size && do_scale && (int)((j >> q) & 1) == outcome) x[k] = v[j];
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const i64 j = i + k * nthr;
      if (j >= size) continue;
      if ((int)((j >> q) & 1) == outcome) {
        if (do_scale) v[j] = make_double2(x[k].x * scale, x[k].y * scale);
      } else {
        v[j] = make_double2(0.0, 0.0);
      }
    }
  }
}

template <typename C, typename R>
__global__ void __launch_bounds__(kSweepThreads) k_scale(C *v, i64 size, R scale) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < size; i += nthr) {
    C x = v[i];
    x.x *= scale;
    x.y *= scale;
    v[i] = x;
  }
}

// ---- argmax ---------------------------------------------------------------
// Order: larger value first, then smaller index -- the first strict maximum
// of the reference's ascending scan.  NaN never wins.
template <typename R>
__device__ __forceinline__ bool better(R v, i64 i, R bv, i64 bi) {
  return v > bv || (v == bv && i < bi);
}

template <typename C, typename R>
__global__ void __launch_bounds__(kReduceThreads)
    k_argmax(const C *v, i64 size, ReduceSlot *out) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  R bv = (R)-1;
  i64 bi = size;
  for (i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x; i < size; i += nthr) {
    C x = v[i];
    R p = (x.x * x.x) + (x.y * x.y);
    if (better(p, i, bv, bi)) {
      bv = p;
      bi = i;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    R ov = __shfl_xor_sync(0xffffffffu, bv, o);
    i64 oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (better(ov, oi, bv, bi)) {
      bv = ov;
      bi = oi;
    }
  }
  __shared__ R sv[kReduceThreads / 32];
  __shared__ i64 si[kReduceThreads / 32];
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sv[w] = bv;
    si[w] = bi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); k++)
      if (better(sv[k], si[k], bv, bi)) {
        bv = sv[k];
        bi = si[k];
      }
    out[blockIdx.x].a = (double)bv;
    out[blockIdx.x].b = (double)bi;
  }
}

// complex64: units of two amplitudes (one 16-byte load), four in flight per
// thread; the same order (larger |a|^2, then smaller index) makes the result
// independent of which thread saw which amplitude.
__global__ void __launch_bounds__(kReduceThreads)
    k_argmax_c64(const float4 *v, i64 units, ReduceSlot *out) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  float bv = -1.f;
  i64 bi = 2 * units;
  for (i64 u = (i64)blockIdx.x * blockDim.x + threadIdx.x; u < units; u += 4 * nthr) {
    float4 x[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const i64 uu = u + k * nthr;
      if (uu < units) x[k] = v[uu];
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const i64 uu = u + k * nthr;
      if (uu >= units) continue;
      const float p0 = (x[k].x * x[k].x) + (x[k].y * x[k].y);
      const float p1 = (x[k].z * x[k].z) + (x[k].w * x[k].w);
      if (better(p0, 2 * uu, bv, bi)) {
        bv = p0;
        bi = 2 * uu;
      }
      if (better(p1, 2 * uu + 1, bv, bi)) {
        bv = p1;
        bi = 2 * uu + 1;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
    const i64 oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (better(ov, oi, bv, bi)) {
      bv = ov;
      bi = oi;
    }
  }
  __shared__ float sv[kReduceThreads / 32];
  __shared__ i64 si[kReduceThreads / 32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sv[w] = bv;
    si[w] = bi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); k++)
      if (better(sv[k], si[k], bv, bi)) {
        bv = sv[k];
        bi = si[k];
      }
    out[blockIdx.x].a = (double)bv;
    out[blockIdx.x].b = (double)bi;
  }
}

__global__ void k_argmax_finalize(const ReduceSlot *p, int nblocks, double *result) {
  if (threadIdx.x != 0) return;
  double bv = -1.0, bi = 9.0e18;
  for (int k = 0; k < nblocks; k++)
    if (p[k].a > bv || (p[k].a == bv && p[k].b < bi)) {
      bv = p[k].a;
      bi = p[k].b;
    }
  result[0] = bv;
  result[1] = bi;
}

// ---- shot sampling: sampler.cuh -------------------------------------------------

// ---- host side -----------------------------------------------------------------

static int reduce(qcs_cuda_state *s, int op, int q, double *res, int nres) {
  const DeviceInfo &d = s->dev;
  const double Ns = (double)s->size * (s->prec == QCS_CUDA_C128 ? 16 : 8);
  prof_begin(s);
  if (s->prec == QCS_CUDA_C128) {
    const double2 *v = (const double2 *)s->vec;
    if (op == OP_NORM) k_reduce_c128<OP_NORM><<<d.reduce_blocks, kReduceThreads, 0, s->stream>>>(v, s->size, q, s->d_partials);
    else if (op == OP_MASK) k_reduce_c128<OP_MASK><<<d.reduce_blocks, kReduceThreads, 0, s->stream>>>(v, s->size, q, s->d_partials);
    else k_reduce_c128<OP_SUM><<<d.reduce_blocks, kReduceThreads, 0, s->stream>>>(v, s->size, q, s->d_partials);
  } else {
    const float4 *v = (const float4 *)s->vec;
    i64 units = s->size / 2;
    if (op == OP_NORM) k_reduce_c64<OP_NORM><<<d.reduce_blocks, kReduceThreads, 0, s->stream>>>(v, units, q, s->d_partials);
    else if (op == OP_MASK) k_reduce_c64<OP_MASK><<<d.reduce_blocks, kReduceThreads, 0, s->stream>>>(v, units, q, s->d_partials);
    else k_reduce_c64<OP_SUM><<<d.reduce_blocks, kReduceThreads, 0, s->stream>>>(v, units, q, s->d_partials);
  }
  int rc = launched(s, KC_REDUCE, Ns, "reduce");
  if (rc) return rc;
  double *dst = (op == OP_SUM) ? s->d_result + 4 : s->d_result;
  prof_begin(s);
  k_finalize<<<1, 32, 0, s->stream>>>(s->d_partials, d.reduce_blocks, dst);
  rc = launched(s, KC_OTHER, d.reduce_blocks * 32.0, "reduce finalize");
  if (rc || !res) return rc;
  rc = copy_d2h(s, s->h_result, s->d_result, 8 * sizeof(double), "reduce readback");
  if (!rc) rc = check_cuda(cudaStreamSynchronize(s->stream), "reduce sync");
  if (rc) return rc;
  for (int i = 0; i < nres; i++) res[i] = s->h_result[(op == OP_SUM ? 4 : 0) + i];
  return QCS_CUDA_OK;
}

static int scale_state(qcs_cuda_state *s, double inv) {
  int g = grid_for(s->size, kSweepThreads, s->dev, 8);
  prof_begin(s);
  if (s->prec == QCS_CUDA_C128)
    k_scale<double2, double><<<g, kSweepThreads, 0, s->stream>>>((double2 *)s->vec, s->size, inv);
  else
    k_scale<float2, float><<<g, kSweepThreads, 0, s->stream>>>((float2 *)s->vec, s->size, (float)inv);
  return launched(s, KC_COLLAPSE, 2.0 * s->size * (s->prec == QCS_CUDA_C128 ? 16 : 8),
                  "normalize");
}

int diffusion(qcs_cuda_state *s) {
  const DeviceInfo &d = s->dev;
  const double Ns = (double)s->size * (s->prec == QCS_CUDA_C128 ? 16 : 8);
  int rc;
  if (s->sem == QCS_CUDA_REFERENCE) {
    rc = reduce(s, OP_SUM, 0, nullptr, 0);
    if (rc) return rc;
    void *src = s->vec;
    s->vec = s->scratch;
    s->scratch = src;
    int g = grid_for(s->size, kSweepThreads, d, 8);
    prof_begin(s);
    if (s->prec == QCS_CUDA_C128)
      k_diffuse_reference<double2><<<g, kSweepThreads, 0, s->stream>>>(
          (double2 *)s->vec, (const double2 *)src, s->size, s->d_result + 4);
    else
      k_diffuse_reference<float2><<<g, kSweepThreads, 0, s->stream>>>(
          (float2 *)s->vec, (const float2 *)src, s->size, s->d_result + 4);
    invalidate_sum(s);
    return launched(s, KC_DIFFUSE, 2 * Ns, "diffusion");
  }
  if (!s->sum_valid) {
    rc = reduce(s, OP_SUM, 0, nullptr, 0);
    if (rc) return rc;
  }
  double inv_n = ldexp(1.0, -s->n);
  prof_begin(s);
  if (s->prec == QCS_CUDA_C128)
    k_diffuse_c128<<<d.reduce_blocks, kReduceThreads, 0, s->stream>>>(
        (double2 *)s->vec, s->size, s->d_result + 4, inv_n, s->d_partials);
  else
    k_diffuse_c64<<<d.reduce_blocks, kReduceThreads, 0, s->stream>>>(
        (float4 *)s->vec, s->size / 2, s->d_result + 4, inv_n, s->d_partials);
  rc = launched(s, KC_DIFFUSE, 2 * Ns, "diffusion");
  if (rc) return rc;
  prof_begin(s);
  k_finalize<<<1, 32, 0, s->stream>>>(s->d_partials, d.reduce_blocks, s->d_result + 4);
  rc = launched(s, KC_OTHER, d.reduce_blocks * 32.0, "diffusion finalize");
  if (rc) return rc;
  s->sum_valid = 1;
  return QCS_CUDA_OK;
}

int norm_sq(qcs_cuda_state *s, double *out) { return reduce(s, OP_NORM, 0, out, 1); }

// The cached amplitude sum, computed now unless it is valid.
int ensure_sum(qcs_cuda_state *s) {
  if (s->sum_valid) return QCS_CUDA_OK;
  int rc = reduce(s, OP_SUM, 0, nullptr, 0);
  if (!rc) s->sum_valid = 1;
  return rc;
}

// A kernel left per-part sums of the new amplitudes in d_partials[0..nslots):
// combine them (fixed order) into the cached sum.
int finalize_sum(qcs_cuda_state *s, int nslots) {
  prof_begin(s);
  k_finalize<<<1, 32, 0, s->stream>>>(s->d_partials, nslots, s->d_result + 4);
  int rc = launched(s, KC_OTHER, nslots * 32.0, "sum finalize");
  if (!rc) s->sum_valid = 1;
  return rc;
}

}  // namespace qcs

using namespace qcs;

extern "C" {

int qcs_cuda_diffusion(qcs_cuda_state *s) {
  QCS_CHECK_STATE(s);
  return diffusion(s);
}

int qcs_cuda_norm_sq(qcs_cuda_state *s, double *out) {
  QCS_CHECK_STATE(s);
  if (!out) return set_error(QCS_CUDA_EINVAL, "null out");
  return norm_sq(s, out);
}

int qcs_cuda_normalize(qcs_cuda_state *s) {
  QCS_CHECK_STATE(s);
  double total;
  int rc = norm_sq(s, &total);
  if (rc) return rc;
  if (total > 1e-12 && total != 1.0) {
    invalidate_sum(s);
    return scale_state(s, 1.0 / sqrt(total));
  }
  return QCS_CUDA_OK;
}

int qcs_cuda_prob_zero(qcs_cuda_state *s, int qubit, double *p0) {
  QCS_CHECK_STATE(s);
  if (!p0) return set_error(QCS_CUDA_EINVAL, "null out");
  if (qubit < 0 || qubit >= s->n) return set_error(QCS_CUDA_EINVAL, "qubit %d out of range", qubit);
  double r[2];
  int rc = reduce(s, OP_MASK, qubit, r, 2);
  if (!rc) *p0 = r[0];
  return rc;
}

int qcs_cuda_expect_z(qcs_cuda_state *s, int qubit, double *out) {
  QCS_CHECK_STATE(s);
  if (!out) return set_error(QCS_CUDA_EINVAL, "null out");
  if (qubit < 0 || qubit >= s->n) return set_error(QCS_CUDA_EINVAL, "qubit %d out of range", qubit);
  double r[2];
  int rc = reduce(s, OP_MASK, qubit, r, 2);
  if (!rc) *out = r[0] - r[1];
  return rc;
}

int qcs_cuda_measure(qcs_cuda_state *s, int qubit, double random_val, int *outcome) {
  QCS_CHECK_STATE(s);
  if (!outcome) return set_error(QCS_CUDA_EINVAL, "null out");
  if (qubit < 0 || qubit >= s->n) return set_error(QCS_CUDA_EINVAL, "qubit %d out of range", qubit);
  double r[2];
  int rc = reduce(s, OP_MASK, qubit, r, 2);
  if (rc) return rc;
  int o = (random_val <= r[0]) ? 0 : 1;
  double kept = o ? r[1] : r[0];
  int do_scale = (kept > 1e-12 && kept != 1.0);
  double inv = do_scale ? 1.0 / sqrt(kept) : 1.0;
  prof_begin(s);
  if (s->prec == QCS_CUDA_C128)
    k_collapse_c128<<<s->dev.reduce_blocks, kReduceThreads, 0, s->stream>>>(
        (double2 *)s->vec, s->size, qubit, o, inv, do_scale);
  else
    k_collapse_c64<<<s->dev.reduce_blocks, kReduceThreads, 0, s->stream>>>(
        (float4 *)s->vec, s->size / 2, qubit, o, (float)inv, do_scale);
  invalidate_sum(s);
  rc = launched(s, KC_COLLAPSE, 1.5 * s->size * (s->prec == QCS_CUDA_C128 ? 16 : 8),
                "measure collapse");
  if (rc) return rc;
  *outcome = o;
  return QCS_CUDA_OK;
}

int qcs_cuda_probability(qcs_cuda_state *s, long long index, double *p) {
  QCS_CHECK_STATE(s);
  if (!p) return set_error(QCS_CUDA_EINVAL, "null out");
  if (index < 0 || index >= s->size) {
    *p = 0.0;  // qc_get_probability returns 0.0 out of range (src/qcs.c:392-393)
    return QCS_CUDA_OK;
  }
  size_t bytes = s->prec == QCS_CUDA_C128 ? 16 : 8;
  int rc = copy_d2h(s, s->h_result, (char *)s->vec + (size_t)index * bytes, bytes,
                    "probability readback");
  if (!rc) rc = check_cuda(cudaStreamSynchronize(s->stream), "probability sync");
  if (rc) return rc;
  if (s->prec == QCS_CUDA_C128) {
    double re = s->h_result[0], im = s->h_result[1];
    *p = (re * re) + (im * im);
  } else {
    const float *f = (const float *)s->h_result;
    *p = ((double)f[0] * (double)f[0]) + ((double)f[1] * (double)f[1]);
  }
  return QCS_CUDA_OK;
}

int qcs_cuda_argmax(qcs_cuda_state *s, long long *index, double *prob) {
  QCS_CHECK_STATE(s);
  if (!index) return set_error(QCS_CUDA_EINVAL, "null out");
  const DeviceInfo &d = s->dev;
  prof_begin(s);
  if (s->prec == QCS_CUDA_C128)
    k_argmax<double2, double><<<d.reduce_blocks, kReduceThreads, 0, s->stream>>>(
        (const double2 *)s->vec, s->size, s->d_partials);
  else if (s->size >= 2)
    k_argmax_c64<<<d.reduce_blocks, kReduceThreads, 0, s->stream>>>(
        (const float4 *)s->vec, s->size / 2, s->d_partials);
  else
    k_argmax<float2, float><<<d.reduce_blocks, kReduceThreads, 0, s->stream>>>(
        (const float2 *)s->vec, s->size, s->d_partials);
  int rc = launched(s, KC_REDUCE, (double)s->size * (s->prec == QCS_CUDA_C128 ? 16 : 8),
                    "argmax");
  if (rc) return rc;
  prof_begin(s);
  k_argmax_finalize<<<1, 32, 0, s->stream>>>(s->d_partials, d.reduce_blocks, s->d_result);
  rc = launched(s, KC_OTHER, d.reduce_blocks * 32.0, "argmax finalize");
  if (!rc) rc = copy_d2h(s, s->h_result, s->d_result, 2 * sizeof(double), "argmax readback");
  if (!rc) rc = check_cuda(cudaStreamSynchronize(s->stream), "argmax sync");
  if (rc) return rc;
  *index = (long long)s->h_result[1];
  if (prob) return qcs_cuda_probability(s, *index, prob);
  return QCS_CUDA_OK;
}

int qcs_cuda_sample(qcs_cuda_state *s, const double *random_vals, int shots,
                    long long *out_index) {
  QCS_CHECK_STATE(s);
  if (shots < 0 || (shots > 0 && (!random_vals || !out_index)))
    return set_error(QCS_CUDA_EINVAL, "bad shot arguments");
  if (shots == 0) return QCS_CUDA_OK;
  int rc = ensure_sample_scratch(s, shots);
  if (rc) return rc;
  const i64 tile = s->size / s->n_tiles;
  const DeviceInfo &d = s->dev;
  int G = 1;
  i64 per = 1;
  smp_ranges(s->n_tiles, d.num_sms, d.num_sms * 8, &G, &per);
  double *in = s->d_tile_prefix, *boff = s->d_tile_prefix + s->n_tiles;
  const double sb = s->prec == QCS_CUDA_C128 ? 16 : 8;
  prof_begin(s);
  if (s->prec == QCS_CUDA_C128)
    k_smp_tile_sums<double2><<<G, kSampleThreads, 0, s->stream>>>(
        (const double2 *)s->vec, tile, s->n_tiles, per, in, boff);
  else
    k_smp_tile_sums<float2><<<G, kSampleThreads, 0, s->stream>>>(
        (const float2 *)s->vec, tile, s->n_tiles, per, in, boff);
  rc = launched(s, KC_SAMPLE, s->size * sb, "sample tile sums");
  if (rc) return rc;
  prof_begin(s);
  k_smp_prefix<<<1, 1024, 0, s->stream>>>(boff, G);
  rc = launched(s, KC_SAMPLE, 16.0 * G, "sample prefix");
  if (rc) return rc;
  memcpy(s->h_draws, random_vals, (size_t)shots * sizeof(double));
  rc = copy_h2d(s, s->d_draws, s->h_draws, (size_t)shots * sizeof(double), "sample draws upload");
  if (rc) return rc;
  int threads = 256;
  int blocks = (int)(((i64)shots * 32 + threads - 1) / threads);
  if (blocks > d.num_sms * 16) blocks = d.num_sms * 16;
  prof_begin(s);
  if (s->prec == QCS_CUDA_C128)
    k_smp_sample<double2><<<blocks, threads, 0, s->stream>>>(
        (const double2 *)s->vec, tile, s->n_tiles, per, in, boff, G, s->d_draws, shots,
        s->d_samples);
  else
    k_smp_sample<float2><<<blocks, threads, 0, s->stream>>>(
        (const float2 *)s->vec, tile, s->n_tiles, per, in, boff, G, s->d_draws, shots,
        s->d_samples);
  rc = launched(s, KC_SAMPLE, (double)shots * tile * sb, "sample");
  if (!rc) rc = copy_d2h(s, s->h_samples, s->d_samples, (size_t)shots * sizeof(i64),
                         "sample readback");
  if (!rc) rc = check_cuda(cudaStreamSynchronize(s->stream), "sample sync");
  if (rc) return rc;
  memcpy(out_index, s->h_samples, (size_t)shots * sizeof(i64));
  return QCS_CUDA_OK;
}

}  // extern "C"
