// gates.cu -- per-gate amplitude sweeps (the plain path).
//
// The reference applies every gate as a full out-of-place sweep plus a copy
// (src/q_gates.c:131-148, :277-297).  Here PHYSICAL semantics sweep in
// place and touch only the amplitudes a gate changes:
//
//   dense 1q (H, X, Y, RX, RY)      all pairs (lo, lo + 2^t)       2*N*s bytes
//   diagonal 1q with U00 == 1 (Z,P) amplitudes with bit t set        N*s
//   diagonal 1q (RZ)                all amplitudes, no pairing     2*N*s
//   controlled 2x2 (CNOT)           pairs with the control bit set   N*s
//   controlled diagonal (CPHASE)    amplitudes with both bits set   N*s/2
//
// REFERENCE semantics keep the reference's out-of-place sweeps, the buffer
// swap and the [[U00,U01],[0,1]] controlled rule so that results match its
// sequential build bit for bit in complex128.
//
// All kernels are grid-stride loops over 64-bit indices; each thread keeps
// kUnroll independent pairs in flight to cover HBM latency.
#include <type_traits>

#include "common.cuh"

namespace qcs {

constexpr int kUnroll = 4;
constexpr int kSweepBlocksPerSM = 8;

// Dense 2x2 on every pair (lo, lo + 2^t).  OOP selects dst != src (REFERENCE
// semantics); in place otherwise.  Output per pair is exactly
// c_add(c_mul(g0,v0), c_mul(g1,v1)), c_add(c_mul(g2,v0), c_mul(g3,v1)).
template <typename C>
__global__ void __launch_bounds__(kSweepThreads)
    k_dense1q(C *dst, const C *src, i64 npairs, int t, Mat2<C> m) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  const i64 tb = 1LL << t;
  i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  for (; p + (kUnroll - 1) * nthr < npairs; p += kUnroll * nthr) {
    C v0[kUnroll], v1[kUnroll];
    i64 lo[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      lo[u] = insert_zero(p + u * nthr, t);
      v0[u] = src[lo[u]];
      v1[u] = src[lo[u] + tb];
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      dst[lo[u]] = cadd(cmul(m.g[0], v0[u]), cmul(m.g[1], v1[u]));
      dst[lo[u] + tb] = cadd(cmul(m.g[2], v0[u]), cmul(m.g[3], v1[u]));
    }
  }
  for (; p < npairs; p += nthr) {
    i64 lo = insert_zero(p, t);
    C v0 = src[lo], v1 = src[lo + tb];
    dst[lo] = cadd(cmul(m.g[0], v0), cmul(m.g[1], v1));
    dst[lo + tb] = cadd(cmul(m.g[2], v0), cmul(m.g[3], v1));
  }
}

// diag(d0, d1) on every amplitude: psi_i *= d_{bit t of i}.  Equal to the
// dense formula (the off-diagonal products are +-0).
template <typename C>
__global__ void __launch_bounds__(kSweepThreads)
    k_diag1q(C *v, i64 size, int t, C d0, C d1) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i + (kUnroll - 1) * nthr < size; i += kUnroll * nthr) {
    C a[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) a[u] = v[i + u * nthr];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      i64 j = i + u * nthr;
      v[j] = cmul(((j >> t) & 1) ? d1 : d0, a[u]);
    }
  }
  for (; i < size; i += nthr) v[i] = cmul(((i >> t) & 1) ? d1 : d0, v[i]);
}

// psi_i *= phase for every i whose bits b0 and b1 are both set (b1 < 0: only
// b0).  Z, P (b1 < 0) and CPHASE (control, target).
template <typename C>
__global__ void __launch_bounds__(kSweepThreads)
    k_phase_mask(C *v, i64 count, int blo, int bhi, i64 setmask, C phase) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  for (; p + (kUnroll - 1) * nthr < count; p += kUnroll * nthr) {
    C a[kUnroll];
    i64 idx[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      i64 x = insert_zero(p + u * nthr, blo);
      if (bhi >= 0) x = insert_zero(x, bhi);
      idx[u] = x | setmask;
      a[u] = v[idx[u]];
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++) v[idx[u]] = cmul(phase, a[u]);
  }
  for (; p < count; p += nthr) {
    i64 x = insert_zero(p, blo);
    if (bhi >= 0) x = insert_zero(x, bhi);
    x |= setmask;
    v[x] = cmul(phase, v[x]);
  }
}

// complex64 with both bits above bit 0 (blo >= 1): the amplitudes 2x, 2x+1
// of a 16-byte unit x share every bit but bit 0, so they are changed
// together; unit p of the affected ones is x = p with zeros inserted at
// blo-1 (and bhi-1), or'ed with setmask >> 1.  Four units in flight.
__global__ void __launch_bounds__(kSweepThreads)
    k_phase_mask_v2(float4 *v, i64 units, int blo, int bhi, i64 setmask, float2 phase) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  for (; p < units; p += kUnroll * nthr) {
    float4 a[kUnroll];
    i64 idx[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      i64 x = insert_zero(p + u * nthr, blo - 1);
      if (bhi >= 0) x = insert_zero(x, bhi - 1);
      idx[u] = x | (setmask >> 1);
      if (p + u * nthr < units) a[u] = v[idx[u]];
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      if (p + u * nthr >= units) continue;
      const float2 y0 = cmul(phase, make_float2(a[u].x, a[u].y));
      const float2 y1 = cmul(phase, make_float2(a[u].z, a[u].w));
      v[idx[u]] = make_float4(y0.x, y0.y, y1.x, y1.y);
    }
  }
}

// complex64 with the lower bit at bit 0 (blo == 0): the odd amplitude of
// every 16-byte unit whose bit bhi - 1 is set (bhi < 0: of every unit) gets
// the phase.  Whole units are moved, so a warp's accesses fill the 32-byte
// sectors the touched amplitudes lie in.
__global__ void __launch_bounds__(kSweepThreads)
    k_phase_mask_odd(float4 *v, i64 units, int bhi, float2 phase) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  const i64 set = bhi >= 1 ? 1LL << (bhi - 1) : 0;
  i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  for (; p < units; p += kUnroll * nthr) {
    float4 a[kUnroll];
    i64 idx[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      idx[u] = bhi >= 1 ? (insert_zero(p + u * nthr, bhi - 1) | set) : p + u * nthr;
      if (p + u * nthr < units) a[u] = v[idx[u]];
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      if (p + u * nthr >= units) continue;
      const float2 y = cmul(phase, make_float2(a[u].z, a[u].w));
      v[idx[u]] = make_float4(a[u].x, a[u].y, y.x, y.y);
    }
  }
}

// Unitary controlled-U, in place: pairs (lo, lo + 2^t) whose control bit is
// set.  lo enumerates indices with bit c = 1 and bit t = 0.
template <typename C>
__global__ void __launch_bounds__(kSweepThreads)
    k_ctrl1q(C *v, i64 npairs, int blo, int bhi, i64 cmask, int t, Mat2<C> m) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  const i64 tb = 1LL << t;
  i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  for (; p + (kUnroll - 1) * nthr < npairs; p += kUnroll * nthr) {
    C v0[kUnroll], v1[kUnroll];
    i64 lo[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      lo[u] = insert_zero(insert_zero(p + u * nthr, blo), bhi) | cmask;
      v0[u] = v[lo[u]];
      v1[u] = v[lo[u] + tb];
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      v[lo[u]] = cadd(cmul(m.g[0], v0[u]), cmul(m.g[1], v1[u]));
      v[lo[u] + tb] = cadd(cmul(m.g[2], v0[u]), cmul(m.g[3], v1[u]));
    }
  }
  for (; p < npairs; p += nthr) {
    i64 lo = insert_zero(insert_zero(p, blo), bhi) | cmask;
    C v0 = v[lo], v1 = v[lo + tb];
    v[lo] = cadd(cmul(m.g[0], v0), cmul(m.g[1], v1));
    v[lo + tb] = cadd(cmul(m.g[2], v0), cmul(m.g[3], v1));
  }
}

// complex64 controlled-U with control and target above bit 0: pairs of
// 16-byte units (lo, lo + 2^(t-1)), each unit two amplitudes that share the
// control and target bits.  Same per-amplitude arithmetic as k_ctrl1q.
__global__ void __launch_bounds__(kSweepThreads)
    k_ctrl1q_v2(float4 *v, i64 npairs, int blo, int bhi, i64 cmask, int t, Mat2<float2> m) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  const i64 tb = 1LL << (t - 1);
  i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  for (; p < npairs; p += kUnroll * nthr) {
    float4 a[kUnroll], b[kUnroll];
    i64 lo[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      lo[u] = insert_zero(insert_zero(p + u * nthr, blo - 1), bhi - 1) | (cmask >> 1);
      if (p + u * nthr < npairs) {
        a[u] = v[lo[u]];
        b[u] = v[lo[u] + tb];
      }
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      if (p + u * nthr >= npairs) continue;
      const float2 a0 = make_float2(a[u].x, a[u].y), a1 = make_float2(a[u].z, a[u].w);
      const float2 b0 = make_float2(b[u].x, b[u].y), b1 = make_float2(b[u].z, b[u].w);
      const float2 x0 = cadd(cmul(m.g[0], a0), cmul(m.g[1], b0));
      const float2 x1 = cadd(cmul(m.g[0], a1), cmul(m.g[1], b1));
      const float2 y0 = cadd(cmul(m.g[2], a0), cmul(m.g[3], b0));
      const float2 y1 = cadd(cmul(m.g[2], a1), cmul(m.g[3], b1));
      v[lo[u]] = make_float4(x0.x, x0.y, x1.x, x1.y);
      v[lo[u] + tb] = make_float4(y0.x, y0.y, y1.x, y1.y);
    }
  }
}

// Exchange gates, m = [[0, m01], [m10, 0]] (X, Y, and CNOT on its control=1
// pairs), in place: v0' = m01 v1, v1' = m10 v0.  The dense formula's other
// two products are +-0, so the values equal c_add(c_mul(g0,v0), c_mul(g1,v1))
// (at most the sign of a zero differs) with a third of its operations: on a
// complex128 state, whose sweeps GB300's FP64 rate bounds, that is the time.
// CTRL: pairs with the control bit set, lo enumerated as in k_ctrl1q.
template <typename C, bool CTRL>
__global__ void __launch_bounds__(kSweepThreads)
    k_exch1q(C *v, i64 npairs, int blo, int bhi, i64 cmask, int t, C m01, C m10) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  const i64 tb = 1LL << t;
  i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  for (; p < npairs; p += kUnroll * nthr) {
    C v0[kUnroll], v1[kUnroll];
    i64 lo[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      const i64 q = p + u * nthr;
      lo[u] = CTRL ? (insert_zero(insert_zero(q, blo), bhi) | cmask) : insert_zero(q, t);
      if (q < npairs) {
        v0[u] = v[lo[u]];
        v1[u] = v[lo[u] + tb];
      }
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      if (p + u * nthr >= npairs) continue;
      v[lo[u]] = cmul(m01, v1[u]);
      v[lo[u] + tb] = cmul(m10, v0[u]);
    }
  }
}

// The reference's controlled sweep (src/q_gates.c:277-297), out of place:
// every pair is copied, except that control=1 pairs get
// lo := c_add(c_mul(g0,v0), c_mul(g1,v1)) and keep hi := v1.
// FORM 1 (U01 = 0, e.g. CPHASE) and FORM 2 (U00 = 0, e.g. CNOT) leave out
// the product with the zero entry: the values are the full formula's (that
// product is +-0).
template <typename C, int FORM>
__global__ void __launch_bounds__(kSweepThreads)
    k_ctrl1q_reference(C *dst, const C *src, i64 npairs, int t, i64 cmask, Mat2<C> m) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  const i64 tb = 1LL << t;
  for (i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += nthr) {
    i64 lo = insert_zero(p, t);
    C v0 = src[lo], v1 = src[lo + tb];
    C x = v0;
    if (lo & cmask)
      x = FORM == 1 ? cmul(m.g[0], v0)
          : FORM == 2 ? cmul(m.g[1], v1)
                      : cadd(cmul(m.g[0], v0), cmul(m.g[1], v1));
    dst[lo] = x;
    dst[lo + tb] = v1;
  }
}

// REFERENCE semantics' one-qubit sweep, out of place, for a diagonal (FORM 1)
// or exchange (FORM 2) 2x2: each output is one complex product, whose value
// equals the full formula's (the other product is +-0).
template <typename C, int FORM>
__global__ void __launch_bounds__(kSweepThreads)
    k_oop1q(C *dst, const C *src, i64 npairs, int t, Mat2<C> m) {
  const i64 nthr = (i64)gridDim.x * blockDim.x;
  const i64 tb = 1LL << t;
  i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  for (; p < npairs; p += kUnroll * nthr) {
    C v0[kUnroll], v1[kUnroll];
    i64 lo[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      lo[u] = insert_zero(p + u * nthr, t);
      if (p + u * nthr < npairs) {
        v0[u] = src[lo[u]];
        v1[u] = src[lo[u] + tb];
      }
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      if (p + u * nthr >= npairs) continue;
      dst[lo[u]] = FORM == 1 ? cmul(m.g[0], v0[u]) : cmul(m.g[1], v1[u]);
      dst[lo[u] + tb] = FORM == 1 ? cmul(m.g[3], v1[u]) : cmul(m.g[2], v0[u]);
    }
  }
}

// Phase flip on one amplitude.  PHYSICAL: in place; also keeps the cached
// amplitude sum (sum[0..1]) in step when `sum` is non-null.  REFERENCE: the
// host has already swapped buffers, so dst is the stale buffer and the value
// comes from the current one (src/q_gates.c:311-316).
template <typename C>
__global__ void k_flip(C *dst, const C *src, i64 index, double *sum) {
  C a = src[index];
  dst[index] = make_c<C>(-(double)a.x, -(double)a.y);
  if (sum) {
    sum[0] -= 2.0 * (double)a.x;
    sum[1] -= 2.0 * (double)a.y;
  }
}

static bool is_zero(const double *z) { return z[0] == 0.0 && z[1] == 0.0; }
static bool is_one(const double *z) { return z[0] == 1.0 && z[1] == 0.0; }

static void swap_buffers(qcs_cuda_state *s) {
  void *t = s->vec;
  s->vec = s->scratch;
  s->scratch = t;
}

template <typename C>
static int apply_1q_t(qcs_cuda_state *s, const double m[8], int t) {
  const DeviceInfo &d = s->dev;
  const double Ns = (double)s->size * sizeof(C);
  Mat2<C> g = to_mat2<C>(m);
  C *v = (C *)s->vec;
  if (s->sem == QCS_CUDA_REFERENCE) {
    i64 np = s->size / 2;
    const int gr = grid_for(np, kSweepThreads * kUnroll, d, kSweepBlocksPerSM);
    prof_begin(s);
    if (is_zero(m + 2) && is_zero(m + 4))
      k_oop1q<C, 1><<<gr, kSweepThreads, 0, s->stream>>>((C *)s->scratch, v, np, t, g);
    else if (is_zero(m) && is_zero(m + 6))
      k_oop1q<C, 2><<<gr, kSweepThreads, 0, s->stream>>>((C *)s->scratch, v, np, t, g);
    else
      k_dense1q<C><<<gr, kSweepThreads, 0, s->stream>>>((C *)s->scratch, v, np, t, g);
    int rc = launched(s, KC_DENSE1Q, 2 * Ns, "apply_1q");
    if (rc) return rc;
    swap_buffers(s);
    return QCS_CUDA_OK;
  }
  bool diag = is_zero(m + 2) && is_zero(m + 4);
  if (diag && is_one(m)) {
    if (is_one(m + 6)) return QCS_CUDA_OK;  // identity: 1*v + 0*v == v
    i64 cnt = s->size / 2;
    prof_begin(s);
    if (std::is_same<C, float2>::value && t >= 1)
      k_phase_mask_v2<<<grid_for(cnt / 2, kSweepThreads * kUnroll, d, kSweepBlocksPerSM),
                        kSweepThreads, 0, s->stream>>>((float4 *)v, cnt / 2, t, -1, 1LL << t,
                                                       make_float2((float)m[6], (float)m[7]));
    else if (std::is_same<C, float2>::value)  // t == 0
      k_phase_mask_odd<<<grid_for(cnt, kSweepThreads * kUnroll, d, kSweepBlocksPerSM),
                         kSweepThreads, 0, s->stream>>>((float4 *)v, cnt, -1,
                                                        make_float2((float)m[6], (float)m[7]));
    else
      k_phase_mask<C><<<grid_for(cnt, kSweepThreads * kUnroll, d, kSweepBlocksPerSM),
                        kSweepThreads, 0, s->stream>>>(v, cnt, t, -1, 1LL << t, g.g[3]);
    return launched(s, KC_PHASE_MASK, Ns, "apply_1q (phase)");
  }
  if (diag) {
    prof_begin(s);
    k_diag1q<C><<<grid_for(s->size, kSweepThreads * kUnroll, d, kSweepBlocksPerSM), kSweepThreads,
                  0, s->stream>>>(v, s->size, t, g.g[0], g.g[3]);
    return launched(s, KC_DIAG1Q, 2 * Ns, "apply_1q (diagonal)");
  }
  i64 np = s->size / 2;
  prof_begin(s);
  if (std::is_same<C, double2>::value && is_zero(m) && is_zero(m + 6))  // X, Y
    k_exch1q<C, false><<<grid_for(np, kSweepThreads * kUnroll, d, kSweepBlocksPerSM),
                         kSweepThreads, 0, s->stream>>>(v, np, -1, -1, 0, t, g.g[1], g.g[2]);
  else
    k_dense1q<C><<<grid_for(np, kSweepThreads * kUnroll, d, kSweepBlocksPerSM), kSweepThreads,
                   0, s->stream>>>(v, v, np, t, g);
  return launched(s, KC_DENSE1Q, 2 * Ns, "apply_1q");
}

template <typename C>
static int apply_ctrl_t(qcs_cuda_state *s, const double m[8], int c, int t) {
  const DeviceInfo &d = s->dev;
  const double Ns = (double)s->size * sizeof(C);
  Mat2<C> g = to_mat2<C>(m);
  C *v = (C *)s->vec;
  i64 cmask = 1LL << c;
  if (s->sem == QCS_CUDA_REFERENCE) {
    i64 np = s->size / 2;
    prof_begin(s);
    const int gr = grid_for(np, kSweepThreads, d, kSweepBlocksPerSM);
    if (is_zero(m + 2))
      k_ctrl1q_reference<C, 1><<<gr, kSweepThreads, 0, s->stream>>>((C *)s->scratch, v, np, t,
                                                                     cmask, g);
    else if (is_zero(m))
      k_ctrl1q_reference<C, 2><<<gr, kSweepThreads, 0, s->stream>>>((C *)s->scratch, v, np, t,
                                                                     cmask, g);
    else
      k_ctrl1q_reference<C, 0><<<gr, kSweepThreads, 0, s->stream>>>((C *)s->scratch, v, np, t,
                                                                     cmask, g);
    int rc = launched(s, KC_CTRL1Q, 2 * Ns, "apply_controlled");
    if (rc) return rc;
    swap_buffers(s);
    return QCS_CUDA_OK;
  }
  int blo = c < t ? c : t, bhi = c < t ? t : c;
  bool diag = is_zero(m + 2) && is_zero(m + 4);
  if (diag && is_one(m)) {
    if (is_one(m + 6)) return QCS_CUDA_OK;
    i64 cnt = s->size / 4;
    prof_begin(s);
    if (std::is_same<C, float2>::value && blo >= 1)
      k_phase_mask_v2<<<grid_for(cnt / 2, kSweepThreads * kUnroll, d, kSweepBlocksPerSM),
                        kSweepThreads, 0, s->stream>>>((float4 *)v, cnt / 2, blo, bhi,
                                                       cmask | (1LL << t),
                                                       make_float2((float)m[6], (float)m[7]));
    else if (std::is_same<C, float2>::value)  // blo == 0: units with bit bhi set
      k_phase_mask_odd<<<grid_for(cnt, kSweepThreads * kUnroll, d, kSweepBlocksPerSM),
                         kSweepThreads, 0, s->stream>>>((float4 *)v, cnt, bhi,
                                                        make_float2((float)m[6], (float)m[7]));
    else
      k_phase_mask<C><<<grid_for(cnt, kSweepThreads * kUnroll, d, kSweepBlocksPerSM),
                        kSweepThreads, 0, s->stream>>>(v, cnt, blo, bhi, cmask | (1LL << t),
                                                       g.g[3]);
    return launched(s, KC_PHASE_MASK, Ns / 2, "apply_controlled (phase)");
  }
  i64 np = s->size / 4;
  prof_begin(s);
  if (std::is_same<C, float2>::value && blo >= 1)
    k_ctrl1q_v2<<<grid_for(np / 2, kSweepThreads * kUnroll, d, kSweepBlocksPerSM), kSweepThreads,
                  0, s->stream>>>((float4 *)v, np / 2, blo, bhi, cmask, t, to_mat2<float2>(m));
  else if (std::is_same<C, double2>::value && is_zero(m) && is_zero(m + 6))  // CNOT
    k_exch1q<C, true><<<grid_for(np, kSweepThreads * kUnroll, d, kSweepBlocksPerSM),
                        kSweepThreads, 0, s->stream>>>(v, np, blo, bhi, cmask, t, g.g[1], g.g[2]);
  else
    k_ctrl1q<C><<<grid_for(np, kSweepThreads * kUnroll, d, kSweepBlocksPerSM), kSweepThreads, 0,
                  s->stream>>>(v, np, blo, bhi, cmask, t, g);
  return launched(s, KC_CTRL1Q, Ns, "apply_controlled");
}

// The 2x2 travels in the kernel's parameters: 4 complex values.
static void count_matrix(qcs_cuda_state *s) {
  s->h2d_bytes += s->prec == QCS_CUDA_C128 ? 64 : 32;
}

int apply_1q(qcs_cuda_state *s, const double m[8], int t) {
  invalidate_sum(s);
  count_matrix(s);
  return s->prec == QCS_CUDA_C128 ? apply_1q_t<double2>(s, m, t) : apply_1q_t<float2>(s, m, t);
}

int apply_ctrl(qcs_cuda_state *s, const double m[8], int c, int t) {
  invalidate_sum(s);
  count_matrix(s);
  return s->prec == QCS_CUDA_C128 ? apply_ctrl_t<double2>(s, m, c, t)
                                  : apply_ctrl_t<float2>(s, m, c, t);
}

int phase_flip(qcs_cuda_state *s, i64 index) {
  void *src = s->vec;
  void *dst = s->vec;
  double *sum = nullptr;
  if (s->sem == QCS_CUDA_REFERENCE) {
    swap_buffers(s);
    dst = s->vec;  // the stale buffer becomes live
  } else if (s->sum_valid) {
    sum = s->d_result + 4;
  }
  prof_begin(s);
  if (s->prec == QCS_CUDA_C128)
    k_flip<double2><<<1, 1, 0, s->stream>>>((double2 *)dst, (const double2 *)src, index, sum);
  else
    k_flip<float2><<<1, 1, 0, s->stream>>>((float2 *)dst, (const float2 *)src, index, sum);
  if (s->sem == QCS_CUDA_REFERENCE) invalidate_sum(s);
  return launched(s, KC_OTHER, s->prec == QCS_CUDA_C128 ? 32.0 : 16.0, "phase_flip");
}

// Gate matrices of the qc_<gate> wrappers (src/q_gates.c:362-491), built on
// the host in FP64 with the same libm calls.
void gate_matrix(int kind, double angle, double m[8]) {
  for (int i = 0; i < 8; i++) m[i] = 0.0;
  double ch, sh;
  switch (kind) {
    case QCS_GATE_X:
    case QCS_GATE_CNOT:
      m[2] = 1.0; m[4] = 1.0; break;
    case QCS_GATE_H: {
      double h = 1.0 / sqrt(2.0);
      m[0] = h; m[2] = h; m[4] = h; m[6] = -h; break;
    }
    case QCS_GATE_Y:
      m[3] = -1.0; m[5] = 1.0; break;
    case QCS_GATE_Z:
      m[0] = 1.0; m[6] = -1.0; break;
    case QCS_GATE_P:
    case QCS_GATE_CPHASE:
      m[0] = 1.0; m[6] = cos(angle); m[7] = sin(angle); break;
    case QCS_GATE_RX:
      ch = cos(angle / 2.0); sh = sin(angle / 2.0);
      m[0] = ch; m[3] = -sh; m[5] = -sh; m[6] = ch; break;
    case QCS_GATE_RY:
      ch = cos(angle / 2.0); sh = sin(angle / 2.0);
      m[0] = ch; m[2] = -sh; m[4] = sh; m[6] = ch; break;
    case QCS_GATE_RZ:
      ch = cos(angle / 2.0); sh = sin(angle / 2.0);
      m[0] = ch; m[1] = -sh; m[6] = ch; m[7] = sh; break;
    default:  // identity
      m[0] = 1.0; m[6] = 1.0; break;
  }
}

bool gate_is_controlled(int kind) { return kind == QCS_GATE_CNOT || kind == QCS_GATE_CPHASE; }

bool gate_kind_valid(int kind) { return kind >= QCS_GATE_H && kind <= QCS_GATE_I; }

int check_qubit(const qcs_cuda_state *s, int q, const char *what) {
  if (q < 0 || q >= s->n)
    return set_error(QCS_CUDA_EINVAL, "%s: qubit %d outside [0, %d)", what, q, s->n);
  return QCS_CUDA_OK;
}

}  // namespace qcs

using namespace qcs;

extern "C" {

int qcs_cuda_apply_1q(qcs_cuda_state *s, const double m[8], int target) {
  QCS_CHECK_STATE(s);
  if (!m) return set_error(QCS_CUDA_EINVAL, "null gate matrix");
  int rc = check_qubit(s, target, "apply_1q");
  return rc ? rc : apply_1q(s, m, target);
}

int qcs_cuda_apply_controlled_1q(qcs_cuda_state *s, const double m[8], int control,
                                 int target) {
  QCS_CHECK_STATE(s);
  if (!m) return set_error(QCS_CUDA_EINVAL, "null gate matrix");
  int rc = check_qubit(s, control, "apply_controlled");
  if (!rc) rc = check_qubit(s, target, "apply_controlled");
  if (rc) return rc;
  if (control == target) return set_error(QCS_CUDA_EINVAL, "control equals target (%d)", target);
  return apply_ctrl(s, m, control, target);
}

int qcs_cuda_apply_gate(qcs_cuda_state *s, int kind, int target, int control, double angle) {
  QCS_CHECK_STATE(s);
  if (!gate_kind_valid(kind)) return set_error(QCS_CUDA_EINVAL, "unknown gate kind %d", kind);
  double m[8];
  gate_matrix(kind, angle, m);
  if (gate_is_controlled(kind)) return qcs_cuda_apply_controlled_1q(s, m, control, target);
  return qcs_cuda_apply_1q(s, m, target);
}

int qcs_cuda_phase_flip(qcs_cuda_state *s, long long index) {
  QCS_CHECK_STATE(s);
  if (index < 0 || index >= s->size)
    return set_error(QCS_CUDA_EINVAL, "phase flip index %lld outside [0, %lld)", index, s->size);
  return phase_flip(s, index);
}

}  // extern "C"
