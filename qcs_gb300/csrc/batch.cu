// batch.cu -- many independent circuits in one persistent kernel launch.
//
// The reference simulates one circuit per t_q_circuit, every gate a full
// sweep (src/qcs.c:159-228), and reads results with qc_measure/qc_run_shots
// (:237-284, :575-607).  A batch of thousands of small-to-medium circuits
// (10..22 qubits) is launch-bound that way.  Here one persistent kernel takes
// the whole batch:
//
//  * CTAs pull instances from an atomic queue, largest first (the order is
//    part of the tuned schedule);
//  * an instance of at most `tile_q` qubits lives entirely in shared memory:
//    |0...0> is built there, its gates run there, and <Z_0> and the shots
//    are computed there -- it never touches HBM;
//  * gates run in register groups: the gates of a stage are partitioned
//    greedily into groups on at most 4 tile bits, and one pass over shared
//    memory applies a whole group, each thread holding the 16 amplitudes of
//    one setting of the other bits in registers (one pass per group instead
//    of one per gate);
//  * a larger instance lives in a per-CTA slot of global memory and runs in
//    stages: a stage is a set of tile_q qubits and the gates acting inside
//    it; for every tile (one setting of the other qubits) the CTA gathers the
//    2^tile_q amplitudes into shared memory with coalesced runs, applies the
//    stage's gates there and scatters them back, so a stage costs one read
//    and one write of the state however many gates it holds;
//  * <Z_0> is accumulated in FP64 (FP32 partials over 8 amplitudes) and each
//    shot is drawn from a counter-based generator (splitmix64 of seed,
//    instance, shot), mapped to an index with an FP64 warp scan.
//
// The run is captured once into a CUDA graph (queue reset, kernel, result
// copies) and replayed; new angles only rewrite the pinned gate table the
// graph's upload node reads.  The schedule (threads per CTA, tile size,
// CTAs per SM, instance order) comes from qcs_cuda_batch_autotune, which
// times the candidates on the batch itself.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "fusion.h"

namespace qcs {

struct BInst {
  int n;
  int stage0;
  int nstages;
  int group;  // CTAs that share the instance's stages (1: one CTA)
};

// Bounded spin of one thread on a counter another CTA raises: ~2 s.

struct BStage {
  int group0;
  int ngroups;
  int nt;             // tile qubits (local bits)
  int pad;
  signed char q[24];  // local bit m -> global qubit (ascending)
};

// Up to kGroupQ tile bits whose gates run in one pass: each thread holds the
// 2^r amplitudes of one setting of the other bits in registers and applies
// the group's gates to them in order.
constexpr int kGroupQ = 4;
struct BGroup {
  int gate0;
  int ngates;
  int r;                    // group bits
  signed char q[kGroupQ];   // tile bit of group bit j (ascending)
};

struct BGate {
  float2 m[4];
  int type;  // 0: 2x2 on group bit t; 1: 2x2 on group bit t where bit c is set
  int t, c;
  int form;  // 0: dense; 1: exchange (X, CNOT: m = [[0,1],[1,0]]); 2: diagonal
};

struct BatchTune {
  int threads;      // 256, 512 or 1024
  int tile_q;       // 12, 13 or 14
  int ctas_per_sm;  // 1, 2 or 4 (as many as shared memory and registers allow)
  int order;        // 0: largest first, 1: given order
  int split_q;      // instances above split_q qubits run on 2^(n - split_q) CTAs
};

}  // namespace qcs

struct qcs_cuda_batch {
  int count;
  int shots;
  unsigned long long seed;
  int max_n;
  std::vector<int> nq;            // qubits per instance
  std::vector<qcs_cuda_op> ops;   // all ops, instance after instance
  std::vector<int> op_off;        // count + 1
  // plan (for the current tile size)
  std::vector<qcs::BInst> insts;
  std::vector<qcs::BStage> stages;
  std::vector<qcs::BGroup> groups;
  // planned gates in group order: gate i is the product of the ops
  // fold_ops[fold_off[i] .. fold_off[i+1]) (one-qubit gates on one qubit with
  // nothing else on that qubit between them fold into one 2x2)
  std::vector<int> fold_off;
  std::vector<int> fold_ops;
  std::vector<int> gate_tc;       // its group-local target | control << 8 (control 0xFF: none)
  std::vector<int> order;         // instance order
  std::vector<int2> items;        // (instance, member) in queue order
  qcs::BatchTune tune;
  int planned_tile_q;
  // device
  cudaStream_t stream;
  qcs::DeviceInfo dev;
  qcs::BInst *d_insts;
  qcs::BStage *d_stages;
  qcs::BGroup *d_groups;
  qcs::BGate *d_gates;
  qcs::BGate *h_gates;  // pinned; the graph's upload node reads it
  int2 *d_items;
  int *d_queue;
  int *d_stage_done;  // per instance: member stage completions this launch
  int *d_lead;        // per instance: 1 + CTA of member 0 (its slot holds the state)
  double *d_z;
  double *h_z;          // pinned
  qcs::i64 *d_samples;
  qcs::i64 *h_samples;  // pinned
  float2 *d_slots;      // one global slot per CTA for instances above tile_q
  int *d_err;
  long long wait_captured;  // wait limit the captured graph's kernel carries
  size_t slot_amps;
  int grid;
  size_t cap_gates, cap_stages;
  cudaGraphExec_t graph;
  float last_ms;
};

namespace qcs {

constexpr int kMassTile = 4096;  // sampling tile (amplitudes)

__device__ __forceinline__ u64 splitmix64(u64 x) {
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  return x ^ (x >> 31);
}

// Uniform draw in [0, 1) for (seed, instance, shot), 53 random bits.
__host__ __device__ inline double shot_draw(u64 seed, u64 inst, u64 shot) {
  u64 x = seed ^ (inst * 0xD1B54A32D192ED03ULL) ^ (shot * 0x8CB92BA72F3D8DD7ULL);
  x += 0x9E3779B97F4A7C15ULL;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
  x ^= x >> 31;
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ double bwarp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

template <int T>
__device__ double block_sum(double v, double *red) {
  v = bwarp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = l < T / 32 ? red[l] : 0.0;
    r = bwarp_sum(r);
  }
  return r;  // valid in thread 0
}

// Shared-memory position of tile amplitude i: the low 4 bits are XORed with
// the next 4, a bijection that spreads a warp's accesses over the banks
// whichever tile bits a gate group holds (without it, a group on bits 0..3
// sends all 32 lanes of a warp to one bank).
__device__ __forceinline__ int swz(int i) { return i ^ ((i >> 4) & 15); }

// One 2x2 on register bit TB of the R amplitudes a[] (controlled: only where
// register bit c is set).  Static indices keep a[] in registers.
template <int R, int TB>
__device__ __forceinline__ void reg_gate(float2 (&a)[1 << kGroupQ], const BGate &g) {
  if (g.form == 1) {  // exchange: no arithmetic
#pragma unroll
    for (int e = 0; e < R; e++) {
      if (e & (1 << TB)) continue;
      if (g.type && !((e >> g.c) & 1)) continue;
      const float2 v0 = a[e];
      a[e] = a[e | (1 << TB)];
      a[e | (1 << TB)] = v0;
    }
  } else if (g.form == 2) {  // diagonal: one complex product per amplitude
#pragma unroll
    for (int e = 0; e < R; e++) {
      if (e & (1 << TB)) continue;
      if (g.type && !((e >> g.c) & 1)) continue;
      a[e] = cmul(g.m[0], a[e]);
      a[e | (1 << TB)] = cmul(g.m[3], a[e | (1 << TB)]);
    }
  } else {
#pragma unroll
    for (int e = 0; e < R; e++) {
      if (e & (1 << TB)) continue;
      if (g.type && !((e >> g.c) & 1)) continue;
      const float2 v0 = a[e], v1 = a[e | (1 << TB)];
      a[e] = cadd(cmul(g.m[0], v0), cmul(g.m[1], v1));
      a[e | (1 << TB)] = cadd(cmul(g.m[2], v0), cmul(g.m[3], v1));
    }
  }
}

// Apply one group to a tile of 2^nt amplitudes in shared memory.
template <int T, int RB>
__device__ __forceinline__ void smem_group_r(float2 *S, int nt, const BGroup &G,
                                             const BGate *gates) {
  constexpr int R = 1 << RB;
  const int np = 1 << (nt - RB);
  int qb[kGroupQ];
#pragma unroll
  for (int j = 0; j < RB; j++) qb[j] = G.q[j];
  for (int p = threadIdx.x; p < np; p += T) {
    int base = p;
#pragma unroll
    for (int j = 0; j < RB; j++)  // ascending: insert a zero at tile bit qb[j]
      base = ((base >> qb[j]) << (qb[j] + 1)) | (base & ((1 << qb[j]) - 1));
    // offset of register e: base with group bit j of e at tile bit qb[j]
    auto off = [&](int e) {
      int o = base;
#pragma unroll
      for (int j = 0; j < RB; j++)
        if ((e >> j) & 1) o |= 1 << qb[j];
      return o;
    };
    float2 a[1 << kGroupQ];
#pragma unroll
    for (int e = 0; e < R; e++) a[e] = S[swz(off(e))];
    for (int gi = 0; gi < G.ngates; gi++) {
      const BGate g = gates[G.gate0 + gi];
      switch (g.t) {
        case 0: reg_gate<R, 0>(a, g); break;
        case 1: if constexpr (RB > 1) reg_gate<R, 1>(a, g); break;
        case 2: if constexpr (RB > 2) reg_gate<R, 2>(a, g); break;
        default: if constexpr (RB > 3) reg_gate<R, 3>(a, g); break;
      }
    }
#pragma unroll
    for (int e = 0; e < R; e++) S[swz(off(e))] = a[e];
  }
}

template <int T>
__device__ __forceinline__ void smem_group(float2 *S, int nt, const BGroup &G, const BGate *gates) {
  switch (G.r) {
    case 1: smem_group_r<T, 1>(S, nt, G, gates); break;
    case 2: smem_group_r<T, 2>(S, nt, G, gates); break;
    case 3: smem_group_r<T, 3>(S, nt, G, gates); break;
    default: smem_group_r<T, 4>(S, nt, G, gates); break;
  }
}

// Shots of one instance: prefix of tile masses in shared memory, one warp per
// shot, FP64 scan.  amp(i) reads amplitude i (shared or global).
template <int T, typename AmpFn>
__device__ void sample_shots(const double *prefix, int n_tiles, int tile, int shots, u64 seed,
                             int inst, i64 *out, AmpFn amp) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int s = warp; s < shots; s += T / 32) {
    const double r = shot_draw(seed, (u64)inst, (u64)s);
    i64 result = -1;
    if (r < prefix[n_tiles]) {
      int lo = 0, hi = n_tiles - 1;
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (r < prefix[mid + 1]) hi = mid;
        else lo = mid + 1;
      }
      double cum = prefix[lo];
      i64 last_nonzero = (i64)lo * tile;
      for (i64 base = (i64)lo * tile; base < (i64)(lo + 1) * tile && result < 0; base += 32) {
        double p = 0.0;
        if (lane < tile) {
          float2 a = amp(base + lane);
          p = (double)a.x * a.x + (double)a.y * a.y;
        }
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

// Exclusive prefix of m values in shared memory (m <= 1024), total at [m].
template <int T>
__device__ void smem_prefix(double *x, int m) {
  __syncthreads();
  if (threadIdx.x == 0) {
    double run = 0.0;
    for (int i = 0; i < m; i++) {
      const double t = x[i];
      x[i] = run;
      run += t;
    }
    x[m] = run;
  }
  __syncthreads();
}

// Thread 0 waits until *cnt >= target, at most `limit` clock cycles; false
// on timeout or abort.
__device__ bool wait_count(const int *cnt, int target, int *err, int where, long long limit) {
  const long long t0 = clock64();
  while (*(volatile const int *)cnt < target) {
    if (*(volatile const int *)err) return false;
    if (clock64() - t0 > limit) {
      atomicCAS(err, 0, where);
      return false;
    }
    __nanosleep(200);
  }
  __threadfence();
  return true;
}

// 64 registers a thread: two CTAs of 512 threads (or one of 1024) fit an SM.
// Work items are (instance, member): an instance of `group` > 1 is shared by
// `group` CTAs that split the tiles of each stage and meet at a counter
// after every stage; the grid never exceeds the CTAs that fit the GPU at
// once, so every member of a group runs concurrently with the others.
template <int T>
__global__ void __launch_bounds__(T, 1024 / T)
    k_batch(const BInst *insts, const BStage *stages, const BGroup *groups, const BGate *gates,
            const int2 *items, int n_items, int shots, u64 seed, int tile_q, float2 *slots,
            i64 slot_amps, int *queue, int *stage_done, int *lead, int *err, double *z_out,
            i64 *samples_out, long long wait) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *S = reinterpret_cast<float2 *>(smem_raw);               // 2^tile_q amplitudes
  double *prefix = reinterpret_cast<double *>(S + (1 << tile_q));  // up to 1025 tile masses
  __shared__ double red[T / 32];
  __shared__ int s_item;
  __shared__ int s_ok;
  __shared__ i64 goff_lo[64];
  __shared__ i64 goff_hi[256];

  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
    __syncthreads();
    const int qi = s_item;
    if (qi >= n_items) break;
    const int inst = items[qi].x;
    const int member = items[qi].y;
    const BInst I = insts[inst];
    const int G = I.group;
    const i64 size = 1LL << I.n;
    double z = 0.0;
    // the instance's amplitudes live in the slot of its member-0 CTA
    float2 *slot = slots + (i64)blockIdx.x * slot_amps;
    if (G > 1) {
      if (threadIdx.x == 0) {
        s_ok = 1;
        if (member == 0) {
          atomicExch(&lead[inst], blockIdx.x + 1);
        } else {
          s_ok = wait_count(&lead[inst], 1, err, 1, wait) ? 1 : 0;
        }
      }
      __syncthreads();
      if (!s_ok) return;
      slot = slots + (i64)(*(volatile int *)&lead[inst] - 1) * slot_amps;
    }
    if (I.n <= tile_q) {
      // ---- shared-memory resident instance ----
      const int L = 1 << I.n;
      for (int i = threadIdx.x; i < L; i += T) S[swz(i)] = make_float2(i == 0 ? 1.f : 0.f, 0.f);
      __syncthreads();
      const BStage st = stages[I.stage0];
      for (int gi = 0; gi < st.ngroups; gi++) {
        smem_group<T>(S, I.n, groups[st.group0 + gi], gates);
        __syncthreads();
      }
      const int tile = L < kMassTile ? L : kMassTile;
      const int n_tiles = L / tile;
      for (int t = 0; t < n_tiles; t++) {
        double zp = 0.0, mp = 0.0;
        for (int j = threadIdx.x; j < tile; j += T) {
          const int i = t * tile + j;
          const float2 a = S[swz(i)];
          const float p = a.x * a.x + a.y * a.y;
          mp += (double)p;
          zp += (i & 1) ? -(double)p : (double)p;
        }
        const double ms = block_sum<T>(mp, red);
        const double zs = block_sum<T>(zp, red);
        if (threadIdx.x == 0) {
          prefix[t] = ms;
          z += zs;
        }
      }
      smem_prefix<T>(prefix, n_tiles);
      sample_shots<T>(prefix, n_tiles, tile, shots, seed, inst, samples_out + (i64)inst * shots,
                      [&](i64 i) { return S[swz((int)i)]; });
    } else {
      // ---- global-slot instance, run in stages ----
      for (int si = 0; si < I.nstages; si++) {
        const BStage st = stages[I.stage0 + si];
        const int nt = st.nt;
        const int L = 1 << nt;
        // offset tables for this stage: local index l = lo | hi << 6
        __syncthreads();
        for (int e = threadIdx.x; e < 64 + 256; e += T) {
          const bool is_lo = e < 64;
          const int v = is_lo ? e : e - 64;
          i64 o = 0;
          for (int m = 0; m < nt; m++) {
            const int bit = is_lo ? m : m - 6;
            if ((is_lo && m < 6) || (!is_lo && m >= 6))
              if ((v >> bit) & 1) o |= 1LL << st.q[m];
          }
          if (is_lo) goff_lo[v] = o;
          else goff_hi[v] = o;
        }
        __syncthreads();
        // qubits outside the tile, ascending: the tile id's bits
        i64 outside[40];
        int nout = 0;
        {
          int k = 0;
          for (int q = 0; q < I.n; q++) {
            if (k < nt && st.q[k] == q) {
              k++;
              continue;
            }
            outside[nout++] = q;
          }
        }
        const i64 n_tiles = 1LL << nout;
        for (i64 tt = member; tt < n_tiles; tt += G) {
          i64 base = 0;
          for (int j = 0; j < nout; j++) base |= ((tt >> j) & 1LL) << outside[j];
          for (int l = threadIdx.x; l < L; l += T) {
            const i64 gidx = base + goff_lo[l & 63] + goff_hi[l >> 6];
            S[swz(l)] = si == 0 ? make_float2(gidx == 0 ? 1.f : 0.f, 0.f) : slot[gidx];
          }
          __syncthreads();
          for (int gi = 0; gi < st.ngroups; gi++) {
            smem_group<T>(S, nt, groups[st.group0 + gi], gates);
            __syncthreads();
          }
          for (int l = threadIdx.x; l < L; l += T)
            slot[base + goff_lo[l & 63] + goff_hi[l >> 6]] = S[swz(l)];
          __syncthreads();
        }
        if (G > 1) {  // every member's tiles of this stage are written
          __threadfence();  // each thread's slot writes, before the count
          __syncthreads();
          if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(&stage_done[inst], 1);
            s_ok = wait_count(&stage_done[inst], G * (si + 1), err, 2, wait) ? 1 : 0;
          }
          __syncthreads();
          if (!s_ok) return;
        }
      }
      if (member != 0) continue;  // member 0 reads out the instance
      __threadfence_block();
      __syncthreads();
      // <Z_0> and tile masses in one contiguous pass (deterministic order);
      // at most 1024 sampling tiles
      const i64 mtile = size >> 10 > kMassTile ? size >> 10 : kMassTile;
      const int n_tiles = (int)(size / mtile);
      for (int t = 0; t < n_tiles; t++) {
        double zp = 0.0, mp = 0.0;
        for (i64 j = threadIdx.x; j < mtile; j += T) {
          const i64 i = (i64)t * mtile + j;
          const float2 a = slot[i];
          const float p = a.x * a.x + a.y * a.y;
          mp += (double)p;
          zp += (i & 1) ? -(double)p : (double)p;
        }
        const double ms = block_sum<T>(mp, red);
        const double zs = block_sum<T>(zp, red);
        if (threadIdx.x == 0) {
          prefix[t] = ms;
          z += zs;
        }
      }
      smem_prefix<T>(prefix, n_tiles);
      sample_shots<T>(prefix, n_tiles, (int)mtile, shots, seed, inst,
                      samples_out + (i64)inst * shots, [&](i64 i) { return slot[i]; });
    }
    if (threadIdx.x == 0) z_out[inst] = z;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// The gates of one stage (op indices in order) on tile qubits tq (ascending)
// as register groups of at most kGroupQ tile bits: a greedy partition of the
// stage's gates (commuting only past gates on disjoint qubits).
static void plan_groups(qcs_cuda_batch *b, const std::vector<int> &stage_ops, int n,
                        const std::vector<int> &tq, BStage &st) {
  st.group0 = (int)b->groups.size();
  std::vector<qcs_cuda_op> sub(stage_ops.size());
  for (size_t j = 0; j < stage_ops.size(); j++) sub[j] = b->ops[stage_ops[j]];
  PartitionOptions po;
  po.kmax = kGroupQ;
  po.cost = nullptr;
  po.cost_ctx = nullptr;
  std::vector<PlanItem> items = partition(sub.data(), (int)sub.size(), n, po);
  auto tile_bit = [&](int q) {
    for (size_t m = 0; m < tq.size(); m++)
      if (tq[m] == q) return (int)m;
    return -1;
  };
  for (const PlanItem &it : items) {
    BGroup G;
    memset(&G, 0, sizeof(G));
    G.gate0 = (int)b->gate_tc.size();
    G.r = (int)it.qubits.size();
    for (int j = 0; j < G.r; j++) G.q[j] = (signed char)tile_bit(it.qubits[j]);
    auto group_bit = [&](int q) {
      for (int j = 0; j < G.r; j++)
        if (it.qubits[j] == q) return j;
      return -1;
    };
    // gates of the group in order; pending[j]: index (in this group's gate
    // list) of the one-qubit gate on group bit j that later one-qubit gates
    // on j fold into, -1 after a two-qubit gate touched j
    std::vector<std::vector<int>> glist;
    std::vector<int> gtc;
    int pending[kGroupQ];
    for (int j = 0; j < kGroupQ; j++) pending[j] = -1;
    for (int g : it.gates) {
      const qcs_cuda_op &o = sub[g];
      const int t = group_bit(o.target);
      if (gate_is_controlled(o.kind)) {
        const int c = group_bit(o.control);
        pending[t] = pending[c] = -1;
        glist.push_back({stage_ops[g]});
        gtc.push_back(t | (c << 8));
      } else if (pending[t] >= 0) {
        glist[pending[t]].push_back(stage_ops[g]);
      } else {
        pending[t] = (int)glist.size();
        glist.push_back({stage_ops[g]});
        gtc.push_back(t | (0xFF << 8));
      }
    }
    for (size_t e = 0; e < glist.size(); e++) {
      b->fold_off.push_back((int)b->fold_ops.size());
      for (int op : glist[e]) b->fold_ops.push_back(op);
      b->gate_tc.push_back(gtc[e]);
    }
    G.ngates = (int)b->gate_tc.size() - G.gate0;
    b->groups.push_back(G);
  }
  st.ngroups = (int)b->groups.size() - st.group0;
}

static int batch_plan(qcs_cuda_batch *b, int tile_q) {
  b->insts.clear();
  b->stages.clear();
  b->groups.clear();
  b->fold_off.clear();
  b->fold_ops.clear();
  b->gate_tc.clear();
  for (int i = 0; i < b->count; i++) {
    BInst I;
    I.n = b->nq[i];
    I.stage0 = (int)b->stages.size();
    I.group = 1;
    const qcs_cuda_op *ops = b->ops.data() + b->op_off[i];
    const int nops = b->op_off[i + 1] - b->op_off[i];
    if (I.n <= tile_q) {
      BStage st;
      memset(&st, 0, sizeof(st));
      st.nt = I.n;
      std::vector<int> tq(I.n), stage_ops(nops);
      std::iota(tq.begin(), tq.end(), 0);
      std::iota(stage_ops.begin(), stage_ops.end(), b->op_off[i]);
      for (int m = 0; m < I.n; m++) st.q[m] = (signed char)m;
      plan_groups(b, stage_ops, I.n, tq, st);
      b->stages.push_back(st);
      I.nstages = 1;
    } else {
      PartitionOptions po;
      po.kmax = tile_q - 3;
      po.cost = nullptr;
      po.cost_ctx = nullptr;
      std::vector<PlanItem> plan = partition(ops, nops, I.n, po);
      if (plan.empty()) {  // no gates: one empty stage still writes |0...0>
        PlanItem empty;
        empty.kind = 0;
        empty.op = -1;
        plan.push_back(empty);
      }
      for (const PlanItem &it : plan) {
        BStage st;
        memset(&st, 0, sizeof(st));
        std::vector<char> in(I.n, 0);
        for (int q : it.qubits) in[q] = 1;
        int cnt = (int)it.qubits.size();
        for (int q = 0; q < I.n && cnt < tile_q; q++)
          if (!in[q]) {
            in[q] = 1;
            cnt++;
          }
        std::vector<int> tq;
        for (int q = 0; q < I.n; q++)
          if (in[q]) tq.push_back(q);
        st.nt = (int)tq.size();
        for (int m = 0; m < st.nt; m++) st.q[m] = (signed char)tq[m];
        std::vector<int> stage_ops;
        for (int g : it.gates) stage_ops.push_back(b->op_off[i] + g);
        plan_groups(b, stage_ops, I.n, tq, st);
        b->stages.push_back(st);
      }
      I.nstages = (int)plan.size();
    }
    b->insts.push_back(I);
  }
  b->fold_off.push_back((int)b->fold_ops.size());
  b->planned_tile_q = tile_q;
  return QCS_CUDA_OK;
}

// Gate table from the ops and the current angles (group-local bits): each
// entry is the FP64 product of its folded ops, rounded once to FP32.
static void batch_fill_gates(qcs_cuda_batch *b) {
  const size_t ng = b->gate_tc.size();
  for (size_t gi = 0; gi < ng; gi++) {
    double acc[8] = {1, 0, 0, 0, 0, 0, 1, 0};
    int kind = 0;
    for (int f = b->fold_off[gi]; f < b->fold_off[gi + 1]; f++) {
      const qcs_cuda_op &o = b->ops[b->fold_ops[f]];
      kind = o.kind;
      double m[8], r[8];
      gate_matrix(o.kind, o.angle, m);
      for (int i = 0; i < 2; i++)  // acc := m * acc
        for (int j = 0; j < 2; j++) {
          double re = 0.0, im = 0.0;
          for (int l = 0; l < 2; l++) {
            const double *x = m + 2 * (2 * i + l), *y = acc + 2 * (2 * l + j);
            re += x[0] * y[0] - x[1] * y[1];
            im += x[0] * y[1] + x[1] * y[0];
          }
          r[2 * (2 * i + j)] = re;
          r[2 * (2 * i + j) + 1] = im;
        }
      memcpy(acc, r, sizeof(acc));
    }
    BGate g;
    memset(&g, 0, sizeof(g));
    for (int e = 0; e < 4; e++) g.m[e] = make_float2((float)acc[2 * e], (float)acc[2 * e + 1]);
    g.type = gate_is_controlled(kind) ? 1 : 0;
    // exact zeros decide the form: the exchange and diagonal paths give the
    // same numbers as the dense one (the skipped terms are products with 0)
    const bool off0 = acc[2] == 0.0 && acc[3] == 0.0 && acc[4] == 0.0 && acc[5] == 0.0;
    const bool swap = acc[0] == 0.0 && acc[1] == 0.0 && acc[6] == 0.0 && acc[7] == 0.0 &&
                      acc[2] == 1.0 && acc[3] == 0.0 && acc[4] == 1.0 && acc[5] == 0.0;
    g.form = swap ? 1 : (off0 ? 2 : 0);
    g.t = b->gate_tc[gi] & 0xFF;
    g.c = g.type ? (b->gate_tc[gi] >> 8) & 0xFF : 0;
    b->h_gates[gi] = g;
  }
}

static void batch_free_device(qcs_cuda_batch *b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  cudaFree(b->d_insts);
  cudaFree(b->d_stages);
  cudaFree(b->d_groups);
  cudaFree(b->d_gates);
  if (b->h_gates) cudaFreeHost(b->h_gates);
  cudaFree(b->d_items);
  b->d_insts = nullptr;
  b->d_stages = nullptr;
  b->d_groups = nullptr;
  b->d_gates = nullptr;
  b->h_gates = nullptr;
  b->d_items = nullptr;
}

static size_t smem_for(int tile_q) { return ((size_t)8 << tile_q) + 1025 * sizeof(double); }

template <int T>
static int set_smem_attr(int tile_q) {
  return check_cuda(cudaFuncSetAttribute(k_batch<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem_for(tile_q)),
                    "cudaFuncSetAttribute(batch)");
}

static int batch_upload(qcs_cuda_batch *b) {
  batch_free_device(b);
  int rc = check_cuda(cudaMalloc((void **)&b->d_insts, b->insts.size() * sizeof(BInst)), "cudaMalloc(batch)");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&b->d_stages, b->stages.size() * sizeof(BStage)), "cudaMalloc(batch)");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&b->d_groups, std::max<size_t>(1, b->groups.size()) * sizeof(BGroup)), "cudaMalloc(batch)");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&b->d_gates, std::max<size_t>(1, b->gate_tc.size()) * sizeof(BGate)), "cudaMalloc(batch)");
  if (!rc) rc = check_cuda(cudaMallocHost((void **)&b->h_gates, std::max<size_t>(1, b->gate_tc.size()) * sizeof(BGate)), "cudaMallocHost(batch)");
  if (rc) return rc;
  batch_fill_gates(b);
  // grid: CTAs per SM from the tune, but never more than fit the GPU at once
  // (members of a group wait for each other); every CTA owns a global slot
  int fit = 0;
  switch (b->tune.threads) {
    case 256: rc = set_smem_attr<256>(b->tune.tile_q); break;
    case 512: rc = set_smem_attr<512>(b->tune.tile_q); break;
    default: rc = set_smem_attr<1024>(b->tune.tile_q); break;
  }
  if (rc) return rc;
  switch (b->tune.threads) {
    case 256: rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k_batch<256>, 256, smem_for(b->tune.tile_q)), "occupancy"); break;
    case 512: rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k_batch<512>, 512, smem_for(b->tune.tile_q)), "occupancy"); break;
    default: rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k_batch<1024>, 1024, smem_for(b->tune.tile_q)), "occupancy"); break;
  }
  if (rc) return rc;
  if (fit < 1) return set_error(QCS_CUDA_EUNSUP, "batch kernel does not fit an SM");
  const int grid = b->dev.num_sms * std::min(b->tune.ctas_per_sm, fit);
  // group sizes: 2^(n - split_q) CTAs above split_q qubits (never below the
  // tile, at most half the grid)
  for (int i = 0; i < b->count; i++) {
    BInst &I = b->insts[i];
    int G = 1;
    if (I.n > b->tune.tile_q && I.n > b->tune.split_q) {
      const int e = I.n - b->tune.split_q;
      G = e >= 20 ? (1 << 20) : (1 << e);
      G = std::min(G, std::max(1, grid / 2));
    }
    I.group = G;
  }
  // instance order
  b->order.resize(b->count);
  std::iota(b->order.begin(), b->order.end(), 0);
  if (b->tune.order == 0) {
    std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) {
      const double cx = (double)(b->op_off[x + 1] - b->op_off[x]) * std::ldexp(1.0, b->nq[x]);
      const double cy = (double)(b->op_off[y + 1] - b->op_off[y]) * std::ldexp(1.0, b->nq[y]);
      return cx > cy;
    });
  }
  rc = check_cuda(cudaMemcpy(b->d_insts, b->insts.data(), b->insts.size() * sizeof(BInst), cudaMemcpyHostToDevice), "upload");
  if (!rc) rc = check_cuda(cudaMemcpy(b->d_stages, b->stages.data(), b->stages.size() * sizeof(BStage), cudaMemcpyHostToDevice), "upload");
  if (!rc && !b->groups.empty()) rc = check_cuda(cudaMemcpy(b->d_groups, b->groups.data(), b->groups.size() * sizeof(BGroup), cudaMemcpyHostToDevice), "upload");
  b->items.clear();
  for (int inst : b->order)
    for (int g = 0; g < b->insts[inst].group; g++) b->items.push_back(make_int2(inst, g));
  if (!rc) rc = check_cuda(cudaMalloc((void **)&b->d_items, b->items.size() * sizeof(int2)), "cudaMalloc(batch)");
  if (!rc) rc = check_cuda(cudaMemcpy(b->d_items, b->items.data(), b->items.size() * sizeof(int2), cudaMemcpyHostToDevice), "upload");
  if (rc) return rc;
  if (grid != b->grid) {
    cudaFree(b->d_slots);
    b->d_slots = nullptr;
    b->grid = grid;
    const size_t slot = b->max_n > 12 ? ((size_t)1 << b->max_n) : 4096;
    b->slot_amps = slot;
    rc = check_cuda(cudaMalloc((void **)&b->d_slots, slot * grid * sizeof(float2)), "cudaMalloc(batch slots)");
    if (rc) return rc;
  }
  return rc;
}

static int batch_enqueue(qcs_cuda_batch *b) {
  const size_t gbytes = std::max<size_t>(1, b->gate_tc.size()) * sizeof(BGate);
  int rc = check_cuda(cudaMemcpyAsync(b->d_gates, b->h_gates, gbytes, cudaMemcpyHostToDevice, b->stream),
                      "batch gate upload");
  if (!rc) rc = check_cuda(cudaMemsetAsync(b->d_queue, 0, sizeof(int), b->stream), "batch queue reset");
  if (!rc) rc = check_cuda(cudaMemsetAsync(b->d_stage_done, 0, b->count * sizeof(int), b->stream), "batch counters");
  if (!rc) rc = check_cuda(cudaMemsetAsync(b->d_lead, 0, b->count * sizeof(int), b->stream), "batch counters");
  if (!rc) rc = check_cuda(cudaMemsetAsync(b->d_err, 0, sizeof(int), b->stream), "batch error flag");
  if (rc) return rc;
  const size_t smem = smem_for(b->tune.tile_q);
  const int tq = b->tune.tile_q;
#define QCS_LAUNCH_BATCH(T)                                                                       \
  k_batch<T><<<b->grid, T, smem, b->stream>>>(                                                    \
      b->d_insts, b->d_stages, b->d_groups, b->d_gates, b->d_items, (int)b->items.size(),           \
      b->shots, b->seed, tq, b->d_slots, (i64)b->slot_amps, b->d_queue, b->d_stage_done, b->d_lead, \
      b->d_err, b->d_z, b->d_samples, b->wait_captured)
  switch (b->tune.threads) {
    case 256: QCS_LAUNCH_BATCH(256); break;
    case 512: QCS_LAUNCH_BATCH(512); break;
    default: QCS_LAUNCH_BATCH(1024); break;
  }
#undef QCS_LAUNCH_BATCH
  rc = check_launch("batch kernel");
  if (!rc) rc = check_cuda(cudaMemcpyAsync(b->h_z, b->d_z, b->count * sizeof(double), cudaMemcpyDeviceToHost, b->stream), "batch results");
  if (!rc && b->shots > 0)
    rc = check_cuda(cudaMemcpyAsync(b->h_samples, b->d_samples, (size_t)b->count * b->shots * sizeof(i64), cudaMemcpyDeviceToHost, b->stream), "batch samples");
  return rc;
}

static int batch_capture(qcs_cuda_batch *b) {
  b->wait_captured = wait_cycles();  // the graph's kernel node keeps this limit
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  cudaGraph_t g = nullptr;
  int rc = check_cuda(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
  if (rc) return rc;
  int rc2 = batch_enqueue(b);
  rc = check_cuda(cudaStreamEndCapture(b->stream, &g), "graph capture end");
  if (rc2) {
    if (g) cudaGraphDestroy(g);
    return rc2;
  }
  if (rc) return rc;
  rc = check_cuda(cudaGraphInstantiate(&b->graph, g, 0), "graph instantiate");
  cudaGraphDestroy(g);
  return rc;
}

static int batch_apply_tune(qcs_cuda_batch *b, const BatchTune &t) {
  b->tune = t;
  int rc = QCS_CUDA_OK;
  if (b->planned_tile_q != t.tile_q) rc = batch_plan(b, t.tile_q);
  if (!rc) rc = batch_upload(b);
  if (!rc) rc = batch_capture(b);
  return rc;
}

static int batch_launch_timed(qcs_cuda_batch *b, float *ms) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, b->stream);
  int rc = check_cuda(cudaGraphLaunch(b->graph, b->stream), "graph launch");
  cudaEventRecord(e1, b->stream);
  if (!rc) rc = check_cuda(cudaEventSynchronize(e1), "batch sync");
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ms) *ms = t;
  return rc;
}

// A timed replay whose device error flag is checked afterwards.
static int batch_launch_checked(qcs_cuda_batch *b, float *ms) {
  int rc = batch_launch_timed(b, ms);
  if (rc) return rc;
  int flag = 0;
  rc = check_cuda(cudaMemcpy(&flag, b->d_err, sizeof(int), cudaMemcpyDeviceToHost), "batch error flag");
  if (rc) return rc;
  if (flag)
    return set_error(QCS_CUDA_ETIMEOUT, "batch: a group of CTAs gave up waiting (site %d)", flag);
  return QCS_CUDA_OK;
}

static void batch_destroy(qcs_cuda_batch *b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_free_device(b);
  cudaFree(b->d_queue);
  cudaFree(b->d_stage_done);
  cudaFree(b->d_lead);
  cudaFree(b->d_z);
  cudaFree(b->d_samples);
  cudaFree(b->d_slots);
  cudaFree(b->d_err);
  if (b->h_z) cudaFreeHost(b->h_z);
  if (b->h_samples) cudaFreeHost(b->h_samples);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

}  // namespace qcs

using namespace qcs;

extern "C" {

int qcs_cuda_batch_create(int count, const int *num_qubits, const int *op_offsets,
                          const qcs_cuda_op *ops, int shots, unsigned long long seed,
                          qcs_cuda_batch **out) {
  if (!out) return set_error(QCS_CUDA_EINVAL, "null out");
  *out = nullptr;
  if (count < 1 || !num_qubits || !op_offsets || (op_offsets[count] > 0 && !ops) || shots < 0)
    return set_error(QCS_CUDA_EINVAL, "bad batch arguments");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(QCS_CUDA_ENODEV, "no CUDA device visible");
  }
  qcs_cuda_batch *b = new qcs_cuda_batch();
  b->count = count;
  b->shots = shots;
  b->seed = seed;
  b->max_n = 0;
  b->nq.assign(num_qubits, num_qubits + count);
  b->op_off.assign(op_offsets, op_offsets + count + 1);
  b->ops.assign(ops, ops + op_offsets[count]);
  for (int i = 0; i < count; i++) {
    const int n = b->nq[i];
    if (n < 1 || n > 26 || b->op_off[i + 1] < b->op_off[i]) {
      delete b;
      return set_error(QCS_CUDA_EINVAL, "instance %d: %d qubits (1..26) or bad op range", i, n);
    }
    b->max_n = std::max(b->max_n, n);
    for (int j = b->op_off[i]; j < b->op_off[i + 1]; j++) {
      const qcs_cuda_op &o = b->ops[j];
      const bool ctl = gate_is_controlled(o.kind);
      if (!gate_kind_valid(o.kind) || o.target < 0 || o.target >= n ||
          (ctl && (o.control < 0 || o.control >= n || o.control == o.target))) {
        delete b;
        return set_error(QCS_CUDA_EINVAL, "instance %d op %d: not a valid gate", i, j);
      }
    }
  }
  int dev = 0;
  int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (!rc) rc = device_info(dev, &b->dev);
  if (!rc) rc = check_cuda(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&b->d_queue, sizeof(int)), "cudaMalloc(batch)");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&b->d_stage_done, count * sizeof(int)), "cudaMalloc(batch)");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&b->d_lead, count * sizeof(int)), "cudaMalloc(batch)");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&b->d_err, sizeof(int)), "cudaMalloc(batch)");
  if (!rc) rc = check_cuda(cudaMalloc((void **)&b->d_z, count * sizeof(double)), "cudaMalloc(batch)");
  if (!rc) rc = check_cuda(cudaMallocHost((void **)&b->h_z, count * sizeof(double)), "cudaMallocHost(batch)");
  if (!rc && shots > 0) {
    rc = check_cuda(cudaMalloc((void **)&b->d_samples, (size_t)count * shots * sizeof(i64)), "cudaMalloc(batch)");
    if (!rc) rc = check_cuda(cudaMallocHost((void **)&b->h_samples, (size_t)count * shots * sizeof(i64)), "cudaMallocHost(batch)");
  }
  BatchTune t;
  t.threads = 512;
  t.tile_q = 13;
  t.ctas_per_sm = 2;
  t.order = 0;
  t.split_q = 19;
  if (!rc) rc = batch_apply_tune(b, t);
  if (rc) {
    batch_destroy(b);
    return rc;
  }
  *out = b;
  return QCS_CUDA_OK;
}

int qcs_cuda_batch_destroy(qcs_cuda_batch *b) {
  if (!b) return set_error(QCS_CUDA_EINVAL, "null batch");
  batch_destroy(b);
  return QCS_CUDA_OK;
}

int qcs_cuda_batch_set_angles(qcs_cuda_batch *b, const double *angles) {
  if (!b || !angles) return set_error(QCS_CUDA_EINVAL, "null argument");
  int rc = check_cuda(cudaStreamSynchronize(b->stream), "batch sync");
  if (rc) return rc;
  for (size_t j = 0; j < b->ops.size(); j++) b->ops[j].angle = angles[j];
  batch_fill_gates(b);  // the captured graph uploads this pinned table on its next replay
  return QCS_CUDA_OK;
}

int qcs_cuda_batch_traffic(qcs_cuda_batch *b, double *hbm_bytes) {
  if (!b || !hbm_bytes) return set_error(QCS_CUDA_EINVAL, "null batch argument");
  double bytes = 8.0 * b->count * (1.0 + b->shots);
  for (const BInst &I : b->insts)
    if (I.n > b->planned_tile_q)  // 2 nstages - 1 stage passes, 1 read-out pass
      bytes += ldexp(8.0, I.n) * (2.0 * I.nstages);
  *hbm_bytes = bytes;
  return QCS_CUDA_OK;
}

int qcs_cuda_batch_run(qcs_cuda_batch *b, double *expect_z0, long long *samples, double *ms) {
  if (!b) return set_error(QCS_CUDA_EINVAL, "null batch");
  float t = 0.f;
  int rc = QCS_CUDA_OK;
  if (b->wait_captured != wait_cycles()) rc = batch_capture(b);  // the wait limit changed
  if (!rc) rc = batch_launch_checked(b, &t);
  if (rc) return rc;
  b->last_ms = t;
  if (ms) *ms = t;
  if (expect_z0) memcpy(expect_z0, b->h_z, b->count * sizeof(double));
  if (samples && b->shots > 0)
    memcpy(samples, b->h_samples, (size_t)b->count * b->shots * sizeof(i64));
  return QCS_CUDA_OK;
}

int qcs_cuda_batch_autotune(qcs_cuda_batch *b, int repeats, int *chosen) {
  if (!b) return set_error(QCS_CUDA_EINVAL, "null batch");
  if (repeats < 1) repeats = 1;
  auto time_tune = [&](const BatchTune &t, float *out) {
    int rc = batch_apply_tune(b, t);
    float ms = 0.f, sum = 0.f;
    if (!rc) rc = batch_launch_checked(b, &ms);  // warm-up
    for (int r = 0; !rc && r < repeats; r++) {
      rc = batch_launch_checked(b, &ms);
      sum += ms;
    }
    *out = sum / repeats;
    return rc;
  };
  const int threads[] = {256, 512, 1024};
  const int tiles[] = {12, 13, 14};
  const int ctas[] = {1, 2, 4};
  BatchTune best = b->tune;
  float best_ms = 1e30f;
  for (int th : threads)
    for (int tq : tiles)
      for (int cp : ctas)
        for (int ord = 0; ord < 2; ord++) {
          // the CTAs of an SM must fit its shared memory, and four only
          // with 256 threads (64 registers a thread)
          if (smem_for(tq) * cp > 220 * 1024 || th * cp > 1024) continue;
          BatchTune t = b->tune;
          t.threads = th;
          t.tile_q = tq;
          t.ctas_per_sm = cp;
          t.order = ord;
          float ms = 0.f;
          int rc = time_tune(t, &ms);
          if (rc) return rc;
          if (ms < best_ms) {
            best_ms = ms;
            best = t;
          }
        }
  // then how far large instances spread over CTAs (27: never)
  const int splits[] = {17, 18, 19, 20, 27};
  const BatchTune base = best;
  for (int sq : splits) {
    if (sq == base.split_q) continue;
    BatchTune t = base;
    t.split_q = sq;
    float ms = 0.f;
    int rc = time_tune(t, &ms);
    if (rc) return rc;
    if (ms < best_ms) {
      best_ms = ms;
      best = t;
    }
  }
  int rc = batch_apply_tune(b, best);
  if (rc) return rc;
  if (chosen) {
    chosen[0] = best.threads;
    chosen[1] = best.tile_q;
    chosen[2] = best.ctas_per_sm;
    chosen[3] = best.order;
  }
  return QCS_CUDA_OK;
}

int qcs_cuda_batch_split(qcs_cuda_batch *b, int split_q) {
  if (!b) return set_error(QCS_CUDA_EINVAL, "null batch");
  if (split_q < 1 || split_q > 27) return set_error(QCS_CUDA_EINVAL, "split_q %d outside 1..27", split_q);
  BatchTune t = b->tune;
  t.split_q = split_q;
  return batch_apply_tune(b, t);
}

int qcs_cuda_batch_schedule(qcs_cuda_batch *b, int *schedule) {
  if (!b || !schedule) return set_error(QCS_CUDA_EINVAL, "null argument");
  schedule[0] = b->tune.threads;
  schedule[1] = b->tune.tile_q;
  schedule[2] = std::min(b->tune.ctas_per_sm, b->grid / std::max(1, b->dev.num_sms));
  schedule[3] = b->tune.order;
  schedule[4] = b->tune.split_q;
  return QCS_CUDA_OK;
}

int qcs_cuda_batch_config(qcs_cuda_batch *b, int threads, int tile_q, int ctas_per_sm,
                          int order) {
  if (!b) return set_error(QCS_CUDA_EINVAL, "null batch");
  if ((threads != 256 && threads != 512 && threads != 1024) || tile_q < 10 || tile_q > 14 ||
      ctas_per_sm < 1 || ctas_per_sm > 4 || ctas_per_sm == 3 || order < 0 || order > 1 ||
      threads * ctas_per_sm > 1024)
    return set_error(QCS_CUDA_EINVAL, "bad batch schedule");
  if (smem_for(tile_q) * ctas_per_sm > 220 * 1024)
    return set_error(QCS_CUDA_EINVAL, "%d CTAs of tile 2^%d do not fit one SM", ctas_per_sm,
                     tile_q);
  BatchTune t = b->tune;
  t.threads = threads;
  t.tile_q = tile_q;
  t.ctas_per_sm = ctas_per_sm;
  t.order = order;
  return batch_apply_tune(b, t);
}

}  // extern "C"
