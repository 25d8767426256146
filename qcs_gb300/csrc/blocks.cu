// blocks.cu -- dense k-qubit block application (SIMT engine) and qcs_cuda_run.
//
// A block on qubit set Q (k qubits) maps every "column" of the state (one
// setting of the other n-k qubits) through the 2^k x 2^k matrix U.  A CTA
// works on tiles of 2^k x 2^c amplitudes: T = Q plus the c lowest qubits
// outside Q, so every tile is a union of contiguous runs of at least
// 2^min(7, n-k) amplitudes and its gather/scatter is fully coalesced
// whatever Q is.  The tile goes through shared memory as S[a][col] (row
// stride C+1 to spread banks); each thread owns one column and forms
// out[a'] = sum_a U[a'][a] * S[a][col] with U read from kernel parameters
// (a uniform, broadcast operand).
//
// HBM traffic per block: 2 * N * s bytes (one read, one write), however many
// gates the block holds.  FP32 work: 8 * 2^k flops per amplitude, so this
// engine stays bandwidth-bound up to k = 4 on GB300's CUDA cores; larger
// blocks belong on the tensor cores (blocks_tc.cu).
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "costmodel.h"
#include "fusion.h"

namespace qcs {

int apply_1q(qcs_cuda_state *s, const double m[8], int t);
int apply_ctrl(qcs_cuda_state *s, const double m[8], int c, int t);
int phase_flip(qcs_cuda_state *s, i64 index);
int diffusion(qcs_cuda_state *s);
int check_qubit(const qcs_cuda_state *s, int q, const char *what);
int apply_block_tc(qcs_cuda_state *s, int k, const int *qubits, const double *u,
                   bool known_unitary, const BlockFuse *fuse);
bool tc_supported(const qcs_cuda_state *s, int k);

constexpr int kBlockThreads = 128;  // = max columns per tile
constexpr int kMaxColBits = 7;
constexpr int kSimtMaxK = 5;

// Tile geometry, computed on the host.  Local index l of a tile has nT bits;
// bit m stands for qubit tq[m] (ascending).  l = lo | hi << 6 and every
// per-element quantity is a sum of a lo-table and a hi-table entry.
struct TileGeom {
  int n, k, c, nT;
  i64 n_tiles;
  int nfree;
  signed char freeq[40];  // qubits outside T, ascending (tile id bits)
  i64 goff_lo[64];
  i64 goff_hi[64];
  unsigned char a_lo[64], a_hi[64];
  unsigned char col_lo[64], col_hi[64];
};

template <typename C, int K> struct BlockU { C u[K * K]; };

template <typename C, int K>
__global__ void __launch_bounds__(kBlockThreads)
    k_block_simt(C *v, const __grid_constant__ TileGeom g, const __grid_constant__ BlockU<C, K> U) {
  const int Cn = 1 << g.c;        // columns per tile
  const int stride = Cn + 1;      // smem row stride (elements)
  const int L = 1 << g.nT;        // elements per tile
  extern __shared__ unsigned char smem_raw[];
  C *S = reinterpret_cast<C *>(smem_raw);
  // The lo/hi tables are indexed per lane; kernel parameters live in the
  // constant bank, which serialises divergent reads, so they go to shared
  // memory first.
  __shared__ i64 goff[128];
  __shared__ unsigned char acol[256];
  const int tid = threadIdx.x;
  for (int e = tid; e < 64; e += kBlockThreads) {
    goff[e] = g.goff_lo[e];
    goff[64 + e] = g.goff_hi[e];
    acol[e] = g.a_lo[e];
    acol[64 + e] = g.a_hi[e];
    acol[128 + e] = g.col_lo[e];
    acol[192 + e] = g.col_hi[e];
  }
  __syncthreads();
  for (i64 tile = blockIdx.x; tile < g.n_tiles; tile += gridDim.x) {
    i64 base = 0;
    for (int j = 0; j < g.nfree; j++) base |= ((tile >> j) & 1LL) << g.freeq[j];
    // gather (global order, coalesced)
    for (int l = tid; l < L; l += kBlockThreads) {
      const int lo = l & 63, hi = l >> 6;
      const i64 off = goff[lo] + goff[64 + hi];
      const int a = acol[lo] + acol[64 + hi];
      const int col = acol[128 + lo] + acol[192 + hi];
      S[a * stride + col] = v[base + off];
    }
    __syncthreads();
    if (tid < Cn) {
      C in[K];
#pragma unroll
      for (int a = 0; a < K; a++) in[a] = S[a * stride + tid];
#pragma unroll
      for (int r = 0; r < K; r++) {
        C acc = cmul(U.u[r * K], in[0]);
#pragma unroll
        for (int a = 1; a < K; a++) acc = cadd(acc, cmul(U.u[r * K + a], in[a]));
        S[r * stride + tid] = acc;
      }
    }
    __syncthreads();
    for (int l = tid; l < L; l += kBlockThreads) {
      const int lo = l & 63, hi = l >> 6;
      const i64 off = goff[lo] + goff[64 + hi];
      const int a = acol[lo] + acol[64 + hi];
      const int col = acol[128 + lo] + acol[192 + hi];
      v[base + off] = S[a * stride + col];
    }
    __syncthreads();
  }
}

// qubits[] in caller order (bit j of the block index is qubits[j]).
static void make_geom(const qcs_cuda_state *s, int k, const int *qubits, TileGeom &g) {
  memset(&g, 0, sizeof(g));
  g.n = s->n;
  g.k = k;
  int c = s->n - k < kMaxColBits ? s->n - k : kMaxColBits;
  g.c = c;
  g.nT = k + c;
  std::vector<int> role(s->n, -1);  // -1 free, >=0 block bit, -2 column
  for (int j = 0; j < k; j++) role[qubits[j]] = j;
  int taken = 0;
  for (int q = 0; q < s->n && taken < c; q++)
    if (role[q] == -1) { role[q] = -2; taken++; }
  std::vector<int> tq;
  for (int q = 0; q < s->n; q++) {
    if (role[q] == -1) g.freeq[g.nfree++] = (signed char)q;
    else tq.push_back(q);
  }
  g.n_tiles = 1LL << g.nfree;
  // per T position: global offset bit, block bit, column bit
  std::vector<i64> gbit(g.nT);
  std::vector<int> abit(g.nT, 0), cbit(g.nT, 0);
  int colj = 0;
  for (int m = 0; m < g.nT; m++) {
    int q = tq[m];
    gbit[m] = 1LL << q;
    if (role[q] >= 0) abit[m] = 1 << role[q];
    else cbit[m] = 1 << (colj++);
  }
  for (int e = 0; e < 64; e++) {
    i64 go = 0, gh = 0;
    int al = 0, ah = 0, cl = 0, ch = 0;
    for (int m = 0; m < g.nT; m++) {
      if (m < 6) {
        if ((e >> m) & 1) { go += gbit[m]; al += abit[m]; cl += cbit[m]; }
      } else {
        if ((e >> (m - 6)) & 1) { gh += gbit[m]; ah += abit[m]; ch += cbit[m]; }
      }
    }
    g.goff_lo[e] = go;
    g.goff_hi[e] = gh;
    g.a_lo[e] = (unsigned char)al;
    g.a_hi[e] = (unsigned char)ah;
    g.col_lo[e] = (unsigned char)cl;
    g.col_hi[e] = (unsigned char)ch;
  }
}

template <typename C, int K>
static int launch_block(qcs_cuda_state *s, const TileGeom &g, const double *u) {
  BlockU<C, K> U;
  for (int i = 0; i < K * K; i++) U.u[i] = make_c<C>(u[2 * i], u[2 * i + 1]);
  size_t smem = (size_t)K * ((1 << g.c) + 1) * sizeof(C);
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(k_block_simt<C, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         96 * 1024);
    configured = true;
  }
  i64 want = g.n_tiles;
  i64 cap = (i64)s->dev.num_sms * 8;
  int grid = (int)(want < cap ? want : cap);
  s->h2d_bytes += (long long)sizeof(U);  // the block matrix rides in the parameters
  prof_begin(s);
  k_block_simt<C, K><<<grid, kBlockThreads, smem, s->stream>>>((C *)s->vec, g, U);
  return launched(s, KC_BLOCK_SIMT, 2.0 * s->size * sizeof(C), "apply_block (SIMT)");
}

template <typename C>
static int apply_block_simt_t(qcs_cuda_state *s, int k, const int *qubits, const double *u) {
  TileGeom g;
  make_geom(s, k, qubits, g);
  switch (k) {
    case 1: return launch_block<C, 2>(s, g, u);
    case 2: return launch_block<C, 4>(s, g, u);
    case 3: return launch_block<C, 8>(s, g, u);
    case 4: return launch_block<C, 16>(s, g, u);
    case 5: return launch_block<C, 32>(s, g, u);
    default: return set_error(QCS_CUDA_EUNSUP, "SIMT block engine supports k <= %d", kSimtMaxK);
  }
}

// A k-qubit block as a 5-qubit one: the lowest qubits it does not touch are
// appended as block bits k..4, where the matrix acts as the identity.
static void widen_to_5(const qcs_cuda_state *s, int k, const int *qubits, const double *u,
                       int *q5, std::vector<double> &u5) {
  const int K = 1 << k;
  int kk = k;
  for (int j = 0; j < k; j++) q5[j] = qubits[j];
  for (int q = 0; q < s->n && kk < 5; q++) {
    bool used = false;
    for (int j = 0; j < k; j++) used = used || qubits[j] == q;
    if (!used) q5[kk++] = q;
  }
  u5.assign(2 * 32 * 32, 0.0);
  for (int a = 0; a < 32; a++)
    for (int b = 0; b < 32; b++)
      if ((a >> k) == (b >> k)) {
        const size_t src = 2 * ((size_t)(a & (K - 1)) * K + (b & (K - 1)));
        u5[2 * (a * 32 + b)] = u[src];
        u5[2 * (a * 32 + b) + 1] = u[src + 1];
      }
}

// Engine choice: the tensor cores take the blocks they support (k = 5, 6 on
// complex64 states) unless SIMT is asked for.  AUTO and TENSOR also send
// 2..4-qubit blocks to the tensor cores, widened to 5 qubits: at 30 qubits
// the CUDA-core kernel takes 6.3 / 5.8 / 6.9 ms for k = 2 / 3 / 4 against
// 3.0 ms for a 5-qubit tensor-core block.  `strict` (explicit
// single-block calls) refuses a TENSOR request the tensor engine cannot
// serve instead of running it on the CUDA cores.
// The engine apply_block picks for a block of k qubits: 1 when the tensor
// cores take it (widened to 5 qubits for k = 2..4), 0 for the CUDA cores.
static bool block_on_tensor_cores(const qcs_cuda_state *s, int k, int engine) {
  if (engine == QCS_FUSE_SIMT) return false;
  if (tc_supported(s, k) && (engine == QCS_FUSE_TENSOR || k > 4)) return true;
  return k >= 2 && k <= 4 && tc_supported(s, 5);
}

int apply_block(qcs_cuda_state *s, int k, const int *qubits, const double *u, int engine,
                bool strict, const BlockFuse *fuse) {
  const bool tc_ok = tc_supported(s, k);
  const bool widen = engine != QCS_FUSE_SIMT && k >= 2 && k <= 4 && tc_supported(s, 5);
  if (engine == QCS_FUSE_TENSOR && strict && !tc_ok && !widen)
    return set_error(QCS_CUDA_EUNSUP, "tensor-core block engine: unsupported k=%d / precision", k);
  // blocks from the planner (strict == false) are products of unitary gates;
  // the tensor-core path keeps or sets the cached sum itself
  if (tc_ok && (engine == QCS_FUSE_TENSOR || (engine == QCS_FUSE_AUTO && k > 4)))
    return apply_block_tc(s, k, qubits, u, !strict, fuse);
  if (widen) {
    int q5[5];
    std::vector<double> u5;
    widen_to_5(s, k, qubits, u, q5, u5);
    return apply_block_tc(s, 5, q5, u5.data(), !strict, fuse);
  }
  if (fuse && (fuse->diffuse_in || fuse->sum_out))
    return set_error(QCS_CUDA_EUNSUP, "fused diffusion needs the tensor-core engine");
  invalidate_sum(s);
  if (s->prec == QCS_CUDA_C128) return apply_block_simt_t<double2>(s, k, qubits, u);
  return apply_block_simt_t<float2>(s, k, qubits, u);
}

static int validate_ops(const qcs_cuda_state *s, const qcs_cuda_op *ops, int count) {
  for (int i = 0; i < count; i++) {
    const qcs_cuda_op &o = ops[i];
    if (o.kind == QCS_OP_DIFFUSION) continue;
    if (o.kind == QCS_OP_PHASE_FLIP) {
      if (o.index < 0 || o.index >= s->size)
        return set_error(QCS_CUDA_EINVAL, "op %d: phase flip index %lld out of range", i, o.index);
      continue;
    }
    if (!gate_kind_valid(o.kind)) return set_error(QCS_CUDA_EINVAL, "op %d: unknown kind %d", i, o.kind);
    if (o.target < 0 || o.target >= s->n)
      return set_error(QCS_CUDA_EINVAL, "op %d: target %d out of range", i, o.target);
    if (gate_is_controlled(o.kind) &&
        (o.control < 0 || o.control >= s->n || o.control == o.target))
      return set_error(QCS_CUDA_EINVAL, "op %d: bad control %d", i, o.control);
  }
  return QCS_CUDA_OK;
}

static int apply_op(qcs_cuda_state *s, const qcs_cuda_op &o) {
  if (o.kind == QCS_OP_PHASE_FLIP) return phase_flip(s, o.index);
  if (o.kind == QCS_OP_DIFFUSION) return diffusion(s);
  double m[8];
  gate_matrix(o.kind, o.angle, m);
  if (gate_is_controlled(o.kind)) return apply_ctrl(s, m, o.control, o.target);
  return apply_1q(s, m, o.target);
}

static int apply_block_item(qcs_cuda_state *s, const PlanItem &it, int engine,
                            const std::vector<cd> &u, const BlockFuse *fuse);

static int apply_item(qcs_cuda_state *s, const qcs_cuda_op *ops, const PlanItem &it, int engine,
                      std::vector<cd> &u) {
  if (it.kind == 1) return apply_op(s, ops[it.op]);
  if (it.gates.size() == 1) return apply_op(s, ops[it.gates[0]]);
  block_matrix(ops, it, u);
  return apply_block_item(s, it, engine, u, nullptr);
}

// The widest block the tensor cores take on this state (0: none).
static int tc_max(const qcs_cuda_state *s, int engine) {
  if (engine == QCS_FUSE_SIMT) return 0;
  for (int k = 7; k >= 5; k--)
    if (tc_supported(s, k)) return k;
  return 0;
}

static int fusion_cap(const qcs_cuda_state *s, int k, int engine) {
  int kcap = kSimtMaxK;
  if (engine != QCS_FUSE_SIMT && tc_supported(s, 7)) kcap = 7;
  else if (engine != QCS_FUSE_SIMT && tc_supported(s, 6)) kcap = 6;
  if (k > kcap) k = kcap;
  if (k > s->n) k = s->n;
  return k;
}

// The plan of the last fused run, with its block matrices, kept per state:
// circuits are usually run many times over (shots in separate runs, sweeps
// of the same circuit, benchmarks), and planning -- above all the learned
// partitioner, which scores many candidate plans with the MLP -- costs host
// time before the first kernel can start.  The key is the exact op bytes
// plus everything the plan depends on.
struct PlanCache {
  std::vector<qcs_cuda_op> ops;
  int n = -1, k = 0, engine = 0, partitioner = 0;
  const qcs_cuda_costmodel *cm = nullptr;
  unsigned long long cm_gen = 0;
  std::vector<PlanItem> plan;
  std::vector<std::vector<cd>> mats;  // per item: the block matrix, or empty
  std::vector<TcResident *> res;      // per item: a resident tensor-core block, or null
  void clear_blocks() {
    for (TcResident *r : res) tc_free_resident(r);
    res.clear();
    mats.clear();
  }
  ~PlanCache() { clear_blocks(); }
};

// Block matrices (host) and resident tensor-core images (device) are kept
// while their total stays under this many bytes.
constexpr size_t kPlanCacheMatBytes = 64u << 20;

// A plain run (one kernel per op) kept as a CUDA graph.  Small states run
// circuits of short kernels whose launches, one per gate, take as long as
// the kernels (a 20-qubit complex128 QFT phase: ~3 us of work).  The same op
// list, byte for byte, is captured into a graph on its second run in a row
// and replayed from then on: one graph launch per circuit.  The cached
// amplitude sum is reset before the capture and before every replay, so the
// reductions the graph recorded are the ones a fresh run would make.
// REFERENCE semantics sweep out of place and swap the state's two buffers
// on the host after each sweep: a recording holds the buffers it started
// from, so a list with an odd number of swaps needs one recording per
// starting buffer (two at most), and each replay swaps the host's pointers
// as the recorded run did.
struct PlainGraph {
  std::vector<qcs_cuda_op> ops;
  int seen = 0;  // runs of this op list in a row
  struct Rec {
    void *start = nullptr;          // the buffer holding the state at the start
    cudaGraphExec_t exec = nullptr;
    bool swapped = false;           // the run ends in the other buffer
    long long launches = 0;         // kernels in the graph
    int sum_valid_end = 0;          // the cached-sum flag after a run
  } rec[2];
  ~PlainGraph() {
    for (Rec &r : rec)
      if (r.exec) cudaGraphExecDestroy(r.exec);
  }
};

constexpr int kPlainGraphMaxQubits = 26;  // above, a gate's kernel outlasts its launch
constexpr int kPlainGraphMinOps = 16;

void plan_cache_free(qcs_cuda_state *s) {
  delete s->plans;
  s->plans = nullptr;
  delete s->plain_graph;
  s->plain_graph = nullptr;
}

static bool plan_cache_hit(const PlanCache *c, const qcs_cuda_op *ops, int count, int n, int k,
                           int engine, int partitioner, const qcs_cuda_costmodel *cm,
                           unsigned long long gen) {
  return c && c->n == n && c->k == k && c->engine == engine && c->partitioner == partitioner &&
         c->cm == cm && c->cm_gen == gen && (int)c->ops.size() == count &&
         (count == 0 || memcmp(c->ops.data(), ops, (size_t)count * sizeof(qcs_cuda_op)) == 0);
}

static bool item_is_block(const PlanItem &it) { return it.kind == 0 && it.gates.size() > 1; }

static int apply_block_item(qcs_cuda_state *s, const PlanItem &it, int engine,
                            const std::vector<cd> &u, const BlockFuse *fuse) {
  const int kb = (int)it.qubits.size();
  if (kb == 1) {
    double m[8] = {u[0].real(), u[0].imag(), u[1].real(), u[1].imag(),
                   u[2].real(), u[2].imag(), u[3].real(), u[3].imag()};
    return apply_1q(s, m, it.qubits[0]);
  }
  return apply_block(s, kb, it.qubits.data(), reinterpret_cast<const double *>(u.data()), engine,
                     false, fuse);
}

static bool item_is_op(const qcs_cuda_op *ops, const PlanItem &it, int kind) {
  return it.kind == 1 && ops[it.op].kind == kind;
}

// Executes a plan.  Two fusions across Grover-style barriers, for blocks the
// tensor cores run: a diffusion directly followed by such a block runs
// inside it (the block acts on 2m - psi), and such a block followed by phase
// flips and then a diffusion leaves the amplitude sum that diffusion needs
// (the flips correct it), so neither costs a pass over the state.  Block
// matrices come from `use_mats` where present, else are formed here and,
// within the budget, kept in `store_mats`.
static int execute_plan(qcs_cuda_state *s, const qcs_cuda_op *ops,
                        const std::vector<PlanItem> &plan, int engine, PlanCache *use,
                        PlanCache *store) {
  auto on_tc = [&](const PlanItem &it) {
    return item_is_block(it) && it.qubits.size() >= 2 &&
           block_on_tensor_cores(s, (int)it.qubits.size(), engine);
  };
  std::vector<cd> u;
  size_t kept = 0;
  bool diffusion_pending = false;
  for (size_t i = 0; i < plan.size(); i++) {
    const PlanItem &it = plan[i];
    int rc;
    if (item_is_op(ops, it, QCS_OP_DIFFUSION) && i + 1 < plan.size() && on_tc(plan[i + 1])) {
      diffusion_pending = true;  // applied by the next block
      continue;
    }
    if (!item_is_block(it)) {
      rc = apply_item(s, ops, it, engine, u);
    } else {
      BlockFuse f;
      f.diffuse_in = diffusion_pending;
      f.sum_out = false;
      if (on_tc(it)) {
        size_t j = i + 1;
        while (j < plan.size() && item_is_op(ops, plan[j], QCS_OP_PHASE_FLIP)) j++;
        f.sum_out = j < plan.size() && item_is_op(ops, plan[j], QCS_OP_DIFFUSION);
      }
      diffusion_pending = false;
      const BlockFuse *fp = (f.diffuse_in || f.sum_out) ? &f : nullptr;
      if (use && use->res[i]) {
        rc = tc_launch_resident(s, use->res[i], fp);
      } else if (use && !use->mats[i].empty()) {
        rc = apply_block_item(s, it, engine, use->mats[i], fp);
      } else {
        block_matrix(ops, it, u);
        const size_t bytes = u.size() * sizeof(cd);
        if (store && kept + bytes <= kPlanCacheMatBytes && on_tc(it)) {
          // keep it on the device, prepared (widened to 5 qubits for k < 5)
          const int kb = (int)it.qubits.size();
          TcResident *r = nullptr;
          if (tc_supported(s, kb) && (engine == QCS_FUSE_TENSOR || kb > 4)) {
            rc = tc_make_resident(s, kb, it.qubits.data(),
                                  reinterpret_cast<const double *>(u.data()), true, &r);
          } else {
            int q5[5];
            std::vector<double> u5;
            widen_to_5(s, kb, it.qubits.data(), reinterpret_cast<const double *>(u.data()), q5,
                       u5);
            rc = tc_make_resident(s, 5, q5, u5.data(), true, &r);
          }
          if (!rc) {
            store->res[i] = r;
            kept += tc_resident_bytes(r);
            rc = tc_launch_resident(s, r, fp);
          }
        } else {
          rc = apply_block_item(s, it, engine, u, fp);
          if (store && kept + bytes <= kPlanCacheMatBytes) {
            store->mats[i] = u;
            kept += bytes;
          }
        }
      }
    }
    if (rc) return rc;
  }
  return QCS_CUDA_OK;
}

static int run_plain(qcs_cuda_state *s, const qcs_cuda_op *ops, int count) {
  for (int i = 0; i < count; i++) {
    int rc = apply_op(s, ops[i]);
    if (rc) return rc;
  }
  return QCS_CUDA_OK;
}

static int replay_plain(qcs_cuda_state *s, const PlainGraph::Rec &r) {
  invalidate_sum(s);
  int rc = check_cuda(cudaGraphLaunch(r.exec, s->stream), "plain graph launch");
  if (rc) return rc;
  if (r.swapped) {
    void *t = s->vec;
    s->vec = s->scratch;
    s->scratch = t;
  }
  s->launches += r.launches;
  s->sum_valid = r.sum_valid_end;
  return QCS_CUDA_OK;
}

// The plain run through the kept graph (see PlainGraph).
static int run_plain_kept(qcs_cuda_state *s, const qcs_cuda_op *ops, int count) {
  PlainGraph *g = s->plain_graph;
  const bool same = g && (int)g->ops.size() == count &&
                    memcmp(g->ops.data(), ops, (size_t)count * sizeof(qcs_cuda_op)) == 0;
  if (!same) {
    delete g;
    g = new PlainGraph();
    g->ops.assign(ops, ops + count);
    s->plain_graph = g;
  }
  g->seen++;
  for (const PlainGraph::Rec &r : g->rec)
    if (r.exec && r.start == s->vec) return replay_plain(s, r);
  PlainGraph::Rec *slot = !g->rec[0].exec ? &g->rec[0] : !g->rec[1].exec ? &g->rec[1] : nullptr;
  if (g->seen < 2 || !slot) return run_plain(s, ops, count);
  // second run in a row (from this buffer): record it, then launch the
  // recording; the host-side swaps made while recording leave the pointers
  // as the recorded run leaves them
  invalidate_sum(s);
  const long long l0 = s->launches;
  void *start = s->vec, *start_scratch = s->scratch;
  int rc = check_cuda(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal),
                      "plain graph capture");
  if (rc) return rc;
  rc = run_plain(s, ops, count);
  cudaGraph_t graph = nullptr;
  const int rc_end = check_cuda(cudaStreamEndCapture(s->stream, &graph), "plain graph capture end");
  if (!rc) rc = rc_end;
  cudaGraphExec_t exec = nullptr;
  if (!rc) rc = check_cuda(cudaGraphInstantiate(&exec, graph, 0), "plain graph instantiate");
  if (graph) cudaGraphDestroy(graph);
  const long long n_launch = s->launches - l0;
  const bool swapped = s->vec != start;
  const int sum_end = s->sum_valid;
  s->launches = l0;  // nothing ran while recording
  s->vec = start;
  s->scratch = start_scratch;
  if (rc) return rc;
  slot->start = start;
  slot->exec = exec;
  slot->swapped = swapped;
  slot->launches = n_launch;
  slot->sum_valid_end = sum_end;
  return replay_plain(s, *slot);
}

int run_ops(qcs_cuda_state *s, const qcs_cuda_op *ops, int count, const qcs_cuda_run_options *opt) {
  int rc = validate_ops(s, ops, count);
  if (rc) return rc;
  int k = opt ? opt->fusion_k : 0;
  if (k <= 1 || s->sem == QCS_CUDA_REFERENCE) {
    const bool keep = !(opt && (opt->flags & QCS_RUN_NO_PLAN_CACHE)) && !s->prof &&
                      s->n <= kPlainGraphMaxQubits && count >= kPlainGraphMinOps;
    return keep ? run_plain_kept(s, ops, count) : run_plain(s, ops, count);
  }
  const int engine = opt->fusion_engine;
  k = fusion_cap(s, k, engine);
  const bool learned = opt->partitioner == QCS_PARTITION_LEARNED && costmodel_ready(s->cm);
  const int part = learned ? QCS_PARTITION_LEARNED : QCS_PARTITION_GREEDY;
  const qcs_cuda_costmodel *cm = learned ? s->cm : nullptr;
  const unsigned long long gen = learned ? costmodel_generation(s->cm) : 0;
  const bool use_cache = !(opt->flags & QCS_RUN_NO_PLAN_CACHE);
  if (use_cache && plan_cache_hit(s->plans, ops, count, s->n, k, engine, part, cm, gen))
    return execute_plan(s, ops, s->plans->plan, engine, s->plans, nullptr);
  std::vector<PlanItem> plan;
  if (learned) {
    plan = partition_learned(ops, count, s->n, k, s->cm, tc_max(s, engine), nullptr, nullptr,
                             nullptr);
  } else {
    PartitionOptions po;
    po.kmax = k;
    po.cost = nullptr;
    po.cost_ctx = nullptr;
    plan = partition(ops, count, s->n, po);
  }
  PlanCache *c = nullptr;
  if (use_cache) {
    if (!s->plans) s->plans = new PlanCache();
    c = s->plans;
    c->n = -1;  // invalid until the run completes
    c->ops.assign(ops, ops + count);
    c->clear_blocks();
    c->mats.assign(plan.size(), std::vector<cd>());
    c->res.assign(plan.size(), nullptr);
  }
  rc = execute_plan(s, ops, plan, engine, nullptr, c);
  if (rc) return rc;
  if (c) {
    c->plan = std::move(plan);
    c->n = s->n;
    c->k = k;
    c->engine = engine;
    c->partitioner = part;
    c->cm = cm;
    c->cm_gen = gen;
  }
  return QCS_CUDA_OK;
}

int collect_timings(qcs_cuda_state *s, const qcs_cuda_op *ops, int count, int kmax, int engine,
                    float *feats, float *ms, int max, int *written) {
  int rc = validate_ops(s, ops, count);
  if (rc) return rc;
  kmax = fusion_cap(s, kmax < 1 ? 1 : kmax, engine);
  PartitionOptions po;
  po.kmax = kmax;
  po.cost = nullptr;
  po.cost_ctx = nullptr;
  std::vector<PlanItem> plan = partition(ops, count, s->n, po);
  const int tcm = tc_max(s, engine);
  std::vector<cudaEvent_t> ev;
  std::vector<int> rec;  // item index of each recorded pair
  std::vector<cd> u;
  for (size_t i = 0; i < plan.size(); i++) {
    const bool timed = plan[i].kind == 0 && (int)rec.size() < max;
    // the block matrix is formed before the opening event: host work while
    // the stream waits must not count as the kernel's time
    const bool block = item_is_block(plan[i]);
    if (block) block_matrix(ops, plan[i], u);
    cudaEvent_t a = nullptr, b = nullptr;
    if (timed) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      cudaEventRecord(a, s->stream);
    }
    rc = block ? apply_block_item(s, plan[i], engine, u, nullptr)
               : apply_item(s, ops, plan[i], engine, u);
    if (timed) {
      cudaEventRecord(b, s->stream);
      ev.push_back(a);
      ev.push_back(b);
      rec.push_back((int)i);
    }
    if (rc) break;
  }
  if (!rc) rc = check_cuda(cudaStreamSynchronize(s->stream), "collect sync");
  for (size_t r = 0; r < rec.size(); r++) {
    float t = 0.f;
    cudaEventElapsedTime(&t, ev[2 * r], ev[2 * r + 1]);
    const PlanItem &it = plan[rec[r]];
    const int cat = item_category(ops, it, tcm);
    item_features(cat, s->n, (int)it.qubits.size(), (int)it.gates.size(), it.qubits.data(),
                  feats + r * kCostFeatures);
    ms[r] = t;
  }
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  if (written) *written = (int)rec.size();
  return rc;
}

}  // namespace qcs

using namespace qcs;

extern "C" {

int qcs_cuda_apply_block(qcs_cuda_state *s, int k, const int *qubits, const double *u,
                         int engine) {
  QCS_CHECK_STATE(s);
  if (!qubits || !u) return set_error(QCS_CUDA_EINVAL, "null block argument");
  if (k < 1 || k > 7 || k > s->n) return set_error(QCS_CUDA_EINVAL, "block size k=%d unsupported", k);
  if (s->sem == QCS_CUDA_REFERENCE)
    return set_error(QCS_CUDA_EUNSUP, "dense blocks need PHYSICAL semantics");
  i64 seen = 0;
  for (int j = 0; j < k; j++) {
    int rc = check_qubit(s, qubits[j], "apply_block");
    if (rc) return rc;
    if (seen & (1LL << qubits[j])) return set_error(QCS_CUDA_EINVAL, "repeated qubit %d", qubits[j]);
    seen |= 1LL << qubits[j];
  }
  return apply_block(s, k, qubits, u, engine, true, nullptr);
}

int qcs_cuda_plan(const qcs_cuda_op *ops, int count, int num_qubits, int kmax, int *order,
                  int *item, int *num_items) {
  if (count < 0 || (count > 0 && (!ops || !order || !item)) || !num_items)
    return set_error(QCS_CUDA_EINVAL, "bad plan arguments");
  if (num_qubits < 1 || num_qubits > 36) return set_error(QCS_CUDA_EINVAL, "bad qubit count");
  qcs_cuda_state shape;
  memset(&shape, 0, sizeof(shape));
  shape.n = num_qubits;
  shape.size = 1LL << num_qubits;
  int rc = validate_ops(&shape, ops, count);
  if (rc) return rc;
  PartitionOptions po;
  po.kmax = kmax < 1 ? 1 : (kmax > 7 ? 7 : kmax);
  po.cost = nullptr;
  po.cost_ctx = nullptr;
  std::vector<PlanItem> plan = partition(ops, count, num_qubits, po);
  int j = 0;
  for (size_t it = 0; it < plan.size(); it++) {
    if (plan[it].kind == 1) {
      order[j] = plan[it].op;
      item[j++] = (int)it;
    } else {
      for (int g : plan[it].gates) {
        order[j] = g;
        item[j++] = (int)it;
      }
    }
  }
  *num_items = (int)plan.size();
  return QCS_CUDA_OK;
}

int qcs_cuda_collect_timings(qcs_cuda_state *s, const qcs_cuda_op *ops, int count, int kmax,
                             int engine, float *features, float *ms, int max, int *written) {
  QCS_CHECK_STATE(s);
  if (count < 0 || (count > 0 && !ops) || max < 0 || (max > 0 && (!features || !ms)))
    return set_error(QCS_CUDA_EINVAL, "bad collect arguments");
  return collect_timings(s, ops, count, kmax, engine, features, ms, max, written);
}

int qcs_cuda_state_set_costmodel(qcs_cuda_state *s, qcs_cuda_costmodel *m) {
  QCS_CHECK_STATE(s);
  if (m && costmodel_features(m) != kCostFeatures)
    return set_error(QCS_CUDA_EINVAL, "cost model must take %d features", kCostFeatures);
  s->cm = m;
  return QCS_CUDA_OK;
}

int qcs_cuda_item_features(int category, int n, int k, const int *qubits, int ngates, float *out) {
  if (category < 0 || category > 6 || k < 1 || k > 8 || !qubits || !out)
    return set_error(QCS_CUDA_EINVAL, "bad item");
  item_features(category, n, k, ngates, qubits, out);
  return QCS_CUDA_OK;
}

int qcs_cuda_plan_learned(const qcs_cuda_op *ops, int count, int num_qubits, int kmax,
                          qcs_cuda_costmodel *m, int *order, int *item, int *num_items,
                          double *pred_ms, double *greedy_ms, int *choice) {
  if (count < 0 || (count > 0 && (!ops || !order || !item)) || !num_items || !m)
    return set_error(QCS_CUDA_EINVAL, "bad plan arguments");
  if (!costmodel_ready(m) || costmodel_features(m) != kCostFeatures)
    return set_error(QCS_CUDA_EINVAL, "cost model not ready");
  qcs_cuda_state shape;
  memset(&shape, 0, sizeof(shape));
  shape.n = num_qubits;
  shape.size = 1LL << num_qubits;
  int rc = validate_ops(&shape, ops, count);
  if (rc) return rc;
  if (kmax > 7) kmax = 7;
  // the tensor cores take k-qubit blocks on states of at least k + 7 qubits
  const int tcm = num_qubits >= 14 ? 7 : num_qubits >= 13 ? 6 : num_qubits >= 12 ? 5 : 0;
  std::vector<PlanItem> plan =
      partition_learned(ops, count, num_qubits, kmax, m, tcm, pred_ms, greedy_ms, choice);
  int j = 0;
  for (size_t it = 0; it < plan.size(); it++) {
    if (plan[it].kind == 1) {
      order[j] = plan[it].op;
      item[j++] = (int)it;
    } else {
      for (int g : plan[it].gates) {
        order[j] = g;
        item[j++] = (int)it;
      }
    }
  }
  *num_items = (int)plan.size();
  return QCS_CUDA_OK;
}

int qcs_cuda_run(qcs_cuda_state *s, const qcs_cuda_op *ops, int count,
                 const qcs_cuda_run_options *options) {
  QCS_CHECK_STATE(s);
  if (count < 0 || (count > 0 && !ops)) return set_error(QCS_CUDA_EINVAL, "bad op list");
  return run_ops(s, ops, count, options);
}

}  // extern "C"
