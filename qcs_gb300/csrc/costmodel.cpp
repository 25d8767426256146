// costmodel.cpp -- features of plan items and the learned partitioner.
//
// The greedy fixed-k planner (fusion.cpp) fuses as wide as k allows.  Wider
// is not always faster: a 5-qubit block on the CUDA cores is FP32-bound, a
// lone diagonal gate touches half the state, the tensor-core engine has a
// per-launch cost.  A small MLP trained on timings of this simulator's own
// kernels predicts each item's device time from the features below; the
// learned partitioner scores several candidate plans with it and keeps the
// cheapest, with the greedy width-k plan as the fallback and the judge.
#include <math.h>
#include <string.h>

#include <algorithm>

#include "costmodel.h"

namespace qcs {

void item_features(int cat, int n, int k, int ngates, const int *qubits, float *f) {
  memset(f, 0, kCostFeatures * sizeof(float));
  f[cat] = 1.f;
  f[7] = n / 32.f;
  f[8] = k / 8.f;
  f[9] = ngates / 64.f;
  int low = 0, top = 0;
  for (int j = 0; j < k; j++) {
    const int q = qubits[j];
    if (q < 8) f[10 + q] = 1.f;
    if (q < 7) low++;
    if (q > top) top = q;
  }
  f[18] = low / 7.f;
  f[19] = top / 32.f;
}

static bool is_zero(const double *z) { return z[0] == 0.0 && z[1] == 0.0; }
static bool is_one(const double *z) { return z[0] == 1.0 && z[1] == 0.0; }

int item_category(const qcs_cuda_op *ops, const PlanItem &it, int tc_max) {
  const int k = (int)it.qubits.size();
  if (it.gates.size() == 1 || k == 1) {
    // a single gate, or a product of one-qubit gates on one qubit: plain kernel
    double m[8];
    int kind = ops[it.gates[0]].kind;
    bool ctl = gate_is_controlled(kind);
    if (it.gates.size() == 1) {
      gate_matrix(kind, ops[it.gates[0]].angle, m);
    } else {
      // product of the 2x2s (same qubit): classify the result
      double a[8] = {1, 0, 0, 0, 0, 0, 1, 0};
      for (int g : it.gates) {
        double b[8], r[8];
        gate_matrix(ops[g].kind, ops[g].angle, b);
        for (int i = 0; i < 2; i++)
          for (int j = 0; j < 2; j++) {
            double re = 0, im = 0;
            for (int l = 0; l < 2; l++) {
              const double *x = b + 2 * (2 * i + l), *y = a + 2 * (2 * l + j);
              re += x[0] * y[0] - x[1] * y[1];
              im += x[0] * y[1] + x[1] * y[0];
            }
            r[2 * (2 * i + j)] = re;
            r[2 * (2 * i + j) + 1] = im;
          }
        memcpy(a, r, sizeof(a));
      }
      memcpy(m, a, sizeof(a));
    }
    const bool diag = is_zero(m + 2) && is_zero(m + 4);
    if (ctl) return (diag && is_one(m)) ? CAT_CPHASE : CAT_CTRL;
    if (diag && is_one(m)) return CAT_PHASE;
    if (diag) return CAT_DIAG;
    return CAT_DENSE;
  }
  // AUTO runs 2..4-qubit blocks on the tensor cores, widened to 5 qubits
  if (tc_max >= 5 && k >= 2 && k <= tc_max) return CAT_TC;
  return CAT_SIMT;
}

struct PlanScore {
  const qcs_cuda_costmodel *m;
  const qcs_cuda_op *ops;
  int n;
  int tc_max;
};

static double item_ms(const PlanScore &ps, const PlanItem &it) {
  if (it.kind == 1) return 0.0;  // non-gate ops are the same in every plan
  float f[kCostFeatures];
  const int cat = item_category(ps.ops, it, ps.tc_max);
  item_features(cat, ps.n, (int)it.qubits.size(), (int)it.gates.size(), it.qubits.data(), f);
  return exp2((double)costmodel_predict_host(ps.m, f));
}

static double plan_ms(const PlanScore &ps, const std::vector<PlanItem> &plan) {
  double t = 0.0;
  for (const PlanItem &it : plan) t += item_ms(ps, it);
  return t;
}

// Growth hook: predicted time of a block of k qubits and ngates gates.
static double grow_cost(int n, int k, int ngates, const int *qubits, void *ctx) {
  const PlanScore &ps = *static_cast<const PlanScore *>(ctx);
  int cat;
  if (k == 1) cat = CAT_DENSE;
  else if (ps.tc_max >= 5 && k <= ps.tc_max) cat = CAT_TC;
  else cat = CAT_SIMT;
  float f[kCostFeatures];
  item_features(cat, n, k, ngates, qubits, f);
  return exp2((double)costmodel_predict_host(ps.m, f));
}

// Cheapest predicted way to run one block's gates: the block itself, or its
// gates re-partitioned greedily at every narrower width (width 1: every gate
// on its own, or merged with same-qubit neighbours).  The block's gate order is a valid execution order of those
// gates, so each alternative may replace the block in place.  Returns true
// (and fills *out) when an alternative is predicted faster.
static bool refine_block(const PlanScore &ps, const PlanItem &it, std::vector<PlanItem> *out) {
  const int m = (int)it.gates.size();
  const int k = (int)it.qubits.size();
  if (it.kind != 0 || m < 2 || k < 2) return false;
  std::vector<qcs_cuda_op> sub(m);
  for (int j = 0; j < m; j++) sub[j] = ps.ops[it.gates[j]];
  PlanScore sps = ps;
  sps.ops = sub.data();
  const double t_block = item_ms(sps, [&] {
    PlanItem local = it;
    for (int j = 0; j < m; j++) local.gates[j] = j;
    return local;
  }());
  double best = t_block;
  std::vector<PlanItem> best_items;
  for (int kk = 1; kk < k; kk++) {
    PartitionOptions po;
    po.kmax = kk;
    po.cost = nullptr;
    po.cost_ctx = nullptr;
    std::vector<PlanItem> cand = partition(sub.data(), m, ps.n, po);
    const double t = plan_ms(sps, cand);
    if (t < best) {
      best = t;
      best_items = std::move(cand);
    }
  }
  if (best_items.empty()) return false;
  for (PlanItem &x : best_items)
    for (int &g : x.gates) g = it.gates[g];
  *out = std::move(best_items);
  return true;
}

std::vector<PlanItem> partition_learned(const qcs_cuda_op *ops, int count, int n, int kmax,
                                        const qcs_cuda_costmodel *m, int tc_max,
                                        double *pred_ms, double *greedy_ms, int *choice) {
  PlanScore ps{m, ops, n, tc_max};
  PartitionOptions po;
  po.kmax = kmax;
  po.cost = nullptr;
  po.cost_ctx = nullptr;
  std::vector<PlanItem> best = partition(ops, count, n, po);
  const double judge = plan_ms(ps, best);
  double best_ms = judge;
  // 2..7: greedy width; + 100: model-stopped growth; + 200: lookahead ties
  int best_choice = kmax;
  for (int k = 2; k <= kmax; k++)
    for (int tie = 0; tie < 2; tie++)
      for (int grown = 0; grown < 2; grown++) {
        if (!grown && !tie && k == kmax) continue;  // the judge itself
        po.kmax = k;
        po.tie = tie;
        po.cost = grown ? grow_cost : nullptr;
        po.cost_ctx = grown ? &ps : nullptr;
        std::vector<PlanItem> cand = partition(ops, count, n, po);
        const double t = plan_ms(ps, cand);
        if (t < best_ms) {
          best_ms = t;
          best = std::move(cand);
          best_choice = k + (grown ? 100 : 0) + (tie ? 200 : 0);
        }
      }
  // Block by block: split the blocks the model predicts slower than their
  // parts (a wide block holding a few diagonal gates, say).
  std::vector<PlanItem> refined;
  refined.reserve(best.size());
  int splits = 0;
  for (PlanItem &it : best) {
    std::vector<PlanItem> parts;
    if (refine_block(ps, it, &parts)) {
      for (PlanItem &x : parts) refined.push_back(std::move(x));
      splits++;
    } else {
      refined.push_back(std::move(it));
    }
  }
  best = std::move(refined);  // every item was moved into `refined`
  if (splits) best_ms = plan_ms(ps, best);
  if (pred_ms) *pred_ms = best_ms;
  if (greedy_ms) *greedy_ms = judge;
  if (choice) *choice = best_choice + 1000 * splits;
  return best;
}

}  // namespace qcs
