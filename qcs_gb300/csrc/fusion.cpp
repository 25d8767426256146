// fusion.cpp -- greedy fixed-k partition of a gate list into dense blocks.
//
// Algorithm (per segment between non-gate operations):
//   1. Seed a block with the earliest unscheduled gate (always ready: every
//      earlier gate is scheduled).
//   2. Repeatedly add the ready gate that grows the block's qubit set least
//      (ties: earliest), provided the union stays within kmax qubits.  A
//      gate is ready when, on each of its qubits, it is the next unscheduled
//      gate; moving it into the block therefore commutes it only past gates
//      on disjoint qubits.
//   3. When no ready gate fits, close the block and go to 1.
// With a cost hook, step 2 also stops when adding the gate would raise the
// estimated time per gate of the block.  With tie = 1, step 2 breaks ties
// between gates of equal growth by a one-step lookahead instead of by age.
#include <algorithm>
#include <cmath>

#include "fusion.h"

namespace qcs {

static int op_qubits(const qcs_cuda_op &o, int q[2]) {
  q[0] = o.target;
  if (gate_is_controlled(o.kind)) {
    q[1] = o.control;
    return 2;
  }
  return 1;
}

static void partition_segment(const qcs_cuda_op *ops, int first, int last, int n,
                              const PartitionOptions &opt, std::vector<PlanItem> &plan) {
  // per-qubit ordered gate lists
  std::vector<std::vector<int>> onq(n);
  for (int i = first; i < last; i++) {
    int q[2];
    int m = op_qubits(ops[i], q);
    for (int j = 0; j < m; j++) onq[q[j]].push_back(i);
  }
  std::vector<size_t> head(n, 0);
  std::vector<char> done(last - first, 0);
  int remaining = last - first;
  int scan = first;  // earliest possibly-unscheduled gate
  auto next_on = [&](int q) -> int { return head[q] < onq[q].size() ? onq[q][head[q]] : -1; };
  auto ready = [&](int g) {
    int q[2];
    int m = op_qubits(ops[g], q);
    for (int j = 0; j < m; j++)
      if (next_on(q[j]) != g) return false;
    return true;
  };
  auto schedule = [&](int g) {
    int q[2];
    int m = op_qubits(ops[g], q);
    for (int j = 0; j < m; j++) head[q[j]]++;
    done[g - first] = 1;
    remaining--;
  };
  const int kmax = opt.kmax < 1 ? 1 : opt.kmax;
  while (remaining > 0) {
    while (done[scan - first]) scan++;
    PlanItem item;
    item.kind = 0;
    item.op = -1;
    std::vector<char> inb(n, 0);
    int kb = 0;
    int seed = scan;
    {
      int q[2];
      int m = op_qubits(ops[seed], q);
      for (int j = 0; j < m; j++)
        if (!inb[q[j]]) { inb[q[j]] = 1; kb++; }
      schedule(seed);
      item.gates.push_back(seed);
    }
    double best_rate = 0.0;
    if (opt.cost) {
      std::vector<int> qs;
      for (int q = 0; q < n; q++) if (inb[q]) qs.push_back(q);
      best_rate = opt.cost(n, kb, 1, qs.data(), opt.cost_ctx);
    }
    // gates that fit the block at no growth once gate `cand` has joined it
    auto lookahead = [&](int cand) {
      std::vector<char> in2 = inb;
      int qc[2];
      const int mc = op_qubits(ops[cand], qc);
      for (int j = 0; j < mc; j++) in2[qc[j]] = 1;
      int score = 0;
      for (int q2 = 0; q2 < n; q2++) {
        if (!in2[q2]) continue;
        size_t h = head[q2] + (next_on(q2) == cand ? 1 : 0);
        for (; h < onq[q2].size(); h++) {
          int qg[2];
          const int mg = op_qubits(ops[onq[q2][h]], qg);
          bool inside = true;
          for (int j = 0; j < mg; j++) inside = inside && in2[qg[j]];
          if (!inside) break;
          score++;
        }
      }
      return score;
    };
    for (;;) {
      int best = -1, best_grow = 1 << 30;
      for (int q = 0; q < n; q++) {
        int g = next_on(q);
        if (g < 0 || !ready(g)) continue;
        int qq[2];
        int m = op_qubits(ops[g], qq);
        int grow = 0;
        for (int j = 0; j < m; j++) grow += inb[qq[j]] ? 0 : 1;
        if (kb + grow > kmax) continue;
        if (grow < best_grow) {
          best = g;
          best_grow = grow;
        } else if (grow == best_grow && g != best) {
          const bool take = (opt.tie == 1 && grow > 0) ? lookahead(g) > lookahead(best) ||
                                                             (lookahead(g) == lookahead(best) && g < best)
                                                       : g < best;
          if (take) best = g;
        }
      }
      if (best < 0) break;
      if (opt.cost && best_grow > 0) {
        std::vector<int> qs;
        int qq[2];
        int m = op_qubits(ops[best], qq);
        for (int q = 0; q < n; q++) if (inb[q]) qs.push_back(q);
        for (int j = 0; j < m; j++) if (!inb[qq[j]]) qs.push_back(qq[j]);
        std::sort(qs.begin(), qs.end());
        int ng = (int)item.gates.size() + 1;
        double t_new = opt.cost(n, kb + best_grow, ng, qs.data(), opt.cost_ctx);
        // time per gate must not get worse by growing the block
        if (t_new / ng > best_rate / (ng - 1)) break;
        best_rate = t_new;
      }
      int qq[2];
      int m = op_qubits(ops[best], qq);
      for (int j = 0; j < m; j++)
        if (!inb[qq[j]]) { inb[qq[j]] = 1; kb++; }
      schedule(best);
      item.gates.push_back(best);
    }
    for (int q = 0; q < n; q++)
      if (inb[q]) item.qubits.push_back(q);
    plan.push_back(std::move(item));
  }
}

std::vector<PlanItem> partition(const qcs_cuda_op *ops, int count, int n,
                                const PartitionOptions &opt) {
  std::vector<PlanItem> plan;
  int seg = 0;
  for (int i = 0; i <= count; i++) {
    bool barrier = (i == count) || !gate_kind_valid(ops[i].kind);
    if (!barrier) continue;
    if (i > seg) partition_segment(ops, seg, i, n, opt, plan);
    if (i < count) {
      PlanItem item;
      item.kind = 1;
      item.op = i;
      plan.push_back(item);
    }
    seg = i + 1;
  }
  return plan;
}

void block_matrix(const qcs_cuda_op *ops, const PlanItem &item, std::vector<cd> &u) {
  const int k = (int)item.qubits.size();
  const int K = 1 << k;
  u.assign((size_t)K * K, cd(0.0, 0.0));
  for (int a = 0; a < K; a++) u[(size_t)a * K + a] = cd(1.0, 0.0);
  auto bit_of = [&](int q) {
    for (int j = 0; j < k; j++)
      if (item.qubits[j] == q) return j;
    return -1;
  };
  for (int g : item.gates) {
    const qcs_cuda_op &o = ops[g];
    double m[8];
    gate_matrix(o.kind, o.angle, m);
    cd g00(m[0], m[1]), g01(m[2], m[3]), g10(m[4], m[5]), g11(m[6], m[7]);
    int tb = 1 << bit_of(o.target);
    int cb = gate_is_controlled(o.kind) ? (1 << bit_of(o.control)) : 0;
    // U := G * U, i.e. apply the gate to every column of U
    for (int a = 0; a < K; a++) {
      if (a & tb) continue;
      if (cb && !(a & cb)) continue;
      cd *r0 = &u[(size_t)a * K];
      cd *r1 = &u[(size_t)(a | tb) * K];
      for (int col = 0; col < K; col++) {
        cd v0 = r0[col], v1 = r1[col];
        r0[col] = g00 * v0 + g01 * v1;
        r1[col] = g10 * v0 + g11 * v1;
      }
    }
  }
}

}  // namespace qcs
