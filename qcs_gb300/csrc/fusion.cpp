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

// U := G U for one gate, on the rows (a, a | tb) of every control setting.
// U is held as separate real and imaginary planes (row-major K x K), so the
// column loops are plain FP64 streams.  Only the columns that can be nonzero
// are visited: starting from the identity, after gates on the block bits in
// `touched`, U[a][c] = 0 unless a and c agree outside `touched`.  Three gate
// shapes: diagonal (Z, P, RZ, CPHASE: each row scaled, rows equal to 1 left
// alone), exchange (X, Y, CNOT: rows swapped and scaled) and dense.  Each
// element is computed as g00*v0 + g01*v1 with the zero terms of the first
// two shapes left out, which changes no value (at most the sign of a zero).
struct Planes {
  int K;
  std::vector<double> re, im;
};

static inline void cmul_into(double gr, double gi, double vr, double vi, double &or_, double &oi) {
  or_ = gr * vr - gi * vi;
  oi = gr * vi + gi * vr;
}

static void apply_gate_planes(Planes &P, const double m[8], int tb, int cb, int touched) {
  const int K = P.K;
  const bool diag = m[2] == 0.0 && m[3] == 0.0 && m[4] == 0.0 && m[5] == 0.0;
  const bool exch = m[0] == 0.0 && m[1] == 0.0 && m[6] == 0.0 && m[7] == 0.0;
  const bool full = touched == K - 1;  // every column may be nonzero
  const int free_mask = (K - 1) & ~touched;
  for (int a = 0; a < K; a++) {
    if (a & tb) continue;
    if (cb && !(a & cb)) continue;
    double *r0r = &P.re[(size_t)a * K], *r0i = &P.im[(size_t)a * K];
    double *r1r = &P.re[(size_t)(a | tb) * K], *r1i = &P.im[(size_t)(a | tb) * K];
    // the columns to visit: c = (a & free_mask) | sub for every subset sub
    // of `touched` (all K columns once every bit is touched)
    const int cbase = a & free_mask;
    auto each_col = [&](auto &&f) {
      if (full) {
        for (int c = 0; c < K; c++) f(c);
      } else {
        int sub = 0;
        do {
          f(cbase | sub);
          sub = (sub - touched) & touched;
        } while (sub != 0);
      }
    };
    if (diag) {
      const bool one0 = m[0] == 1.0 && m[1] == 0.0, one1 = m[6] == 1.0 && m[7] == 0.0;
      if (!one0)
        each_col([&](int c) {
          double xr, xi;
          cmul_into(m[0], m[1], r0r[c], r0i[c], xr, xi);
          r0r[c] = xr;
          r0i[c] = xi;
        });
      if (!one1)
        each_col([&](int c) {
          double xr, xi;
          cmul_into(m[6], m[7], r1r[c], r1i[c], xr, xi);
          r1r[c] = xr;
          r1i[c] = xi;
        });
    } else if (exch) {
      const bool swap_only = m[2] == 1.0 && m[3] == 0.0 && m[4] == 1.0 && m[5] == 0.0;
      each_col([&](int c) {
        const double v0r = r0r[c], v0i = r0i[c], v1r = r1r[c], v1i = r1i[c];
        if (swap_only) {
          r0r[c] = v1r;
          r0i[c] = v1i;
          r1r[c] = v0r;
          r1i[c] = v0i;
        } else {
          cmul_into(m[2], m[3], v1r, v1i, r0r[c], r0i[c]);
          cmul_into(m[4], m[5], v0r, v0i, r1r[c], r1i[c]);
        }
      });
    } else {
      each_col([&](int c) {
        const double v0r = r0r[c], v0i = r0i[c], v1r = r1r[c], v1i = r1i[c];
        double ar, ai, br, bi;
        cmul_into(m[0], m[1], v0r, v0i, ar, ai);
        cmul_into(m[2], m[3], v1r, v1i, br, bi);
        r0r[c] = ar + br;
        r0i[c] = ai + bi;
        cmul_into(m[4], m[5], v0r, v0i, ar, ai);
        cmul_into(m[6], m[7], v1r, v1i, br, bi);
        r1r[c] = ar + br;
        r1i[c] = ai + bi;
      });
    }
  }
}

void block_matrix(const qcs_cuda_op *ops, const PlanItem &item, std::vector<cd> &u) {
  const int k = (int)item.qubits.size();
  const int K = 1 << k;
  Planes P;
  P.K = K;
  P.re.assign((size_t)K * K, 0.0);
  P.im.assign((size_t)K * K, 0.0);
  for (int a = 0; a < K; a++) P.re[(size_t)a * K + a] = 1.0;
  auto bit_of = [&](int q) {
    for (int j = 0; j < k; j++)
      if (item.qubits[j] == q) return j;
    return -1;
  };
  int touched = 0;
  for (int g : item.gates) {
    const qcs_cuda_op &o = ops[g];
    double m[8];
    gate_matrix(o.kind, o.angle, m);
    const int tb = 1 << bit_of(o.target);
    const int cb = gate_is_controlled(o.kind) ? (1 << bit_of(o.control)) : 0;
    touched |= tb | cb;
    apply_gate_planes(P, m, tb, cb, touched);
  }
  u.resize((size_t)K * K);
  for (size_t i = 0; i < (size_t)K * K; i++) u[i] = cd(P.re[i], P.im[i]);
}

}  // namespace qcs
