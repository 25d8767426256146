// fusion.h -- gate-list partitioning into dense k-qubit blocks (host side).
//
// The reference has no fusion pass: every qc_<gate> call is its own sweep
// (src/qcs.c:159-228).  Here a gate list is cut into segments at the
// operations that are not gates (phase flip, diffusion), and each segment
// is partitioned into blocks of at most kmax qubits; a block's 2^k x 2^k
// matrix is the ordered product of its gates, formed in FP64.
#pragma once

#include <complex>
#include <vector>

#include "qcs_cuda.h"

namespace qcs {

typedef std::complex<double> cd;

struct PlanItem {
  // kind == 0: fused block; kind == 1: a single op applied as is
  int kind;
  int op;                    // the op index for kind == 1
  std::vector<int> gates;    // op indices of the block, in application order
  std::vector<int> qubits;   // ascending; bit j of the block index is qubits[j]
};

// Cost-model hook: estimated device time (arbitrary units) of one block of
// k qubits holding `ngates` gates on an n-qubit state; the greedy partitioner
// calls it to decide whether closing a block early pays.  nullptr: pure
// greedy (grow while the block fits).
typedef double (*BlockCostFn)(int n, int k, int ngates, const int *qubits, void *ctx);

struct PartitionOptions {
  int kmax;
  BlockCostFn cost;
  void *cost_ctx;
  // Tie-break among ready gates that grow the block by the same (non-zero)
  // number of qubits: 0 takes the earliest; 1 takes the one after which the
  // most further gates fit the block at no growth (one step of lookahead).
  int tie = 0;
};

// Greedy fixed-k partition of ops[0..count).
std::vector<PlanItem> partition(const qcs_cuda_op *ops, int count, int n,
                                const PartitionOptions &opt);

// Dense matrix of a block: row-major K x K, U[out][in].
void block_matrix(const qcs_cuda_op *ops, const PlanItem &item, std::vector<cd> &u);

// The 2x2 of a named gate (src/q_gates.c:362-491), FP64.
void gate_matrix(int kind, double angle, double m[8]);
bool gate_is_controlled(int kind);
bool gate_kind_valid(int kind);

}  // namespace qcs
