// costmodel.h -- learned fusion cost model: features of a plan item and the
// partitioner that uses the model.
#pragma once

#include <vector>

#include "fusion.h"
#include "qcs_cuda.h"

namespace qcs {

constexpr int kMlpHidden = 64;     // width of the three hidden layers
constexpr int kCostFeatures = 20;  // QCS_COSTMODEL_FEATURES

// Item categories (one-hot features 0..6).
enum ItemCat {
  CAT_DENSE = 0,   // one dense 2x2 sweep
  CAT_DIAG = 1,    // diagonal 2x2 on every amplitude
  CAT_PHASE = 2,   // phase on the amplitudes with one bit set
  CAT_CTRL = 3,    // controlled dense 2x2
  CAT_CPHASE = 4,  // controlled phase
  CAT_SIMT = 5,    // fused block, CUDA cores
  CAT_TC = 6       // fused block, tensor cores
};

// Features of one item: category, n, k, gate count, which of qubits 0..7 it
// touches, how many of its qubits are below 7, its highest qubit.
void item_features(int cat, int n, int k, int ngates, const int *qubits, float *f);

// Category the executor will use for a plan item.  tc_max: the widest block
// the tensor cores take on this state (5, 6 or 7; 0 when they take none);
// 2..4-qubit blocks go there widened to 5 when tc_max >= 5.
int item_category(const qcs_cuda_op *ops, const PlanItem &it, int tc_max);

struct CostModelView;  // opaque handle used by the partitioner

// Learned partition: candidate plans (greedy with every width up to kmax, and
// greedy growth stopped by the model), each scored by the model's predicted
// time; the greedy width-kmax plan judges -- the candidate replaces it only
// when predicted faster.  *chosen receives a short description.
std::vector<PlanItem> partition_learned(const qcs_cuda_op *ops, int count, int n, int kmax,
                                        const struct ::qcs_cuda_costmodel *m, int tc_max,
                                        double *pred_ms, double *greedy_ms, int *choice);

float costmodel_predict_host(const struct ::qcs_cuda_costmodel *m, const float *x);
bool costmodel_ready(const struct ::qcs_cuda_costmodel *m);
// Changes whenever the model's parameters change (training, set_params).
unsigned long long costmodel_generation(const struct ::qcs_cuda_costmodel *m);
int costmodel_features(const struct ::qcs_cuda_costmodel *m);

}  // namespace qcs
