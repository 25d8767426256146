// mlp.cu -- learned fusion cost model kernels (placeholder).
#include "common.cuh"
