// batch.cu -- batched variational circuits (placeholder; filled in below).
#include "common.cuh"
