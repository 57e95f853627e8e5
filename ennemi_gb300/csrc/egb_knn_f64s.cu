// All-FP64 slab (k+1)-NN tile kernels (see egb_knn.cuh).
#include "egb_knn.cuh"
EGB_KNN_TU(true, true)
EGB_KNN_DEFER_TU(true)
