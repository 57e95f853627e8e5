// FP32-filter brute-force (k+1)-NN tile kernels (see egb_knn.cuh).
#include "egb_knn.cuh"
EGB_KNN_TU(false, false)
