// egb_matrix.cu -- the pairwise MI matrix and normalize_mi on the device.
//
// pairwise_mi collects the estimate of every pair i < j into a symmetric
// nvar x nvar matrix with a NaN diagonal (ennemi/_driver.py:716-721), and
// normalize_mi maps each value v to sqrt(1 - exp(-2 v)) when v > 0, leaving
// the others (zero, negative, -inf, NaN) unchanged (_driver.py:77-81).
// Elementwise work: one thread per matrix entry or value.
#include "egb_internal.cuh"

namespace egb {
namespace {

constexpr int MX_THREADS = 256;

__device__ __forceinline__ double normalize_one(double v) {
  return v <= 0.0 ? v : sqrt(1.0 - exp(-2.0 * v));
}

__global__ void fill_nan_kernel(double* __restrict__ out, int64_t n) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = nan;
}

__global__ void pairwise_kernel(const double* __restrict__ vals, const int32_t* __restrict__ pairs,
                                int ntasks, int nvar, int normalize, double* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntasks) return;
  const int i = pairs[2 * t], j = pairs[2 * t + 1];
  if ((unsigned)i >= (unsigned)nvar || (unsigned)j >= (unsigned)nvar) return;
  const double v = normalize ? normalize_one(vals[t]) : vals[t];
  out[(int64_t)i * nvar + j] = v;
  out[(int64_t)j * nvar + i] = v;
}

__global__ void normalize_kernel(const double* __restrict__ in, int64_t n, double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = normalize_one(in[i]);
}

int blocks_for(int64_t n) {
  const int64_t b = (n + MX_THREADS - 1) / MX_THREADS;
  return (int)(b < 1 ? 1 : b > 65535 ? 65535 : b);
}

}  // namespace

void launch_pairwise_matrix(const double* vals_d, const int32_t* pairs_d, int ntasks, int nvar,
                            int normalize, double* out_d, cudaStream_t st) {
  const int64_t nn = (int64_t)nvar * nvar;
  if (nn <= 0) return;
  fill_nan_kernel<<<blocks_for(nn), MX_THREADS, 0, st>>>(out_d, nn);
  count_launch();
  if (ntasks <= 0) return;
  pairwise_kernel<<<(ntasks + MX_THREADS - 1) / MX_THREADS, MX_THREADS, 0, st>>>(
      vals_d, pairs_d, ntasks, nvar, normalize, out_d);
  count_launch();
}

void launch_normalize(const double* in_d, int64_t n, double* out_d, cudaStream_t st) {
  if (n <= 0) return;
  normalize_kernel<<<blocks_for(n), MX_THREADS, 0, st>>>(in_d, n, out_d);
  count_launch();
}

}  // namespace egb
