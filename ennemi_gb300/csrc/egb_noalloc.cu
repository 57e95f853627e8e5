// egb_noalloc.cu -- egb_knn_eps_noalloc(): the (k+1)-NN distance query of
// egb_knn_eps() for callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc: a plugin embedded in a larger GPU
// application that owns a fixed, pre-reserved memory pool; a latency-bound
// loop where the implicit device synchronisation of cudaMalloc/cudaFree is not
// acceptable; a process running close to the device's memory limit where an
// allocation may fail mid-run.  This entry point takes device pointers for
// its input and output, and keeps every intermediate buffer in one file-scope
// __device__ array of fixed size (EGB_NOALLOC_SCRATCH_BYTES).  Every GPU that
// loads the library holds that array until the process exits.
//
// Limits: n <= EGB_NOALLOC_MAX_POINTS, d <= EGB_NOALLOC_MAX_DIM, k + 1 <= 32.
// Larger requests are rejected with EGB_ERR_ARG before anything is launched.
//
// The search itself is the all-FP64 brute-force tile kernel of egb_knn.cuh
// (the same code the plain comparator runs), so results equal egb_knn_eps()
// bit for bit.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "egb_internal.cuh"
#include "ennemi_gb.h"

namespace {

constexpr int64_t NOALLOC_MAX_POINTS = EGB_NOALLOC_MAX_POINTS;
constexpr int NOALLOC_MAX_DIM = EGB_NOALLOC_MAX_DIM;
constexpr int NOALLOC_MAX_DEVICES = 64;

// The scratch: job descriptor, work items, counters, then the SoA copy of the
// points.  Shared by every call on a device; its contents persist between
// calls, so everything that must start at zero is cleared by the set-up
// kernel of each call.
static __device__ __align__(256) unsigned char g_noalloc_scratch[EGB_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch per device, looked up once per device.
// In host code the array's name is only a stand-in, never a device address.
unsigned char* g_scratch_dev[NOALLOC_MAX_DEVICES] = {};
int g_num_sms[NOALLOC_MAX_DEVICES] = {};
std::mutex g_setup_mutex;

struct Layout {
  size_t job, items, counters, idx, c64, end;
};

Layout layout_for(int64_t n, int d, int nitems) {
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  const int64_t lds = (n + 31) / 32 * 32;
  Layout L{};
  L.job = 0;
  L.items = up(L.job + sizeof(egb::JobDev));
  L.counters = up(L.items + sizeof(egb::WorkItem) * (size_t)nitems);
  L.idx = up(L.counters + 64);  // work counter, error word, 4 x u64 stats
  L.c64 = up(L.idx + sizeof(int32_t) * (size_t)lds);
  L.end = up(L.c64 + sizeof(double) * (size_t)d * (size_t)lds);
  return L;
}

// One thread block: clear the counters, write the job descriptor and the
// work items; every block: copy the row-major points into the SoA columns.
__global__ void noalloc_setup_kernel(unsigned char* scratch, Layout L, const double* points,
                                     int64_t n, int d, int K, int qb, int nitems, double* eps) {
  const int64_t lds = (n + 31) / 32 * 32;
  double* c64 = reinterpret_cast<double*>(scratch + L.c64);
  int32_t* idx = reinterpret_cast<int32_t*>(scratch + L.idx);
  if (blockIdx.x == 0) {
    unsigned char* cnt = scratch + L.counters;
    for (int i = threadIdx.x; i < 64; i += blockDim.x) cnt[i] = 0;
    egb::WorkItem* items = reinterpret_cast<egb::WorkItem*>(scratch + L.items);
    for (int i = threadIdx.x; i < nitems; i += blockDim.x) items[i] = egb::WorkItem{0, i * qb, 0, 0};
    if (threadIdx.x == 0) {
      egb::JobDev J;
      memset(&J, 0, sizeof(J));
      J.c64 = c64;
      J.idx = idx;
      J.eps = eps;
      J.jflags = reinterpret_cast<uint32_t*>(cnt + 8);  // never read by the plain kernel
      J.stats = reinterpret_cast<unsigned long long*>(cnt + 32);
      J.lds = lds;
      J.len = (int32_t)n;
      J.K = K;
      J.sp.d = d;
      for (int c = 0; c < d; ++c) J.sp.cols[c] = (int8_t)c;
      *reinterpret_cast<egb::JobDev*>(scratch + L.job) = J;
    }
  }
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < lds;
       p += (int64_t)gridDim.x * blockDim.x) {
    idx[p] = p < n ? (int32_t)p : 0;
    for (int c = 0; c < d; ++c) c64[(int64_t)c * lds + p] = p < n ? points[p * d + c] : 0.0;
  }
}

int setup_device(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return EGB_ERR_ARG;
  if (g_scratch_dev[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return EGB_ERR_CUDA;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      cudaGetLastError();
      return EGB_ERR_CUDA;
    }
    g_num_sms[dev] = sms > 0 ? sms : 1;
    g_scratch_dev[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_dev[dev];
  return EGB_OK;
}

}  // namespace

extern "C" int egb_knn_eps_noalloc(const double* points, int64_t n, int32_t d, int32_t k,
                                   double* eps, void* stream) {
  if (!points || !eps || n < 1 || n > NOALLOC_MAX_POINTS || d < 1 || d > NOALLOC_MAX_DIM ||
      k < 1 || k + 1 > EGB_KREG_MAX)
    return EGB_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return EGB_ERR_CUDA;
  }
  unsigned char* scratch = nullptr;
  int rc = setup_device(dev, &scratch);
  if (rc != EGB_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  const int K = k + 1;
  const int kclass = K <= 4 ? 4 : K <= 8 ? 8 : K <= 16 ? 16 : 32;
  const int dclass = (d >= 2 && d <= 4) ? d : 0;
  const int qb = egb::knn_shape(kclass, dclass, /*plain=*/1, /*slab=*/0, d).queries();
  const int nitems = (int)((n + qb - 1) / qb);
  const Layout L = layout_for(n, d, nitems);
  if (L.end > sizeof(g_noalloc_scratch)) return EGB_ERR_ARG;

  // An error the caller left pending stays pending: only a different error
  // raised by this call's own launches is consumed and reported.
  const cudaError_t prior = cudaPeekAtLastError();
  auto own_error = [prior]() {
    const cudaError_t now = cudaPeekAtLastError();
    if (now == cudaSuccess || now == prior) return false;
    cudaGetLastError();
    return true;
  };
  int blocks = (int)((n + 255) / 256);
  if (blocks > 256) blocks = 256;
  noalloc_setup_kernel<<<blocks, 256, 0, st>>>(scratch, L, points, n, d, K, qb, nitems, eps);
  unsigned char* cnt = scratch + L.counters;
  egb::launch_knn_tile(reinterpret_cast<const egb::JobDev*>(scratch + L.job),
                       reinterpret_cast<const egb::WorkItem*>(scratch + L.items), nitems, kclass,
                       dclass, /*plain=*/1, /*slab=*/0, d, reinterpret_cast<int*>(cnt),
                       reinterpret_cast<uint32_t*>(cnt + 4), nullptr, nullptr, g_num_sms[dev], st);
  if (own_error()) return EGB_ERR_CUDA;
  uint32_t err = 0;
  if (cudaMemcpyAsync(&err, cnt + 4, sizeof(err), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    own_error();
    return EGB_ERR_CUDA;
  }
  return err ? EGB_ERR_DEVICE : EGB_OK;
}
