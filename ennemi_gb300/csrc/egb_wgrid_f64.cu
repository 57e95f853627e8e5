// Warp-level grid kernels, all FP64 (see egb_wgrid.cuh).
#include "egb_wgrid.cuh"
namespace egb {
void launch_knn_wgrid_f64(int kclass, int dclass, const JobDev* jobs, const WorkItem* items,
                           int nitems, int* ctr, int dmax, int sms, cudaStream_t st) {
  wgrid_detail::WgridDispatch<true>::knn(kclass, dclass, jobs, items, nitems, ctr, dmax, sms, st);
}
void launch_count_wgrid_f64(int dclass, const JobDev* jobs, const WorkItem* items, int nitems,
                             int* ctr, int dmax, int sms, cudaStream_t st) {
  wgrid_detail::WgridDispatch<true>::count(dclass, jobs, items, nitems, ctr, dmax, sms, st);
}
}  // namespace egb
