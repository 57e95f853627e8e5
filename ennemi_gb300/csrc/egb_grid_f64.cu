// Grid (strip layout) kNN and count kernels, all FP64 (see egb_grid.cuh).
#include "egb_grid.cuh"
namespace egb {
TileShape grid_shape_f64(int dclass, int dmax) {
  return grid_detail::GridDispatch<true>::shape(dclass, dmax);
}
void launch_knn_grid_f64(int kclass, int dclass, const JobDev* jobs, const WorkItem* items,
                          int nitems, int* ctr, uint32_t* err, int dmax, DeferEntry* df, int* dc,
                          int sms, cudaStream_t st) {
  grid_detail::GridDispatch<true>::knn(kclass, dclass, jobs, items, nitems, ctr, err, dmax, df, dc,
                                      sms, st);
}
void launch_count_grid_f64(int dclass, const JobDev* jobs, const WorkItem* items, int nitems,
                            int* ctr, uint32_t* err, int dmax, DeferEntry* df, int* dc, int sms,
                            cudaStream_t st) {
  grid_detail::GridDispatch<true>::count(dclass, jobs, items, nitems, ctr, err, dmax, df, dc, sms,
                                        st);
}
}  // namespace egb
