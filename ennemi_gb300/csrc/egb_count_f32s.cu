// FP32-filter slab ball-count kernels (see egb_count.cuh).
#include "egb_count.cuh"
namespace egb {
TileShape count_shape_f32s(int dclass, int dmax) {
  return count_detail::CountDispatch<false, true>::shape(dclass, dmax);
}
void launch_count_f32s(int dclass, const JobDev* jobs, const WorkItem* items, int nitems,
                       int* counter, uint32_t* err, int dmax, DeferEntry* df, int* dc, int num_sms,
                       cudaStream_t st) {
  count_detail::CountDispatch<false, true>::launch(dclass, jobs, items, nitems, counter, err,
                                                    dmax, df, dc, num_sms, st);
}
void count_defer_f32s(int dclass, const JobDev* jobs, const DeferEntry* list, const int* count,
                      int cap, int num_sms, cudaStream_t st) {
  count_detail::CountDispatch<false, true>::defer(dclass, jobs, list, count, cap, num_sms, st);
}
}  // namespace egb
