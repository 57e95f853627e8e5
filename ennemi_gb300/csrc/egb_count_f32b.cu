// FP32-filter brute-force ball-count kernels (see egb_count.cuh).
#include "egb_count.cuh"
namespace egb {
TileShape count_shape_f32b(int dclass, int dmax) {
  return count_detail::CountDispatch<false, false>::shape(dclass, dmax);
}
void launch_count_f32b(int dclass, const JobDev* jobs, const WorkItem* items, int nitems,
                       int* counter, uint32_t* err, int dmax, DeferEntry* df, int* dc, int num_sms,
                       cudaStream_t st) {
  count_detail::CountDispatch<false, false>::launch(dclass, jobs, items, nitems, counter, err,
                                                    dmax, df, dc, num_sms, st);
}
}  // namespace egb
