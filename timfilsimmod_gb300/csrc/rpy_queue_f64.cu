// rpy_queue_f64.cu -- FP64 instantiations of the work-queue kernel:
// (threads per CTA, targets per thread, sources per tile, minimum resident
// CTAs); index = variant.
#include "rpy_queue.cuh"

namespace tfs {

const QueueVariant g_qvariants_f64[kNumQueueVariantsF64] = {
    {128, 1, 128, 1}, {64, 1, 128, 1}, {128, 2, 128, 1}};

const QueueFn g_queue_f64[kNumQueueVariantsF64][kNumQueueSources] = {
    TFS_QUEUE_ROW(double, 128, 1, 128, 1), TFS_QUEUE_ROW(double, 64, 1, 128, 1),
    TFS_QUEUE_ROW(double, 128, 2, 128, 1)};

}  // namespace tfs
