// rpy_queue_f32.cu -- FP32 (compensated) instantiations of the work-queue
// kernel: (threads per CTA, targets per thread, sources per tile, minimum
// resident CTAs); index = variant.
#include "rpy_queue.cuh"

namespace tfs {

const QueueVariant g_qvariants_f32[kNumQueueVariantsF32] = {
    {128, 1, 256, 8}, {128, 2, 256, 6}, {64, 2, 256, 10}, {128, 4, 256, 4}, {256, 1, 256, 4}};

const QueueFn g_queue_f32[kNumQueueVariantsF32][kNumQueueSources] = {
    TFS_QUEUE_ROW(float, 128, 1, 256, 8), TFS_QUEUE_ROW(float, 128, 2, 256, 6),
    TFS_QUEUE_ROW(float, 64, 2, 256, 10), TFS_QUEUE_ROW(float, 128, 4, 256, 4),
    TFS_QUEUE_ROW(float, 256, 1, 256, 4)};

}  // namespace tfs
