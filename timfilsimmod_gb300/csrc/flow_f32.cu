// flow_f32.cu -- FP32 (compensated) instantiations of the flow-field kernel.
#include "flow_kernels.cuh"

namespace tfs {

const FlowVariant g_flow_variants_f32[kFlowVariantsF32] = {
    {128, 2, 256}, {128, 4, 256}, {256, 2, 256}, {64, 4, 256}};

const FlowFn g_flow_f32[kFlowVariantsF32][2] = {
    TFS_FLOW_ROW(float, 128, 2, 256), TFS_FLOW_ROW(float, 128, 4, 256),
    TFS_FLOW_ROW(float, 256, 2, 256), TFS_FLOW_ROW(float, 64, 4, 256)};

}  // namespace tfs
