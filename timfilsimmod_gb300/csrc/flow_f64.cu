// flow_f64.cu -- FP64 instantiations of the flow-field kernel.
#include "flow_kernels.cuh"

namespace tfs {

const FlowVariant g_flow_variants_f64[kFlowVariantsF64] = {
    {128, 1, 128}, {128, 2, 128}, {64, 2, 128}};

const FlowFn g_flow_f64[kFlowVariantsF64][2] = {
    TFS_FLOW_ROW(double, 128, 1, 128), TFS_FLOW_ROW(double, 128, 2, 128),
    TFS_FLOW_ROW(double, 64, 2, 128)};

}  // namespace tfs
