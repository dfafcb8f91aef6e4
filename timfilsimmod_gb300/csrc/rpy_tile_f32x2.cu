// rpy_tile_f32x2.cu -- instantiations of the packed FP32x2 tile kernel.
#include "rpy_tile_x2.cuh"

namespace tfs {

// variants kNumVariantsF32Scalar + 0, 1, 2 of g_variants_f32
const TileFn g_tile_f32x2[kNumVariantsF32X2][kNumCombos] = {
    TFS_TILE_X2_ROW(128, 4, 256), TFS_TILE_X2_ROW(128, 8, 256), TFS_TILE_X2_ROW(64, 8, 256)};

}  // namespace tfs
