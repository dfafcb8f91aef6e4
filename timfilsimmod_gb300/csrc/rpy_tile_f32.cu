// rpy_tile_f32.cu -- FP32 (compensated) instantiations of the tile kernel.
#include "rpy_tile.cuh"

namespace tfs {

// (threads per CTA, targets per thread, sources per tile); index = variant.
// Variants kNumVariantsF32Scalar.. are the packed FP32x2 kernels
// (rpy_tile_f32x2.cu).
const TileVariant g_variants_f32[kNumVariantsF32] = {
    {128, 4, 256, 0}, {128, 2, 256, 0}, {256, 2, 256, 0}, {64, 4, 256, 0}, {128, 8, 256, 0},
    {256, 4, 256, 0}, {128, 4, 256, 1}, {128, 8, 256, 1}, {64, 8, 256, 1}};

const TileFn g_tile_f32[kNumVariantsF32Scalar][kNumCombos] = {
    TFS_TILE_ROW(float, 128, 4, 256), TFS_TILE_ROW(float, 128, 2, 256),
    TFS_TILE_ROW(float, 256, 2, 256), TFS_TILE_ROW(float, 64, 4, 256),
    TFS_TILE_ROW(float, 128, 8, 256), TFS_TILE_ROW(float, 256, 4, 256)};

}  // namespace tfs
