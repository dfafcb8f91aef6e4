// rpy_tile_f32.cu -- FP32 (compensated) instantiations of the tile kernel.
#include "rpy_tile.cuh"

namespace tfs {

// (threads per CTA, targets per thread, sources per tile); index = variant.
// Variants kNumVariantsF32Scalar.. are the packed FP32x2 kernels
// (rpy_tile_f32x2.cu).
const TileVariant g_variants_f32[kNumVariantsF32] = {
    {128, 4, 256, 0, 0}, {128, 2, 256, 0, 0}, {256, 2, 256, 0, 0}, {64, 4, 256, 0, 0},
    {128, 8, 256, 0, 0}, {128, 2, 256, 0, 6}, {128, 1, 256, 0, 8}, {64, 2, 256, 0, 12},
    {128, 4, 256, 1, 0}, {128, 8, 256, 1, 0}, {64, 8, 256, 1, 0}};

const TileFn g_tile_f32[kNumVariantsF32Scalar][kNumCombos] = {
    TFS_TILE_ROW(float, 128, 4, 256, 1), TFS_TILE_ROW(float, 128, 2, 256, 1),
    TFS_TILE_ROW(float, 256, 2, 256, 1), TFS_TILE_ROW(float, 64, 4, 256, 1),
    TFS_TILE_ROW(float, 128, 8, 256, 1), TFS_TILE_ROW(float, 128, 2, 256, 6),
    TFS_TILE_ROW(float, 128, 1, 256, 8), TFS_TILE_ROW(float, 64, 2, 256, 12)};

}  // namespace tfs
