// rpy_tile_f32.cu -- FP32 (compensated) instantiations of the tile kernel.
#include "rpy_tile.cuh"

namespace tfs {

// (threads per CTA, targets per thread, sources per tile); index = variant.
const TileVariant g_variants_f32[kNumVariantsF32] = {
    {128, 4, 256}, {128, 2, 256}, {256, 2, 256}, {64, 4, 256}, {128, 8, 256}, {256, 4, 256}};

const TileFn g_tile_f32[kNumVariantsF32][kNumCombos] = {
    TFS_TILE_ROW(float, 128, 4, 256), TFS_TILE_ROW(float, 128, 2, 256),
    TFS_TILE_ROW(float, 256, 2, 256), TFS_TILE_ROW(float, 64, 4, 256),
    TFS_TILE_ROW(float, 128, 8, 256), TFS_TILE_ROW(float, 256, 4, 256)};

}  // namespace tfs
