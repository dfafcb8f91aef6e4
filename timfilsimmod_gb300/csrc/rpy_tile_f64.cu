// rpy_tile_f64.cu -- FP64 instantiations of the tile kernel.
#include "rpy_tile.cuh"

namespace tfs {

// (threads per CTA, targets per thread, sources per tile); index = variant.
const TileVariant g_variants_f64[kNumVariantsF64] = {
    {128, 1, 128, 0, 0}, {64, 1, 128, 0, 0}, {128, 2, 128, 0, 0}, {256, 1, 128, 0, 0},
    {32, 1, 128, 0, 0}};

const TileFn g_tile_f64[kNumVariantsF64][kNumCombos] = {
    TFS_TILE_ROW(double, 128, 1, 128, 1), TFS_TILE_ROW(double, 64, 1, 128, 1),
    TFS_TILE_ROW(double, 128, 2, 128, 1), TFS_TILE_ROW(double, 256, 1, 128, 1),
    TFS_TILE_ROW(double, 32, 1, 128, 1)};

}  // namespace tfs
