// k_tile_defer.cu — K4 launches with deferred colour (the kernel is in k_tile.cuh).
#include "k_tile.cuh"

namespace mtgl {

int dispatch_tile_deferred(const TileArgs &a, cudaStream_t s, bool occ_only)
{
    return dispatch_tile_size<true>(a, s, occ_only);
}

}  // namespace mtgl
