// k_tile.cu — K4 launches without deferred colour (the kernel is in k_tile.cuh).
#include "k_tile.cuh"

namespace mtgl {

int launch_tile(const TileArgs &a, cudaStream_t s)
{
    if (a.ntiles == 0) return 0;
    return a.defer ? dispatch_tile_deferred(a, s, false) : dispatch_tile_size<false>(a, s, false);
}

int tile_occupancy(const TileArgs &a)
{
    return a.defer ? dispatch_tile_deferred(a, nullptr, true) : dispatch_tile_size<false>(a, nullptr, true);
}

}  // namespace mtgl
