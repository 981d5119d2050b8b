// pyramid.cu — single-launch Hi-Z depth pyramid (blz_pyramid_build).
//
// The reference builds the pyramid with one dispatch per mip and a barrier between them
// (src/Renderer/BlitzenDX12/dx12Draw.cpp:248-277, src/Renderer/BlitzenVulkan/vulkanDraw.cpp:579-614).
// Here one launch builds every mip: one block per 32x32 tile of mip 0 reduces it through mip 5, and
// the block that finishes last builds the few remaining small mips and rewinds the context's
// counter (pyramid_tile.cuh holds the steps and the texel rules of both forms). Pyramid builds of
// one context are therefore ordered on the device, as all of a context's work is.
#include "pyramid_tile.cuh"

namespace blz {

constexpr int kPyrThreads = 256;

template <uint32_t MODE>
__global__ void __launch_bounds__(kPyrThreads) pyramid_kernel(const __grid_constant__ PyramidBuildParams p) {
    __shared__ float sA[kPyrSmemA];
    __shared__ float sB[kPyrSmemB];
    pdl_wait();
    pdl_launch_next();
    pyramid_tile<MODE, kPyrThreads>(p, blockIdx.x * kPyrTile, blockIdx.y * kPyrTile, sA, sB);
    // the levels above 5 span several tiles: the last block to finish builds them
    if (p.mipCount > kPyrInTileLevels + 1) pyramid_tile_finish<MODE, kPyrThreads>(p, gridDim.x * gridDim.y, p.done, nullptr, sA, sB);
}

cudaError_t launch_pyramid_build(const PyramidBuildParams& p, cudaStream_t s, uint32_t* launches) {
    dim3 grid((p.width + kPyrTile - 1) / kPyrTile, (p.height + kPyrTile - 1) / kPyrTile);
    cudaError_t e;
    if (p.mode == BLZ_HIZ_VULKAN) e = launch_pdl(pyramid_kernel<BLZ_HIZ_VULKAN>, grid, dim3(kPyrThreads), 0, s, p);
    else e = launch_pdl(pyramid_kernel<BLZ_HIZ_D3D12>, grid, dim3(kPyrThreads), 0, s, p);
    if (launches) *launches += 1u;
    return e;
}

}  // namespace blz
