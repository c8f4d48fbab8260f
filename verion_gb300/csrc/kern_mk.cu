// Megakernel variants (shaders/pathtrace.slang).
#include "kernels.cuh"
#include "launch.h"

namespace vgx {

template <bool L, bool R, typename A>
static cudaError_t mk(dim3 grid, cudaStream_t s, const vgd::Ctx& c)
{
    vgk::mk_pathtrace<L, R, A><<<grid, 128, 0, s>>>(c);
    return cudaGetLastError();
}

cudaError_t launch_megakernel(Variant v, dim3 grid, cudaStream_t s, const vgd::Ctx& c)
{
    switch (v.index()) {
    case 0: return mk<false, false, float>(grid, s, c);
    case 1: return mk<true, false, float>(grid, s, c);
    case 2: return mk<false, true, float>(grid, s, c);
    case 3: return mk<true, true, float>(grid, s, c);
    case 4: return mk<false, false, double>(grid, s, c);
    case 5: return mk<true, false, double>(grid, s, c);
    case 6: return mk<false, true, double>(grid, s, c);
    default: return mk<true, true, double>(grid, s, c);
    }
}

} // namespace vgx
