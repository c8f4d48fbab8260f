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

#include "aov.cuh"

namespace vgx {

cudaError_t launch_aov_normals(cudaStream_t s, const vgd::Ctx& c, const float* camera18, float* out)
{
    vga::CameraRecord cam;
    for (int i = 0; i < 18; i++)
        cam.v[i] = camera18[i];
    uint32_t w = (uint32_t)cam.v[0], h = (uint32_t)cam.v[1];
    dim3 grid((w + 15) / 16, (h + 7) / 8);
    vga::aov_normals<<<grid, 128, 0, s>>>(c, cam, out);
    return cudaGetLastError();
}

cudaError_t launch_aov_main(cudaStream_t s, const vgd::Ctx& c, const float* camera18, float* albedo_depth,
                            uint32_t* object_ids, uint32_t* material_ids, float* coverage)
{
    vga::CameraRecord cam;
    for (int i = 0; i < 18; i++)
        cam.v[i] = camera18[i];
    uint32_t w = (uint32_t)cam.v[0], h = (uint32_t)cam.v[1];
    dim3 grid((w + 15) / 16, (h + 7) / 8);
    vga::aov_main<<<grid, 128, 0, s>>>(c, cam, albedo_depth, object_ids, material_ids, coverage);
    return cudaGetLastError();
}

} // namespace vgx
