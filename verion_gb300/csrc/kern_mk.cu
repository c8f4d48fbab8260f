// Megakernel variants (shaders/pathtrace.slang).
#include "kernels.cuh"
#include "launch.h"

namespace vgx {

// Persistent form: resident blocks per SM times the SMs, the work counter cleared first; else one
// 16 x 8 tile per block.
template <bool L, bool R, typename A>
static cudaError_t mk(int sms, uint32_t w, uint32_t h, cudaStream_t s, const vgd::Ctx& c, uint32_t* next)
{
    if constexpr (vgk::mk_persistent(R)) {
        static int per_sm = 0;
        if (per_sm == 0) {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, vgk::mk_pathtrace<L, R, A>, 128, 0) != cudaSuccess ||
                per_sm < 1)
                per_sm = 1;
        }
        cudaError_t e = cudaMemsetAsync(next, 0, 4, s);
        if (e != cudaSuccess)
            return e;
        vgk::mk_pathtrace<L, R, A><<<per_sm * sms, 128, 0, s>>>(c, next);
    } else {
        vgk::mk_pathtrace<L, R, A><<<dim3((w + 15) / 16, (h + 7) / 8), 128, 0, s>>>(c, next);
    }
    return cudaGetLastError();
}

cudaError_t launch_megakernel(Variant v, int sms, uint32_t w, uint32_t h, cudaStream_t s, const vgd::Ctx& c,
                              uint32_t* next)
{
    switch (v.index()) {
    case 0: return mk<false, false, float>(sms, w, h, s, c, next);
    case 1: return mk<true, false, float>(sms, w, h, s, c, next);
    case 2: return mk<false, true, float>(sms, w, h, s, c, next);
    case 3: return mk<true, true, float>(sms, w, h, s, c, next);
    case 4: return mk<false, false, double>(sms, w, h, s, c, next);
    case 5: return mk<true, false, double>(sms, w, h, s, c, next);
    case 6: return mk<false, true, double>(sms, w, h, s, c, next);
    default: return mk<true, true, double>(sms, w, h, s, c, next);
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
