// The streaming-wavefront kernels compiled with ReSTIR (kernels.cuh, RESTIR = true): a translation
// unit of their own so the build compiles them beside the plain variants (kern_wf.cu). Under
// ReSTIR the host runs one sample per launch sequence, so the reservoirs of the previous sample
// (the other frame parity) are complete before any path of the current sample reads them, as in
// the reference's one-sample dispatches (crates/verion-gpu-metal/src/renderer.rs:459-463).
#include "kernels.cuh"
#include "launch.h"

namespace vgx {

template <bool L, typename A>
static int rshade_occ()
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_stream_shade<L, A, true>, 128, 0);
    return n > 0 ? n : 1;
}

cudaError_t launch_stream_shade_restir(Variant v, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                       uint32_t wave)
{
    if (v.light && v.f64)
        vgk::wf_stream_shade<true, double, true><<<blocks, 128, 0, s>>>(c, w, wave);
    else if (v.light)
        vgk::wf_stream_shade<true, float, true><<<blocks, 128, 0, s>>>(c, w, wave);
    else if (v.f64)
        vgk::wf_stream_shade<false, double, true><<<blocks, 128, 0, s>>>(c, w, wave);
    else
        vgk::wf_stream_shade<false, float, true><<<blocks, 128, 0, s>>>(c, w, wave);
    return cudaGetLastError();
}

int stream_shade_restir_blocks_per_sm(Variant v)
{
    if (v.light && v.f64)
        return rshade_occ<true, double>();
    if (v.light)
        return rshade_occ<true, float>();
    if (v.f64)
        return rshade_occ<false, double>();
    return rshade_occ<false, float>();
}

cudaError_t launch_stream_tail_restir(Variant v, uint32_t max_slots, cudaStream_t s, const vgd::Ctx& c,
                                      const vgk::Wave& w, uint32_t wave)
{
    unsigned blocks = (max_slots + 127) / 128;
    if (blocks == 0)
        return cudaSuccess;
    if (v.light && v.f64)
        vgk::wf_stream_tail<true, double, false, true><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    else if (v.light)
        vgk::wf_stream_tail<true, float, false, true><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    else if (v.f64)
        vgk::wf_stream_tail<false, double, false, true><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    else
        vgk::wf_stream_tail<false, float, false, true><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    return cudaGetLastError();
}

cudaError_t launch_stream_shade_deferred_restir(bool f64, bool sorted, int blocks, cudaStream_t s, const vgd::Ctx& c,
                                                const vgk::Wave& w, uint32_t wave)
{
    if (f64 && sorted)
        vgk::wf_stream_shade_deferred<double, false, true, true><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    else if (f64)
        vgk::wf_stream_shade_deferred<double, false, true><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    else if (sorted)
        vgk::wf_stream_shade_deferred<float, false, true, true><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    else
        vgk::wf_stream_shade_deferred<float, false, true><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    return cudaGetLastError();
}

cudaError_t launch_stream_shadow_restir(bool f64, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                        uint32_t wave)
{
    if (f64)
        vgk::wf_stream_shadow<double, true><<<blocks, 128, 0, s>>>(c, w, wave);
    else
        vgk::wf_stream_shadow<float, true><<<blocks, 128, 0, s>>>(c, w, wave);
    return cudaGetLastError();
}

cudaError_t launch_stream_finish_restir(bool f64, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                        uint32_t wave)
{
    if (f64)
        vgk::wf_stream_finish<double, true><<<blocks, 128, 0, s>>>(c, w, wave);
    else
        vgk::wf_stream_finish<float, true><<<blocks, 128, 0, s>>>(c, w, wave);
    return cudaGetLastError();
}

int stream_deferred_restir_blocks_per_sm(bool f64)
{
    int n = 0;
    if (f64)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_stream_shade_deferred<double, false, true, true>, 128, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_stream_shade_deferred<float, false, true, true>, 128, 0);
    return n > 0 ? n : 1;
}

} // namespace vgx
