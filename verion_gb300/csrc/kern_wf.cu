// Wavefront kernel variants (shaders/wf_*.slang) and the traversal-only kernels.
#include "kernels.cuh"
#include "launch.h"

namespace vgx {

template <bool L, bool R, typename A>
static cudaError_t shade(int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w, uint32_t d)
{
    vgk::wf_shade<L, R, A><<<blocks, 128, 0, s>>>(c, w, d);
    return cudaGetLastError();
}

template <bool L, bool R, typename A>
static int shade_occ()
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_shade<L, R, A>, 128, 0);
    return n > 0 ? n : 1;
}

cudaError_t launch_wf_shade(Variant v, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w, uint32_t d)
{
    switch (v.index()) {
    case 0: return shade<false, false, float>(blocks, s, c, w, d);
    case 1: return shade<true, false, float>(blocks, s, c, w, d);
    case 2: return shade<false, true, float>(blocks, s, c, w, d);
    case 3: return shade<true, true, float>(blocks, s, c, w, d);
    case 4: return shade<false, false, double>(blocks, s, c, w, d);
    case 5: return shade<true, false, double>(blocks, s, c, w, d);
    case 6: return shade<false, true, double>(blocks, s, c, w, d);
    default: return shade<true, true, double>(blocks, s, c, w, d);
    }
}

int wf_shade_blocks_per_sm(Variant v)
{
    switch (v.index()) {
    case 0: return shade_occ<false, false, float>();
    case 1: return shade_occ<true, false, float>();
    case 2: return shade_occ<false, true, float>();
    case 3: return shade_occ<true, true, float>();
    case 4: return shade_occ<false, false, double>();
    case 5: return shade_occ<true, false, double>();
    case 6: return shade_occ<false, true, double>();
    default: return shade_occ<true, true, double>();
    }
}

cudaError_t launch_wf_begin(cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w)
{
    vgk::wf_begin<<<1, 64, 0, s>>>(c, w);
    return cudaGetLastError();
}

cudaError_t launch_wf_select(bool f64, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w)
{
    unsigned blocks = (w.n + 255) / 256;
    if (f64)
        vgk::wf_select<double><<<blocks, 256, 0, s>>>(c, w);
    else
        vgk::wf_select<float><<<blocks, 256, 0, s>>>(c, w);
    return cudaGetLastError();
}

cudaError_t launch_wf_extend(bool stats, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                             uint32_t d)
{
    if (stats)
        vgk::wf_extend<true><<<blocks, 128, 0, s>>>(c, w, d);
    else
        vgk::wf_extend<false><<<blocks, 128, 0, s>>>(c, w, d);
    return cudaGetLastError();
}

int wf_extend_blocks_per_sm()
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_extend<false>, 128, 0);
    return n > 0 ? n : 1;
}

cudaError_t launch_trace_rays(int blocks, cudaStream_t s, const vgd::Ctx& c, const float* rays, uint4* out, uint32_t n,
                              uint32_t* fetch)
{
    vgk::trace_rays<<<blocks, 128, 0, s>>>(c, rays, out, n, fetch);
    return cudaGetLastError();
}

cudaError_t launch_occlusion_rays(cudaStream_t s, const vgd::Ctx& c, const float* rays, uint32_t* out, uint32_t n)
{
    vgk::occlusion_rays<<<(n + 127) / 128, 128, 0, s>>>(c, rays, out, n);
    return cudaGetLastError();
}

} // namespace vgx

namespace vgx {

template <bool L, typename A>
static cudaError_t sshade(int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w, uint32_t wave)
{
    vgk::wf_stream_shade<L, A><<<blocks, 128, 0, s>>>(c, w, wave);
    return cudaGetLastError();
}

template <bool L, typename A>
static int sshade_occ()
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_stream_shade<L, A>, 128, 0);
    return n > 0 ? n : 1;
}

cudaError_t launch_stream_start(Variant v, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w)
{
    unsigned blocks = (w.n + 255) / 256;
    if (v.light && v.f64)
        vgk::wf_stream_start<true, double><<<blocks, 256, 0, s>>>(c, w, vgk::CacheWave{});
    else if (v.light)
        vgk::wf_stream_start<true, float><<<blocks, 256, 0, s>>>(c, w, vgk::CacheWave{});
    else if (v.f64)
        vgk::wf_stream_start<false, double><<<blocks, 256, 0, s>>>(c, w, vgk::CacheWave{});
    else
        vgk::wf_stream_start<false, float><<<blocks, 256, 0, s>>>(c, w, vgk::CacheWave{});
    return cudaGetLastError();
}

cudaError_t launch_stream_extend(bool stats, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                 uint32_t wave)
{
    if (stats)
        vgk::wf_stream_extend<true><<<blocks, 128, 0, s>>>(c, w, wave);
    else
        vgk::wf_stream_extend<false><<<blocks, 128, 0, s>>>(c, w, wave);
    return cudaGetLastError();
}

cudaError_t launch_stream_shade(Variant v, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                uint32_t wave)
{
    if (v.restir)
        return launch_stream_shade_restir(v, blocks, s, c, w, wave);
    if (v.light && v.f64)
        return sshade<true, double>(blocks, s, c, w, wave);
    if (v.light)
        return sshade<true, float>(blocks, s, c, w, wave);
    if (v.f64)
        return sshade<false, double>(blocks, s, c, w, wave);
    return sshade<false, float>(blocks, s, c, w, wave);
}

int stream_shade_blocks_per_sm(Variant v)
{
    if (v.restir)
        return stream_shade_restir_blocks_per_sm(v);
    if (v.light && v.f64)
        return sshade_occ<true, double>();
    if (v.light)
        return sshade_occ<true, float>();
    if (v.f64)
        return sshade_occ<false, double>();
    return sshade_occ<false, float>();
}

} // namespace vgx

namespace vgx {

cudaError_t launch_stream_tail(Variant v, uint32_t max_slots, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                               uint32_t wave)
{
    if (v.restir)
        return launch_stream_tail_restir(v, max_slots, s, c, w, wave);
    unsigned blocks = (max_slots + 127) / 128;
    if (blocks == 0)
        return cudaSuccess;
    if (v.light && v.f64)
        vgk::wf_stream_tail<true, double><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    else if (v.light)
        vgk::wf_stream_tail<true, float><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    else if (v.f64)
        vgk::wf_stream_tail<false, double><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    else
        vgk::wf_stream_tail<false, float><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    return cudaGetLastError();
}

} // namespace vgx

namespace vgx {

cudaError_t launch_stream_shade_deferred(bool f64, bool sorted, int blocks, cudaStream_t s, const vgd::Ctx& c,
                                         const vgk::Wave& w, uint32_t wave)
{
    if (f64 && sorted)
        vgk::wf_stream_shade_deferred<double, false, false, true><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    else if (f64)
        vgk::wf_stream_shade_deferred<double><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    else if (sorted)
        vgk::wf_stream_shade_deferred<float, false, false, true><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    else
        vgk::wf_stream_shade_deferred<float><<<blocks, 128, 0, s>>>(c, w, wave, vgk::CacheWave{});
    return cudaGetLastError();
}

cudaError_t launch_stream_classify(int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w, uint32_t wave)
{
    vgk::wf_stream_classify<<<blocks, 256, 0, s>>>(c, w, wave);
    return cudaGetLastError();
}

// Radiance-cache frames (lighting split off): start without the training pixels, shade with the
// cache hook, and the tail with it.
cudaError_t launch_stream_cache_start(bool f64, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                      const vgk::CacheWave& q)
{
    unsigned blocks = (w.n + 255) / 256;
    if (f64)
        vgk::wf_stream_start<false, double, true><<<blocks, 256, 0, s>>>(c, w, q);
    else
        vgk::wf_stream_start<false, float, true><<<blocks, 256, 0, s>>>(c, w, q);
    return cudaGetLastError();
}

cudaError_t launch_stream_cache_shade(bool f64, bool sorted, int blocks, cudaStream_t s, const vgd::Ctx& c,
                                      const vgk::Wave& w, uint32_t wave, const vgk::CacheWave& q)
{
    if (f64 && sorted)
        vgk::wf_stream_shade_deferred<double, true, false, true><<<blocks, 128, 0, s>>>(c, w, wave, q);
    else if (f64)
        vgk::wf_stream_shade_deferred<double, true><<<blocks, 128, 0, s>>>(c, w, wave, q);
    else if (sorted)
        vgk::wf_stream_shade_deferred<float, true, false, true><<<blocks, 128, 0, s>>>(c, w, wave, q);
    else
        vgk::wf_stream_shade_deferred<float, true><<<blocks, 128, 0, s>>>(c, w, wave, q);
    return cudaGetLastError();
}

int stream_cache_shade_blocks_per_sm(bool f64)
{
    int n = 0;
    if (f64)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_stream_shade_deferred<double, true>, 128, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_stream_shade_deferred<float, true>, 128, 0);
    return n > 0 ? n : 1;
}

cudaError_t launch_stream_cache_tail(bool f64, uint32_t max_slots, cudaStream_t s, const vgd::Ctx& c,
                                     const vgk::Wave& w, uint32_t wave, const vgk::CacheWave& q)
{
    unsigned blocks = (max_slots + 127) / 128;
    if (blocks == 0)
        return cudaSuccess;
    if (f64)
        vgk::wf_stream_tail<false, double, true><<<blocks, 128, 0, s>>>(c, w, wave, q);
    else
        vgk::wf_stream_tail<false, float, true><<<blocks, 128, 0, s>>>(c, w, wave, q);
    return cudaGetLastError();
}

cudaError_t launch_stream_shadow(bool f64, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                 uint32_t wave)
{
    if (f64)
        vgk::wf_stream_shadow<double><<<blocks, 128, 0, s>>>(c, w, wave);
    else
        vgk::wf_stream_shadow<float><<<blocks, 128, 0, s>>>(c, w, wave);
    return cudaGetLastError();
}

int stream_finish_blocks_per_sm(bool f64)
{
    static int n[2] = {0, 0};
    int& k = n[f64 ? 1 : 0];
    if (k == 0) {
        if (f64)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, vgk::wf_stream_finish<double>, 128, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, vgk::wf_stream_finish<float>, 128, 0);
        k = k > 0 ? k : 1;
    }
    return k;
}

int stream_deferred_blocks_per_sm(bool f64, int* shadow)
{
    int n = 0, m = 0;
    if (f64) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_stream_shade_deferred<double>, 128, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, vgk::wf_stream_shadow<double>, 128, 0);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_stream_shade_deferred<float>, 128, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m, vgk::wf_stream_shadow<float>, 128, 0);
    }
    *shadow = m > 0 ? m : 1;
    return n > 0 ? n : 1;
}

} // namespace vgx

namespace vgx {

cudaError_t launch_stream_extend_dyn(bool stats, bool coop, int blocks, cudaStream_t s, const vgd::Ctx& c,
                                     const vgk::Wave& w, uint32_t wave)
{
    if (stats && coop)
        vgk::wf_stream_extend_dyn<true, true><<<blocks, 128, 0, s>>>(c, w, wave);
    else if (stats)
        vgk::wf_stream_extend_dyn<true, false><<<blocks, 128, 0, s>>>(c, w, wave);
    else if (coop)
        vgk::wf_stream_extend_dyn<false, true><<<blocks, 128, 0, s>>>(c, w, wave);
    else
        vgk::wf_stream_extend_dyn<false, false><<<blocks, 128, 0, s>>>(c, w, wave);
    return cudaGetLastError();
}

cudaError_t launch_stream_shadow_trace(bool stats, bool coop, int blocks, cudaStream_t s, const vgd::Ctx& c,
                                       const vgk::Wave& w, uint32_t wave)
{
    if (stats && coop)
        vgk::wf_stream_shadow_trace<true, true><<<blocks, 128, 0, s>>>(c, w, wave);
    else if (stats)
        vgk::wf_stream_shadow_trace<true, false><<<blocks, 128, 0, s>>>(c, w, wave);
    else if (coop)
        vgk::wf_stream_shadow_trace<false, true><<<blocks, 128, 0, s>>>(c, w, wave);
    else
        vgk::wf_stream_shadow_trace<false, false><<<blocks, 128, 0, s>>>(c, w, wave);
    return cudaGetLastError();
}

int stream_shadow_trace_blocks_per_sm()
{
    static int n = 0;
    if (n == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_stream_shadow_trace<false, false>, 128, 0);
        n = n > 0 ? n : 1;
    }
    return n;
}

int stream_trace_blocks_per_sm(bool coop)
{
    int n = 0;
    if (coop)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_stream_extend_dyn<false, true>, 128, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, vgk::wf_stream_extend_dyn<false, false>, 128, 0);
    return n > 0 ? n : 1;
}

cudaError_t launch_stream_finish(bool f64, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                 uint32_t wave)
{
    if (f64)
        vgk::wf_stream_finish<double><<<blocks, 128, 0, s>>>(c, w, wave);
    else
        vgk::wf_stream_finish<float><<<blocks, 128, 0, s>>>(c, w, wave);
    return cudaGetLastError();
}

} // namespace vgx
