// Host-side launchers of the kernel variants. The variants are compiled in separate translation
// units (kern_mk.cu, kern_wf.cu) so the build runs them in parallel.
#pragma once
#include <cuda_runtime.h>

#include "ctx.h"

namespace vgx {

// Compile-time variant of the path core: lighting split on, ReSTIR compiled in (the reference's
// `restirCompiled` specialisation constant, pt_core.slang:51-53), double-precision sums.
struct Variant {
    bool light;
    bool restir;
    bool f64;
    int index() const { return (light ? 1 : 0) | (restir ? 2 : 0) | (f64 ? 4 : 0); }
};

// The megakernel over a w x h frame; `next` is a device word (its pixel counter).
cudaError_t launch_megakernel(Variant v, int sms, uint32_t w, uint32_t h, cudaStream_t s, const vgd::Ctx& c,
                              uint32_t* next);
cudaError_t launch_wf_shade(Variant v, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w, uint32_t d);
int wf_shade_blocks_per_sm(Variant v);

cudaError_t launch_wf_begin(cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w);
cudaError_t launch_wf_select(bool f64, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w);
cudaError_t launch_wf_extend(bool stats, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w, uint32_t d);
int wf_extend_blocks_per_sm();
// Streaming wavefront (path regeneration); see kernels.cuh.
cudaError_t launch_stream_start(Variant v, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w);
cudaError_t launch_stream_extend(bool stats, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                 uint32_t wave);
cudaError_t launch_stream_shade(Variant v, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                uint32_t wave);
int stream_shade_blocks_per_sm(Variant v);
// Three-stage wave (lighting split off): shade without traversal, then the shadow stage.
cudaError_t launch_stream_cache_start(bool f64, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                      const vgk::CacheWave& q);
cudaError_t launch_stream_cache_shade(bool f64, bool sorted, int blocks, cudaStream_t s, const vgd::Ctx& c,
                                      const vgk::Wave& w, uint32_t wave, const vgk::CacheWave& q);
int stream_cache_shade_blocks_per_sm(bool f64);
cudaError_t launch_stream_cache_tail(bool f64, uint32_t max_slots, cudaStream_t s, const vgd::Ctx& c,
                                     const vgk::Wave& w, uint32_t wave, const vgk::CacheWave& q);
// With `sorted` the shade stage takes the wave's slots class by class (launch_stream_classify first).
cudaError_t launch_stream_shade_deferred(bool f64, bool sorted, int blocks, cudaStream_t s, const vgd::Ctx& c,
                                         const vgk::Wave& w, uint32_t wave);
cudaError_t launch_stream_classify(int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w, uint32_t wave);
cudaError_t launch_stream_shadow(bool f64, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                 uint32_t wave);
int stream_deferred_blocks_per_sm(bool f64, int* shadow);
// Dynamic-fetch traversal stages: extend, the shadow trace of opaque scenes, then finish.
// With `coop` the warp-cooperative leaf testing of traverse.cuh (the same hits).
cudaError_t launch_stream_extend_dyn(bool stats, bool coop, int blocks, cudaStream_t s, const vgd::Ctx& c,
                                     const vgk::Wave& w, uint32_t wave);
cudaError_t launch_stream_shadow_trace(bool stats, bool coop, int blocks, cudaStream_t s, const vgd::Ctx& c,
                                       const vgk::Wave& w, uint32_t wave);
int stream_trace_blocks_per_sm(bool coop);
// Resident 128-thread blocks per SM of the finish stage and of the shadow stage (their grids fill
// the SMs once).
int stream_finish_blocks_per_sm(bool f64);
int stream_shadow_trace_blocks_per_sm();
cudaError_t launch_stream_finish(bool f64, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                 uint32_t wave);
// The same streaming stages compiled with ReSTIR (kern_wf_restir.cu); the host runs them one
// sample per launch sequence.
cudaError_t launch_stream_shade_restir(Variant v, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                       uint32_t wave);
int stream_shade_restir_blocks_per_sm(Variant v);
cudaError_t launch_stream_tail_restir(Variant v, uint32_t max_slots, cudaStream_t s, const vgd::Ctx& c,
                                      const vgk::Wave& w, uint32_t wave);
cudaError_t launch_stream_shade_deferred_restir(bool f64, bool sorted, int blocks, cudaStream_t s, const vgd::Ctx& c,
                                                const vgk::Wave& w, uint32_t wave);
int stream_deferred_restir_blocks_per_sm(bool f64);
cudaError_t launch_stream_shadow_restir(bool f64, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                        uint32_t wave);
cudaError_t launch_stream_finish_restir(bool f64, int blocks, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                                        uint32_t wave);
// Finishes every slot still live after `wave` (at most max_slots of them) in one launch.
cudaError_t launch_stream_tail(Variant v, uint32_t max_slots, cudaStream_t s, const vgd::Ctx& c, const vgk::Wave& w,
                               uint32_t wave);
// Primary-hit AOVs (normals.slang, aov.slang); camera18 is the reference's camera record.
cudaError_t launch_aov_normals(cudaStream_t s, const vgd::Ctx& c, const float* camera18, float* out);
cudaError_t launch_aov_main(cudaStream_t s, const vgd::Ctx& c, const float* camera18, float* albedo_depth,
                            uint32_t* object_ids, uint32_t* material_ids, float* coverage);
cudaError_t launch_trace_rays(int blocks, cudaStream_t s, const vgd::Ctx& c, const float* rays, uint4* out, uint32_t n,
                              uint32_t* fetch);
cudaError_t launch_occlusion_rays(cudaStream_t s, const vgd::Ctx& c, const float* rays, uint32_t* out, uint32_t n);

} // namespace vgx
