// Host-side launchers of the radiance-cache kernels (kern_nrc.cu).
#pragma once
#include <cuda_runtime.h>

#include "ctx.h"
#include "nrc.cuh"

// Adam settings; the step count t lives on the device (nrc_launch_step advances it), so a captured
// training sequence replays with the right bias corrections.
struct NrcAdam {
    float lr, beta1, beta2, eps;
    const uint32_t* step;
};

// Path-kernel outputs: query records (one per pixel at most) and training records.
struct NrcPathArgs {
    float spread;
    uint32_t train_stride, train_offset;
    float* qrec;
    uint32_t* qcount;
    uint32_t qcap;
    float* trec;
    uint32_t* tcount;
    uint32_t tcap;
};

namespace vgx {

// Training pixels of a frame: those with (pixel + offset) % stride == 0 among px pixels; the
// smallest is *first, the others follow every `stride` pixels.
inline uint32_t nrc_train_pixels(uint64_t px, uint32_t stride, uint32_t offset, uint32_t* first)
{
    *first = (stride - offset % stride) % stride;
    return *first < px ? (uint32_t)((px - 1 - *first) / stride + 1) : 0u;
}

// Sets the cache kernels' shared-memory limits (once; before any stream capture).
void nrc_prepare();

// Input tiles of records [offset, offset + limit) of the first min(*count, cap) (kern_nrc.cu).
cudaError_t nrc_launch_encode(int blocks, cudaStream_t s, const vgn::CacheDev& cd, const float* rec,
                              const uint32_t* count, uint32_t cap, uint32_t offset, uint32_t limit, uint8_t* X);
cudaError_t nrc_launch_scatter(int blocks, cudaStream_t s, const vgn::CacheDev& cd, const float* rec,
                               const uint32_t* count, uint32_t cap, uint32_t offset, uint32_t limit, const float* GX);
cudaError_t nrc_launch_infer(int blocks, cudaStream_t s, const vgn::CacheDev& cd, const uint8_t* X, const float* rec,
                             const uint32_t* count, uint32_t cap, float* out, void* accum, int accum_bits);
cudaError_t nrc_launch_train(int blocks, cudaStream_t s, const vgn::CacheDev& cd, const uint8_t* X, const float* rec,
                             const uint32_t* count, uint32_t cap, uint32_t offset, uint32_t batch, float* GX);
cudaError_t nrc_launch_adam(cudaStream_t s, float* p, float* g, float* m, float* v, size_t n, const uint32_t* count,
                            uint32_t cap, uint32_t offset, uint32_t batch, const NrcAdam& a, void* half_out,
                            bool lazy);
cudaError_t nrc_launch_step(cudaStream_t s, uint32_t* step);
cudaError_t nrc_launch_to_half(cudaStream_t s, const float* p, void* out, size_t n);
cudaError_t nrc_launch_pack(cudaStream_t s, const float* w, uint8_t* img);
// Query paths over the 16 x 8 pixel tiles of `grid`; the training paths of the frame.
cudaError_t nrc_launch_query_paths(bool f64, dim3 grid, cudaStream_t s, const vgd::Ctx& c, const NrcPathArgs& a);
cudaError_t nrc_launch_train_paths(bool f64, cudaStream_t s, const vgd::Ctx& c, const NrcPathArgs& a);

} // namespace vgx
