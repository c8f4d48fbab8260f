// Radiance-cache kernels (no reference counterpart; see nrc.cuh for the record and network
// layout): the hash-grid encoding, inference and training on the fifth-generation tensor cores
// (tcgen05 MMA, operands in shared memory, accumulators in tensor memory), Adam, the bf16 weight
// image, and the path kernel that ends paths at the cache.
#include <cuda_fp16.h>

#include <algorithm>

#include "launch_nrc.h"
#include "nrc_device.cuh"
#include "pt_device.cuh"

namespace vgnk {

using namespace vgd;
using namespace vgn;
using namespace vgtc;
using namespace vgnd;

// ---- encoding kernel ----------------------------------------------------------------------------

// Rows [offset, end) of the first min(*count, cap) records, end = min(that, offset + limit),
// encoded as the network's input tiles: tile t holds rows offset + 128 t ... in the MMA operand
// layout (128 x 64 bf16, 128-byte swizzle), so a tile moves to shared memory in one bulk copy.
// The padding rows of the last tile are zero.
__global__ void __launch_bounds__(256) nrc_encode(CacheDev cd, const float* __restrict__ rec, const uint32_t* count,
                                                  uint32_t cap, uint32_t offset, uint32_t limit, uint8_t* X)
{
    uint32_t n = min(*count, cap);
    uint32_t end = offset < n ? min(n, offset + limit) : offset;
    uint32_t rows = end - offset;
    uint32_t padded = (rows + TILE - 1) / TILE * TILE;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < padded; r += gridDim.x * blockDim.x) {
        float v[64];
        if (r < rows) {
            input_row(cd, rec + (size_t)(offset + r) * REC_WORDS, v);
        } else {
#pragma unroll
            for (int k = 0; k < 64; k++)
                v[k] = 0.0f;
        }
        store_row(X + (size_t)(r / TILE) * 16384u, r % TILE, v);
    }
}

// Scatters the input-gradient grid columns of rows [offset, end) (GX: 32 floats per row, row r of
// the batch at GX + 32 r) to the table gradient.
__global__ void __launch_bounds__(256) nrc_grid_scatter(CacheDev cd, const float* __restrict__ rec,
                                                        const uint32_t* count, uint32_t cap, uint32_t offset,
                                                        uint32_t limit, const float* __restrict__ GX)
{
    uint32_t n = min(*count, cap);
    uint32_t end = offset < n ? min(n, offset + limit) : offset;
    uint32_t rows = end - offset;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        float g[32];
        const float4* src = reinterpret_cast<const float4*>(GX + (size_t)r * 32);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            float4 q = src[k];
            g[4 * k] = q.x, g[4 * k + 1] = q.y, g[4 * k + 2] = q.z, g[4 * k + 3] = q.w;
        }
        grid_backward(cd, rec + (size_t)(offset + r) * REC_WORDS, g);
    }
}

// ---- inference ----------------------------------------------------------------------------------

// Over the encoded tiles X of the first min(*count, cap) records. MODE 0: out[3 i + k] =
// prediction k of record i. MODE 1: the prediction, clamped at zero and times the record's
// throughput, is added to the record's pixel in `accum`. Each CTA walks tiles blockIdx.x,
// blockIdx.x + gridDim.x, ... with two input buffers: the next tile's bulk copy runs while the
// current one goes through the five layers (MMA into tensor memory, then bias-free ReLU epilogue
// back into the same buffer as the next layer's operand).
template <int MODE, typename A>
__global__ void __launch_bounds__(128) nrc_infer(CacheDev cd, const uint8_t* __restrict__ X,
                                                 const float* __restrict__ rec, const uint32_t* count, uint32_t cap,
                                                 float* out, A* accum)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* sm = align1024(smem_raw);
    uint8_t* W = sm;
    uint8_t* buf[2] = {sm + IMG_FWD_BYTES, sm + IMG_FWD_BYTES + 16384};
    __shared__ uint64_t mbar, lbar[2];
    __shared__ uint32_t tslot;
    uint32_t tid = threadIdx.x, warp = tid >> 5;
    uint32_t n = min(*count, cap);
    uint32_t tiles = (n + TILE - 1) / TILE;
    for (uint32_t i = tid; i < IMG_FWD_BYTES / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(W)[i] = __ldg(reinterpret_cast<const uint4*>(cd.img) + i);
    if (tid == 0) {
        bar_init(&mbar, 1);
        bar_init(&lbar[0], 1);
        bar_init(&lbar[1], 1);
        fence_bar_init();
    }
    if (warp == 0)
        tmem_alloc(&tslot, 64);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    uint32_t issued[2] = {0, 0}, used[2] = {0, 0}; // bulk copies per buffer (issued by thread 0)
    if (tid == 0) {
        for (uint32_t b = 0; b < 2; b++) {
            uint32_t t = blockIdx.x + b * gridDim.x;
            if (t < tiles) {
                bar_expect_tx(&lbar[b], 16384);
                bulk_g2s(buf[b], X + (size_t)t * 16384u, 16384, &lbar[b]);
                issued[b]++;
            }
        }
    }
    uint32_t tmem = tslot;
    uint32_t lane_addr = tmem + ((warp * 32u) << 16);
    uint32_t phase = 0;
    bool ok = true;
    uint32_t k = 0;
    for (uint32_t t = blockIdx.x; t < tiles && ok; t += gridDim.x, k++) {
        uint8_t* H = buf[k & 1u];
        ok = __syncthreads_and(wait_mma(&lbar[k & 1u], (k >> 1) & 1u)) != 0;
        if (!ok)
            break;
        used[k & 1u]++;
        float v[64];
        for (uint32_t l = 0; l < 5 && ok; l++) {
            fence_async_smem();
            __syncthreads();
            tc_fence_after();
            if (tid == 0) {
                const uint8_t* B = W + (l < 4 ? IMG_W + l * 8192u : IMG_W4);
                issue_layer(tmem, H, 0, B, 0, l < 4 ? 64u : 16u, 4, false);
                mma_commit(&mbar);
            }
            bool done = wait_mma(&mbar, phase);
            phase ^= 1u;
            ok = __syncthreads_and(done) != 0;
            if (!ok)
                break;
            tc_fence_after();
            load_acc(lane_addr, v, l < 4 ? 64 : 16);
            tc_fence_before();
            if (l < 4) {
#pragma unroll
                for (int q = 0; q < 64; q++)
                    v[q] = fmaxf(v[q], 0.0f);
                store_row(H, tid, v);
            }
        }
        if (!ok)
            break;
        uint32_t i = t * TILE + tid;
        if (i < n) {
            if (MODE == 0) {
                out[3 * (size_t)i] = v[0];
                out[3 * (size_t)i + 1] = v[1];
                out[3 * (size_t)i + 2] = v[2];
            } else {
                const float* r = rec + (size_t)i * REC_WORDS;
                uint32_t px = __float_as_uint(r[19]);
                A* a = accum + 3 * (size_t)px;
                a[0] += (A)(r[16] * fmaxf(v[0], 0.0f));
                a[1] += (A)(r[17] * fmaxf(v[1], 0.0f));
                a[2] += (A)(r[18] * fmaxf(v[2], 0.0f));
            }
        }
        // The buffer is free (its last reader, the output layer's MMA, has completed): refill it
        // with the tile after next once the generic writes are ordered before the async copy.
        fence_async_smem();
        __syncthreads();
        uint32_t nt = t + 2 * gridDim.x;
        if (tid == 0 && nt < tiles) {
            bar_expect_tx(&lbar[k & 1u], 16384);
            bulk_g2s(H, X + (size_t)nt * 16384u, 16384, &lbar[k & 1u]);
            issued[k & 1u]++;
        }
    }
    // After an early stop, a copy still in flight must land (bounded wait) before the CTA exits.
    if (!ok && tid == 0) {
        atomicOr(cd.err, ERR_MMA_TIMEOUT);
        for (uint32_t b = 0; b < 2; b++)
            if (issued[b] > used[b])
                wait_mma(&lbar[b], used[b] & 1u);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        tmem_free(tmem, 64);
}

// ---- training -----------------------------------------------------------------------------------

// Shared-memory plan of the training kernel (bytes from a 1024-aligned base).
constexpr uint32_t T_H = IMG_BYTES;            // 128 x 64 inputs, then activations (forward A operand)
constexpr uint32_t T_HT = T_H + 16384;         // 5 transposed activations, 64 x 128 each
constexpr uint32_t T_G = T_HT + 5 * 16384;     // 128 x 64 gradients (backward A operand)
constexpr uint32_t T_GT = T_G + 16384;         // 128 x 128 transposed gradients, rows 64..127 zero
constexpr uint32_t T_END = T_GT + 32768;       // 223,232
constexpr uint32_t TRAIN_SMEM = T_END + 1024;  // with the alignment slack
constexpr uint32_t INFER_SMEM = IMG_FWD_BYTES + 2 * 16384 + 1024;

// One training pass over the encoded tiles X of records [offset, end) (end as in nrc_encode):
// the relative L2 loss sum_k (p_k - y_k)^2 / (p_k^2 + 0.01) (denominator held constant) is
// summed into cd.loss and its weight gradients into cd.mlp_grad; the gradient of the 32 grid
// inputs of batch row r goes to GX + 32 r (nrc_grid_scatter takes it to the table). Per
// 128-record tile: forward (5 MMA layers), then for each layer from the last, the weight
// gradient dW_l += G^T H_l (accumulated in tensor memory over the tiles of this CTA) and the
// data gradient G W_l, masked by the ReLU of the layer below.
__global__ void __launch_bounds__(128, 1) nrc_train(CacheDev cd, const uint8_t* __restrict__ X,
                                                    const float* __restrict__ rec, const uint32_t* count,
                                                    uint32_t cap, uint32_t offset, uint32_t batch, float* GX)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* sm = align1024(smem_raw);
    uint8_t* W = sm;
    uint8_t* H = sm + T_H;
    uint8_t* HT = sm + T_HT;
    uint8_t* G = sm + T_G;
    uint8_t* GT = sm + T_GT;
    __shared__ uint64_t mbar, lbar;
    __shared__ uint32_t tslot;
    __shared__ float red[4];
    uint32_t tid = threadIdx.x, warp = tid >> 5;
    for (uint32_t i = tid; i < IMG_BYTES / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(W)[i] = __ldg(reinterpret_cast<const uint4*>(cd.img) + i);
    for (uint32_t i = tid; i < 32768 / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(GT)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        bar_init(&mbar, 1);
        bar_init(&lbar, 1);
        fence_bar_init();
    }
    if (warp == 0)
        tmem_alloc(&tslot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    uint32_t tmem = tslot;
    uint32_t lane_addr = tmem + ((warp * 32u) << 16);
    uint32_t n = min(*count, cap);
    uint32_t end = offset < n ? min(n, offset + batch) : offset;
    uint32_t tiles = end > offset ? (end - offset + TILE - 1) / TILE : 0;
    uint32_t phase = 0, lphase = 0;
    bool ok = true, first = true, copy_late = false;
    float loss = 0.0f;
    for (uint32_t t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        // The previous tile is done with H: bring in this tile's inputs.
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            bar_expect_tx(&lbar, 16384);
            bulk_g2s(H, X + (size_t)t * 16384u, 16384, &lbar);
        }
        ok = __syncthreads_and(wait_mma(&lbar, lphase)) != 0;
        if (!ok) {
            copy_late = true;
            break;
        }
        lphase ^= 1u;
        uint32_t row = t * TILE + tid;
        uint32_t i = offset + row;
        bool valid = i < end;
        const float* r = rec + (size_t)i * REC_WORDS;
        float v[64];
#pragma unroll
        for (uint32_t j = 0; j < 8; j++) {
            uint4 q = *reinterpret_cast<const uint4*>(H + tid * 128u + (((j ^ tid) & 7u) << 4));
            const __nv_bfloat162* h2 = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                float2 f = __bfloat1622float2(h2[e]);
                v[8 * j + 2 * e] = f.x;
                v[8 * j + 2 * e + 1] = f.y;
            }
        }
        store_col(HT, 8192, tid, v);
        uint32_t mask[4][2];
        // Forward.
#pragma unroll
        for (uint32_t l = 0; l < 5; l++) {
            fence_async_smem();
            __syncthreads();
            tc_fence_after();
            if (tid == 0) {
                const uint8_t* B = W + (l < 4 ? IMG_W + l * 8192u : IMG_W4);
                issue_layer(tmem, H, 0, B, 0, l < 4 ? 64u : 16u, 4, false);
                mma_commit(&mbar);
            }
            bool done = wait_mma(&mbar, phase);
            phase ^= 1u;
            ok = __syncthreads_and(done) != 0;
            if (!ok)
                break;
            tc_fence_after();
            load_acc(lane_addr, v, l < 4 ? 64 : 16);
            tc_fence_before();
            if (l < 4) {
                uint32_t m0 = 0, m1 = 0;
#pragma unroll
                for (int q = 0; q < 64; q++) {
                    bool on = v[q] > 0.0f;
                    if (q < 32)
                        m0 |= (on ? 1u : 0u) << q;
                    else
                        m1 |= (on ? 1u : 0u) << (q - 32);
                    v[q] = on ? v[q] : 0.0f;
                }
                mask[l][0] = m0;
                mask[l][1] = m1;
                store_row(H, tid, v);
                store_col(HT + (l + 1) * 16384u, 8192, tid, v);
            }
        }
        if (!ok)
            break;
        // Loss gradient of the three outputs.
        float g[64];
#pragma unroll
        for (int q = 0; q < 64; q++)
            g[q] = 0.0f;
        if (valid) {
#pragma unroll
            for (int q = 0; q < 3; q++) {
                float d = v[q] - r[16 + q];
                float den = v[q] * v[q] + 0.01f;
                loss += d * d / den;
                g[q] = 2.0f * d / den;
            }
        }
        store_row(G, tid, g);
        store_col(GT, 16384, tid, g);
        // Backward.
#pragma unroll
        for (int l = 4; l >= 0; l--) {
            fence_async_smem();
            __syncthreads();
            tc_fence_after();
            if (tid == 0) {
                issue_layer(tmem + 64u + 64u * l, GT, 16384, HT + l * 16384u, 8192, 64, 8, !first);
                const uint8_t* B = W + (l == 4 ? IMG_W4T : IMG_WT + l * 8192u);
                issue_layer(tmem, G, 0, B, 0, 64, l == 4 ? 1u : 4u, false);
                mma_commit(&mbar);
            }
            bool done = wait_mma(&mbar, phase);
            phase ^= 1u;
            ok = __syncthreads_and(done) != 0;
            if (!ok)
                break;
            tc_fence_after();
            load_acc(lane_addr, g, l > 0 ? 64 : 32);
            tc_fence_before();
            if (l > 0) {
#pragma unroll
                for (int q = 0; q < 64; q++) {
                    uint32_t bit = q < 32 ? (mask[l - 1][0] >> q) & 1u : (mask[l - 1][1] >> (q - 32)) & 1u;
                    g[q] = bit ? g[q] : 0.0f;
                }
                store_row(G, tid, g);
                store_col(GT, 16384, tid, g);
            } else if (valid) {
                float4* dst = reinterpret_cast<float4*>(GX + (size_t)row * 32);
#pragma unroll
                for (int q = 0; q < 8; q++)
                    dst[q] = make_float4(g[4 * q], g[4 * q + 1], g[4 * q + 2], g[4 * q + 3]);
            }
        }
        first = false;
    }
    // Weight gradients: rows 0..63 of each accumulator (0..15 for the output layer) live in the
    // lanes of warps 0 and 1.
    if (ok && !first && warp < 2) {
        tc_fence_after();
        for (uint32_t l = 0; l < 5; l++) {
            float v[64];
            load_acc(lane_addr + 64u + 64u * l, v, 64);
            uint32_t rows = l < 4 ? 64u : 16u;
            if (tid < rows) {
                float* dst = cd.mlp_grad + mlp_offset(l) + tid * WIDTH;
#pragma unroll
                for (int q = 0; q < 64; q++)
                    atomicAdd(dst + q, v[q]);
            }
        }
    }
    if (!ok && tid == 0) {
        atomicOr(cd.err, ERR_MMA_TIMEOUT);
        if (copy_late)
            wait_mma(&lbar, lphase); // the input copy must land before the CTA exits
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        loss += __shfl_xor_sync(FULLM, loss, o);
    if ((tid & 31u) == 0)
        red[warp] = loss;
    tc_fence_before();
    __syncthreads();
    if (tid == 0 && cd.loss)
        atomicAdd(cd.loss, (double)red[0] + (double)red[1] + (double)red[2] + (double)red[3]);
    if (warp == 0)
        tmem_free(tmem, 512);
}

// ---- optimiser and weight image ---------------------------------------------------------------

// Adam (Kingma and Ba 2015) on the gradient sums of the step, scaled by 1 / (3 x records used);
// a step without records changes nothing. The gradient sums are cleared. With `half_out` the
// updated parameter is also written as fp16 (the grid table).
// With `lazy`, entries whose gradient sum is exactly zero are left alone (their moments do not
// decay): the grid table, where a step touches a small fraction of the entries.
__global__ void nrc_adam(float* p, float* g, float* m, float* v, size_t n, const uint32_t* count, uint32_t cap,
                         uint32_t offset, uint32_t batch, NrcAdam a, __half* half_out, bool lazy)
{
    uint32_t avail = min(*count, cap);
    uint32_t used = avail > offset ? min(batch, avail - offset) : 0u;
    if (used == 0)
        return;
    float scale = 1.0f / (3.0f * (float)used);
    float t = (float)*a.step;
    float bc1 = 1.0f - powf(a.beta1, t), bc2 = 1.0f - powf(a.beta2, t);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float gs = g[i];
        if (lazy && gs == 0.0f)
            continue;
        float gi = gs * scale;
        g[i] = 0.0f;
        float mi = a.beta1 * m[i] + (1.0f - a.beta1) * gi;
        float vi = a.beta2 * v[i] + (1.0f - a.beta2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        float pi = p[i] - a.lr * (mi / bc1) / (sqrtf(vi / bc2) + a.eps);
        p[i] = pi;
        if (half_out)
            half_out[i] = __float2half_rn(pi);
    }
}

// Advances the Adam step count.
__global__ void nrc_step(uint32_t* step) { *step += 1u; }

// fp16 copy of the f32 grid parameters.
__global__ void nrc_to_half(const float* p, __half* out, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __float2half_rn(p[i]);
}

// The bf16 weight image from the f32 parameters (see nrc.cuh).
__global__ void nrc_pack(const float* w, uint8_t* img)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= MLP_PARAMS)
        return;
    __nv_bfloat16 b = __float2bfloat16_rn(w[i]);
    uint32_t l = min(i / (WIDTH * WIDTH), 4u);
    uint32_t j = i - l * WIDTH * WIDTH;
    uint32_t o = j / WIDTH, k = j % WIDTH;
    if (l < 4) {
        *reinterpret_cast<__nv_bfloat16*>(img + IMG_W + l * 8192u + sw128(o, k)) = b;
        *reinterpret_cast<__nv_bfloat16*>(img + IMG_WT + l * 8192u + sw128(k, o)) = b;
    } else {
        *reinterpret_cast<__nv_bfloat16*>(img + IMG_W4 + sw128(o, k)) = b;
        *reinterpret_cast<__nv_bfloat16*>(img + IMG_W4T + sw128(k, o)) = b;
    }
}

// ---- path kernel --------------------------------------------------------------------------------

constexpr uint32_t MAX_TRAIN_VERTICES = 16;

// Reserves k consecutive slots per lane with one atomic per warp; every lane of the warp calls it.
static __device__ __forceinline__ uint32_t warp_reserve(uint32_t* ctr, uint32_t k)
{
    uint32_t lane = threadIdx.x & 31u;
    uint32_t incl = k;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(FULLM, incl, o);
        if (lane >= o)
            incl += y;
    }
    uint32_t total = __shfl_sync(FULLM, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && total)
        base = atomicAdd(ctr, total);
    base = __shfl_sync(FULLM, base, 31);
    return base + incl - k;
}

static_assert(REC_WORDS == CACHE_REC_WORDS, "cache record layout");

// One sample per pixel (sample index P_SAMPLE). A path ends at the first vertex where its
// spread passes the threshold and leaves a query record (its radiance past that vertex comes
// from the cache); one pixel in `train_stride` (offset by the frame) traces a training path
// instead, which never ends for a query and leaves one training record per vertex with the
// radiance the rest of the path brought, divided by the throughput reaching the vertex.
// The two kinds run as separate kernels, so that the short query paths of a warp are not held
// up by a training path's full depth: mk_cache_query over 16 x 8 pixel tiles (training pixels
// idle), mk_cache_train over the training pixels only.
static __device__ __forceinline__ bool is_train_pixel(const NrcPathArgs& a, uint32_t pixel)
{
    return (pixel + a.train_offset) % a.train_stride == 0;
}

// Minimum resident 128-thread blocks per SM requested for the whole-path kernels of the cache
// integrator (a register cap; 0: none). Unlike the megakernel they gain little: per sample of the
// Cornell box's cache frames 1.22 ms with no cap, 1.28 at 8 blocks and 1.52 at 16 blocks for the
// one-kernel query paths; on the wavefront (training paths only) within 2%.
#ifndef VG_CACHE_PATH_MIN_BLOCKS
#define VG_CACHE_PATH_MIN_BLOCKS 0
#endif
#if VG_CACHE_PATH_MIN_BLOCKS > 0
#define VG_CACHE_PATH_BOUNDS __launch_bounds__(128, VG_CACHE_PATH_MIN_BLOCKS)
#else
#define VG_CACHE_PATH_BOUNDS __launch_bounds__(128)
#endif

template <typename A>
__global__ void VG_CACHE_PATH_BOUNDS mk_cache_query(const __grid_constant__ Ctx c, NrcPathArgs a)
{
    uint32_t x = blockIdx.x * 16 + (threadIdx.x & 15u);
    uint32_t y = blockIdx.y * 8 + (threadIdx.x >> 4);
    uint32_t pixel = y * c.p[P_WIDTH] + x;
    bool inside = x < c.p[P_WIDTH] && y < c.p[P_HEIGHT] && !is_train_pixel(a, pixel);
    CacheHook hk;
    hk.c = a.spread;
    hk.train = false;
    hk.a0 = hk.a = 0.0f;
    hk.query = false;
    bool query = false;
    PathState<false> st;
    if (inside) {
        st = generatePathFor<false>(c, x, y, c.p[P_SAMPLE]);
        for (uint32_t depth = 0; depth < c.p[P_MAX_DEPTH]; depth++) {
            bool alive = shadePathCall<false, false, false, true>(c, st, traceClosest(c, st.org, st.dir), depth, pixel,
                                                              nullptr, &hk);
            if (hk.query) {
                query = true;
                break;
            }
            if (!alive)
                break;
        }
        finishPath<false, A>(c, st, pixel);
    }
    bool ok = inside && !bad3(st.parts.total);
    uint32_t q = warp_reserve(a.qcount, (query && ok) ? 1u : 0u);
    if (query && ok && q < a.qcap)
        cacheQueryRecord(a.qrec + (size_t)q * REC_WORDS, hk, pixel);
}

// Training pixels: pixel = first + k * train_stride for thread k, first = the smallest pixel with
// (pixel + train_offset) % train_stride == 0; each traces the frame's P_SAMPLES_PER_DISPATCH
// samples one after the other.
template <typename A>
__global__ void VG_CACHE_PATH_BOUNDS mk_cache_train(const __grid_constant__ Ctx c, NrcPathArgs a, uint32_t first,
                                                      uint32_t count)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    bool inside = k < count;
    uint32_t pixel = first + k * a.train_stride;
    uint32_t w = c.p[P_WIDTH];
    uint32_t x = inside ? pixel % w : 0u, y = inside ? pixel / w : 0u;
    CacheHook hk;
    hk.c = a.spread;
    hk.train = true;
    hk.a0 = hk.a = 0.0f;
    hk.query = false;
    float feat[MAX_TRAIN_VERTICES][16];
    V3 thr[MAX_TRAIN_VERTICES], Lb[MAX_TRAIN_VERTICES];
    for (uint32_t ks = 0; ks < c.p[P_SAMPLES_PER_DISPATCH]; ks++) {
        uint32_t nv = 0;
        hk.a0 = hk.a = 0.0f;
        PathState<false> st;
        if (inside) {
            st = generatePathFor<false>(c, x, y, c.p[P_SAMPLE] + ks);
            for (uint32_t depth = 0; depth < c.p[P_MAX_DEPTH]; depth++) {
                bool alive = shadePathCall<false, false, false, true>(c, st, traceClosest(c, st.org, st.dir), depth, pixel,
                                                                  nullptr, &hk);
                if (hk.vertex && nv < MAX_TRAIN_VERTICES) {
                    cacheFeatures(feat[nv], hk);
                    thr[nv] = hk.thr;
                    Lb[nv] = hk.L;
                    nv++;
                }
                if (!alive)
                    break;
            }
            finishPath<false, A>(c, st, pixel);
        }
        bool ok = inside && !bad3(st.parts.total);
        uint32_t nt = ok ? nv : 0u;
        uint32_t t0 = warp_reserve(a.tcount, nt);
        for (uint32_t j = 0; j < nt; j++) {
            if (t0 + j >= a.tcap)
                break;
            float* d = a.trec + (size_t)(t0 + j) * REC_WORDS;
            V3 rest = st.parts.total - Lb[j];
            V3 t = thr[j];
            for (int q = 0; q < 16; q++)
                d[q] = feat[j][q];
            d[16] = t.x > 0.0f ? rest.x / t.x : 0.0f;
            d[17] = t.y > 0.0f ? rest.y / t.y : 0.0f;
            d[18] = t.z > 0.0f ? rest.z / t.z : 0.0f;
            d[19] = 0.0f;
        }
    }
}

} // namespace vgnk

namespace vgx {

using namespace vgnk;

void nrc_prepare()
{
    static bool done = false;
    if (done)
        return;
    cudaFuncSetAttribute(nrc_infer<0, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, INFER_SMEM);
    cudaFuncSetAttribute(nrc_infer<1, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, INFER_SMEM);
    cudaFuncSetAttribute(nrc_infer<1, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, INFER_SMEM);
    cudaFuncSetAttribute(nrc_train, cudaFuncAttributeMaxDynamicSharedMemorySize, TRAIN_SMEM);
    done = true;
}

cudaError_t nrc_launch_encode(int blocks, cudaStream_t s, const vgn::CacheDev& cd, const float* rec,
                              const uint32_t* count, uint32_t cap, uint32_t offset, uint32_t limit, uint8_t* X)
{
    nrc_encode<<<blocks, 256, 0, s>>>(cd, rec, count, cap, offset, limit, X);
    return cudaGetLastError();
}

cudaError_t nrc_launch_scatter(int blocks, cudaStream_t s, const vgn::CacheDev& cd, const float* rec,
                               const uint32_t* count, uint32_t cap, uint32_t offset, uint32_t limit, const float* GX)
{
    nrc_grid_scatter<<<blocks, 256, 0, s>>>(cd, rec, count, cap, offset, limit, GX);
    return cudaGetLastError();
}

cudaError_t nrc_launch_infer(int blocks, cudaStream_t s, const vgn::CacheDev& cd, const uint8_t* X, const float* rec,
                             const uint32_t* count, uint32_t cap, float* out, void* accum, int accum_bits)
{
    nrc_prepare();
    if (!accum)
        nrc_infer<0, float><<<blocks, 128, INFER_SMEM, s>>>(cd, X, rec, count, cap, out, (float*)nullptr);
    else if (accum_bits == 64)
        nrc_infer<1, double><<<blocks, 128, INFER_SMEM, s>>>(cd, X, rec, count, cap, nullptr, (double*)accum);
    else
        nrc_infer<1, float><<<blocks, 128, INFER_SMEM, s>>>(cd, X, rec, count, cap, nullptr, (float*)accum);
    return cudaGetLastError();
}

cudaError_t nrc_launch_train(int blocks, cudaStream_t s, const vgn::CacheDev& cd, const uint8_t* X, const float* rec,
                             const uint32_t* count, uint32_t cap, uint32_t offset, uint32_t batch, float* GX)
{
    nrc_prepare();
    nrc_train<<<blocks, 128, TRAIN_SMEM, s>>>(cd, X, rec, count, cap, offset, batch, GX);
    return cudaGetLastError();
}

cudaError_t nrc_launch_adam(cudaStream_t s, float* p, float* g, float* m, float* v, size_t n, const uint32_t* count,
                            uint32_t cap, uint32_t offset, uint32_t batch, const NrcAdam& a, void* half_out, bool lazy)
{
    int blocks = (int)std::min<size_t>((n + 255) / 256, 8192);
    nrc_adam<<<blocks, 256, 0, s>>>(p, g, m, v, n, count, cap, offset, batch, a, (__half*)half_out, lazy);
    return cudaGetLastError();
}

cudaError_t nrc_launch_step(cudaStream_t s, uint32_t* step)
{
    nrc_step<<<1, 1, 0, s>>>(step);
    return cudaGetLastError();
}

cudaError_t nrc_launch_to_half(cudaStream_t s, const float* p, void* out, size_t n)
{
    int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
    nrc_to_half<<<blocks, 256, 0, s>>>(p, (__half*)out, n);
    return cudaGetLastError();
}

cudaError_t nrc_launch_pack(cudaStream_t s, const float* w, uint8_t* img)
{
    nrc_pack<<<(vgn::MLP_PARAMS + 255) / 256, 256, 0, s>>>(w, img);
    return cudaGetLastError();
}

cudaError_t nrc_launch_query_paths(bool f64, dim3 grid, cudaStream_t s, const vgd::Ctx& c, const NrcPathArgs& a)
{
    if (f64)
        mk_cache_query<double><<<grid, 128, 0, s>>>(c, a);
    else
        mk_cache_query<float><<<grid, 128, 0, s>>>(c, a);
    return cudaGetLastError();
}

cudaError_t nrc_launch_train_paths(bool f64, cudaStream_t s, const vgd::Ctx& c, const NrcPathArgs& a)
{
    uint32_t first;
    uint32_t count = nrc_train_pixels((uint64_t)c.p[P_WIDTH] * c.p[P_HEIGHT], a.train_stride, a.train_offset, &first);
    if (count == 0)
        return cudaSuccess;
    if (f64)
        mk_cache_train<double><<<(count + 127) / 128, 128, 0, s>>>(c, a, first, count);
    else
        mk_cache_train<float><<<(count + 127) / 128, 128, 0, s>>>(c, a, first, count);
    return cudaGetLastError();
}

} // namespace vgx
