// Device helpers of the radiance cache shared by its kernels (kern_nrc.cu) and the batch
// kernel (kern_batch.cu): the hash-grid encoding and its gradient scatter, the network input row,
// operand-tile stores, TMEM loads, MMA issue and bounded waits.
#pragma once
#include <cuda_fp16.h>

#include "nrc.cuh"
#include "tc.cuh"

namespace vgnd {

using namespace vgn;
using namespace vgtc;

constexpr uint32_t FULLM = 0xffffffffu;
constexpr unsigned long long WAIT_NS = 2000000000ull; // an MMA completion wait gives up after 2 s

static __device__ __forceinline__ uint8_t* align1024(uint8_t* p)
{
    uint32_t a = smem_u32(p);
    return p + (((a + 1023u) & ~1023u) - a);
}

static __device__ __forceinline__ unsigned long long now_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the MMA phase; false once WAIT_NS have passed (the caller stops issuing work).
static __device__ __forceinline__ bool wait_mma(uint64_t* bar, uint32_t parity)
{
    unsigned long long t0 = now_ns();
    for (;;) {
        if (bar_wait(bar, parity, 64))
            return true;
        if (now_ns() - t0 > WAIT_NS)
            return false;
    }
}

// ---- encoding ---------------------------------------------------------------------------------

// Trilinear hash-grid features of a world position, 2 per level (levels past cd.levels are 0).
// The corner weights are ((wx * wy) * wz) and the corners are summed in the order 0..7
// (bit 0 = x, bit 1 = y, bit 2 = z), in single precision.
static __device__ __forceinline__ void grid_features(const CacheDev& cd, const float* rec, float* f)
{
    float x = fminf(fmaxf((rec[0] - cd.lo[0]) * cd.inv_extent, 0.0f), 1.0f);
    float y = fminf(fmaxf((rec[1] - cd.lo[1]) * cd.inv_extent, 0.0f), 1.0f);
    float z = fminf(fmaxf((rec[2] - cd.lo[2]) * cd.inv_extent, 0.0f), 1.0f);
    uint32_t mask = (1u << cd.log2_t) - 1u;
#pragma unroll
    for (uint32_t l = 0; l < MAX_LEVELS; l++) {
        float a0 = 0.0f, a1 = 0.0f;
        if (l < cd.levels) {
            uint32_t res = cd.res[l];
            float sx = x * (float)res, sy = y * (float)res, sz = z * (float)res;
            uint32_t ix = min((uint32_t)sx, res - 1u), iy = min((uint32_t)sy, res - 1u), iz = min((uint32_t)sz, res - 1u);
            float fx = sx - (float)ix, fy = sy - (float)iy, fz = sz - (float)iz;
            bool dense = (cd.dense_mask >> l) & 1u;
            const uint32_t* g = cd.grid + ((size_t)l << cd.log2_t);
#pragma unroll
            for (uint32_t k = 0; k < 8; k++) {
                float w = ((k & 1u) ? fx : 1.0f - fx) * ((k & 2u) ? fy : 1.0f - fy);
                w = w * ((k & 4u) ? fz : 1.0f - fz);
                uint32_t e = __ldg(g + grid_index(ix + (k & 1u), iy + ((k >> 1) & 1u), iz + ((k >> 2) & 1u), res, dense, mask));
                __half2 h = *reinterpret_cast<__half2*>(&e);
                float2 v = __half22float2(h);
                a0 = a0 + w * v.x;
                a1 = a1 + w * v.y;
            }
        }
        f[2 * l] = a0;
        f[2 * l + 1] = a1;
    }
}

// Gradient of the grid features scattered to the table entries (f32 atomics).
static __device__ __forceinline__ void grid_backward(const CacheDev& cd, const float* rec, const float* g)
{
    float x = fminf(fmaxf((rec[0] - cd.lo[0]) * cd.inv_extent, 0.0f), 1.0f);
    float y = fminf(fmaxf((rec[1] - cd.lo[1]) * cd.inv_extent, 0.0f), 1.0f);
    float z = fminf(fmaxf((rec[2] - cd.lo[2]) * cd.inv_extent, 0.0f), 1.0f);
    uint32_t mask = (1u << cd.log2_t) - 1u;
    for (uint32_t l = 0; l < cd.levels; l++) {
        float g0 = g[2 * l], g1 = g[2 * l + 1];
        if (g0 == 0.0f && g1 == 0.0f)
            continue;
        uint32_t res = cd.res[l];
        float sx = x * (float)res, sy = y * (float)res, sz = z * (float)res;
        uint32_t ix = min((uint32_t)sx, res - 1u), iy = min((uint32_t)sy, res - 1u), iz = min((uint32_t)sz, res - 1u);
        float fx = sx - (float)ix, fy = sy - (float)iy, fz = sz - (float)iz;
        bool dense = (cd.dense_mask >> l) & 1u;
        float* gg = cd.grid_grad + ((size_t)l << cd.log2_t) * 2;
        for (uint32_t k = 0; k < 8; k++) {
            float w = ((k & 1u) ? fx : 1.0f - fx) * ((k & 2u) ? fy : 1.0f - fy);
            w = w * ((k & 4u) ? fz : 1.0f - fz);
            uint32_t e = grid_index(ix + (k & 1u), iy + ((k >> 1) & 1u), iz + ((k >> 2) & 1u), res, dense, mask);
            // Both features of the entry in one 8-byte atomic (an entry's pair is 8-byte aligned).
            atomicAdd(reinterpret_cast<float2*>(gg + 2 * (size_t)e), make_float2(w * g0, w * g1));
        }
    }
}

// The 64 network inputs of a record.
static __device__ __forceinline__ void input_row(const CacheDev& cd, const float* rec, float* v)
{
    grid_features(cd, rec, v);
#pragma unroll
    for (int k = 0; k < 6; k++)
        v[32 + k] = rec[3 + k] * 0.5f + 0.5f;
#pragma unroll
    for (int k = 0; k < 6; k++)
        v[38 + k] = rec[9 + k];
    v[44] = 1.0f;
#pragma unroll
    for (int k = 45; k < 64; k++)
        v[k] = 0.0f;
}

// Row m of a [rows x 64] swizzled bf16 tile.
static __device__ __forceinline__ void store_row(uint8_t* tile, uint32_t m, const float* v)
{
#pragma unroll
    for (uint32_t j = 0; j < 8; j++) {
        uint4 q;
        q.x = pack_bf16(v[8 * j], v[8 * j + 1]);
        q.y = pack_bf16(v[8 * j + 2], v[8 * j + 3]);
        q.z = pack_bf16(v[8 * j + 4], v[8 * j + 5]);
        q.w = pack_bf16(v[8 * j + 6], v[8 * j + 7]);
        *reinterpret_cast<uint4*>(tile + m * 128u + (((j ^ m) & 7u) << 4)) = q;
    }
}

// Column m (0..127) of a transposed tile: rows 0..63 of K-regions of `region` bytes each.
static __device__ __forceinline__ void store_col(uint8_t* tile, uint32_t region, uint32_t m, const float* v)
{
    uint8_t* base = tile + (m >> 6) * region;
    uint32_t c = m & 63u;
#pragma unroll
    for (uint32_t j = 0; j < 64; j++)
        *reinterpret_cast<__nv_bfloat16*>(base + sw128(j, c)) = __float2bfloat16_rn(v[j]);
}

// 64 (or 16) accumulator columns of this thread's row.
static __device__ __forceinline__ void load_acc(uint32_t taddr, float* v, int cols)
{
    tmem_ld16(taddr, v);
    if (cols > 16)
        tmem_ld16(taddr + 16, v + 16);
    if (cols > 32) {
        tmem_ld16(taddr + 32, v + 32);
        tmem_ld16(taddr + 48, v + 48);
    }
}

// Makes the tile writes visible to the tensor core, then thread 0 issues `steps` MMAs of one layer.
static __device__ __forceinline__ void issue_layer(uint32_t d, const uint8_t* A, uint32_t a_region, const uint8_t* B,
                                                   uint32_t b_region, uint32_t n, uint32_t steps, bool accumulate)
{
    uint32_t id = idesc_bf16(128, n);
    uint32_t a = smem_u32(A), b = smem_u32(B);
    for (uint32_t s = 0; s < steps; s++) {
        uint32_t ao = (s >> 2) * a_region + (s & 3u) * 32u;
        uint32_t bo = (s >> 2) * b_region + (s & 3u) * 32u;
        mma_bf16(d, sdesc(a + ao), sdesc(b + bo), id, (accumulate || s > 0) ? 1u : 0u);
    }
}


} // namespace vgnd
