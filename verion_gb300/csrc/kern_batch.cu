// Batched rendering (vg_batch_render; no reference counterpart): the work items of many requests
// (each a 16 x 8 pixel tile of one request with all of that request's samples) in one persistent
// launch. CTAs take items in the order the host laid them out (shortest request first) with one
// atomic each. A plain request's tile runs exactly what the megakernel runs (pathtrace.slang:9-26),
// so its sums equal a megakernel accumulate bit for bit. A cached request's tile ends its paths at
// the radiance cache and evaluates the cache for its 128 pixels in the same CTA: the tile is one
// M = 128 tcgen05 MMA tile, so the queries never leave the SM (the fused form of nrc_encode +
// nrc_infer).
#include <algorithm>

#include "batch.h"
#include "launch_batch.h"
#include "nrc_device.cuh"
#include "pt_device.cuh"

namespace vgbk {

using namespace vgd;
using namespace vgn;
using namespace vgtc;
using namespace vgnd;
using namespace vgb;

constexpr uint32_t BATCH_SMEM = IMG_FWD_BYTES + 16384 + 1024;

// Register cap of the batch kernel: at least this many 128-thread CTAs per SM.
#ifndef VG_BATCH_MIN_BLOCKS
#define VG_BATCH_MIN_BLOCKS 3
#endif
constexpr uint32_t MAX_TRAIN_VERTICES = 16;
static_assert(sizeof(BatchReq) % 16 == 0, "BatchReq is copied to shared memory in 16-byte words");

// Reserves k consecutive slots per lane with one atomic per warp; every lane of the warp calls it.
static __device__ __forceinline__ uint32_t reserve(uint32_t* ctr, uint32_t k)
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

template <typename A>
static __device__ __forceinline__ void plain_tile(const Ctx& c, uint32_t x, uint32_t y, bool inside)
{
    if (!inside)
        return;
    uint32_t pixel = y * c.p[P_WIDTH] + x;
    uint32_t n = c.p[P_SAMPLES_PER_DISPATCH];
    if (n == 0)
        return;
    // One loop over bounces, a path's end starting the pixel's next sample (mk_pathtrace).
    uint32_t k = 0, depth = 0;
    PathState<false> st = generatePathFor<false>(c, x, y, c.p[P_SAMPLE]);
    for (;;) {
        if (shadePathCall<false, false>(c, st, traceClosest(c, st.org, st.dir), depth, pixel) &&
            depth + 1 < c.p[P_MAX_DEPTH]) {
            depth++;
            continue;
        }
        finishPath<false, A>(c, st, pixel);
        if (++k >= n)
            break;
        depth = 0;
        st = generatePathFor<false>(c, x, y, c.p[P_SAMPLE] + k);
    }
}

// One sample of a cached tile, one pixel per thread: the query path of mk_cache_query, or the
// training path of mk_cache_train for a training pixel; returns whether this thread's path left a
// query, with its record in `q`.
template <typename A>
static __device__ __forceinline__ bool cache_sample(const BatchReq& R, uint32_t x, uint32_t y, bool inside,
                                                    uint32_t sample, float* q)
{
    const Ctx& c = R.c;
    uint32_t pixel = y * c.p[P_WIDTH] + x;
    uint32_t offset = (sample * 2654435761u) % R.train_stride;
    CacheHook hk;
    hk.c = R.spread;
    hk.train = inside && (pixel + offset) % R.train_stride == 0;
    hk.a0 = hk.a = 0.0f;
    hk.query = false;
    float feat[MAX_TRAIN_VERTICES][16];
    V3 thr[MAX_TRAIN_VERTICES], Lb[MAX_TRAIN_VERTICES];
    uint32_t nv = 0;
    bool query = false;
    PathState<false> st;
    if (inside) {
        st = generatePathFor<false>(c, x, y, sample);
        for (uint32_t depth = 0; depth < c.p[P_MAX_DEPTH]; depth++) {
            bool alive = shadePathCall<false, false, false, true>(c, st, traceClosest(c, st.org, st.dir), depth, pixel,
                                                              nullptr, &hk);
            if (hk.vertex && hk.train && nv < MAX_TRAIN_VERTICES) {
                cacheFeatures(feat[nv], hk);
                thr[nv] = hk.thr;
                Lb[nv] = hk.L;
                nv++;
            }
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
    uint32_t nt = (hk.train && ok) ? nv : 0u;
    uint32_t t0 = reserve(R.tcount, nt);
    for (uint32_t k = 0; k < nt; k++) {
        if (t0 + k >= R.tcap)
            break;
        float* d = R.trec + (size_t)(t0 + k) * REC_WORDS;
        V3 rest = st.parts.total - Lb[k];
        V3 t = thr[k];
        for (int j = 0; j < 16; j++)
            d[j] = feat[k][j];
        d[16] = t.x > 0.0f ? rest.x / t.x : 0.0f;
        d[17] = t.y > 0.0f ? rest.y / t.y : 0.0f;
        d[18] = t.z > 0.0f ? rest.z / t.z : 0.0f;
        d[19] = 0.0f;
    }
    if (query && ok) {
        cacheFeatures(q, hk);
        q[16] = hk.thr.x, q[17] = hk.thr.y, q[18] = hk.thr.z;
        return true;
    }
    return false;
}

__global__ void __launch_bounds__(128, VG_BATCH_MIN_BLOCKS) batch_render(const BatchReq* __restrict__ reqs, uint32_t nreq, uint32_t items,
                                                    uint32_t* next, BatchDone* done, uint32_t* err)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* sm = align1024(smem_raw);
    uint8_t* W = sm;
    uint8_t* H = sm + IMG_FWD_BYTES;
    __shared__ __align__(16) BatchReq R;
    __shared__ uint32_t s_item, s_req;
    __shared__ const uint8_t* s_img;
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    uint32_t tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) {
        bar_init(&bar, 1);
        fence_bar_init();
        s_img = nullptr;
    }
    if (warp == 0)
        tmem_alloc(&tslot, 64);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    uint32_t tmem = tslot;
    uint32_t lane_addr = tmem + ((warp * 32u) << 16);
    uint32_t phase = 0;
    bool ok = true;
    for (;;) {
        if (tid == 0) {
            uint32_t it = atomicAdd(next, 1u);
            uint32_t r = 0;
            if (it < items)
                while (r + 1 < nreq && reqs[r + 1].item_begin <= it)
                    r++;
            s_item = it;
            s_req = r;
        }
        __syncthreads();
        uint32_t it = s_item;
        if (it >= items)
            break;
        const uint4* src = reinterpret_cast<const uint4*>(reqs + s_req);
        for (uint32_t i = tid; i < sizeof(BatchReq) / 16; i += blockDim.x)
            reinterpret_cast<uint4*>(&R)[i] = src[i];
        __syncthreads();
        if (R.cached && s_img != R.cd.img) {
            for (uint32_t i = tid; i < IMG_FWD_BYTES / 16; i += blockDim.x)
                reinterpret_cast<uint4*>(W)[i] = __ldg(reinterpret_cast<const uint4*>(R.cd.img) + i);
            __syncthreads();
            if (tid == 0)
                s_img = R.cd.img;
        }
        uint32_t tile = it - R.item_begin;
        uint32_t x = (tile % R.tiles_x) * 16 + (tid & 15u);
        uint32_t y = (tile / R.tiles_x) * 8 + (tid >> 4);
        bool inside = x < R.c.p[P_WIDTH] && y < R.c.p[P_HEIGHT];
        if (!R.cached) {
            if (R.f64)
                plain_tile<double>(R.c, x, y, inside);
            else
                plain_tile<float>(R.c, x, y, inside);
        } else {
            uint32_t pixel = y * R.c.p[P_WIDTH] + x;
            for (uint32_t k = 0; k < R.c.p[P_SAMPLES_PER_DISPATCH] && ok; k++) {
                float q[20];
                bool has = R.f64 ? cache_sample<double>(R, x, y, inside, R.c.p[P_SAMPLE] + k, q)
                                 : cache_sample<float>(R, x, y, inside, R.c.p[P_SAMPLE] + k, q);
                float v[64];
                if (has) {
                    input_row(R.cd, q, v);
                } else {
#pragma unroll
                    for (int j = 0; j < 64; j++)
                        v[j] = 0.0f;
                }
                store_row(H, tid, v);
                for (uint32_t l = 0; l < 5; l++) {
                    fence_async_smem();
                    __syncthreads();
                    tc_fence_after();
                    if (tid == 0) {
                        const uint8_t* B = W + (l < 4 ? IMG_W + l * 8192u : IMG_W4);
                        issue_layer(tmem, H, 0, B, 0, l < 4 ? 64u : 16u, 4, false);
                        mma_commit(&bar);
                    }
                    bool fin = wait_mma(&bar, phase);
                    phase ^= 1u;
                    ok = __syncthreads_and(fin) != 0;
                    if (!ok)
                        break;
                    tc_fence_after();
                    load_acc(lane_addr, v, l < 4 ? 64 : 16);
                    tc_fence_before();
                    if (l < 4) {
#pragma unroll
                        for (int j = 0; j < 64; j++)
                            v[j] = fmaxf(v[j], 0.0f);
                        store_row(H, tid, v);
                    }
                }
                if (ok && has) {
                    if (R.f64) {
                        double* a = (double*)R.c.accum + 3 * (size_t)pixel;
                        a[0] += (double)(q[16] * fmaxf(v[0], 0.0f));
                        a[1] += (double)(q[17] * fmaxf(v[1], 0.0f));
                        a[2] += (double)(q[18] * fmaxf(v[2], 0.0f));
                    } else {
                        float* a = (float*)R.c.accum + 3 * (size_t)pixel;
                        a[0] += q[16] * fmaxf(v[0], 0.0f);
                        a[1] += q[17] * fmaxf(v[1], 0.0f);
                        a[2] += q[18] * fmaxf(v[2], 0.0f);
                    }
                }
            }
            if (!ok)
                break;
        }
        // The request's sums of this tile are written: count the tile, and time the last one.
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            if (atomicSub(&done[s_req].remaining, 1u) == 1u)
                done[s_req].done_ns = now_ns();
        }
    }
    if (!ok && tid == 0)
        atomicOr(err, ERR_MMA_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        tmem_free(tmem, 64);
}

// The batch's start time on the device clock.
__global__ void batch_clock(unsigned long long* t) { *t = now_ns(); }

} // namespace vgbk

namespace vgx {

using namespace vgbk;

static cudaError_t g_occ_err = cudaSuccess;

int batch_blocks_per_sm()
{
    static int n = -1;
    if (n < 0) {
        cudaError_t e = cudaFuncSetAttribute(batch_render, cudaFuncAttributeMaxDynamicSharedMemorySize, BATCH_SMEM);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(batch_render, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared);
        // From the kernel's own resource use: registers (allocated per warp in units of 256) and
        // shared memory (its static and dynamic bytes plus the driver's 1 KB per block).
        cudaFuncAttributes a{};
        if (e == cudaSuccess)
            e = cudaFuncGetAttributes(&a, batch_render);
        int dev = 0, regs_sm = 65536, smem_sm = 233472;
        if (e == cudaSuccess && cudaGetDevice(&dev) == cudaSuccess) {
            cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
            cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        }
        g_occ_err = e;
        int warp_regs = ((a.numRegs * 32 + 255) / 256) * 256;
        int by_regs = a.numRegs > 0 ? regs_sm / (warp_regs * 4) : 1;
        int by_smem = smem_sm / (int)(BATCH_SMEM + a.sharedSizeBytes + 1024);
        n = std::max(1, std::min(std::min(by_regs, by_smem), 16));
    }
    return n;
}

int batch_kernel_info(int* regs, int* local_bytes, int* static_smem, int* error)
{
    int b = batch_blocks_per_sm();
    cudaFuncAttributes a{};
    cudaError_t e = cudaFuncGetAttributes(&a, batch_render);
    *regs = a.numRegs;
    *local_bytes = (int)a.localSizeBytes;
    *static_smem = (int)a.sharedSizeBytes;
    *error = g_occ_err != cudaSuccess ? (int)g_occ_err : (int)e;
    return b;
}

cudaError_t launch_batch(int blocks, cudaStream_t s, const vgb::BatchReq* reqs, uint32_t nreq, uint32_t items,
                         uint32_t* next, vgb::BatchDone* done, uint32_t* err, unsigned long long* t0)
{
    batch_blocks_per_sm();
    batch_clock<<<1, 1, 0, s>>>(t0);
    batch_render<<<blocks, 128, BATCH_SMEM, s>>>(reqs, nreq, items, next, done, err);
    return cudaGetLastError();
}

} // namespace vgx
