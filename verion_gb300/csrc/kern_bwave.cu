// The batch wavefront (vg_batch_render; no reference counterpart): the streaming wavefront of
// kernels.cuh over the pixels of many requests at once. A slot of the wave buffers traces one pixel
// of one request with all of that request's samples, in order, as the streaming wavefront does for
// one frame; when the pixel's last sample is added the slot takes the next pixel of the batch (the
// host lays the requests' pixels out shortest request first), so small requests share the GPU with
// the others instead of running one at a time on a half-empty machine. Each slot reads its
// request's parameter block and scene from the request table, and the traversal stages walk each
// ray in its own scene's BVH. Per pixel the samples are added one at a time in order by the same
// functions, so a request's sums equal a megakernel accumulate of it bit for bit.
//
// A request with a radiance cache runs the cache integrator's paths: a query path ends where its
// spread passes the cache's threshold and leaves a query record; a training pixel of the sample
// (the pixel test of mk_cache_train) runs its full path and records its vertices, which become
// training records when the path ends. After each wave's finish stage one kernel evaluates every
// cache's queries of that wave (encoding and MMA layers per 128-record tile, the cache's weights
// in shared memory) and adds each answer times the path throughput to its pixel. So per pixel the
// sums take path radiance and cache answer of one sample before those of the next, as the
// megakernel cache integrator adds them, and the sums match it bit for bit while the cache is
// fixed; the caches take their training steps after the batch.
//
// The bounce loop runs on the device: the host captures start, a loop body of two waves (so that
// the queue parity of each launch is fixed) ending in a kernel that sets the loop's condition
// (cudaGraphSetConditional on a WHILE node), and the tail kernel (batches without caches), in one
// CUDA graph, which later batches of the same shape replay.
#include <algorithm>

#include "batch.h"
#include "kernels.cuh"
#include "launch_batch.h"
#include "nrc_device.cuh"

namespace vgbw {

using namespace vgd;
using namespace vgk;
using namespace vgn;
using namespace vgtc;
using namespace vgnd;
using vgb::NO_CACHE;
using vgb::WaveBatch;
using vgb::WaveCache;
using vgb::WaveReq;

// Shading classes: the four material classes of a plain request's slot, then the same four of a
// cached request's slot (shaded by the cache instantiation of bw_shade).
constexpr uint32_t BW_CLASSES = 2 * SHADE_CLASSES;
static_assert(sizeof(WaveReq) % 16 == 0 && sizeof(WaveCache) % 16 == 0, "request and cache tables are 16-byte records");
constexpr uint32_t ANSWER_SMEM = IMG_FWD_BYTES + 16384 + 1024;

// Training pixel test of a cached request's sample (mk_cache_train's, per sample).
static __device__ __forceinline__ bool training_pixel(const WaveReq& R, uint32_t pix, uint32_t sample)
{
    uint32_t offset = (sample * 2654435761u) % R.train_stride;
    return (pix + offset) % R.train_stride == 0;
}

// Request of work item `item`: the last request whose first item is at or before it.
static __device__ __forceinline__ uint32_t item_request(const WaveBatch& b, uint32_t item)
{
    uint32_t lo = 0, hi = b.nreq - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) >> 1;
        if (b.reqs[mid].item_begin <= item)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Slot p starts work item `item`: the first sample of that pixel.
static __device__ __forceinline__ void begin_item(const WaveBatch& b, const Wave& w, uint32_t p, uint32_t item)
{
    uint32_t r = item_request(b, item);
    const WaveReq& R = b.reqs[r];
    uint32_t pix = item - R.item_begin;
    uint32_t width = R.c.p[P_WIDTH];
    PathState<false> st = generatePathFor<false>(R.c, pix % width, pix / width, R.c.p[P_SAMPLE]);
    storePath<false>(w, st, p);
    w.meta[p] = 0;
    b.slot_req[p] = r;
    b.slot_pix[p] = pix;
    if (b.tnv)
        b.tnv[p] = 0;
}

// A pixel's last sample is added: count it, and time the request's last pixel.
static __device__ __forceinline__ void pixel_done(const WaveBatch& b, uint32_t r)
{
    __threadfence();
    if (atomicSub(&b.done[r].remaining, 1u) == 1u)
        b.done[r].done_ns = now_ns();
}

// Lanes with `want` take the next work items (one atomic per warp) and start them; returns
// whether this lane's slot has a pixel again. Every lane of the warp calls it.
static __device__ __forceinline__ bool take_items(const WaveBatch& b, const Wave& w, uint32_t p, bool want)
{
    uint32_t need = __ballot_sync(FULL, want);
    if (need == 0)
        return false;
    uint32_t base = 0;
    if (lane_id() == 0)
        base = atomicAdd(b.next, __popc(need));
    base = __shfl_sync(FULL, base, 0);
    if (!want)
        return false;
    uint32_t item = base + __popc(need & ((1u << lane_id()) - 1u));
    if (item >= b.items)
        return false;
    begin_item(b, w, p, item);
    return true;
}

// The first wave's queue: slot i takes work item i. Also sets the request counters, the item
// counter, the loop counter and the start time.
__global__ void __launch_bounds__(256) bw_start(WaveBatch b, Wave w)
{
    __shared__ uint32_t slot[8];
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t first = min(w.n, b.items);
    if (p == 0) {
        *b.next = first;
        b.loop[0] = 0;
        *b.t0 = now_ns();
    }
    if (p < b.nreq) {
        b.done[p].remaining = b.reqs[p].pixels;
        b.done[p].done_ns = 0;
    }
    bool live = p < first;
    if (live)
        begin_item(b, w, p, p);
    block_append<8>(&w.counts[0], w.queue[0], live, p, slot);
}

// Closest hits of the wave's rays, each in its request's scene (wf_stream_extend_dyn).
__global__ void __launch_bounds__(128, VG_TRACE_MIN_BLOCKS) bw_extend(WaveBatch b, Wave w, uint32_t wave)
{
    uint32_t in = wave & 1u, out = in ^ 1u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.counts[out] = 0;
        w.fetch[2 + in] = 0;
        w.fetch[4 + in] = 0;
        w.fetch[6 + in] = 0;
        w.fetch[8 + in] = 0;
    }
    // The previous wave's queries are answered: this wave's start empty.
    if (blockIdx.x == 0)
        for (uint32_t j = threadIdx.x; j < b.ncache; j += blockDim.x)
            *b.caches[j].qcount = 0;
    uint32_t count = w.counts[in];
    const uint32_t* qin = w.queue[in];
    vgt::trace_queue_scenes<false>(
        &w.fetch[in], count, b.err, w.refill, w.steps,
        [&](uint32_t i, V3& o, V3& d, float& tmax, const uint4*& nodes, const float4*& tris) {
            uint32_t p = qin[i];
            const DeviceScene& s = b.reqs[b.slot_req[p]].c.s;
            nodes = s.nodes;
            tris = s.tris;
            float4 a = w.state[p];
            float4 e = w.state[w.n + p];
            o = v3(a.x, a.y, a.z);
            d = v3(e.x, e.y, e.z);
            tmax = 1.0e30f;
            return true;
        },
        [&](uint32_t i, const vgt::TraceHit& q) {
            w.hits[qin[i]] = make_uint4(q.hit ? 1u : 0u, q.hit ? q.inst : 0u, q.hit ? q.prim : 0u,
                                        __float_as_uint(q.hit ? q.t : 0.0f));
        });
}

// Material classes of the wave's slots (wf_stream_classify), each from its request's scene; a
// cached request's slots in classes SHADE_CLASSES and up.
__global__ void __launch_bounds__(256) bw_classify(WaveBatch b, Wave w, uint32_t wave)
{
    uint32_t in = wave & 1u, out = in ^ 1u;
    if (blockIdx.x == 0 && threadIdx.x < BW_CLASSES)
        w.scount[out * BW_CLASSES + threadIdx.x] = 0;
    uint32_t count = w.counts[in];
    const uint32_t* qin = w.queue[in];
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += stride) {
        uint32_t i = base + threadIdx.x;
        bool have = i < count;
        uint32_t p = have ? qin[i] : 0u;
        uint32_t k = BW_CLASSES;
        if (have) {
            const WaveReq& R = b.reqs[b.slot_req[p]];
            k = shadeClass(R.c, w.hits[p]) + (R.cache != NO_CACHE ? SHADE_CLASSES : 0u);
        }
        for (uint32_t cls = 0; cls < BW_CLASSES; cls++)
            warp_append(&w.scount[in * BW_CLASSES + cls], w.squeue + (size_t)cls * w.n, k == cls, p);
    }
}

// Shading of the wave's hits, class by class, with the light sample left as a shadow request
// (wf_stream_shade_deferred with material sorting): the plain requests' slots, or with CACHE the
// cached requests' slots, whose paths may end at the cache (a query record for the wave's answer
// stage) or, on a training pixel, record their vertices.
template <bool CACHE>
__global__ void __launch_bounds__(128, VG_SHADE_MIN_BLOCKS) bw_shade(WaveBatch b, Wave w, uint32_t wave)
{
    uint32_t in = wave & 1u;
    uint32_t n = w.n;
    const uint32_t c0 = CACHE ? SHADE_CLASSES : 0u;
    uint32_t seg[SHADE_CLASSES + 1] = {0, 0, 0, 0, 0};
    for (uint32_t k = 0; k < SHADE_CLASSES; k++)
        seg[k + 1] = seg[k] + w.scount[in * BW_CLASSES + c0 + k];
    uint32_t count = seg[SHADE_CLASSES];
    for (;;) {
        uint32_t base = warp_fetch(&w.fetch[(CACHE ? 8 : 2) + in]);
        if (base >= count)
            break;
        uint32_t i = base + lane_id();
        bool query = false;
        uint32_t r = 0, pix = 0;
        CacheHook hk;
        if (i < count) {
            uint32_t k = i >= seg[1] ? (i >= seg[2] ? (i >= seg[3] ? 3u : 2u) : 1u) : 0u;
            uint32_t p = w.squeue[(size_t)(c0 + k) * n + (i - seg[k])];
            r = b.slot_req[p];
            pix = b.slot_pix[p];
            const WaveReq& R = b.reqs[r];
            const Ctx& c = R.c;
            uint32_t meta = w.meta[p];
            uint32_t depth = meta & 0xffu;
            PathState<false> st = loadState<false>(w, p);
            uint4 hr = w.hits[p];
            Hit h;
            h.hit = hr.x != 0;
            h.inst = hr.y;
            h.prim = hr.z;
            h.t = __uint_as_float(hr.w);
            ShadowReq req;
            bool train = false;
            if (CACHE) {
                // The spread starts at zero with each sample.
                float2 sp = depth > 0 ? b.spread[p] : make_float2(0.0f, 0.0f);
                train = training_pixel(R, pix, c.p[P_SAMPLE] + (meta >> 8));
                hk.c = R.spread;
                hk.train = train;
                hk.a0 = sp.x;
                hk.a = sp.y;
            }
            bool alive = shadePath<false, false, true, CACHE>(c, st, h, depth, pix, &req, CACHE ? &hk : nullptr) &&
                         depth + 1 < c.p[P_MAX_DEPTH];
            if (CACHE) {
                if (hk.vertex && train) {
                    uint32_t nv = b.tnv[p];
                    if (nv < vgb::WAVE_MAX_TRAIN_VERTICES) {
                        float f[16];
                        cacheFeatures(f, hk);
                        float4* v = b.tvert + ((size_t)p * vgb::WAVE_MAX_TRAIN_VERTICES + nv) * vgb::WAVE_VERTEX_VEC4;
                        for (int j = 0; j < 4; j++)
                            v[j] = make_float4(f[4 * j], f[4 * j + 1], f[4 * j + 2], f[4 * j + 3]);
                        v[4] = make_float4(hk.thr.x, hk.thr.y, hk.thr.z, hk.L.x);
                        v[5] = make_float4(hk.L.y, hk.L.z, 0.0f, 0.0f);
                        b.tnv[p] = nv + 1;
                    }
                }
                query = hk.query && !bad3(st.parts.total);
                if (alive)
                    b.spread[p] = make_float2(hk.a0, hk.a);
            }
            if (alive)
                storePath<false>(w, st, p);
            else
                w.state[3 * n + p] = make_float4(st.parts.total.x, st.parts.total.y, st.parts.total.z, st.qPrev);
            uint32_t flags = (req.valid ? 1u : 0u) | (alive ? 2u : 0u);
            w.sreq[n + p] = make_float4(req.d.x, req.d.y, req.d.z, __uint_as_float(flags));
            if (req.valid) {
                w.sreq[p] = make_float4(req.o.x, req.o.y, req.o.z, req.tmax);
                w.sreq[2 * n + p] = make_float4(req.c.x, req.c.y, req.c.z, 0.0f);
            }
        }
        if (CACHE && __ballot_sync(FULL, query)) {
            // Records of one cache together: one atomic per cache present in the warp.
            uint32_t j = query ? b.reqs[r].cache : 0xffffffffu;
            uint32_t grp = __match_any_sync(FULL, j);
            uint32_t leader = __ffs(grp) - 1u;
            uint32_t first = 0;
            if (query && lane_id() == leader)
                first = atomicAdd(b.caches[j].qcount, __popc(grp));
            first = __shfl_sync(FULL, first, leader);
            if (query) {
                uint32_t slot = first + __popc(grp & ((1u << lane_id()) - 1u));
                cacheQueryRecord(b.caches[j].qrec + (size_t)slot * CACHE_REC_WORDS, hk, (r << 22) | pix);
            }
        }
        __syncwarp();
    }
}

// Shadow rays of the wave's light samples, any hit, each in its request's scene. A scene with
// translucent surfaces leaves its rays to the finish stage (occluded(): layers with opacity).
__global__ void __launch_bounds__(128, VG_TRACE_MIN_BLOCKS) bw_shadow_trace(WaveBatch b, Wave w, uint32_t wave)
{
    uint32_t in = wave & 1u;
    uint32_t count = w.counts[in];
    const uint32_t* qin = w.queue[in];
    uint32_t n = w.n;
    vgt::trace_queue_scenes<true>(
        &w.fetch[4 + in], count, b.err, w.shadow_refill, w.shadow_steps,
        [&](uint32_t i, V3& o, V3& d, float& tmax, const uint4*& nodes, const float4*& tris) {
            uint32_t p = qin[i];
            float4 r1 = w.sreq[n + p];
            const DeviceScene& s = b.reqs[b.slot_req[p]].c.s;
            if (!(__float_as_uint(r1.w) & 1u) || !s.shadow_any) {
                tmax = 0.0f;
                return false;
            }
            nodes = s.nodes;
            tris = s.tris;
            float4 r0 = w.sreq[p];
            o = v3(r0.x, r0.y, r0.z);
            d = v3(r1.x, r1.y, r1.z);
            tmax = r0.w;
            return true;
        },
        [&](uint32_t i, const vgt::TraceHit& q) { ((uint32_t*)w.hits)[4 * (size_t)qin[i]] = q.hit ? 1u : 0u; });
}

// The training records of a finished training path (mk_cache_train's): per recorded vertex its
// features and the radiance the rest of the path brought, over the throughput arriving there.
// None for a path whose radiance is not finite; records past the cache's capacity are dropped.
static __device__ __forceinline__ void training_records(const WaveBatch& b, const WaveCache& K, uint32_t p, V3 total)
{
    uint32_t nv = bad3(total) ? 0u : b.tnv[p];
    if (nv == 0)
        return;
    uint32_t t0 = atomicAdd(K.tcount, nv);
    const float4* v = b.tvert + (size_t)p * vgb::WAVE_MAX_TRAIN_VERTICES * vgb::WAVE_VERTEX_VEC4;
    for (uint32_t k = 0; k < nv && t0 + k < K.tcap; k++, v += vgb::WAVE_VERTEX_VEC4) {
        float* d = K.trec + (size_t)(t0 + k) * REC_WORDS;
        for (int j = 0; j < 4; j++) {
            d[4 * j] = v[j].x;
            d[4 * j + 1] = v[j].y;
            d[4 * j + 2] = v[j].z;
            d[4 * j + 3] = v[j].w;
        }
        V3 t = v3(v[4].x, v[4].y, v[4].z);
        V3 rest = total - v3(v[4].w, v[5].x, v[5].y);
        d[16] = t.x > 0.0f ? rest.x / t.x : 0.0f;
        d[17] = t.y > 0.0f ? rest.y / t.y : 0.0f;
        d[18] = t.z > 0.0f ? rest.z / t.z : 0.0f;
        d[19] = 0.0f;
    }
}

// After the shadow rays (finishSlot for a slot of any request): add the unoccluded light sample,
// then queue the path for its next depth, or add it to its pixel and start the pixel's next sample.
// Returns 1 when the slot goes on, 0 when its pixel is finished.
static __device__ __forceinline__ bool finish_slot(const WaveBatch& b, const Wave& w, uint32_t p)
{
    uint32_t n = w.n;
    uint32_t r = b.slot_req[p];
    const WaveReq& R = b.reqs[r];
    const Ctx& c = R.c;
    uint32_t meta = w.meta[p];
    uint32_t depth = meta & 0xffu, k = meta >> 8;
    uint32_t flags = __float_as_uint(w.sreq[n + p].w);
    float4 tot = w.state[3 * n + p];
    V3 total = v3(tot.x, tot.y, tot.z);
    if (flags & 1u) {
        bool blocked;
        if (c.s.shadow_any) {
            blocked = ((const uint32_t*)w.hits)[4 * (size_t)p] != 0u;
        } else {
            float4 r0 = w.sreq[p], r1 = w.sreq[n + p];
            blocked = occluded(c, v3(r0.x, r0.y, r0.z), v3(r1.x, r1.y, r1.z), r0.w);
        }
        if (!blocked) {
            float4 r2 = w.sreq[2 * n + p];
            total += v3(r2.x, r2.y, r2.z);
            if (flags & 2u)
                w.state[3 * n + p] = make_float4(total.x, total.y, total.z, tot.w);
        }
    }
    if (flags & 2u) {
        w.meta[p] = (depth + 1) | (k << 8);
        return true;
    }
    PathState<false> st;
    st.parts.zero();
    st.parts.total = total;
    st.visLit = st.visTotal = 0.0f;
    st.gi = false;
    st.chan = -1;
    uint32_t pix = b.slot_pix[p];
    if (R.f64)
        finishPath<false, double>(c, st, pix);
    else
        finishPath<false, float>(c, st, pix);
    if (R.cache != NO_CACHE && training_pixel(R, pix, c.p[P_SAMPLE] + k))
        training_records(b, b.caches[R.cache], p, total);
    if (k + 1 < c.p[P_SAMPLES_PER_DISPATCH]) {
        uint32_t width = c.p[P_WIDTH];
        PathState<false> nx = generatePathFor<false>(c, pix % width, pix / width, c.p[P_SAMPLE] + k + 1);
        storePath<false>(w, nx, p);
        w.meta[p] = (k + 1) << 8;
        if (b.tnv)
            b.tnv[p] = 0;
        return true;
    }
    pixel_done(b, r);
    return false;
}

__global__ void __launch_bounds__(128, 8) bw_finish(WaveBatch b, Wave w, uint32_t wave)
{
    uint32_t in = wave & 1u, out = in ^ 1u;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        w.fetch[out] = 0;
    uint32_t count = w.counts[in];
    const uint32_t* qin = w.queue[in];
    uint32_t* qout = w.queue[out];
    __shared__ uint32_t slot[4], fetched;
    for (;;) {
        uint32_t base = block_fetch(&w.fetch[6 + in], &fetched);
        if (base >= count)
            break;
        uint32_t i = base + threadIdx.x;
        bool live = false, want = false;
        uint32_t p = 0;
        if (i < count) {
            p = qin[i];
            live = finish_slot(b, w, p);
            want = !live;
        }
        live |= take_items(b, w, p, want);
        block_append<4>(&w.counts[out], qout, live, p, slot);
    }
}

// The wave's cache queries, all caches in one launch: each CTA takes 128-record tiles (the tiles of
// cache 0, then of cache 1, ...), loads the tile's cache weights into shared memory when they
// change, encodes its records (hash grid and the other inputs, one row per thread), runs the five
// MMA layers with TMEM accumulators, and adds each clamped answer times the record's throughput to
// its request's pixel (the fused form of nrc_encode + nrc_infer of the cache integrator).
__global__ void __launch_bounds__(128) bw_answer(WaveBatch b)
{
    uint32_t total = 0;
    for (uint32_t j = 0; j < b.ncache; j++)
        total += (*b.caches[j].qcount + TILE - 1) / TILE;
    if (blockIdx.x >= total)
        return;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* sm = align1024(smem_raw);
    uint8_t* W = sm;
    uint8_t* H = sm + IMG_FWD_BYTES;
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    __shared__ const uint8_t* s_img;
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
    for (uint32_t t = blockIdx.x; t < total && ok; t += gridDim.x) {
        // The tile's cache and its first record.
        uint32_t j = 0, first = t * TILE, n = 0;
        for (;; j++) {
            n = *b.caches[j].qcount;
            uint32_t tiles = (n + TILE - 1) / TILE;
            if (first < tiles * TILE)
                break;
            first -= tiles * TILE;
        }
        const WaveCache& K = b.caches[j];
        if (s_img != K.cd.img) {
            __syncthreads();
            for (uint32_t i = tid; i < IMG_FWD_BYTES / 16; i += blockDim.x)
                reinterpret_cast<uint4*>(W)[i] = __ldg(reinterpret_cast<const uint4*>(K.cd.img) + i);
            __syncthreads();
            if (tid == 0)
                s_img = K.cd.img;
        }
        uint32_t i = first + tid;
        bool has = i < n;
        const float* q = K.qrec + (size_t)i * CACHE_REC_WORDS;
        float v[64];
        if (has) {
            input_row(K.cd, q, v);
        } else {
#pragma unroll
            for (int x = 0; x < 64; x++)
                v[x] = 0.0f;
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
                for (int x = 0; x < 64; x++)
                    v[x] = fmaxf(v[x], 0.0f);
                store_row(H, tid, v);
            }
        }
        if (ok && has) {
            uint32_t tag = __float_as_uint(q[19]);
            const WaveReq& R = b.reqs[tag >> 22];
            size_t o = 3 * (size_t)(tag & ((1u << 22) - 1u));
            if (R.f64) {
                double* a = (double*)R.c.accum + o;
                a[0] += (double)(q[16] * fmaxf(v[0], 0.0f));
                a[1] += (double)(q[17] * fmaxf(v[1], 0.0f));
                a[2] += (double)(q[18] * fmaxf(v[2], 0.0f));
            } else {
                float* a = (float*)R.c.accum + o;
                a[0] += q[16] * fmaxf(v[0], 0.0f);
                a[1] += q[17] * fmaxf(v[1], 0.0f);
                a[2] += q[18] * fmaxf(v[2], 0.0f);
            }
        }
        __syncthreads();
    }
    if (!ok && tid == 0)
        atomicOr(b.err, ERR_MMA_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        tmem_free(tmem, 64);
}

// The loop's condition after each body (two waves, so the next wave reads queue 0): go on while
// more than b.tail slots are live, at most b.max_iter times.
__global__ void bw_condition(WaveBatch b, Wave w, cudaGraphConditionalHandle loop)
{
    uint32_t it = ++b.loop[0];
    cudaGraphSetConditional(loop, (w.counts[0] > b.tail && it < b.max_iter) ? 1u : 0u);
}

// The tail: one thread per live slot (a grid-stride loop over queue 0) runs its path, the rest of
// its pixel's samples and then further work items to the end, trace and shade in a loop as the
// megakernel does.
__global__ void __launch_bounds__(128, VG_TAIL_MIN_BLOCKS) bw_tail(WaveBatch b, Wave w)
{
    uint32_t count = w.counts[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        uint32_t p = w.queue[0][i];
        uint32_t meta = w.meta[p];
        uint32_t depth = meta & 0xffu, k = meta >> 8;
        uint32_t r = b.slot_req[p], pix = b.slot_pix[p];
        PathState<false> st = loadState<false>(w, p);
        for (;;) {
            const WaveReq& R = b.reqs[r];
            const Ctx& c = R.c;
            if (shadePathCall<false, false>(c, st, traceClosest(c, st.org, st.dir), depth, pix) &&
                depth + 1 < c.p[P_MAX_DEPTH]) {
                depth++;
                continue;
            }
            if (R.f64)
                finishPath<false, double>(c, st, pix);
            else
                finishPath<false, float>(c, st, pix);
            uint32_t width = c.p[P_WIDTH];
            depth = 0;
            if (k + 1 < c.p[P_SAMPLES_PER_DISPATCH]) {
                k++;
                st = generatePathFor<false>(c, pix % width, pix / width, c.p[P_SAMPLE] + k);
                continue;
            }
            pixel_done(b, r);
            uint32_t item = atomicAdd(b.next, 1u);
            if (item >= b.items)
                break;
            r = item_request(b, item);
            pix = item - b.reqs[r].item_begin;
            k = 0;
            const Ctx& c2 = b.reqs[r].c;
            st = generatePathFor<false>(c2, pix % c2.p[P_WIDTH], pix / c2.p[P_WIDTH], c2.p[P_SAMPLE]);
        }
    }
}

} // namespace vgbw

namespace vgx {

using namespace vgbw;

cudaError_t bwave_capture_start(cudaStream_t s, const vgb::WaveBatch& b, const vgk::Wave& w)
{
    bw_start<<<(w.n + 255) / 256, 256, 0, s>>>(b, w);
    return cudaGetLastError();
}

cudaError_t bwave_capture_body(cudaStream_t s, int trace_blocks, int shade_blocks, int sms, const vgb::WaveBatch& b,
                               const vgk::Wave& w, cudaGraphConditionalHandle loop, bool condition)
{
    for (uint32_t wave = 0; wave < 2; wave++) {
        bw_extend<<<trace_blocks, 128, 0, s>>>(b, w, wave);
        bw_classify<<<sms * 4, 256, 0, s>>>(b, w, wave);
        bw_shade<false><<<shade_blocks, 128, 0, s>>>(b, w, wave);
        if (b.ncache)
            bw_shade<true><<<shade_blocks, 128, 0, s>>>(b, w, wave);
        bw_shadow_trace<<<trace_blocks, 128, 0, s>>>(b, w, wave);
        bw_finish<<<trace_blocks, 128, 0, s>>>(b, w, wave);
        if (b.ncache)
            bw_answer<<<sms * 2, 128, ANSWER_SMEM, s>>>(b);
    }
    if (condition)
        bw_condition<<<1, 1, 0, s>>>(b, w, loop);
    return cudaGetLastError();
}

cudaError_t bwave_capture_tail(cudaStream_t s, const vgb::WaveBatch& b, const vgk::Wave& w)
{
    bw_tail<<<std::max(1u, (b.tail + 127) / 128), 128, 0, s>>>(b, w);
    return cudaGetLastError();
}

// Resident blocks per SM of the traversal and shade stages (their grids fill the SMs once); also
// lets the answer kernel have its shared memory.
void bwave_blocks_per_sm(int* trace, int* shade)
{
    static int t = -1, sh = -1;
    if (t < 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&t, bw_extend, 128, 0) != cudaSuccess || t < 1)
            t = 1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sh, bw_shade<true>, 128, 0) != cudaSuccess || sh < 1)
            sh = 1;
        cudaFuncSetAttribute(bw_answer, cudaFuncAttributeMaxDynamicSharedMemorySize, ANSWER_SMEM);
    }
    *trace = t;
    *shade = sh;
}

} // namespace vgx
