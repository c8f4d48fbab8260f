// Kernels of the CUDA backend (sm_103a): the megakernel and the wavefront stages.
//
// Reference entry points: shaders/pathtrace.slang (megakernel), shaders/wf_select.slang,
// shaders/wf_args.slang, shaders/wf_extend.slang, shaders/wf_shade.slang, with the path state of
// shaders/include/wf_state.slang.
//
// GB300 design:
// * Extend and shade are persistent kernels: a grid sized to fill the 152 SMs once, each warp
//   fetching 32 consecutive queue entries with one atomic until the depth's queue is drained.
//   The queue length is read on the device, so no indirect dispatch (wf_args) and no host wait
//   sit between depths.
// * Compaction (live paths into the next depth's queue, pixels into the depth-0 queue) is warp
//   aggregated: one ballot, one atomic per warp, each lane writes at its rank.
// * Path state is structure-of-arrays in 16-byte planes: a path's 16 words are four 128-bit
//   loads, each plane contiguous over paths.
#pragma once
#include "pt_device.cuh"

namespace vgk {

using namespace vgd;

constexpr uint32_t FULL = 0xffffffffu;

// Minimum resident 128-thread blocks per SM requested for the shade kernels (a register cap), and
// for the deferred shade stage's ReSTIR instantiations, whose candidate loop waits on memory: on
// the many-light ReSTIR frame 4 blocks gave 7.89 ms, 6 blocks 7.43 (then 7.01 with the shared
// candidate target terms), 10 blocks 6.76, 12 blocks 6.72, 16 blocks 6.90. The plain stage keeps
// 4: 5, 6, 8 or 16 blocks are slower (its inlined shadePath spills heavily below 128 registers),
// and so is calling the out-of-line shadePathCall from it (8.99 ms of shading per benchmark step
// inline at 4 blocks; out of line 9.67 at 4 blocks, 10.5 at 8, 10.9 at 12, 11.4 at 16).
#ifndef VG_SHADE_MIN_BLOCKS
#define VG_SHADE_MIN_BLOCKS 4
#endif
#ifndef VG_RESTIR_SHADE_MIN_BLOCKS
#define VG_RESTIR_SHADE_MIN_BLOCKS 12
#endif
// The same for the kernels that run whole paths per thread through the out-of-line shadePathCall
// (the streaming tail, the batch wavefront's tail).
#ifndef VG_TAIL_MIN_BLOCKS
#define VG_TAIL_MIN_BLOCKS VG_SHADE_MIN_BLOCKS
#endif

// State planes (16 bytes each, plane k of path p at state[k * N + p]):
//   0 (org.xyz, rng)  1 (dir.xyz, flags)  2 (thr.xyz, pathLen)  3 (total.xyz, qPrev)
//   with the lighting split: 4 (directDiffuse.xyz, visLit) 5 (indirectDiffuse.xyz, visTotal)
//   6 (specular.xyz, 0) 7 (transmission.xyz, 0) 8 (emission.xyz, 0)
// flags as in wf_state.slang:42: cls bits 0-1, chan + 1 bits 2-3, misPrev bit 4, restir bit 5,
// gi bit 6, prevInst bits 8 and up.

static __device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Appends `pred` lanes of a converged warp to `queue` (counter `count`); returns the slot.
static __device__ __forceinline__ void warp_append(uint32_t* count, uint32_t* queue, bool pred, uint32_t value)
{
    uint32_t b = __ballot_sync(FULL, pred);
    if (b == 0)
        return;
    uint32_t base = 0;
    if (lane_id() == 0)
        base = atomicAdd(count, __popc(b));
    base = __shfl_sync(FULL, base, 0);
    if (pred)
        queue[base + __popc(b & ((1u << lane_id()) - 1u))] = value;
}

// Warp-wide work fetch: 32 consecutive items per atomic.
static __device__ __forceinline__ uint32_t warp_fetch(uint32_t* counter)
{
    uint32_t base = 0;
    if (lane_id() == 0)
        base = atomicAdd(counter, 32u);
    return __shfl_sync(FULL, base, 0);
}

// Block-level compaction: appends the `pred` threads of a block of WARPS warps to `queue` with one
// atomic per block. Every thread of the block calls it. A block-wide exclusive scan over the warps'
// ballot counts (warp 0 scans them with shuffles) gives each warp its offset in the block's range;
// each lane writes at its warp's offset plus its rank in the ballot. `slot` is WARPS words of
// shared memory. Each warp writes and reads only its own word outside the scan, so calls in a loop
// need no barrier after the writes.
template <uint32_t WARPS>
__device__ __forceinline__ void block_append(uint32_t* count, uint32_t* queue, bool pred, uint32_t value, uint32_t* slot)
{
    uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    uint32_t b = __ballot_sync(FULL, pred);
    if (lane == 0)
        slot[warp] = __popc(b);
    __syncthreads();
    if (warp == 0) {
        uint32_t v = lane < WARPS ? slot[lane] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (uint32_t o = 1; o < WARPS; o <<= 1) {
            uint32_t t = __shfl_up_sync(FULL, incl, o);
            if (lane >= o)
                incl += t;
        }
        uint32_t total = __shfl_sync(FULL, incl, WARPS - 1);
        uint32_t base = 0;
        if (lane == 0 && total)
            base = atomicAdd(count, total);
        base = __shfl_sync(FULL, base, 0);
        if (lane < WARPS)
            slot[lane] = base + incl - v;
    }
    __syncthreads();
    if (pred)
        queue[slot[warp] + __popc(b & ((1u << lane) - 1u))] = value;
}

// Block-wide work fetch: blockDim.x consecutive items per atomic (thread 0 takes them, a barrier
// hands them out). `word` is one word of shared memory.
static __device__ __forceinline__ uint32_t block_fetch(uint32_t* counter, uint32_t* word)
{
    if (threadIdx.x == 0)
        *word = atomicAdd(counter, blockDim.x);
    __syncthreads();
    return *word;
}

template <bool LIGHT>
__device__ __forceinline__ void storePath(const Wave& w, const PathState<LIGHT>& s, uint32_t p)
{
    uint32_t n = w.n;
    uint32_t flags = s.cls | ((uint32_t)(s.chan + 1) << 2) | (s.misPrev ? 16u : 0u) | (s.restir ? 32u : 0u) |
                     (s.gi ? 64u : 0u) | (s.prevInst << 8);
    w.state[p] = make_float4(s.org.x, s.org.y, s.org.z, __uint_as_float(s.rng));
    w.state[n + p] = make_float4(s.dir.x, s.dir.y, s.dir.z, __uint_as_float(flags));
    w.state[2 * n + p] = make_float4(s.thr.x, s.thr.y, s.thr.z, s.pathLen);
    w.state[3 * n + p] = make_float4(s.parts.total.x, s.parts.total.y, s.parts.total.z, s.qPrev);
    if (LIGHT) {
        const Parts<LIGHT>& q = s.parts;
        w.state[4 * n + p] = make_float4(q.directDiffuse.x, q.directDiffuse.y, q.directDiffuse.z, s.visLit);
        w.state[5 * n + p] = make_float4(q.indirectDiffuse.x, q.indirectDiffuse.y, q.indirectDiffuse.z, s.visTotal);
        w.state[6 * n + p] = make_float4(q.specular.x, q.specular.y, q.specular.z, 0.0f);
        w.state[7 * n + p] = make_float4(q.transmission.x, q.transmission.y, q.transmission.z, 0.0f);
        w.state[8 * n + p] = make_float4(q.emission.x, q.emission.y, q.emission.z, 0.0f);
    }
}

// wf_state.slang:60-92. Depth 0 keeps no state: the camera path is generated again.
template <bool LIGHT>
__device__ __forceinline__ PathState<LIGHT> loadPath(const Ctx& c, const Wave& w, uint32_t p, uint32_t depth)
{
    if (depth == 0)
        return generatePathFor<LIGHT>(c, p % c.p[P_WIDTH], p / c.p[P_WIDTH], c.p[P_SAMPLE]);
    uint32_t n = w.n;
    PathState<LIGHT> s;
    float4 a = w.state[p];
    float4 b = w.state[n + p];
    float4 t = w.state[2 * n + p];
    float4 r = w.state[3 * n + p];
    s.org = v3(a.x, a.y, a.z);
    s.rng = __float_as_uint(a.w);
    s.dir = v3(b.x, b.y, b.z);
    uint32_t flags = __float_as_uint(b.w);
    s.thr = v3(t.x, t.y, t.z);
    s.pathLen = t.w;
    s.cls = flags & 3u;
    s.chan = (int)((flags >> 2) & 3u) - 1;
    s.misPrev = (flags & 16u) != 0;
    s.restir = (flags & 32u) != 0;
    s.gi = (flags & 64u) != 0;
    s.prevInst = flags >> 8;
    s.qPrev = r.w;
    s.parts.zero();
    s.parts.total = v3(r.x, r.y, r.z);
    s.visLit = 0.0f;
    s.visTotal = 0.0f;
    if (LIGHT) {
        float4 q4 = w.state[4 * n + p], q5 = w.state[5 * n + p], q6 = w.state[6 * n + p], q7 = w.state[7 * n + p],
               q8 = w.state[8 * n + p];
        s.parts.directDiffuse = v3(q4.x, q4.y, q4.z);
        s.visLit = q4.w;
        s.parts.indirectDiffuse = v3(q5.x, q5.y, q5.z);
        s.visTotal = q5.w;
        s.parts.specular = v3(q6.x, q6.y, q6.z);
        s.parts.transmission = v3(q7.x, q7.y, q7.z);
        s.parts.emission = v3(q8.x, q8.y, q8.z);
    }
    return s;
}

// Minimum resident 128-thread blocks per SM requested for the megakernel (a register cap; 0: none).
// Its threads spend most of their time waiting on dependent node loads in the traversal, so
// occupancy pays more than registers: on the 1M-triangle workload at 1080p, 72.8 Mpaths/s with no
// cap (168 registers, 3 blocks per SM), 88.9 at 8 blocks (64 registers), 102.4 at 12, 114.1 at 16
// (32 registers, every warp slot of the SM; the spills mostly stay in L1 and L2).
#ifndef VG_MK_MIN_BLOCKS
#define VG_MK_MIN_BLOCKS 16
#endif
#if VG_MK_MIN_BLOCKS > 0
#define VG_MK_BOUNDS __launch_bounds__(128, VG_MK_MIN_BLOCKS)
#else
#define VG_MK_BOUNDS __launch_bounds__(128)
#endif

// Idle lanes at or above which a megakernel warp takes new pixels (VG_MK_PERSISTENT).
#ifndef VG_MK_REFILL
#define VG_MK_REFILL 4
#endif
#ifndef VG_MK_PERSISTENT
#define VG_MK_PERSISTENT 1
#endif

// Whether a megakernel instantiation is the persistent form. ReSTIR frames keep one tile per block:
// with one sample per launch the refills cost more than they save (the many-light ReSTIR frame
// 15.6 ms persistent against 13.0 ms; plain frames 119.9 against 113.9 Mpaths/s on the
// 1M-triangle workload, 5.9 against 6.7 ms per many-light frame).
__host__ __device__ constexpr bool mk_persistent(bool restir) { return VG_MK_PERSISTENT && !restir; }

// pathtrace.slang:9-26: params[35] samples from params[6] for every pixel, each pixel's samples in
// order in one thread. One loop over bounces: a lane whose path ends adds it and starts its
// pixel's next sample in the same iteration. Persistent (mk_persistent: frames without ReSTIR): a
// grid that fills the SMs once, whose warps take pixels from the work counter `next` (one atomic per
// refill) whenever at least VG_MK_REFILL lanes have finished theirs, so a warp does not idle on its
// longest pixel; else one 16 x 8 tile per block. Same samples, same order per pixel, same sums.
template <bool LIGHT, bool RESTIR, typename A>
__global__ void VG_MK_BOUNDS mk_pathtrace(const __grid_constant__ Ctx c, uint32_t* next)
{
    uint32_t width = c.p[P_WIDTH];
    uint32_t n = c.p[P_SAMPLES_PER_DISPATCH];
    bool adaptive = c.p[P_ADAPTIVE] != 0;
    if constexpr (mk_persistent(RESTIR)) {
        // Work items in 16 x 8 tiles (128 consecutive items per tile), so a warp's 32 pixels are a
        // 16 x 2 block as in the one-tile-per-block form; items outside the frame are skipped.
        uint32_t height = c.p[P_HEIGHT];
        uint32_t tiles_x = (width + 15) / 16;
        uint32_t nitems = tiles_x * ((height + 7) / 8) * 128u;
        uint32_t lane = lane_id(), lt = (1u << lane) - 1u;
        bool active = false, exhausted = n == 0;
        uint32_t pixel = 0, k = 0, depth = 0;
        PathState<LIGHT> st;
        for (;;) {
            uint32_t idle = __ballot_sync(FULL, !active);
            if (!exhausted && (idle == FULL || (uint32_t)__popc(idle) >= VG_MK_REFILL)) {
                uint32_t cnt = __popc(idle), base = 0;
                if (lane == 0)
                    base = atomicAdd(next, cnt);
                base = __shfl_sync(FULL, base, 0);
                exhausted = base + cnt >= nitems;
                if (!active) {
                    uint32_t idx = base + __popc(idle & lt);
                    uint32_t t = idx >> 7, r = idx & 127u;
                    uint32_t x = (t % tiles_x) * 16 + (r & 15u), y = (t / tiles_x) * 8 + (r >> 4);
                    if (idx < nitems && x < width && y < height && !(adaptive && !pixelActive<A>(c, y * width + x))) {
                        pixel = y * width + x;
                        k = 0;
                        depth = 0;
                        st = generatePathFor<LIGHT>(c, x, y, c.p[P_SAMPLE]);
                        active = true;
                    }
                }
            }
            if (__ballot_sync(FULL, active) == 0) {
                if (exhausted)
                    break;
                continue;
            }
            if (active) {
                if (shadePathCall<LIGHT, RESTIR>(c, st, traceClosest(c, st.org, st.dir), depth, pixel) &&
                    depth + 1 < c.p[P_MAX_DEPTH]) {
                    depth++;
                } else {
                    finishPath<LIGHT, A, RESTIR>(c, st, pixel);
                    if (++k < n && !(adaptive && !pixelActive<A>(c, pixel))) {
                        depth = 0;
                        st = generatePathFor<LIGHT>(c, pixel % width, pixel / width, c.p[P_SAMPLE] + k);
                    } else {
                        active = false;
                    }
                }
            }
        }
    } else {
        uint32_t x = blockIdx.x * 16 + (threadIdx.x & 15u);
        uint32_t y = blockIdx.y * 8 + (threadIdx.x >> 4);
        if (x >= width || y >= c.p[P_HEIGHT])
            return;
        uint32_t pixel = y * width + x;
        if (n == 0 || (adaptive && !pixelActive<A>(c, pixel)))
            return;
        uint32_t k = 0, depth = 0;
        PathState<LIGHT> st = generatePathFor<LIGHT>(c, x, y, c.p[P_SAMPLE]);
        for (;;) {
            if (shadePathCall<LIGHT, RESTIR>(c, st, traceClosest(c, st.org, st.dir), depth, pixel) &&
                depth + 1 < c.p[P_MAX_DEPTH]) {
                depth++;
                continue;
            }
            finishPath<LIGHT, A, RESTIR>(c, st, pixel);
            if (++k >= n || (adaptive && !pixelActive<A>(c, pixel)))
                break;
            depth = 0;
            st = generatePathFor<LIGHT>(c, x, y, c.p[P_SAMPLE] + k);
        }
    }
}

// wf_args.slang:9-24 at depth 0: starts a sample. Every pixel's path is live unless adaptive
// sampling fills the depth-0 queue (wf_select); the later queues and all work counters restart.
static __global__ void wf_begin(const __grid_constant__ Ctx c, Wave w)
{
    uint32_t i = threadIdx.x;
    for (uint32_t k = i; k <= w.depth; k += blockDim.x) {
        w.counts[k] = (k == 0 && c.p[P_ADAPTIVE] == 0) ? w.n : 0u;
        w.fetch[k] = 0;
        w.fetch[w.depth + 1 + k] = 0;
    }
}

// wf_select.slang:7-18: queues the pixels that still take samples; one atomic per block of 256
// (the reference takes one per pixel).
template <typename A>
__global__ void __launch_bounds__(256) wf_select(const __grid_constant__ Ctx c, Wave w)
{
    __shared__ uint32_t slot[8];
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    bool active = p < w.n && pixelActive<A>(c, p);
    block_append<8>(&w.counts[0], w.queue[0], active, p, slot);
}

// Sums a per-lane counter over the warp and adds it to a global 64-bit counter (lane 0).
static __device__ __forceinline__ void warp_count(unsigned long long* dst, uint32_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(FULL, v, o);
    if (lane_id() == 0 && v)
        atomicAdd(dst, (unsigned long long)v);
}

// wf_extend.slang:6-30: closest hit for every live path of depth d. STATS also counts rays,
// BVH nodes visited and triangles tested into w.tstats[0..2] (rays at depth > 0 into [3]).
template <bool STATS>
__global__ void __launch_bounds__(128, 8) wf_extend(const __grid_constant__ Ctx c, Wave w, uint32_t d)
{
    uint32_t count = w.counts[d];
    const uint32_t* qin = w.queue[d & 1u];
    bool direct = d == 0 && c.p[P_ADAPTIVE] == 0;
    uint32_t n_rays = 0, n_nodes = 0, n_tests = 0;
    for (;;) {
        uint32_t base = warp_fetch(&w.fetch[d]);
        if (base >= count)
            break;
        uint32_t i = base + lane_id();
        if (i < count) {
            uint32_t p = direct ? i : qin[i];
            V3 org, dir;
            if (d == 0) {
                PathState<false> s = generatePathFor<false>(c, p % c.p[P_WIDTH], p / c.p[P_WIDTH], c.p[P_SAMPLE]);
                org = s.org;
                dir = s.dir;
            } else {
                float4 a = w.state[p];
                float4 b = w.state[w.n + p];
                org = v3(a.x, a.y, a.z);
                dir = v3(b.x, b.y, b.z);
            }
            vgt::TRay r = vgt::make_ray(org, dir);
            vgt::TraceHit q = vgt::trace_bvh<false>(c.s.nodes, c.s.tris, r, 1.0e30f, c.err);
            w.hits[p] = make_uint4(q.hit ? 1u : 0u, q.hit ? q.inst : 0u, q.hit ? q.prim : 0u,
                                   __float_as_uint(q.hit ? q.t : 0.0f));
            if (STATS) {
                n_rays++;
                n_nodes += q.nodes;
                n_tests += q.tests;
            }
        }
        __syncwarp();
    }
    if (STATS) {
        warp_count(&w.tstats[0], n_rays);
        warp_count(&w.tstats[1], n_nodes);
        warp_count(&w.tstats[2], n_tests);
        warp_count(&w.tstats[3], d > 0 ? n_rays : 0u);
    }
}

// wf_shade.slang:7-29: shade each live path of depth d, then queue it for d + 1 or finish it.
template <bool LIGHT, bool RESTIR, typename A>
__global__ void __launch_bounds__(128, VG_SHADE_MIN_BLOCKS) wf_shade(const __grid_constant__ Ctx c, Wave w, uint32_t d)
{
    uint32_t count = w.counts[d];
    const uint32_t* qin = w.queue[d & 1u];
    uint32_t* qout = w.queue[(d + 1) & 1u];
    bool direct = d == 0 && c.p[P_ADAPTIVE] == 0;
    for (;;) {
        uint32_t base = warp_fetch(&w.fetch[w.depth + 1 + d]);
        if (base >= count)
            break;
        uint32_t i = base + lane_id();
        bool live = false;
        uint32_t p = 0;
        if (i < count) {
            p = direct ? i : qin[i];
            PathState<LIGHT> st = loadPath<LIGHT>(c, w, p, d);
            uint4 hr = w.hits[p];
            Hit h;
            h.hit = hr.x != 0;
            h.inst = hr.y;
            h.prim = hr.z;
            h.t = __uint_as_float(hr.w);
            if (shadePath<LIGHT, RESTIR>(c, st, h, d, p) && d + 1 < w.depth) {
                storePath<LIGHT>(w, st, p);
                live = true;
            } else {
                finishPath<LIGHT, A, RESTIR>(c, st, p);
            }
        }
        __syncwarp();
        warp_append(&w.counts[d + 1], qout, live, p);
    }
}

// ---------------------------------------------------------------------------------------------
// Streaming wavefront (path regeneration). The reference's wavefront runs one sample at a time,
// depth by depth (renderer/wavefront.rs:93-177): 2 x depth launches per sample, most of them on a
// small tail of long paths. Here each pixel's slot runs the batch's params[35] samples back to
// back: when its path ends, the same thread adds it to the pixel's sums and starts the pixel's next
// sample in the same slot. A wave is one extend plus one shade over every live slot, whatever the
// depth of its path. Per pixel the samples are still added in order, one at a time, and adaptive
// sampling still decides before each sample from the statistics of the samples before it, so the
// sums are those of the sample-by-sample loop, bit for bit.
// Counters: queue lengths counts[wave & 1] (in) / counts[~wave & 1] (out), extend work counters
// fetch[0..1], shade work counters fetch[2..3]; each kernel clears the ones the next kernel uses.

// Path state as stored, for any depth (depth 0 included: it was stored when the sample started).
template <bool LIGHT>
__device__ __forceinline__ PathState<LIGHT> loadState(const Wave& w, uint32_t p)
{
    uint32_t n = w.n;
    PathState<LIGHT> s;
    float4 a = w.state[p], b = w.state[n + p], t = w.state[2 * n + p], r = w.state[3 * n + p];
    s.org = v3(a.x, a.y, a.z);
    s.rng = __float_as_uint(a.w);
    s.dir = v3(b.x, b.y, b.z);
    uint32_t flags = __float_as_uint(b.w);
    s.thr = v3(t.x, t.y, t.z);
    s.pathLen = t.w;
    s.cls = flags & 3u;
    s.chan = (int)((flags >> 2) & 3u) - 1;
    s.misPrev = (flags & 16u) != 0;
    s.restir = (flags & 32u) != 0;
    s.gi = (flags & 64u) != 0;
    s.prevInst = flags >> 8;
    s.qPrev = r.w;
    s.parts.zero();
    s.parts.total = v3(r.x, r.y, r.z);
    s.visLit = 0.0f;
    s.visTotal = 0.0f;
    if (LIGHT) {
        float4 q4 = w.state[4 * n + p], q5 = w.state[5 * n + p], q6 = w.state[6 * n + p], q7 = w.state[7 * n + p],
               q8 = w.state[8 * n + p];
        s.parts.directDiffuse = v3(q4.x, q4.y, q4.z);
        s.visLit = q4.w;
        s.parts.indirectDiffuse = v3(q5.x, q5.y, q5.z);
        s.visTotal = q5.w;
        s.parts.specular = v3(q6.x, q6.y, q6.z);
        s.parts.transmission = v3(q7.x, q7.y, q7.z);
        s.parts.emission = v3(q8.x, q8.y, q8.z);
    }
    return s;
}

// Starts the batch: every pixel that takes a sample (wf_select's test) begins sample params[6].
// With CACHE the training pixels of the frame are left out (a kernel of their own traces them).
template <bool LIGHT, typename A, bool CACHE = false>
__global__ void __launch_bounds__(256) wf_stream_start(const __grid_constant__ Ctx c, Wave w, CacheWave q)
{
    __shared__ uint32_t slot[8];
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    bool live = false;
    if (p < w.n && c.p[P_SAMPLES_PER_DISPATCH] > 0 && (c.p[P_ADAPTIVE] == 0 || pixelActive<A>(c, p)) &&
        !(CACHE && (p + q.train_offset) % q.train_stride == 0)) {
        PathState<LIGHT> st = generatePathFor<LIGHT>(c, p % c.p[P_WIDTH], p / c.p[P_WIDTH], c.p[P_SAMPLE]);
        storePath<LIGHT>(w, st, p);
        w.meta[p] = 0;
        live = true;
    }
    block_append<8>(&w.counts[0], w.queue[0], live, p, slot);
}

template <bool STATS>
__global__ void __launch_bounds__(128, 8) wf_stream_extend(const __grid_constant__ Ctx c, Wave w, uint32_t wave)
{
    uint32_t in = wave & 1u, out = in ^ 1u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.counts[out] = 0;
        w.fetch[2 + in] = 0;
        w.fetch[4 + in] = 0;
    }
    uint32_t count = w.counts[in];
    const uint32_t* qin = w.queue[in];
    uint32_t n_rays = 0, n_nodes = 0, n_tests = 0, n_later = 0;
    for (;;) {
        uint32_t base = warp_fetch(&w.fetch[in]);
        if (base >= count)
            break;
        uint32_t i = base + lane_id();
        if (i < count) {
            uint32_t p = qin[i];
            float4 a = w.state[p];
            float4 b = w.state[w.n + p];
            vgt::TRay r = vgt::make_ray(v3(a.x, a.y, a.z), v3(b.x, b.y, b.z));
            vgt::TraceHit q = vgt::trace_bvh<false>(c.s.nodes, c.s.tris, r, 1.0e30f, c.err);
            w.hits[p] = make_uint4(q.hit ? 1u : 0u, q.hit ? q.inst : 0u, q.hit ? q.prim : 0u,
                                   __float_as_uint(q.hit ? q.t : 0.0f));
            if (STATS) {
                n_rays++;
                n_nodes += q.nodes;
                n_tests += q.tests;
                n_later += (w.meta[p] & 0xffu) != 0 ? 1u : 0u;
            }
        }
        __syncwarp();
    }
    if (STATS) {
        warp_count(&w.tstats[0], n_rays);
        warp_count(&w.tstats[1], n_nodes);
        warp_count(&w.tstats[2], n_tests);
        warp_count(&w.tstats[3], n_later);
    }
}

template <bool LIGHT, typename A, bool RESTIR = false>
__global__ void __launch_bounds__(128, VG_SHADE_MIN_BLOCKS) wf_stream_shade(const __grid_constant__ Ctx c, Wave w, uint32_t wave)
{
    uint32_t in = wave & 1u, out = in ^ 1u;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        w.fetch[out] = 0;
    uint32_t count = w.counts[in];
    const uint32_t* qin = w.queue[in];
    uint32_t* qout = w.queue[out];
    uint32_t batch = c.p[P_SAMPLES_PER_DISPATCH];
    for (;;) {
        uint32_t base = warp_fetch(&w.fetch[2 + in]);
        if (base >= count)
            break;
        uint32_t i = base + lane_id();
        bool live = false;
        uint32_t p = 0;
        if (i < count) {
            p = qin[i];
            uint32_t meta = w.meta[p];
            uint32_t depth = meta & 0xffu, k = meta >> 8;
            PathState<LIGHT> st = loadState<LIGHT>(w, p);
            uint4 hr = w.hits[p];
            Hit h;
            h.hit = hr.x != 0;
            h.inst = hr.y;
            h.prim = hr.z;
            h.t = __uint_as_float(hr.w);
            if (shadePath<LIGHT, RESTIR>(c, st, h, depth, p) && depth + 1 < w.depth) {
                storePath<LIGHT>(w, st, p);
                w.meta[p] = (depth + 1) | (k << 8);
                live = true;
            } else {
                finishPath<LIGHT, A, RESTIR>(c, st, p);
                if (k + 1 < batch && (c.p[P_ADAPTIVE] == 0 || pixelActive<A>(c, p))) {
                    PathState<LIGHT> nx =
                        generatePathFor<LIGHT>(c, p % c.p[P_WIDTH], p / c.p[P_WIDTH], c.p[P_SAMPLE] + k + 1);
                    storePath<LIGHT>(w, nx, p);
                    w.meta[p] = (k + 1) << 8;
                    live = true;
                }
            }
        }
        __syncwarp();
        warp_append(&w.counts[out], qout, live, p);
    }
}

// Shading classes of material-sorted shading (SHADE_CLASSES, ctx.h): a missed ray (environment or
// sky), a diffuse surface, a conductor, a dielectric. Only the order in which slots are shaded
// changes (each slot adds to its own pixel), so the sums stay bit-identical.

static __device__ __forceinline__ uint32_t shadeClass(const Ctx& c, uint4 hr)
{
    if (hr.x == 0)
        return 0;
    uint32_t mi = uget(c.s.instances, hr.y * 16 + 2) * 24;
    if (fget(c.s.materials, mi + 8) > 0.0f)
        return 3;
    return fget(c.s.materials, mi + 6) >= 0.5f ? 2u : 1u;
}

// Between extend and shade: every slot of the wave's queue goes to the queue of its shading class
// (one atomic per class present in a warp), so the deferred shade stage's warps mostly run one
// BSDF's code. Clears the other parity's class counts for the next wave (the shade stage of the
// previous wave, their last reader, has finished).
static __global__ void __launch_bounds__(256) wf_stream_classify(const __grid_constant__ Ctx c, Wave w, uint32_t wave)
{
    uint32_t in = wave & 1u, out = in ^ 1u;
    if (blockIdx.x == 0 && threadIdx.x < SHADE_CLASSES)
        w.scount[out * SHADE_CLASSES + threadIdx.x] = 0;
    uint32_t count = w.counts[in];
    const uint32_t* qin = w.queue[in];
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += stride) {
        uint32_t i = base + threadIdx.x;
        bool have = i < count;
        uint32_t p = have ? qin[i] : 0u;
        uint32_t k = have ? shadeClass(c, w.hits[p]) : SHADE_CLASSES;
        for (uint32_t cls = 0; cls < SHADE_CLASSES; cls++)
            warp_append(&w.scount[in * SHADE_CLASSES + cls], w.squeue + (size_t)cls * w.n, k == cls, p);
    }
}

// Streaming wave in three stages (lighting split off): extend, then shade without any traversal,
// then shadow. Shade leaves its emitter / environment light sample as a request per slot
// (w.sreq planes: origin + tmax, direction + flags, contribution); the shadow stage traces it,
// adds the contribution when unoccluded, and only then finishes, restarts or queues the slot.
// flags: bit 0 a request is present, bit 1 the path goes on to the next depth.
// With CACHE a path also ends where its spread passes the cache threshold (shadePath's cache
// hook); it then leaves a query record (one atomic per warp) and finishes like any other.
// With SORTED the wave's slots are taken class by class from the classify stage's queues.
template <typename A, bool CACHE = false, bool RESTIR = false, bool SORTED = false>
__global__ void __launch_bounds__(128, RESTIR ? VG_RESTIR_SHADE_MIN_BLOCKS : VG_SHADE_MIN_BLOCKS) wf_stream_shade_deferred(const __grid_constant__ Ctx c,
                                                                                    Wave w, uint32_t wave,
                                                                                    CacheWave q)
{
    uint32_t in = wave & 1u;
    uint32_t count = w.counts[in];
    const uint32_t* qin = w.queue[in];
    uint32_t n = w.n;
    uint32_t seg[SHADE_CLASSES + 1] = {0, 0, 0, 0, 0};
    if (SORTED)
        for (uint32_t k = 0; k < SHADE_CLASSES; k++)
            seg[k + 1] = seg[k] + w.scount[in * SHADE_CLASSES + k];
    for (;;) {
        uint32_t base = warp_fetch(&w.fetch[2 + in]);
        if (base >= count)
            break;
        uint32_t i = base + lane_id();
        bool query = false;
        uint32_t p = 0, kq = 0;
        CacheHook hk;
        if (i < count) {
            if (SORTED) {
                uint32_t k = i >= seg[1] ? (i >= seg[2] ? (i >= seg[3] ? 3u : 2u) : 1u) : 0u;
                p = w.squeue[(size_t)k * n + (i - seg[k])];
            } else {
                p = qin[i];
            }
            uint32_t meta = w.meta[p];
            uint32_t depth = meta & 0xffu;
            kq = meta >> 8;
            PathState<false> st = loadState<false>(w, p);
            uint4 hr = w.hits[p];
            Hit h;
            h.hit = hr.x != 0;
            h.inst = hr.y;
            h.prim = hr.z;
            h.t = __uint_as_float(hr.w);
            ShadowReq req;
            if (CACHE) {
                // The spread starts at zero with each sample (a path may pass a cut-out surface at
                // depth 0 without meeting the hook).
                float2 sp = depth > 0 ? q.st[p] : make_float2(0.0f, 0.0f);
                hk.c = q.spread;
                hk.train = false;
                hk.a0 = sp.x;
                hk.a = sp.y;
            }
            bool alive = shadePath<false, RESTIR, true, CACHE>(c, st, h, depth, p, &req, &hk) && depth + 1 < w.depth;
            if (CACHE) {
                query = hk.query && !bad3(st.parts.total);
                if (alive)
                    q.st[p] = make_float2(hk.a0, hk.a);
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
            // Records of sample kq go to range kq (one atomic per sample present in the warp).
            uint32_t grp = __match_any_sync(FULL, query ? kq : 0xffffffffu);
            uint32_t leader = __ffs(grp) - 1u;
            uint32_t first = 0;
            if (query && lane_id() == leader)
                first = atomicAdd(q.qcount + kq, __popc(grp));
            first = __shfl_sync(FULL, first, leader);
            uint32_t slot = first + __popc(grp & ((1u << lane_id()) - 1u));
            if (query && slot < q.qcap)
                cacheQueryRecord(q.qrec + ((size_t)kq * q.qcap + slot) * CACHE_REC_WORDS, hk, p);
        }
        __syncwarp();
    }
}

// Finish of one slot after its shadow ray (or with no light sample): add the unoccluded sample,
// then queue the path for its next depth, or finish it and restart the slot with the batch's next
// sample. Returns whether the slot goes to the next wave's queue.
template <typename A, bool RESTIR = false>
__device__ __forceinline__ bool finishSlot(const Ctx& c, const Wave& w, uint32_t p, bool blocked)
{
    uint32_t n = w.n;
    uint32_t meta = w.meta[p];
    uint32_t depth = meta & 0xffu, k = meta >> 8;
    uint32_t flags = __float_as_uint(w.sreq[n + p].w);
    float4 tot = w.state[3 * n + p];
    V3 total = v3(tot.x, tot.y, tot.z);
    if ((flags & 1u) && !blocked) {
        float4 r2 = w.sreq[2 * n + p];
        total += v3(r2.x, r2.y, r2.z);
        if (flags & 2u)
            w.state[3 * n + p] = make_float4(total.x, total.y, total.z, tot.w);
    }
    if (flags & 2u) {
        w.meta[p] = (depth + 1) | (k << 8);
        return true;
    }
    PathState<false> st;
    st.parts.zero();
    st.parts.total = total;
    st.visLit = st.visTotal = 0.0f;
    // The deferred stages never carry ReSTIR GI (the host traces the light sample inside shade
    // when GI is on), so the path's GI flag is false here.
    st.gi = false;
    st.chan = -1;
    finishPath<false, A, RESTIR>(c, st, p);
    if (k + 1 < c.p[P_SAMPLES_PER_DISPATCH] && (c.p[P_ADAPTIVE] == 0 || pixelActive<A>(c, p))) {
        PathState<false> nx = generatePathFor<false>(c, p % c.p[P_WIDTH], p / c.p[P_WIDTH], c.p[P_SAMPLE] + k + 1);
        storePath<false>(w, nx, p);
        w.meta[p] = (k + 1) << 8;
        return true;
    }
    return false;
}

template <typename A, bool RESTIR = false>
__global__ void __launch_bounds__(128, 8) wf_stream_shadow(const __grid_constant__ Ctx c, Wave w, uint32_t wave)
{
    uint32_t in = wave & 1u, out = in ^ 1u;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        w.fetch[out] = 0;
    uint32_t count = w.counts[in];
    const uint32_t* qin = w.queue[in];
    uint32_t* qout = w.queue[out];
    uint32_t n = w.n;
    __shared__ uint32_t slot[4], fetched;
    for (;;) {
        uint32_t base = block_fetch(&w.fetch[4 + in], &fetched);
        if (base >= count)
            break;
        uint32_t i = base + threadIdx.x;
        bool live = false;
        uint32_t p = 0;
        if (i < count) {
            p = qin[i];
            float4 r1 = w.sreq[n + p];
            bool occ = false;
            if (__float_as_uint(r1.w) & 1u) {
                float4 r0 = w.sreq[p];
                occ = occluded(c, v3(r0.x, r0.y, r0.z), v3(r1.x, r1.y, r1.z), r0.w);
            }
            live = finishSlot<A, RESTIR>(c, w, p, occ);
        }
        block_append<4>(&w.counts[out], qout, live, p, slot);
    }
}

// Dynamic-fetch forms of the streaming extend and shadow stages (vgt::trace_queue). A warp refills
// when at least w.refill of its lanes are idle and runs at most w.steps node visits between refills
// (w.shadow_refill, w.shadow_steps for the shadow stage; vg_set_traversal_fetch). Measured on the
// 1M-triangle workload (BVH8 with SAH node cost 0.5, each lane testing its own triangles): refills
// of 4 to 10 lanes are within 0.5% of one another and 2% faster than 16; 24 is 3% slower; 2 or 8
// steps are slower than 4.

// Runs trace_queue, or with COOP trace_queue_coop (warp-cooperative leaf testing; blocks of 128
// threads, the launchers' size): the same hits either way.
template <bool ANY, bool COOP, typename GetRay, typename PutHit>
__device__ __forceinline__ void trace_queue_any(const Ctx& c, uint32_t* fetch, uint32_t count, uint32_t refill,
                                                uint32_t steps, GetRay get, PutHit put)
{
    if (COOP) {
        __shared__ vgt::CoopWarp coop[vgt::COOP_WARPS];
        vgt::trace_queue_coop<ANY>(c.s.nodes, c.s.tris, fetch, count, c.err, refill, steps, coop[threadIdx.x >> 5],
                                   get, put);
    } else {
        vgt::trace_queue<ANY>(c.s.nodes, c.s.tris, fetch, count, c.err, refill, steps, get, put);
    }
}

// Minimum resident 128-thread blocks per SM requested for the dynamic-fetch traversal stages (a
// register cap: 8 blocks leave 64 registers per thread).
#ifndef VG_TRACE_MIN_BLOCKS
#define VG_TRACE_MIN_BLOCKS 8
#endif

template <bool STATS, bool COOP>
__global__ void __launch_bounds__(128, VG_TRACE_MIN_BLOCKS) wf_stream_extend_dyn(const __grid_constant__ Ctx c, Wave w, uint32_t wave)
{
    uint32_t in = wave & 1u, out = in ^ 1u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        w.counts[out] = 0;
        w.fetch[2 + in] = 0;
        w.fetch[4 + in] = 0;
        w.fetch[6 + in] = 0;
    }
    uint32_t count = w.counts[in];
    const uint32_t* qin = w.queue[in];
    uint32_t n_rays = 0, n_nodes = 0, n_tests = 0, n_later = 0;
    trace_queue_any<false, COOP>(
        c, &w.fetch[in], count, w.refill, w.steps,
        [&](uint32_t i, V3& o, V3& d, float& tmax) {
            uint32_t p = qin[i];
            float4 a = w.state[p];
            float4 b = w.state[w.n + p];
            o = v3(a.x, a.y, a.z);
            d = v3(b.x, b.y, b.z);
            tmax = 1.0e30f;
            return true;
        },
        [&](uint32_t i, const vgt::TraceHit& q) {
            uint32_t p = qin[i];
            w.hits[p] = make_uint4(q.hit ? 1u : 0u, q.hit ? q.inst : 0u, q.hit ? q.prim : 0u,
                                   __float_as_uint(q.hit ? q.t : 0.0f));
            if (STATS) {
                n_rays++;
                n_nodes += q.nodes;
                n_tests += q.tests;
                n_later += (w.meta[p] & 0xffu) != 0 ? 1u : 0u;
            }
        });
    if (STATS) {
        warp_count(&w.tstats[0], n_rays);
        warp_count(&w.tstats[1], n_nodes);
        warp_count(&w.tstats[2], n_tests);
        warp_count(&w.tstats[3], n_later);
    }
}

// Shadow rays of the deferred light samples, any hit (opaque scenes: one layer, no opacity roll).
// The result goes to hits[p].x (1 occluded), which the finish stage reads. STATS: the rays traced
// are counted into tstats[4].
// The same for the shadow stage alone (its any-hit rays end at the first occluder; its grid
// follows). 10 or 12 blocks (48 or 40 registers) make the stage 4% and 9% slower than 8.
#ifndef VG_SHADOW_MIN_BLOCKS
#define VG_SHADOW_MIN_BLOCKS VG_TRACE_MIN_BLOCKS
#endif

template <bool STATS, bool COOP>
__global__ void __launch_bounds__(128, VG_SHADOW_MIN_BLOCKS) wf_stream_shadow_trace(const __grid_constant__ Ctx c, Wave w, uint32_t wave)
{
    uint32_t in = wave & 1u;
    uint32_t count = w.counts[in];
    const uint32_t* qin = w.queue[in];
    uint32_t n = w.n;
    uint32_t n_rays = 0;
    trace_queue_any<true, COOP>(
        c, &w.fetch[4 + in], count, w.shadow_refill, w.shadow_steps,
        [&](uint32_t i, V3& o, V3& d, float& tmax) {
            uint32_t p = qin[i];
            float4 r1 = w.sreq[n + p];
            if (!(__float_as_uint(r1.w) & 1u)) {
                tmax = 0.0f;
                return false;
            }
            float4 r0 = w.sreq[p];
            o = v3(r0.x, r0.y, r0.z);
            d = v3(r1.x, r1.y, r1.z);
            tmax = r0.w;
            if (STATS)
                n_rays++;
            return true;
        },
        [&](uint32_t i, const vgt::TraceHit& q) { ((uint32_t*)w.hits)[4 * (size_t)qin[i]] = q.hit ? 1u : 0u; });
    if (STATS)
        warp_count(&w.tstats[4], n_rays);
}

// After the shadow trace: add the unoccluded light sample, then queue, finish or restart each slot
// (the second half of wf_stream_shadow).
// Minimum resident 128-thread blocks per SM requested for the finish stage (a register cap; its grid
// follows). 12 or 16 blocks (40 or 32 registers) are 1.1-1.6% slower per benchmark step than 8.
#ifndef VG_FINISH_MIN_BLOCKS
#define VG_FINISH_MIN_BLOCKS 8
#endif

template <typename A, bool RESTIR = false>
__global__ void __launch_bounds__(128, VG_FINISH_MIN_BLOCKS) wf_stream_finish(const __grid_constant__ Ctx c, Wave w, uint32_t wave)
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
        bool live = false;
        uint32_t p = 0;
        if (i < count) {
            p = qin[i];
            live = finishSlot<A, RESTIR>(c, w, p, ((const uint32_t*)w.hits)[4 * (size_t)p] != 0u);
        }
        block_append<4>(&w.counts[out], qout, live, p, slot);
    }
}

// The tail of a streaming batch: once few slots are live, one thread per remaining slot runs its
// path and the rest of its samples to the end, trace and shade in a loop as the megakernel does,
// instead of one half-empty wave per bounce. Same functions, same order per pixel, same sums.
// With CACHE (lighting split off) paths end at the cache as in wf_stream_shade_deferred.
template <bool LIGHT, typename A, bool CACHE = false, bool RESTIR = false>
__global__ void __launch_bounds__(128, VG_TAIL_MIN_BLOCKS) wf_stream_tail(const __grid_constant__ Ctx c, Wave w,
                                                                          uint32_t wave, CacheWave q)
{
    static_assert(!(CACHE && LIGHT), "the cache runs with the lighting split off");
    uint32_t in = wave & 1u;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.counts[in])
        return;
    uint32_t p = w.queue[in][i];
    uint32_t meta = w.meta[p];
    uint32_t depth = meta & 0xffu, k = meta >> 8;
    uint32_t batch = c.p[P_SAMPLES_PER_DISPATCH];
    PathState<LIGHT> st = loadState<LIGHT>(w, p);
    CacheHook hk;
    if (CACHE) {
        float2 sp = depth > 0 ? q.st[p] : make_float2(0.0f, 0.0f);
        hk.c = q.spread;
        hk.train = false;
        hk.a0 = sp.x;
        hk.a = sp.y;
    }
    for (;;) {
        if (shadePathCall<LIGHT, RESTIR, false, CACHE>(c, st, traceClosest(c, st.org, st.dir), depth, p, nullptr, &hk) &&
            depth + 1 < w.depth) {
            depth++;
            continue;
        }
        if (CACHE && hk.query && !bad3(st.parts.total)) {
            uint32_t slot = atomicAdd(q.qcount + k, 1u);
            if (slot < q.qcap)
                cacheQueryRecord(q.qrec + ((size_t)k * q.qcap + slot) * CACHE_REC_WORDS, hk, p);
        }
        finishPath<LIGHT, A, RESTIR>(c, st, p);
        if (k + 1 < batch && (c.p[P_ADAPTIVE] == 0 || pixelActive<A>(c, p))) {
            k++;
            depth = 0;
            st = generatePathFor<LIGHT>(c, p % c.p[P_WIDTH], p / c.p[P_WIDTH], c.p[P_SAMPLE] + k);
            if (CACHE)
                hk.a0 = hk.a = 0.0f;
            continue;
        }
        break;
    }
}

// Closest hits of caller-given rays (6 floats each: origin, direction): the traversal alone, for
// checking it against an independent implementation and for timing it.
static __global__ void __launch_bounds__(128) trace_rays(const __grid_constant__ Ctx c, const float* rays, uint4* out,
                                                   uint32_t n, uint32_t* fetch)
{
    for (;;) {
        uint32_t base = warp_fetch(fetch);
        if (base >= n)
            break;
        uint32_t i = base + lane_id();
        if (i < n) {
            const float* r = rays + 6 * (size_t)i;
            Hit h = traceClosest(c, v3(r[0], r[1], r[2]), v3(r[3], r[4], r[5]));
            out[i] = make_uint4(h.hit ? 1u : 0u, h.inst, h.prim, __float_as_uint(h.t));
        }
        __syncwarp();
    }
}

// Any-hit queries of caller-given rays (7 floats each: origin, direction, tmax) through the
// shadow-ray path (`occluded`, including translucent layers).
static __global__ void __launch_bounds__(128) occlusion_rays(const __grid_constant__ Ctx c, const float* rays, uint32_t* out,
                                                       uint32_t n)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const float* r = rays + 7 * (size_t)i;
    out[i] = occluded(c, v3(r[0], r[1], r[2]), v3(r[3], r[4], r[5]), r[6]) ? 1u : 0u;
}

} // namespace vgk
