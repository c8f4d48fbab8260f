// Host-side internals of the C ABI shared by its translation units: status and error text,
// device buffers, the context / renderer / accumulation objects and the launch helpers.
#pragma once

#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <string>
#include <mutex>
#include <thread>
#include <vector>
#include "../../include/vgcuda.h"
#include "bvh_build.h"
#include "launch.h"

namespace vgh {
// Error text and out-of-memory figures of the last failing call on this thread (one instance
// across translation units).
inline thread_local std::string g_err;
inline thread_local uint64_t g_oom_needed = 0, g_oom_available = 0;
} // namespace vgh
using vgh::g_err;
using vgh::g_oom_needed;
using vgh::g_oom_available;

using namespace vgl;

struct VgCache;

namespace {


int fail(int status, const std::string& msg)
{
    g_err = msg;
    return status;
}

int cuda_fail(cudaError_t e, const char* what)
{
    if (e == cudaErrorMemoryAllocation)
        return fail(VG_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e));
    return fail(VG_ERR_KERNEL, std::string(what) + ": " + cudaGetErrorString(e));
}

#define VG_CHECK(expr, what)                                                                                        \
    do {                                                                                                            \
        cudaError_t e_ = (expr);                                                                                    \
        if (e_ != cudaSuccess)                                                                                      \
            return cuda_fail(e_, what);                                                                             \
    } while (0)

uint32_t f2u(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

float u2f(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// Host deadline for one blocking call; GPU waits poll against it instead of blocking forever.
double wait_deadline_seconds()
{
    const char* s = getenv("VG_TIMEOUT_S");
    double v = s ? atof(s) : 0.0;
    return v > 0.0 ? v : 600.0;
}

int wait_event(cudaEvent_t ev)
{
    auto t0 = std::chrono::steady_clock::now();
    double limit = wait_deadline_seconds();
    for (;;) {
        cudaError_t e = cudaEventQuery(ev);
        if (e == cudaSuccess)
            return VG_OK;
        if (e != cudaErrorNotReady)
            return cuda_fail(e, "kernel execution");
        double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (dt > limit)
            return fail(VG_ERR_TIMEOUT, "the GPU did not finish within " + std::to_string(limit) + " s");
        std::this_thread::sleep_for(std::chrono::microseconds(dt < 0.01 ? 20 : 200));
    }
}

} // namespace

namespace vgh {
// Device allocations and frees made by this library since it was loaded (all of them go through
// alloc() and DevBuf), readable through vg_debug_allocations.
inline std::atomic<uint64_t> g_mallocs{0}, g_frees{0};
} // namespace vgh

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) {
            cudaFree(p);
            vgh::g_frees++;
        }
        p = nullptr;
        bytes = 0;
    }
};

// Makes `device` the calling thread's current device for one entry-point call and restores the
// caller's device when the call returns (a negative ordinal leaves everything as it is). Every
// object of the C ABI belongs to its context's device; with this guard a caller that drives
// several devices from one thread can interleave calls on their objects freely.
struct DevGuard {
    int prev = -1;
    explicit DevGuard(int device)
    {
        int cur = -1;
        if (device < 0)
            return;
        if (cudaGetDevice(&cur) != cudaSuccess) {
            cudaGetLastError(); // leave no error behind for the call's own launch checks
            return;
        }
        if (cur == device)
            return;
        if (cudaSetDevice(device) == cudaSuccess)
            prev = cur;
        else
            cudaGetLastError();
    }
    ~DevGuard()
    {
        if (prev >= 0)
            cudaSetDevice(prev);
    }
    DevGuard(const DevGuard&) = delete;
    DevGuard& operator=(const DevGuard&) = delete;
};

} // namespace

struct BatchState; // vg_batch_render's device buffers and captured graph (batch.cu)

struct VgContext {
    int device = 0;
    cudaStream_t stream = nullptr;
    int sms = 0;
    uint64_t uploaded = 0;
    BatchState* batch = nullptr;
    int batch_blocks_per_sm = 0; // 0: as many as fit (vg_batch_tune chooses)
    int batch_order = 0;         // VgBatchOrder
    uint64_t batch_wavefront_pixels = 0;          // requests at least this large share the batch wavefront
    uint32_t batch_wave_slots = 1u << 21;         // path slots of the batch wavefront
    bool batch_device_loop = true;                // batch wavefront: bounce loop in the graph (else the host's)
    cudaStream_t side = nullptr;                 // second stream (created on first use): cache training paths
    cudaEvent_t fork = nullptr, join = nullptr;  // ordering between `stream` and `side`
    ~VgContext();
};

struct Restir {
    bool on = false;
    bool di = true, gi = false;
    uint32_t candidates = 4, history = 4;
    bool operator==(const Restir& o) const
    {
        return on == o.on && (!on || (di == o.di && gi == o.gi && candidates == o.candidates && history == o.history));
    }
};

constexpr uint32_t MAX_CACHE_FRAME = 16;           // samples per radiance-cache frame at most
constexpr uint32_t CACHE_WARMUP_SAMPLE = 0x40000000u; // first sample index of cache warm-up frames

struct VgRenderer {
    VgContext* ctx = nullptr;
    int device = -1; // the context's device, kept here so no call dereferences a destroyed context
    DevBuf positions, indices, uvs, vnormals, instances, materials, lights, emitters, emit_cdf, emit_guide, env_pixels,
        env_marginal, env_cond, env_guide, texels, tex_info, nodes, tris, err, scratch;
    vgd::DeviceScene ds{};
    VgSceneInfo info{};
    VgView view{};
    VgBvhInfo bvh{};
    uint32_t instance_count = 0;
    bool multiscatter = true;
    int integrator = VG_MEGAKERNEL;
    bool stage_timing = false;
    bool traversal_stats = false;
    int wavefront_mode = VG_WAVEFRONT_STREAMING;
    uint32_t tail_threshold = 32768; // live slots at or below which the streaming tail runs in one launch
    bool adaptive = false;
    float adaptive_threshold = 0.02f;
    uint32_t adaptive_min_spp = 16;
    Restir restir;
    uint32_t max_depth = DEFAULT_MAX_DEPTH;
    int precision = 64;
    int extend_blocks = 0;
    int shade_blocks[8] = {};
    int stream_shade_blocks[8] = {};
    int deferred_blocks[2] = {};
    int deferred_restir_blocks[2] = {};
    int shadow_blocks[2] = {};
    bool defer_shadows = true; // streaming: shadow rays of the light sample in their own stage
    bool dynamic_fetch = true; // streaming: traversal stages refill idle lanes from the queue
    bool coop_tris = false;    // streaming, dynamic fetch: warp-cooperative leaf testing (measured slower)
    bool material_sort = true; // streaming, deferred shadows: shade the wave's slots class by class
    uint32_t fetch_refill = 8, fetch_steps = 4;               // dynamic fetch, extend stage
    uint32_t shadow_fetch_refill = 8, shadow_fetch_steps = 4; // dynamic fetch, shadow stage
    uint32_t graph_waves = 0;  // streaming: waves per captured CUDA graph (0: launched one by one)
    float bvh_traversal_cost = 0.5f; // SAH node-visit cost the BVH8 was built with (0.5: the fastest measured on the 1M-triangle scene)
    float bounds_lo[3] = {0, 0, 0}, bounds_hi[3] = {0, 0, 0}; // world box of the triangles
    uint64_t texel_key = 0, env_key = 0; // hashes of the uploaded texture and environment tables
    VgCache* cache = nullptr;  // radiance cache integrator when set
    float cache_spread = 0.01f;
    uint32_t cache_train_paths = 16384;
    uint32_t cache_steps = 4;
    uint32_t cache_batch = 16384;
    uint32_t cache_frame = 4;     // integrator WAVEFRONT: samples per cache frame (one cache update per frame)
    uint32_t cache_warmup = 0;    // training-only frames before the first sample of an accumulation
    int cache_shade_blocks[2] = {};
};

struct VgAccum {
    VgRenderer* owner = nullptr;
    int device = -1; // the owner's device (destroying the accumulation must not read the owner)
    uint32_t width = 0, height = 0;
    bool lighting = false;
    int precision = 64;
    uint32_t samples = 0;
    uint32_t first_sample = 0; // sample index of the first sample (vg_accum_set_first_sample)
    double gpu_seconds = 0.0;
    bool stage_ran = false;
    double stage_seconds[2] = {0.0, 0.0};
    uint64_t extend_launches_timed = 0;
    uint64_t launches = 0;
    DevBuf accum, stats, light;
    mutable DevBuf sums32; // f32 copy of f64 sums for vg_accum_read_sums
    bool adaptive_fixed = false; // adaptive setting captured at the first sample
    bool adaptive = false;
    Restir restir;               // captured at the first sample
    DevBuf re_g[2], re_n[2], re_x[2], re_m[2];
    DevBuf re_gx[2], re_gn[2], re_gl[2], re_s[7]; // ReSTIR GI planes
    DevBuf state, hits, queue[2], counts, fetch, tstats, meta, sreq, squeue, scount;
    DevBuf mk_next;                  // the megakernel's pixel counter
    uint32_t* host_counts = nullptr; // pinned ring of wave output counts (streaming wavefront)
    uint32_t last_waves = 0;
    std::vector<uint32_t> wave_live; // last streaming accumulate: live slots after each wave
    std::vector<float> wave_ms;      // with stage timing: extend, shade milliseconds per wave
    float tail_ms = 0.0f;            // with stage timing: the tail launch of the last call
    size_t wave_stages = 2;          // kernels per wave in wave_ms (2, or 3 with deferred shadows)
    ~VgAccum()
    {
        if (host_counts)
            cudaFreeHost(host_counts);
    }
    size_t wavefront_bytes = 0;
    size_t restir_bytes = 0;
    uint32_t last_depth = 0; // max depth of the last wavefront sample
    DevBuf cache_q, cache_t, cache_ctr; // radiance cache: query and training records, their counts
    DevBuf cache_spread;                // radiance cache on the streaming wavefront: a0, a per slot
    uint32_t cache_frame_last = 0;      // samples in the last cache frame (query counters in use)
    double cache_seconds[3] = {0, 0, 0}; // with stage timing: paths, inference, training
};

namespace {

// The device an object of the C ABI belongs to (-1 for a null handle).
int dev_of(const VgContext* ctx) { return ctx ? ctx->device : -1; }
int dev_of(const VgRenderer* r) { return r ? r->device : -1; }
int dev_of(const VgAccum* acc) { return acc ? acc->device : -1; }

int check_fits(size_t bytes)
{
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaMemGetInfo");
    if (bytes > free_b) {
        g_oom_needed = bytes;
        g_oom_available = free_b;
        return fail(VG_ERR_OOM, "out of GPU memory: needed " + std::to_string(bytes) + " bytes, available " +
                                    std::to_string(free_b));
    }
    return VG_OK;
}

int alloc(DevBuf& b, size_t bytes, cudaStream_t s, bool zero)
{
    b.release();
    size_t n = std::max<size_t>(bytes, 16);
    int st = check_fits(n);
    if (st != VG_OK)
        return st;
    cudaError_t e = cudaMalloc(&b.p, n);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    vgh::g_mallocs++;
    b.bytes = n;
    if (zero) {
        e = cudaMemsetAsync(b.p, 0, n, s);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaMemsetAsync");
    }
    return VG_OK;
}

int upload(VgContext* ctx, DevBuf& b, const void* src, size_t bytes)
{
    int st = alloc(b, bytes, ctx->stream, bytes == 0);
    if (st != VG_OK)
        return st;
    if (bytes > 0) {
        if (!src)
            return fail(VG_ERR_INVALID, "null table pointer with non-zero length");
        VG_CHECK(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload");
        ctx->uploaded += bytes;
    }
    return VG_OK;
}

// Checks every index the kernels follow, so a malformed table is an error here instead of an
// out-of-bounds read on the GPU.
int validate(const VgPacked* pk)
{
    if (pk->instance_count == 0 || pk->instances_len == 0)
        return fail(VG_ERR_SCENE, "scene has no instances");
    if (pk->instances_len != (size_t)pk->instance_count * INSTANCE_WORDS)
        return fail(VG_ERR_INVALID, "instance table length does not match the instance count");
    size_t verts = pk->positions_len / 3;
    if (pk->positions_len % 3 != 0 || pk->uvs_len != 2 * verts || pk->vnormals_len != 3 * verts)
        return fail(VG_ERR_INVALID, "vertex tables disagree in length");
    if (pk->materials_len % MATERIAL_WORDS != 0 || pk->materials_len == 0)
        return fail(VG_ERR_INVALID, "material table length is not a multiple of 24");
    size_t materials = pk->materials_len / MATERIAL_WORDS;
    size_t textures = pk->tex_info_len / 4;
    if (pk->tex_info_len % 4 != 0)
        return fail(VG_ERR_INVALID, "texture info length is not a multiple of 4");
    for (size_t t = 0; t < textures; t++) {
        uint64_t off = pk->tex_info[4 * t], w = pk->tex_info[4 * t + 1], h = pk->tex_info[4 * t + 2],
                 levels = pk->tex_info[4 * t + 3];
        if (w == 0 || h == 0 || levels == 0)
            return fail(VG_ERR_INVALID, "texture with zero size");
        uint64_t end = off, lw = w, lh = h;
        for (uint64_t k = 0; k < levels; k++) {
            end += lw * lh;
            lw = std::max<uint64_t>(lw / 2, 1);
            lh = std::max<uint64_t>(lh / 2, 1);
        }
        if (3 * end > pk->texels_len)
            return fail(VG_ERR_INVALID, "texture mip chain beyond the texel table");
    }
    for (size_t m = 0; m < materials; m++) {
        for (int k : {10, 11, 12, 13, 23}) {
            float v = pk->materials[m * MATERIAL_WORDS + k];
            if (!(v >= 0.0f) || v > (float)textures)
                return fail(VG_ERR_INVALID, "material refers to a missing texture");
        }
    }
    uint32_t ec = pk->info.emitter_count;
    if (pk->emitters_len != (size_t)ec * EMITTER_WORDS || pk->emit_cdf_len != ec)
        return fail(VG_ERR_INVALID, "emitter tables disagree with the emitter count");
    uint32_t lc = pk->info.light_count;
    size_t light_need = (size_t)lc * LIGHT_WORDS + ALBEDO_WORDS + 2 * (size_t)pk->instance_count;
    if (pk->lights_len < light_need)
        return fail(VG_ERR_INVALID, "light table shorter than lights + albedo tables + link masks");
    for (uint32_t l = 0; l < lc; l++) {
        uint32_t kind = pk->lights[l * LIGHT_WORDS];
        if (kind > 3)
            return fail(VG_ERR_INVALID, "unknown light kind");
        if (pk->lights[l * LIGHT_WORDS + 13] > 3)
            return fail(VG_ERR_INVALID, "light slot beyond 3");
        uint32_t ies = pk->lights[l * LIGHT_WORDS + 15];
        if (ies != 0 && (size_t)(ies - 1) + 9 + 361 * 181 > pk->lights_len)
            return fail(VG_ERR_INVALID, "IES profile beyond the light table");
    }
    if (pk->mesh_count == 0 || !pk->tlas_mesh)
        return fail(VG_ERR_INVALID, "missing mesh ranges");
    for (size_t i = 0; i < pk->instance_count; i++) {
        const uint32_t* rec = &pk->instances[i * INSTANCE_WORDS];
        uint32_t m = pk->tlas_mesh[i];
        if (m >= pk->mesh_count)
            return fail(VG_ERR_INVALID, "instance refers to a missing mesh");
        const VgMeshRange& mr = pk->meshes[m];
        if (rec[0] != mr.vertex_offset || rec[1] != mr.index_offset)
            return fail(VG_ERR_INVALID, "instance record disagrees with its mesh range");
        if (mr.index_count % 3 != 0 || (uint64_t)mr.index_offset + mr.index_count > pk->indices_len)
            return fail(VG_ERR_INVALID, "mesh index range beyond the index table");
        if ((uint64_t)mr.vertex_offset + mr.vertex_count > verts)
            return fail(VG_ERR_INVALID, "mesh vertex range beyond the vertex table");
        for (uint32_t k = 0; k < mr.index_count; k++)
            if (pk->indices[mr.index_offset + k] >= mr.vertex_count)
                return fail(VG_ERR_INVALID, "triangle index beyond its mesh's vertices");
        if (rec[2] >= materials)
            return fail(VG_ERR_INVALID, "instance refers to a missing material");
        if (rec[3] != 0 && (uint64_t)rec[3] - 1 + mr.index_count / 3 > ec)
            return fail(VG_ERR_INVALID, "instance emitter range beyond the emitter table");
    }
    uint32_t ew = pk->info.env_width, eh = pk->info.env_height;
    if (ew > 0) {
        if (eh == 0 || pk->env_pixels_len != 3 * (size_t)ew * eh || pk->env_marginal_len != eh ||
            pk->env_conditional_len != (size_t)ew * eh)
            return fail(VG_ERR_INVALID, "environment tables disagree with their size");
    }
    return VG_OK;
}

int blocks_for(VgRenderer* r, int per_sm) { return std::max(1, per_sm) * r->ctx->sms; }

// The wavefront buffers of an accumulation (allocated on its first wavefront accumulate).
vgk::Wave wave_of(const VgRenderer* r, const VgAccum* acc)
{
    vgk::Wave w;
    w.state = (float4*)acc->state.p;
    w.hits = (uint4*)acc->hits.p;
    w.queue[0] = (uint32_t*)acc->queue[0].p;
    w.queue[1] = (uint32_t*)acc->queue[1].p;
    w.counts = (uint32_t*)acc->counts.p;
    w.fetch = (uint32_t*)acc->fetch.p;
    w.tstats = (unsigned long long*)acc->tstats.p;
    w.sreq = (float4*)acc->sreq.p;
    w.meta = (uint32_t*)acc->meta.p;
    w.n = acc->width * acc->height;
    w.depth = r->max_depth;
    w.refill = r->fetch_refill;
    w.steps = r->fetch_steps;
    w.shadow_refill = r->shadow_fetch_refill;
    w.shadow_steps = r->shadow_fetch_steps;
    w.squeue = (uint32_t*)acc->squeue.p;
    w.scount = (uint32_t*)acc->scount.p;
    return w;
}

vgx::Variant variant_of(const VgRenderer*, const VgAccum* acc)
{
    vgx::Variant v;
    v.light = acc->lighting;
    v.restir = acc->restir.on;
    v.f64 = acc->precision == 64;
    return v;
}

// pack.rs:828-874, with the renderer's depth in word 7.
void base_params(const VgRenderer* r, const VgAccum* acc, uint32_t* p)
{
    memset(p, 0, PARAM_WORDS * 4);
    p[P_WIDTH] = acc->width;
    p[P_HEIGHT] = acc->height;
    p[P_TAN_HALF_FOV] = f2u(r->view.camera[2]);
    p[P_APERTURE] = f2u(r->view.aperture);
    p[P_FOCUS] = f2u(r->view.focus);
    p[P_LIGHT_COUNT] = r->info.light_count;
    p[P_MAX_DEPTH] = r->max_depth;
    for (int i = 0; i < 12; i++)
        p[P_CAMERA + i] = f2u(r->view.camera[4 + i]);
    for (int i = 0; i < 3; i++)
        p[P_SKY + i] = f2u(r->info.sky[i]);
    p[P_EMITTER_COUNT] = r->info.emitter_count;
    p[P_ENV_W] = r->info.env_width;
    p[P_ENV_H] = r->info.env_height;
    p[P_ENV_PDF_SCALE] = f2u(r->info.env_pdf_scale);
    p[P_PIXEL_CONE] = f2u(2.0f * r->view.camera[2] / (float)acc->height);
    p[P_VIRTUAL_LIGHT] = r->info.virtual_light;
    p[P_TRANSPARENT_BG] = r->info.transparent_background;
    p[P_SHIFT_X] = f2u(r->view.shift[0]);
    p[P_SHIFT_Y] = f2u(r->view.shift[1]);
    p[P_LIGHTING] = acc->lighting ? 1u : 0u;
    p[P_MULTISCATTER] = r->multiscatter ? 1u : 0u;
    if (r->adaptive) {
        p[P_ADAPTIVE] = 1;
        p[P_ADAPTIVE_THRESHOLD] = f2u(r->adaptive_threshold);
        p[P_ADAPTIVE_MIN_SPP] = r->adaptive_min_spp;
    }
    if (r->restir.on) {
        p[P_RESTIR] = (r->restir.di ? 1u : 0u) | (r->restir.gi ? 2u : 0u);
        p[P_RESTIR_CANDIDATES] = r->restir.candidates;
        p[P_RESTIR_HISTORY] = r->restir.history;
    }
}

vgd::Ctx make_ctx(VgRenderer* r, VgAccum* acc)
{
    vgd::Ctx c;
    memset(&c, 0, sizeof(c));
    c.s = r->ds;
    if (acc) {
        base_params(r, acc, c.p);
        c.accum = acc->accum.p;
        c.stats = acc->stats.p;
        c.lighting = (float*)acc->light.p;
        for (int h = 0; h < 2; h++) {
            c.re.g[h] = (float4*)acc->re_g[h].p;
            c.re.n[h] = (float4*)acc->re_n[h].p;
            c.re.x[h] = (float4*)acc->re_x[h].p;
            c.re.m[h] = (float*)acc->re_m[h].p;
            c.re.gx[h] = (float4*)acc->re_gx[h].p;
            c.re.gn[h] = (float4*)acc->re_gn[h].p;
            c.re.gl[h] = (float4*)acc->re_gl[h].p;
        }
        for (int k = 0; k < 7; k++)
            c.re.s[k] = (float4*)acc->re_s[k].p;
    }
    c.err = (uint32_t*)r->err.p;
    return c;
}

int read_err(VgRenderer* r)
{
    uint32_t e = 0;
    VG_CHECK(cudaMemcpyAsync(&e, r->err.p, 4, cudaMemcpyDeviceToHost, r->ctx->stream), "error flag");
    VG_CHECK(cudaStreamSynchronize(r->ctx->stream), "error flag");
    if (e & bvh8::ERR_STACK)
        return fail(VG_ERR_KERNEL, "BVH traversal stack overflow");
    if (e)
        return fail(VG_ERR_KERNEL, "kernel reported error status " + std::to_string(e));
    return VG_OK;
}

} // namespace

struct EventPool {
    std::vector<cudaEvent_t> ev;
    size_t used = 0;
    cudaEvent_t get()
    {
        if (used == ev.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            ev.push_back(e);
        }
        return ev[used++];
    }
    ~EventPool()
    {
        for (auto e : ev)
            cudaEventDestroy(e);
    }
};

// Timed stages of a wavefront accumulate: (stage, (start event, end event)).
using StageEvents = std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>>;

// Streaming wavefront (vgcuda.cu) over `samples` samples per pixel from sample0; with `q` the
// radiance-cache kernel variants.
int stream_samples(VgRenderer* r, VgAccum* acc, vgd::Ctx& c, vgx::Variant v, const vgk::Wave& w, uint32_t sample0,
                   uint32_t samples, bool timed, EventPool& pool, StageEvents& stages, const vgk::CacheWave* q);

// Radiance-cache integrator (cache.cu): the samples of one accumulate call (query paths on the
// streaming wavefront when `w` is given, else in one kernel), and the cache kernels' error status.
int cache_accumulate(VgRenderer* r, VgAccum* acc, vgd::Ctx& c, uint32_t samples, bool timed, const vgk::Wave* w);
int cache_status(VgRenderer* r);
