// C-ABI implementation of the CUDA backend (include/vgcuda.h): context, renderer (table upload,
// validation, BVH build), accumulations and the host loops that issue the kernels.
//
// Reference behaviour restated here:
//   Renderer::build / new      crates/verion-gpu-metal/src/renderer.rs:151-219
//   accumulate                 crates/verion-gpu-metal/src/renderer.rs:775-856
//   encode_megakernel          crates/verion-gpu-metal/src/renderer.rs:449-487 (8 samples a dispatch)
//   run_wavefront              crates/verion-gpu-metal/src/renderer/wavefront.rs:93-177
//   new_accumulation           crates/verion-gpu-metal/src/renderer.rs:858-903
//   base_params                crates/verion-gpu/src/pack.rs:828-874
// The host compiler must not contract floating-point expressions (-ffp-contract=off): the world
// vertices of the BVH are computed with the kernels' transformPoint arithmetic.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/vgcuda.h"
#include "bvh_build.h"
#include "launch.h"

#include "cdf_guide.h"
#include "host.h"

// Sets the thread's error text for translation units compiled without the CUDA headers.
int vg_internal_fail(int status, const char* msg) { return fail(status, msg); }

namespace {

// World-space triangles for the BVH: each instance's mesh through its transform, with the
// arithmetic of transformPoint (pt_core.slang:90-99) so the kernels' vertices match. Builds the
// BVH8 over them and records its statistics and the scene box on the renderer.
int build_world_bvh(VgRenderer* r, const VgPacked* pk, Bvh8Host& bvh)
{
    std::vector<float> verts;
    std::vector<uint32_t> tinst, tprim;
    size_t total = 0;
    for (size_t i = 0; i < pk->instance_count; i++)
        total += pk->meshes[pk->tlas_mesh[i]].index_count / 3;
    if (total > 0xffffffffu / 2)
        return fail(VG_ERR_SCENE, "too many triangles");
    verts.reserve(total * 9);
    tinst.reserve(total);
    tprim.reserve(total);
    for (size_t i = 0; i < pk->instance_count; i++) {
        const uint32_t* rec = &pk->instances[i * INSTANCE_WORDS];
        const VgMeshRange& mr = pk->meshes[pk->tlas_mesh[i]];
        float m[12];
        for (int k = 0; k < 12; k++)
            m[k] = u2f(rec[4 + k]);
        for (uint32_t t = 0; t < mr.index_count / 3; t++) {
            for (int v = 0; v < 3; v++) {
                uint32_t vi = pk->indices[mr.index_offset + 3 * t + v] + rec[0];
                float x = pk->positions[3 * vi], y = pk->positions[3 * vi + 1], z = pk->positions[3 * vi + 2];
                for (int row = 0; row < 3; row++)
                    verts.push_back(m[4 * row] * x + m[4 * row + 1] * y + m[4 * row + 2] * z + m[4 * row + 3]);
            }
            tinst.push_back((uint32_t)i);
            tprim.push_back(t);
        }
    }
    float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    for (size_t i = 0; i < verts.size(); i++) {
        lo[i % 3] = std::min(lo[i % 3], verts[i]);
        hi[i % 3] = std::max(hi[i % 3], verts[i]);
    }
    std::string err;
    if (!build_bvh8(verts.data(), tinst.data(), tprim.data(), (uint32_t)total, bvh, err, r->bvh_traversal_cost))
        return fail(VG_ERR_SCENE, err);
    for (int k = 0; k < 3; k++) {
        r->bounds_lo[k] = lo[k];
        r->bounds_hi[k] = hi[k];
    }
    r->bvh.triangles = bvh.triangles;
    r->bvh.wide_nodes = bvh.wide_nodes;
    r->bvh.wide_depth = bvh.wide_depth;
    r->bvh.binary_nodes = bvh.binary_nodes;
    r->bvh.binary_depth = bvh.binary_depth;
    r->bvh.node_bytes = bvh.nodes.size() * 4;
    r->bvh.triangle_bytes = bvh.tris.size() * 4;
    r->bvh.build_seconds = bvh.build_seconds;
    return VG_OK;
}

// Any translucent material (opacity below 1 or transmission): shadow rays then look past hits.
bool translucent_materials(const VgPacked* pk)
{
    for (size_t m = 0; m < pk->materials_len / MATERIAL_WORDS; m++)
        if (pk->materials[m * MATERIAL_WORDS + 22] < 1.0f || pk->materials[m * MATERIAL_WORDS + 23] > 0.0f)
            return true;
    return false;
}

// Guide tables of the environment's CDF searches (cdf_guide.h; sizes vgd::ENV_GUIDE_M / ENV_GUIDE_C):
// the marginal's, then one per row of the conditional.
std::vector<uint32_t> env_guide(const VgPacked* pk)
{
    uint32_t w = pk->info.env_width, h = pk->info.env_height;
    if (w == 0 || h == 0)
        return std::vector<uint32_t>(vgd::ENV_GUIDE_M + 1, 0u);
    std::vector<uint32_t> g((vgd::ENV_GUIDE_M + 1) + (size_t)h * (vgd::ENV_GUIDE_C + 1));
    cdfg::build_guide(pk->env_marginal, h, vgd::ENV_GUIDE_M, g.data());
    for (uint32_t j = 0; j < h; j++)
        cdfg::build_guide(pk->env_conditional + (size_t)j * w, w, vgd::ENV_GUIDE_C,
                          g.data() + (vgd::ENV_GUIDE_M + 1) + (size_t)j * (vgd::ENV_GUIDE_C + 1));
    return g;
}

// Guide table of the emitter CDF's searches (cdf_guide.h): cdfg::emitter_guide_buckets(n) + 1
// entries.
std::vector<uint32_t> emitter_guide(const VgPacked* pk)
{
    uint32_t n = pk->info.emitter_count;
    uint32_t K = cdfg::emitter_guide_buckets(n);
    std::vector<uint32_t> g(K + 1, 0u);
    if (n > 0)
        cdfg::build_guide(pk->emit_cdf, n, K, g.data());
    return g;
}

// FNV-1a over two tables: whether a re-packed table differs from the uploaded one.
uint64_t table_key(const void* a, size_t a_len, const void* b, size_t b_len)
{
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void* p, size_t words) {
        const uint32_t* w = (const uint32_t*)p;
        for (size_t i = 0; i < words; i++) {
            h ^= w[i];
            h *= 1099511628211ull;
        }
        h ^= words;
        h *= 1099511628211ull;
    };
    if (a)
        mix(a, a_len);
    if (b)
        mix(b, b_len);
    return h;
}

void bind_tables(VgRenderer* r)
{
    r->ds.positions = (const float*)r->positions.p;
    r->ds.indices = (const uint32_t*)r->indices.p;
    r->ds.instances = (const uint32_t*)r->instances.p;
    r->ds.materials = (const float*)r->materials.p;
    r->ds.lights = (const uint32_t*)r->lights.p;
    r->ds.emitters = (const float*)r->emitters.p;
    r->ds.emit_cdf = (const float*)r->emit_cdf.p;
    r->ds.env_pixels = (const float*)r->env_pixels.p;
    r->ds.env_marginal = (const float*)r->env_marginal.p;
    r->ds.env_cond = (const float*)r->env_cond.p;
    r->ds.env_guide = (const uint32_t*)r->env_guide.p;
    r->ds.emit_guide = (const uint32_t*)r->emit_guide.p;
    r->ds.emit_guide_k = cdfg::emitter_guide_buckets(r->info.emitter_count);
    r->ds.uvs = (const float*)r->uvs.p;
    r->ds.texels = (const float*)r->texels.p;
    r->ds.tex_info = (const uint32_t*)r->tex_info.p;
    r->ds.vnormals = (const float*)r->vnormals.p;
    r->ds.nodes = (const uint4*)r->nodes.p;
    r->ds.tris = (const float4*)r->tris.p;
}

} // namespace

// Streaming wavefront over `samples` samples per pixel from sample0 (kernels.cuh): the start, waves
// until no slot is live (the host reads each wave's live count LAG waves later, so the GPU never
// idles on the poll) and a tail launch once few slots are live. With `q` the radiance-cache
// variants run (lighting split off, shadow rays always in their own stage).
int stream_samples(VgRenderer* r, VgAccum* acc, vgd::Ctx& c, vgx::Variant v, const vgk::Wave& w, uint32_t sample0,
                   uint32_t samples, bool timed, EventPool& pool, StageEvents& stages, const vgk::CacheWave* q)
{
    cudaStream_t s = r->ctx->stream;
    int st;
    int eb = blocks_for(r, r->extend_blocks);
    acc->wave_live.clear();
    acc->wave_ms.clear();
    acc->tail_ms = 0.0f;
    int svi = v.index() & 5;
    if (r->stream_shade_blocks[svi] == 0)
        r->stream_shade_blocks[svi] = vgx::stream_shade_blocks_per_sm(v);
    int ssb = blocks_for(r, r->stream_shade_blocks[svi]);
    // Lighting split off: three-stage waves with the shadow rays in their own kernel.
    // ReSTIR GI records the second vertex's direct light while shading it, so with GI the light
    // sample's shadow ray is traced inside shade.
    bool deferred = (!acc->lighting && r->defer_shadows && !(v.restir && acc->restir.gi)) || q;
    if (deferred && r->deferred_blocks[v.f64 ? 1 : 0] == 0)
        r->deferred_blocks[v.f64 ? 1 : 0] =
            vgx::stream_deferred_blocks_per_sm(v.f64, &r->shadow_blocks[v.f64 ? 1 : 0]);
    int dsb = blocks_for(r, r->deferred_blocks[v.f64 ? 1 : 0]);
    if (deferred && v.restir) {
        if (r->deferred_restir_blocks[v.f64 ? 1 : 0] == 0)
            r->deferred_restir_blocks[v.f64 ? 1 : 0] = vgx::stream_deferred_restir_blocks_per_sm(v.f64);
        dsb = blocks_for(r, r->deferred_restir_blocks[v.f64 ? 1 : 0]);
    }
    int csb = 0;
    if (q) {
        if (r->cache_shade_blocks[v.f64 ? 1 : 0] == 0)
            r->cache_shade_blocks[v.f64 ? 1 : 0] = vgx::stream_cache_shade_blocks_per_sm(v.f64);
        csb = blocks_for(r, r->cache_shade_blocks[v.f64 ? 1 : 0]);
    }
    int shb = blocks_for(r, r->shadow_blocks[v.f64 ? 1 : 0]);
    int fnb = blocks_for(r, vgx::stream_finish_blocks_per_sm(v.f64));
    int stb = blocks_for(r, vgx::stream_shadow_trace_blocks_per_sm());
    // Material-sorted shading of the deferred shade stage (plain, ReSTIR and cache waves).
    bool sorted = deferred && r->material_sort && acc->squeue.p != nullptr && acc->scount.p != nullptr &&
                  acc->squeue.bytes >= (size_t)w.n * 4 * vgk::SHADE_CLASSES;
    int clb = r->ctx->sms * 4;
    acc->wave_stages = deferred ? 3 : 2;
    c.p[P_SAMPLE] = sample0;
    c.p[P_SAMPLES_PER_DISPATCH] = samples;
    VG_CHECK(cudaMemsetAsync(acc->counts.p, 0, 2 * 4, s), "counters");
    VG_CHECK(cudaMemsetAsync(acc->fetch.p, 0, 4 * 4, s), "counters");
    if (sorted)
        VG_CHECK(cudaMemsetAsync(acc->scount.p, 0, 2 * vgk::SHADE_CLASSES * 4, s), "counters");
    VG_CHECK((q ? vgx::launch_stream_cache_start(v.f64, s, c, w, *q) : vgx::launch_stream_start(v, s, c, w)), "stream start launch");
    acc->launches++;
    // Waves until no slot is live. The host reads each wave's output count LAG waves later,
    // so the GPU never idles on the poll; extra waves on an empty queue exit at once.
    const uint32_t LAG = 2, RING = 64;
    uint64_t max_waves = (uint64_t)samples * r->max_depth + LAG + 1;
    uint32_t* ring = acc->host_counts;
    std::vector<cudaEvent_t> ring_ev(RING);
    for (auto& e : ring_ev)
        e = pool.get();
    bool done = false;
    uint64_t wave = 0;
    if (r->graph_waves > 0 && !timed) {
        // Captured chunks of graph_waves waves (even, so the queue parity of every wave in a
        // replay matches its place in the sequence), each ending with the live count.
        uint32_t K = r->graph_waves;
        VG_CHECK(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed), "graph capture");
        cudaError_t ce = cudaSuccess;
        for (uint32_t i = 0; i < K && ce == cudaSuccess; i++) {
            ce = r->dynamic_fetch ? vgx::launch_stream_extend_dyn(r->traversal_stats, r->coop_tris, eb, s, c, w, i)
                                  : vgx::launch_stream_extend(r->traversal_stats, eb, s, c, w, i);
            if (ce == cudaSuccess && sorted)
                ce = vgx::launch_stream_classify(clb, s, c, w, i);
            if (ce == cudaSuccess && deferred) {
                ce = (q ? vgx::launch_stream_cache_shade(v.f64, sorted, csb, s, c, w, i, *q) : (v.restir ? vgx::launch_stream_shade_deferred_restir : vgx::launch_stream_shade_deferred)(v.f64, sorted, dsb, s, c, w, i));
                if (ce == cudaSuccess && r->dynamic_fetch && r->ds.shadow_any) {
                    ce = vgx::launch_stream_shadow_trace(r->traversal_stats, r->coop_tris, stb, s, c, w, i);
                    if (ce == cudaSuccess)
                        ce = (v.restir ? vgx::launch_stream_finish_restir : vgx::launch_stream_finish)(v.f64, fnb, s, c, w, i);
                } else if (ce == cudaSuccess)
                    ce = (v.restir ? vgx::launch_stream_shadow_restir : vgx::launch_stream_shadow)(v.f64, shb, s, c, w, i);
            } else if (ce == cudaSuccess)
                ce = vgx::launch_stream_shade(v, ssb, s, c, w, i);
        }
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(&ring[0], (uint32_t*)acc->counts.p + (K & 1u), 4, cudaMemcpyDeviceToHost, s);
        cudaGraph_t g = nullptr;
        cudaError_t ee = cudaStreamEndCapture(s, &g);
        if (ce != cudaSuccess || ee != cudaSuccess) {
            if (g)
                cudaGraphDestroy(g);
            return cuda_fail(ce != cudaSuccess ? ce : ee, "wave graph capture");
        }
        cudaGraphExec_t ge = nullptr;
        ce = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess)
            return cuda_fail(ce, "wave graph instantiation");
        uint32_t per_wave = deferred ? (r->dynamic_fetch && r->ds.shadow_any ? 4 : 3) : 2;
        uint64_t max_rep = (max_waves + K - 1) / K + 2;
        uint64_t rep = 0;
        for (; rep < max_rep && !done; rep++) {
            ce = cudaGraphLaunch(ge, s);
            if (ce == cudaSuccess)
                ce = cudaEventRecord(ring_ev[rep & 1u], s);
            if (ce != cudaSuccess) {
                cudaGraphExecDestroy(ge);
                return cuda_fail(ce, "wave graph launch");
            }
            acc->launches += (uint64_t)K * per_wave;
            if (rep >= 1) {
                if ((st = wait_event(ring_ev[(rep - 1) & 1u])) != VG_OK) {
                    cudaGraphExecDestroy(ge);
                    return st;
                }
                // The count of the last replay that finished (a later one may have overwritten
                // it with a smaller count: live counts never grow).
                uint32_t live = ring[0];
                acc->wave_live.push_back(live);
                done = live == 0;
                if (!done && live <= r->tail_threshold) {
                    ce = (q ? vgx::launch_stream_cache_tail(v.f64, live, s, c, w, (uint32_t)((rep + 1) * K), *q) : vgx::launch_stream_tail(v, live, s, c, w, (uint32_t)((rep + 1) * K)));
                    if (ce != cudaSuccess) {
                        cudaGraphExecDestroy(ge);
                        return cuda_fail(ce, "tail launch");
                    }
                    acc->launches++;
                    done = true;
                }
            }
        }
        wave = rep * K;
        VG_CHECK(cudaStreamSynchronize(s), "waves");
        cudaGraphExecDestroy(ge);
        if (!done && ring[0] != 0)
            return fail(VG_ERR_KERNEL, "streaming wavefront did not drain within its wave bound");
        done = true;
    }
    for (; wave < max_waves && !done; wave++) {
        cudaEvent_t a = nullptr, m = nullptr, b = nullptr;
        if (timed) {
            a = pool.get();
            m = pool.get();
            b = pool.get();
            VG_CHECK(cudaEventRecord(a, s), "event");
        }
        if (r->dynamic_fetch)
            VG_CHECK(vgx::launch_stream_extend_dyn(r->traversal_stats, r->coop_tris, eb, s, c, w, (uint32_t)wave),
                     "extend launch");
        else
            VG_CHECK(vgx::launch_stream_extend(r->traversal_stats, eb, s, c, w, (uint32_t)wave),
                     "extend launch");
        if (timed)
            VG_CHECK(cudaEventRecord(m, s), "event");
        if (sorted) {
            VG_CHECK(vgx::launch_stream_classify(clb, s, c, w, (uint32_t)wave), "classify launch");
            acc->launches++;
        }
        if (deferred) {
            VG_CHECK((q ? vgx::launch_stream_cache_shade(v.f64, sorted, csb, s, c, w, (uint32_t)wave, *q) : (v.restir ? vgx::launch_stream_shade_deferred_restir : vgx::launch_stream_shade_deferred)(v.f64, sorted, dsb, s, c, w, (uint32_t)wave)), "shade launch");
            cudaEvent_t qe = nullptr;
            if (timed) {
                qe = pool.get();
                VG_CHECK(cudaEventRecord(qe, s), "event");
            }
            if (r->dynamic_fetch && r->ds.shadow_any) {
                VG_CHECK(vgx::launch_stream_shadow_trace(r->traversal_stats, r->coop_tris, stb, s, c, w, (uint32_t)wave), "shadow launch");
                VG_CHECK((v.restir ? vgx::launch_stream_finish_restir : vgx::launch_stream_finish)(v.f64, fnb, s, c, w, (uint32_t)wave), "finish launch");
                acc->launches++;
            } else {
                VG_CHECK((v.restir ? vgx::launch_stream_shadow_restir : vgx::launch_stream_shadow)(v.f64, shb, s, c, w, (uint32_t)wave), "shadow launch");
            }
            if (timed) {
                VG_CHECK(cudaEventRecord(b, s), "event");
                stages.push_back({0, {a, m}});
                stages.push_back({1, {m, qe}});
                stages.push_back({3, {qe, b}});
            }
            acc->launches += 3;
        } else {
            VG_CHECK(vgx::launch_stream_shade(v, ssb, s, c, w, (uint32_t)wave), "shade launch");
            if (timed) {
                VG_CHECK(cudaEventRecord(b, s), "event");
                stages.push_back({0, {a, m}});
                stages.push_back({1, {m, b}});
            }
            acc->launches += 2;
        }
        uint32_t slot = (uint32_t)(wave % RING);
        VG_CHECK(cudaMemcpyAsync(&ring[slot], (uint32_t*)acc->counts.p + ((wave + 1) & 1u), 4,
                                 cudaMemcpyDeviceToHost, s),
                 "count readback");
        VG_CHECK(cudaEventRecord(ring_ev[slot], s), "event");
        if (wave >= LAG) {
            uint32_t old = (uint32_t)((wave - LAG) % RING);
            if ((st = wait_event(ring_ev[old])) != VG_OK)
                return st;
            uint32_t live = ring[old];
            done = live == 0;
            acc->wave_live.push_back(live);
            if (!done && live <= r->tail_threshold) {
                // Few slots left: finish them in one launch (the queue after this wave).
                cudaEvent_t a = nullptr, b = nullptr;
                if (timed) {
                    a = pool.get();
                    b = pool.get();
                    VG_CHECK(cudaEventRecord(a, s), "event");
                }
                VG_CHECK((q ? vgx::launch_stream_cache_tail(v.f64, live, s, c, w, (uint32_t)(wave + 1), *q) : vgx::launch_stream_tail(v, live, s, c, w, (uint32_t)(wave + 1))), "tail launch");
                if (timed) {
                    VG_CHECK(cudaEventRecord(b, s), "event");
                    stages.push_back({2, {a, b}});
                }
                acc->launches++;
                done = true;
            }
        }
    }
    acc->last_waves = (uint32_t)wave;
    VG_CHECK(cudaStreamSynchronize(s), "waves");
    for (uint64_t k = wave > LAG ? wave - LAG + 1 : 0; k < wave; k++)
        acc->wave_live.push_back(ring[k % RING]);
    if (!done) {
        VG_CHECK(cudaStreamSynchronize(s), "waves");
        if (ring[(wave - 1) % RING] != 0)
            return fail(VG_ERR_KERNEL, "streaming wavefront did not drain within its wave bound");
    }
    return VG_OK;
}

extern "C" {


size_t vg_last_error(char* buf, size_t len)
{
    if (buf && len > 0) {
        size_t n = std::min(len - 1, g_err.size());
        memcpy(buf, g_err.data(), n);
        buf[n] = 0;
    }
    return g_err.size();
}

void vg_last_oom(uint64_t* needed, uint64_t* available)
{
    if (needed)
        *needed = g_oom_needed;
    if (available)
        *available = g_oom_available;
}

int vg_context_create_on(int device, VgContext** out)
{
    if (!out)
        return fail(VG_ERR_INVALID, "null output pointer");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(VG_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= n)
        return fail(VG_ERR_INVALID, "device ordinal " + std::to_string(device) + " out of range (" +
                                        std::to_string(n) + " devices)");
    cudaDeviceProp prop;
    VG_CHECK(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    if (prop.major != 10 || prop.minor != 3)
        return fail(VG_ERR_UNSUPPORTED, std::string("device ") + prop.name + " is not sm_103 (GB300)");
    DevGuard device_guard(device);
    VgContext* ctx = new VgContext();
    ctx->device = device;
    ctx->sms = prop.multiProcessorCount;
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete ctx;
        return cuda_fail(e, "cudaStreamCreate");
    }
    *out = ctx;
    return VG_OK;
}

int vg_context_create(VgContext** out)
{
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) {
        cudaGetLastError();
        device = 0;
    }
    return vg_context_create_on(device, out);
}

void vg_debug_allocations(uint64_t* mallocs, uint64_t* frees)
{
    if (mallocs)
        *mallocs = vgh::g_mallocs.load();
    if (frees)
        *frees = vgh::g_frees.load();
}

void vg_context_destroy(VgContext* ctx)
{
    DevGuard device_guard(dev_of(ctx));
    if (!ctx)
        return;
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
    if (ctx->side) {
        cudaStreamSynchronize(ctx->side);
        cudaStreamDestroy(ctx->side);
    }
    if (ctx->fork)
        cudaEventDestroy(ctx->fork);
    if (ctx->join)
        cudaEventDestroy(ctx->join);
    delete ctx;
}

int vg_memory(VgContext* ctx, VgMemoryUsage* out)
{
    DevGuard device_guard(dev_of(ctx));
    if (!ctx || !out)
        return fail(VG_ERR_INVALID, "null argument");
    size_t free_b = 0, total_b = 0;
    VG_CHECK(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
    out->budget = total_b;
    out->allocated = total_b - free_b;
    out->uploaded = ctx->uploaded;
    return VG_OK;
}

int vg_renderer_create(VgContext* ctx, const VgPacked* pk, VgRenderer** out)
{
    DevGuard device_guard(dev_of(ctx));
    if (!ctx || !pk || !out)
        return fail(VG_ERR_INVALID, "null argument");
    *out = nullptr;
    int st = validate(pk);
    if (st != VG_OK)
        return st;
    VgRenderer* r = new VgRenderer();
    r->ctx = ctx;
    r->device = ctx->device;
    r->info = pk->info;
    r->view = pk->view;
    r->instance_count = (uint32_t)pk->instance_count;
    Bvh8Host bvh;
    if ((st = build_world_bvh(r, pk, bvh)) != VG_OK) {
        delete r;
        return st;
    }
    bool translucent = translucent_materials(pk);

#define UP(buf, src, n)                                                                                             \
    do {                                                                                                            \
        st = upload(ctx, r->buf, src, (n));                                                                         \
        if (st != VG_OK) {                                                                                          \
            vg_renderer_destroy(r);                                                                                 \
            return st;                                                                                              \
        }                                                                                                           \
    } while (0)
    UP(positions, pk->positions, pk->positions_len * 4);
    UP(indices, pk->indices, pk->indices_len * 4);
    UP(uvs, pk->uvs, pk->uvs_len * 4);
    UP(vnormals, pk->vnormals, pk->vnormals_len * 4);
    UP(instances, pk->instances, pk->instances_len * 4);
    UP(materials, pk->materials, pk->materials_len * 4);
    UP(lights, pk->lights, pk->lights_len * 4);
    UP(emitters, pk->emitters, pk->emitters_len * 4);
    UP(emit_cdf, pk->emit_cdf, pk->emit_cdf_len * 4);
    {
        std::vector<uint32_t> guide = emitter_guide(pk);
        UP(emit_guide, guide.data(), guide.size() * 4);
    }
    UP(env_pixels, pk->env_pixels, pk->env_pixels_len * 4);
    UP(env_marginal, pk->env_marginal, pk->env_marginal_len * 4);
    UP(env_cond, pk->env_conditional, pk->env_conditional_len * 4);
    {
        std::vector<uint32_t> guide = env_guide(pk);
        UP(env_guide, guide.data(), guide.size() * 4);
    }
    UP(texels, pk->texels, pk->texels_len * 4);
    UP(tex_info, pk->tex_info, pk->tex_info_len * 4);
    UP(nodes, bvh.nodes.data(), bvh.nodes.size() * 4);
    UP(tris, bvh.tris.data(), bvh.tris.size() * 4);
#undef UP
    st = alloc(r->err, 16, ctx->stream, true);
    if (st != VG_OK) {
        vg_renderer_destroy(r);
        return st;
    }
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        vg_renderer_destroy(r);
        return cuda_fail(e, "upload");
    }
    r->texel_key = table_key(pk->texels, pk->texels_len, pk->tex_info, pk->tex_info_len);
    r->env_key = table_key(pk->env_pixels, pk->env_pixels_len, pk->env_conditional, pk->env_conditional_len);
    bind_tables(r);
    r->ds.shadow_any = translucent ? 0u : 1u;
    r->extend_blocks = vgx::wf_extend_blocks_per_sm();
    *out = r;
    return VG_OK;
}

void vg_renderer_destroy(VgRenderer* r)
{
    DevGuard device_guard(dev_of(r));
    // As vg_accum_destroy: frees device memory only, independent of the context's lifetime.
    delete r;
}

int vg_renderer_update(VgRenderer* r, const VgPacked* pk, const VgUpdatePlan* plan, VgUpdateReport* out)
{
    DevGuard device_guard(dev_of(r));
    if (!r || !pk || !plan || !out)
        return fail(VG_ERR_INVALID, "null argument");
    memset(out, 0, sizeof(*out));
    int st = validate(pk);
    if (st != VG_OK)
        return st;
    VgContext* ctx = r->ctx;
    if (plan->camera)
        r->view = pk->view;
    if (plan->full) {
        VgRenderer* f = nullptr;
        if ((st = vg_renderer_create(ctx, pk, &f)) != VG_OK)
            return st;
        DevBuf* mine[] = {&r->positions, &r->indices, &r->uvs, &r->vnormals, &r->instances, &r->materials,
                          &r->lights, &r->emitters, &r->emit_cdf, &r->emit_guide, &r->env_pixels, &r->env_marginal, &r->env_cond,
                          &r->env_guide, &r->texels, &r->tex_info, &r->nodes, &r->tris};
        DevBuf* theirs[] = {&f->positions, &f->indices, &f->uvs, &f->vnormals, &f->instances, &f->materials,
                            &f->lights, &f->emitters, &f->emit_cdf, &f->emit_guide, &f->env_pixels, &f->env_marginal, &f->env_cond,
                            &f->env_guide, &f->texels, &f->tex_info, &f->nodes, &f->tris};
        uint64_t bytes = 0;
        for (size_t i = 0; i < sizeof(mine) / sizeof(mine[0]); i++) {
            std::swap(mine[i]->p, theirs[i]->p);
            std::swap(mine[i]->bytes, theirs[i]->bytes);
            bytes += mine[i]->bytes;
        }
        r->info = f->info;
        r->bvh = f->bvh;
        r->instance_count = f->instance_count;
        r->texel_key = f->texel_key;
        r->env_key = f->env_key;
        for (int k = 0; k < 3; k++) {
            r->bounds_lo[k] = f->bounds_lo[k];
            r->bounds_hi[k] = f->bounds_hi[k];
        }
        uint32_t shadow_any = f->ds.shadow_any;
        bind_tables(r);
        r->ds.shadow_any = shadow_any;
        vg_renderer_destroy(f); // frees the old tables
        out->blases_built = pk->mesh_count;
        out->tlas_built = 1;
        out->bytes_uploaded = bytes;
        return VG_OK;
    }
    cudaStream_t s = ctx->stream;
    uint64_t bytes = 0;
    if (plan->vertices) {
        if (std::max<size_t>(pk->positions_len * 4, 16) != r->positions.bytes ||
            std::max<size_t>(pk->uvs_len * 4, 16) != r->uvs.bytes ||
            std::max<size_t>(pk->vnormals_len * 4, 16) != r->vnormals.bytes || (plan->blas_count > 0 && !plan->blases))
            return fail(VG_ERR_SCENE, "a deformed mesh changed its vertex count: that needs a full update");
        for (size_t i = 0; i < plan->blas_count; i++) {
            uint32_t m = plan->blases[i];
            if (m >= pk->mesh_count)
                return fail(VG_ERR_INVALID, "deformed mesh index out of range");
            const VgMeshRange& mr = pk->meshes[m];
            size_t vo = mr.vertex_offset, vc = mr.vertex_count;
            if ((vo + vc) * 3 > pk->positions_len || (vo + vc) * 2 > pk->uvs_len || (vo + vc) * 3 > pk->vnormals_len)
                return fail(VG_ERR_INVALID, "mesh range outside the vertex tables");
            VG_CHECK(cudaMemcpyAsync((float*)r->positions.p + vo * 3, pk->positions + vo * 3, vc * 12,
                                     cudaMemcpyHostToDevice, s),
                     "vertex upload");
            VG_CHECK(cudaMemcpyAsync((float*)r->uvs.p + vo * 2, pk->uvs + vo * 2, vc * 8, cudaMemcpyHostToDevice, s),
                     "vertex upload");
            VG_CHECK(cudaMemcpyAsync((float*)r->vnormals.p + vo * 3, pk->vnormals + vo * 3, vc * 12,
                                     cudaMemcpyHostToDevice, s),
                     "vertex upload");
            bytes += vc * 32;
        }
        out->blases_built = plan->blas_count;
    }
    if (plan->materials) {
        if ((st = upload(ctx, r->materials, pk->materials, pk->materials_len * 4)) != VG_OK)
            return st;
        bytes += pk->materials_len * 4;
        uint64_t key = table_key(pk->texels, pk->texels_len, pk->tex_info, pk->tex_info_len);
        if (key != r->texel_key) {
            if ((st = upload(ctx, r->texels, pk->texels, pk->texels_len * 4)) != VG_OK ||
                (st = upload(ctx, r->tex_info, pk->tex_info, pk->tex_info_len * 4)) != VG_OK)
                return st;
            bytes += (pk->texels_len + pk->tex_info_len) * 4;
            r->texel_key = key;
        }
        r->ds.shadow_any = translucent_materials(pk) ? 0u : 1u;
    }
    if (plan->lights) {
        if ((st = upload(ctx, r->lights, pk->lights, pk->lights_len * 4)) != VG_OK)
            return st;
        bytes += pk->lights_len * 4;
        r->info.light_count = pk->info.light_count;
        for (int k = 0; k < 3; k++)
            r->info.sky[k] = pk->info.sky[k];
        r->info.virtual_light = pk->info.virtual_light;
        r->info.transparent_background = pk->info.transparent_background;
        uint64_t key = table_key(pk->env_pixels, pk->env_pixels_len, pk->env_conditional, pk->env_conditional_len);
        if (key != r->env_key || pk->info.env_width != r->info.env_width || pk->info.env_height != r->info.env_height) {
            if ((st = upload(ctx, r->env_pixels, pk->env_pixels, pk->env_pixels_len * 4)) != VG_OK ||
                (st = upload(ctx, r->env_marginal, pk->env_marginal, pk->env_marginal_len * 4)) != VG_OK ||
                (st = upload(ctx, r->env_cond, pk->env_conditional, pk->env_conditional_len * 4)) != VG_OK)
                return st;
            std::vector<uint32_t> guide = env_guide(pk);
            if ((st = upload(ctx, r->env_guide, guide.data(), guide.size() * 4)) != VG_OK)
                return st;
            bytes += (pk->env_pixels_len + pk->env_marginal_len + pk->env_conditional_len + guide.size()) * 4;
            r->info.env_width = pk->info.env_width;
            r->info.env_height = pk->info.env_height;
            r->info.env_pdf_scale = pk->info.env_pdf_scale;
            r->env_key = key;
        }
    }
    if (plan->emitters) {
        if ((st = upload(ctx, r->emitters, pk->emitters, pk->emitters_len * 4)) != VG_OK ||
            (st = upload(ctx, r->emit_cdf, pk->emit_cdf, pk->emit_cdf_len * 4)) != VG_OK)
            return st;
        std::vector<uint32_t> guide = emitter_guide(pk);
        if ((st = upload(ctx, r->emit_guide, guide.data(), guide.size() * 4)) != VG_OK)
            return st;
        bytes += (pk->emitters_len + pk->emit_cdf_len + guide.size()) * 4;
        r->info.emitter_count = pk->info.emitter_count;
    }
    if (plan->instances) {
        if ((st = upload(ctx, r->instances, pk->instances, pk->instances_len * 4)) != VG_OK)
            return st;
        bytes += pk->instances_len * 4;
        r->instance_count = (uint32_t)pk->instance_count;
    }
    if (plan->tlas || plan->vertices) {
        Bvh8Host bvh;
        if ((st = build_world_bvh(r, pk, bvh)) != VG_OK ||
            (st = upload(ctx, r->nodes, bvh.nodes.data(), bvh.nodes.size() * 4)) != VG_OK ||
            (st = upload(ctx, r->tris, bvh.tris.data(), bvh.tris.size() * 4)) != VG_OK)
            return st;
        bytes += (bvh.nodes.size() + bvh.tris.size()) * 4;
        out->tlas_built = 1;
    }
    VG_CHECK(cudaStreamSynchronize(s), "update");
    uint32_t shadow_any = r->ds.shadow_any;
    bind_tables(r);
    r->ds.shadow_any = shadow_any;
    out->bytes_uploaded = bytes;
    return VG_OK;
}

int vg_set_bvh_traversal_cost(VgRenderer* r, const VgPacked* pk, float cost)
{
    DevGuard device_guard(dev_of(r));
    if (!r || !pk)
        return fail(VG_ERR_INVALID, "null argument");
    if (!(cost > 0.0f && cost <= 16.0f))
        return fail(VG_ERR_INVALID, "SAH traversal cost out of range");
    int st = validate(pk);
    if (st != VG_OK)
        return st;
    if (pk->instance_count != r->instance_count)
        return fail(VG_ERR_SCENE, "the tables are not this renderer's scene");
    float old = r->bvh_traversal_cost;
    r->bvh_traversal_cost = cost;
    Bvh8Host bvh;
    if ((st = build_world_bvh(r, pk, bvh)) != VG_OK || (st = upload(r->ctx, r->nodes, bvh.nodes.data(), bvh.nodes.size() * 4)) != VG_OK ||
        (st = upload(r->ctx, r->tris, bvh.tris.data(), bvh.tris.size() * 4)) != VG_OK) {
        r->bvh_traversal_cost = old;
        return st;
    }
    VG_CHECK(cudaStreamSynchronize(r->ctx->stream), "BVH upload");
    r->ds.nodes = (const uint4*)r->nodes.p;
    r->ds.tris = (const float4*)r->tris.p;
    return VG_OK;
}

int vg_renderer_bvh_info(const VgRenderer* r, VgBvhInfo* out)
{
    if (!r || !out)
        return fail(VG_ERR_INVALID, "null argument");
    *out = r->bvh;
    return VG_OK;
}

int vg_set_camera(VgRenderer* r, const VgView* view)
{
    if (!r || !view)
        return fail(VG_ERR_INVALID, "null argument");
    r->view = *view;
    return VG_OK;
}

int vg_set_multiscatter(VgRenderer* r, int on)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    r->multiscatter = on != 0;
    return VG_OK;
}

int vg_set_integrator(VgRenderer* r, int integrator)
{
    if (!r || (integrator != VG_MEGAKERNEL && integrator != VG_WAVEFRONT))
        return fail(VG_ERR_INVALID, "bad integrator");
    r->integrator = integrator;
    return VG_OK;
}

int vg_integrator(const VgRenderer* r) { return r ? r->integrator : -1; }

int vg_set_stage_timing(VgRenderer* r, int on)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    r->stage_timing = on != 0;
    return VG_OK;
}

int vg_set_wavefront_mode(VgRenderer* r, int mode)
{
    if (!r || (mode != VG_WAVEFRONT_PER_SAMPLE && mode != VG_WAVEFRONT_STREAMING))
        return fail(VG_ERR_INVALID, "bad wavefront mode");
    r->wavefront_mode = mode;
    return VG_OK;
}

uint32_t vg_accum_last_waves(const VgAccum* acc) { return acc ? acc->last_waves : 0; }

int vg_set_stream_tail(VgRenderer* r, uint32_t threshold)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    r->tail_threshold = threshold;
    return VG_OK;
}

double vg_accum_tail_seconds(const VgAccum* acc) { return acc ? acc->tail_ms * 1e-3 : 0.0; }

int vg_set_wavefront_graph(VgRenderer* r, uint32_t waves)
{
    if (!r || (waves & 1u) || waves > 64)
        return fail(VG_ERR_INVALID, "graph waves must be 0 or an even count up to 64");
    r->graph_waves = waves;
    return VG_OK;
}

int vg_set_dynamic_fetch(VgRenderer* r, int on)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    r->dynamic_fetch = on != 0;
    return VG_OK;
}

int vg_set_material_sort(VgRenderer* r, int on)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    r->material_sort = on != 0;
    return VG_OK;
}

int vg_set_coop_triangles(VgRenderer* r, int on)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    r->coop_tris = on != 0;
    return VG_OK;
}

int vg_set_traversal_fetch(VgRenderer* r, uint32_t refill, uint32_t steps, uint32_t shadow_refill,
                           uint32_t shadow_steps)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    if (refill < 1 || refill > 32 || shadow_refill < 1 || shadow_refill > 32 || steps < 1 || steps > 64 ||
        shadow_steps < 1 || shadow_steps > 64)
        return fail(VG_ERR_INVALID, "refill must be 1-32 lanes and steps 1-64 node visits");
    r->fetch_refill = refill;
    r->fetch_steps = steps;
    r->shadow_fetch_refill = shadow_refill;
    r->shadow_fetch_steps = shadow_steps;
    return VG_OK;
}

int vg_set_deferred_shadows(VgRenderer* r, int on)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    r->defer_shadows = on != 0;
    return VG_OK;
}

size_t vg_accum_wave_profile(const VgAccum* acc, float* out, size_t waves)
{
    if (!acc)
        return 0;
    size_t n = std::min(waves, acc->wave_live.size());
    size_t per = acc->wave_stages;
    for (size_t k = 0; out && k < n; k++) {
        out[4 * k] = (float)acc->wave_live[k];
        for (size_t j = 0; j < 3; j++)
            out[4 * k + 1 + j] = j < per && per * k + j < acc->wave_ms.size() ? acc->wave_ms[per * k + j] : 0.0f;
    }
    return acc->wave_live.size();
}

int vg_set_traversal_stats(VgRenderer* r, int on)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    r->traversal_stats = on != 0;
    return VG_OK;
}

int vg_set_adaptive(VgRenderer* r, int on, float threshold, uint32_t min_spp)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    r->adaptive = on != 0;
    r->adaptive_threshold = threshold;
    r->adaptive_min_spp = min_spp;
    return VG_OK;
}

int vg_set_restir(VgRenderer* r, int on, int di, int gi, uint32_t candidates, uint32_t history)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    r->restir.on = on != 0;
    r->restir.di = di != 0;
    r->restir.gi = gi != 0;
    r->restir.candidates = candidates;
    r->restir.history = history;
    return VG_OK;
}

int vg_set_max_depth(VgRenderer* r, uint32_t depth)
{
    if (!r || depth == 0 || depth > 64)
        return fail(VG_ERR_INVALID, "max depth must be in 1..64");
    r->max_depth = depth;
    return VG_OK;
}

int vg_set_accum_precision(VgRenderer* r, int bits)
{
    if (!r || (bits != 32 && bits != 64))
        return fail(VG_ERR_INVALID, "precision must be 32 or 64");
    r->precision = bits;
    return VG_OK;
}

int vg_accum_create(VgRenderer* r, uint32_t width, uint32_t height, int lighting, VgAccum** out)
{
    DevGuard device_guard(dev_of(r));
    if (!r || !out)
        return fail(VG_ERR_INVALID, "null argument");
    *out = nullptr;
    if (width == 0 || height == 0)
        return fail(VG_ERR_SCENE, "image size must be non-zero");
    if ((uint64_t)width * height > 0x7fffffffull)
        return fail(VG_ERR_INVALID, "image too large");
    VgAccum* acc = new VgAccum();
    acc->owner = r;
    acc->device = r->device;
    acc->width = width;
    acc->height = height;
    acc->lighting = lighting != 0;
    acc->precision = r->precision;
    size_t px = (size_t)width * height;
    size_t es = acc->precision == 64 ? 8 : 4;
    int st = alloc(acc->accum, px * 3 * es, r->ctx->stream, true);
    if (st == VG_OK && acc->lighting)
        st = alloc(acc->light, px * LIGHTING_STRIDE * 4, r->ctx->stream, true);
    if (st == VG_OK) {
        cudaError_t e = cudaStreamSynchronize(r->ctx->stream);
        if (e != cudaSuccess)
            st = cuda_fail(e, "accumulation clear");
    }
    if (st != VG_OK) {
        delete acc;
        return st;
    }
    *out = acc;
    return VG_OK;
}

void vg_accum_destroy(VgAccum* acc)
{
    DevGuard device_guard(dev_of(acc));
    // Frees device memory only (cudaFree waits for work in flight); it does not touch the
    // renderer or context, so handles may be destroyed in any order.
    delete acc;
}

int vg_accumulate(VgRenderer* r, VgAccum* acc, uint32_t samples)
{
    DevGuard device_guard(dev_of(r));
    if (!r || !acc || acc->owner != r)
        return fail(VG_ERR_INVALID, "accumulation does not belong to this renderer");
    cudaStream_t s = r->ctx->stream;
    size_t px = (size_t)acc->width * acc->height;
    size_t es = acc->precision == 64 ? 8 : 4;
    int st;
    // Adaptive sampling: the statistics must count every sample from the first one on.
    if (acc->samples == 0) {
        acc->adaptive_fixed = true;
        acc->adaptive = r->adaptive;
    }
    if (acc->adaptive && !acc->stats.p) {
        if ((st = alloc(acc->stats, px * 3 * es, s, true)) != VG_OK)
            return st;
    }
    if (acc->adaptive != r->adaptive)
        return fail(VG_ERR_SCENE, "adaptive sampling was switched mid-accumulation; start a new accumulation");
    if (acc->samples == 0) {
        acc->restir = r->restir;
        for (int h = 0; h < 2; h++) {
            acc->re_g[h].release();
            acc->re_n[h].release();
            acc->re_x[h].release();
            acc->re_m[h].release();
            acc->re_gx[h].release();
            acc->re_gn[h].release();
            acc->re_gl[h].release();
        }
        acc->restir_bytes = 0;
        if (r->restir.on) {
            for (int h = 0; h < 2; h++) {
                if ((st = alloc(acc->re_g[h], px * 16, s, true)) != VG_OK ||
                    (st = alloc(acc->re_n[h], px * 16, s, true)) != VG_OK ||
                    (st = alloc(acc->re_x[h], px * 16, s, true)) != VG_OK ||
                    (st = alloc(acc->re_m[h], px * 4, s, true)) != VG_OK)
                    return st;
                if (r->restir.gi && ((st = alloc(acc->re_gx[h], px * 16, s, true)) != VG_OK ||
                                     (st = alloc(acc->re_gn[h], px * 16, s, true)) != VG_OK ||
                                     (st = alloc(acc->re_gl[h], px * 16, s, true)) != VG_OK))
                    return st;
            }
            for (int k = 0; k < 7; k++) {
                acc->re_s[k].release();
                if (r->restir.gi && (st = alloc(acc->re_s[k], px * 16, s, true)) != VG_OK)
                    return st;
            }
            acc->restir_bytes = px * 2 * (16 * 3 + 4) + (r->restir.gi ? px * (2 * 48 + 7 * 16) : 0);
        }
    }
    if (!(acc->restir == r->restir))
        return fail(VG_ERR_SCENE, "ReSTIR was switched mid-accumulation; start a new accumulation");
    if (acc->first_sample != 0 && (acc->restir.on || r->cache))
        return fail(VG_ERR_SCENE, "a first sample index other than 0 needs plain path tracing (no ReSTIR, no cache)");
    if ((uint64_t)acc->first_sample + acc->samples + samples > 0xffffffffull)
        return fail(VG_ERR_INVALID, "sample index beyond 2^32 - 1");
    const uint32_t sample0 = acc->first_sample + acc->samples; // index of this call's first sample
    bool wavefront = r->integrator == VG_WAVEFRONT && !r->cache;
    const uint32_t max_depth_alloc = 64;
    if (r->integrator == VG_WAVEFRONT && !acc->state.p) {
        uint32_t planes = vgk::BASE_PLANES + (acc->lighting ? vgk::SPLIT_PLANES : 0);
        if ((st = alloc(acc->state, px * planes * 16, s, false)) != VG_OK ||
            (st = alloc(acc->hits, px * 16, s, false)) != VG_OK ||
            (st = alloc(acc->queue[0], px * 4, s, false)) != VG_OK ||
            (st = alloc(acc->queue[1], px * 4, s, false)) != VG_OK ||
            (st = alloc(acc->counts, (max_depth_alloc + 1) * 4, s, true)) != VG_OK ||
            (st = alloc(acc->fetch, 2 * (max_depth_alloc + 1) * 4, s, true)) != VG_OK ||
            (st = alloc(acc->tstats, 8 * 8, s, true)) != VG_OK ||
            (st = alloc(acc->meta, px * 4, s, false)) != VG_OK ||
            (st = alloc(acc->sreq, acc->lighting ? 16 : px * 3 * 16, s, false)) != VG_OK ||
            (st = alloc(acc->squeue, acc->lighting ? 16 : px * 4 * vgk::SHADE_CLASSES, s, false)) != VG_OK ||
            (st = alloc(acc->scount, 2 * vgk::SHADE_CLASSES * 4, s, true)) != VG_OK)
            return st;
        if (!acc->host_counts && cudaHostAlloc((void**)&acc->host_counts, 64 * 4, cudaHostAllocDefault) != cudaSuccess) {
            acc->host_counts = nullptr;
            return fail(VG_ERR_RESOURCE, "pinned host buffer");
        }
        acc->wavefront_bytes = acc->state.bytes + acc->hits.bytes + acc->queue[0].bytes + acc->queue[1].bytes +
                               acc->counts.bytes + acc->fetch.bytes;
    }
    vgd::Ctx c = make_ctx(r, acc);
    vgx::Variant v = variant_of(r, acc);
    EventPool pool;
    cudaEvent_t t0 = pool.get(), t1 = pool.get();
    StageEvents stages;
    bool timed = r->stage_timing && wavefront;
    VG_CHECK(cudaMemsetAsync(r->err.p, 0, 4, s), "error flag");
    VG_CHECK(cudaEventRecord(t0, s), "event");
    bool streamed = false;
    if (r->cache) {
        vgk::Wave w = wave_of(r, acc);
        c.p[P_WF_PATHS] = (uint32_t)px;
        if ((st = cache_accumulate(r, acc, c, samples, r->stage_timing,
                                   r->integrator == VG_WAVEFRONT ? &w : nullptr)) != VG_OK)
            return st;
    } else if (!wavefront) {
        if (!acc->mk_next.p && (st = alloc(acc->mk_next, 16, s, true)) != VG_OK)
            return st;
        uint32_t k = 0;
        while (k < samples) {
            c.p[P_SAMPLE] = sample0 + k;
            c.p[P_SAMPLES_PER_DISPATCH] = std::min<uint32_t>(samples - k, acc->restir.on ? 1u : 8u);
            k += c.p[P_SAMPLES_PER_DISPATCH];
            VG_CHECK(vgx::launch_megakernel(v, r->ctx->sms, acc->width, acc->height, s, c, (uint32_t*)acc->mk_next.p),
                     "megakernel launch");
            acc->launches++;
        }
    } else {
        vgk::Wave w = wave_of(r, acc);
        c.p[P_WF_PATHS] = (uint32_t)px;
        int vi = v.index();
        if (r->shade_blocks[vi] == 0)
            r->shade_blocks[vi] = vgx::wf_shade_blocks_per_sm(v);
        int eb = blocks_for(r, r->extend_blocks);
        int sb = blocks_for(r, r->shade_blocks[vi]);
        bool streaming = r->wavefront_mode == VG_WAVEFRONT_STREAMING;
        if (streaming && samples > 0) {
            streamed = true;
            // Under ReSTIR one sample per launch sequence: a sample's paths read the reservoirs the
            // previous sample left (the other frame parity), which must be complete by then.
            uint32_t per = acc->restir.on ? 1u : samples;
            for (uint32_t k = 0; k < samples; k += per)
                if ((st = stream_samples(r, acc, c, v, w, sample0 + k, per, timed, pool, stages, nullptr)) != VG_OK)
                    return st;
        }
        for (uint32_t k = 0; k < (streaming ? 0u : samples); k++) {
            c.p[P_SAMPLE] = sample0 + k;
            VG_CHECK(vgx::launch_wf_begin(s, c, w), "wf_begin launch");
            acc->launches++;
            if (acc->adaptive) {
                VG_CHECK(vgx::launch_wf_select(v.f64, s, c, w), "wf_select launch");
                acc->launches++;
            }
            for (uint32_t d = 0; d < r->max_depth; d++) {
                c.p[P_WF_DEPTH] = d;
                cudaEvent_t a = nullptr, b = nullptr, m = nullptr;
                if (timed) {
                    a = pool.get();
                    m = pool.get();
                    b = pool.get();
                    VG_CHECK(cudaEventRecord(a, s), "event");
                }
                VG_CHECK(vgx::launch_wf_extend(r->traversal_stats, eb, s, c, w, d), "wf_extend launch");
                if (timed)
                    VG_CHECK(cudaEventRecord(m, s), "event");
                VG_CHECK(vgx::launch_wf_shade(v, sb, s, c, w, d), "wf_shade launch");
                if (timed) {
                    VG_CHECK(cudaEventRecord(b, s), "event");
                    stages.push_back({0, {a, m}});
                    stages.push_back({1, {m, b}});
                }
                acc->launches += 2;
            }
        }
    }
    VG_CHECK(cudaEventRecord(t1, s), "event");
    st = wait_event(t1);
    if (st != VG_OK)
        return st;
    float ms = 0.0f;
    VG_CHECK(cudaEventElapsedTime(&ms, t0, t1), "event");
    acc->gpu_seconds += ms * 1e-3;
    if (timed) {
        acc->stage_ran = true;
        for (auto& sp : stages) {
            float sm = 0.0f;
            VG_CHECK(cudaEventElapsedTime(&sm, sp.second.first, sp.second.second), "event");
            acc->stage_seconds[sp.first >= 2 ? 1 : sp.first] += sm * 1e-3;
            if (sp.first == 2)
                acc->tail_ms = sm;
            else if (streamed)
                acc->wave_ms.push_back(sm);
            if (sp.first == 0)
                acc->extend_launches_timed++;
        }
    }
    st = read_err(r);
    if (st != VG_OK)
        return st;
    if ((st = cache_status(r)) != VG_OK)
        return st;
    if (wavefront && samples > 0)
        acc->last_depth = streamed ? 0 : r->max_depth;
    acc->samples += samples;
    return VG_OK;
}

uint32_t vg_accum_samples(const VgAccum* acc) { return acc ? acc->samples : 0; }

int vg_accum_set_first_sample(VgAccum* acc, uint32_t first)
{
    if (!acc)
        return fail(VG_ERR_INVALID, "null accumulation");
    if (acc->samples != 0)
        return fail(VG_ERR_INVALID, "the first sample index is set before the first sample");
    acc->first_sample = first;
    return VG_OK;
}
double vg_accum_gpu_seconds(const VgAccum* acc) { return acc ? acc->gpu_seconds : 0.0; }

int vg_accum_stage_seconds(const VgAccum* acc, double out[2])
{
    if (!acc || !acc->stage_ran)
        return 0;
    out[0] = acc->stage_seconds[0];
    out[1] = acc->stage_seconds[1];
    return 1;
}

size_t vg_accum_wavefront_bytes(const VgAccum* acc) { return acc ? acc->wavefront_bytes : 0; }
size_t vg_accum_restir_bytes(const VgAccum* acc) { return acc ? acc->restir_bytes : 0; }
int vg_accum_precision(const VgAccum* acc) { return acc ? acc->precision : 0; }
uint64_t vg_accum_launches(const VgAccum* acc) { return acc ? acc->launches : 0; }

double vg_accum_extend_launch_seconds(const VgAccum* acc)
{
    if (!acc || acc->extend_launches_timed == 0)
        return 0.0;
    return acc->stage_seconds[0] / (double)acc->extend_launches_timed;
}

// f64 sums to f32 with round-to-nearest-even, the rounding of the host's (float) cast, so that a
// readback of f32 sums moves half the bytes and needs no conversion on the host.
static __global__ void sums_to_f32(const double* __restrict__ in, float* __restrict__ out, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __double2float_rn(in[i]);
}

static int read_dev(const VgAccum* acc, const DevBuf& b, void* out, size_t bytes)
{
    cudaStream_t s = acc->owner->ctx->stream;
    VG_CHECK(cudaMemcpyAsync(out, b.p, bytes, cudaMemcpyDeviceToHost, s), "readback");
    VG_CHECK(cudaStreamSynchronize(s), "readback");
    return VG_OK;
}

int vg_accum_read_sums(const VgAccum* acc, float* out, size_t len)
{
    DevGuard device_guard(dev_of(acc));
    if (!acc || !out)
        return fail(VG_ERR_INVALID, "null argument");
    size_t n = (size_t)acc->width * acc->height * 3;
    if (len < n)
        return fail(VG_ERR_INVALID, "output too short");
    if (acc->precision == 32)
        return read_dev(acc, acc->accum, out, n * 4);
    // f64 sums: converted on the device, then one copy straight into the caller's buffer (a DMA when
    // it is pinned).
    cudaStream_t s = acc->owner->ctx->stream;
    int st;
    if (!acc->sums32.p || acc->sums32.bytes < n * 4)
        if ((st = alloc(acc->sums32, n * 4, s, false)) != VG_OK)
            return st;
    int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)acc->owner->ctx->sms * 8);
    sums_to_f32<<<blocks, 256, 0, s>>>((const double*)acc->accum.p, (float*)acc->sums32.p, n);
    VG_CHECK(cudaGetLastError(), "sum conversion launch");
    return read_dev(acc, acc->sums32, out, n * 4);
}

int vg_accum_read_sums_f64(const VgAccum* acc, double* out, size_t len)
{
    DevGuard device_guard(dev_of(acc));
    if (!acc || !out)
        return fail(VG_ERR_INVALID, "null argument");
    size_t n = (size_t)acc->width * acc->height * 3;
    if (len < n)
        return fail(VG_ERR_INVALID, "output too short");
    if (acc->precision == 64)
        return read_dev(acc, acc->accum, out, n * 8);
    std::vector<float> tmp(n);
    int st = read_dev(acc, acc->accum, tmp.data(), n * 4);
    if (st != VG_OK)
        return st;
    for (size_t i = 0; i < n; i++)
        out[i] = tmp[i];
    return VG_OK;
}

int vg_accum_read_lighting(const VgAccum* acc, float* out, size_t len)
{
    DevGuard device_guard(dev_of(acc));
    if (!acc || !out)
        return fail(VG_ERR_INVALID, "null argument");
    if (!acc->lighting)
        return fail(VG_ERR_INVALID, "accumulation has no lighting split");
    size_t n = (size_t)acc->width * acc->height * LIGHTING_STRIDE;
    if (len < n)
        return fail(VG_ERR_INVALID, "output too short");
    return read_dev(acc, acc->light, out, n * 4);
}

int vg_accum_read_stats(const VgAccum* acc, float* out, size_t len)
{
    DevGuard device_guard(dev_of(acc));
    if (!acc || !out)
        return fail(VG_ERR_INVALID, "null argument");
    if (!acc->stats.p)
        return fail(VG_ERR_INVALID, "adaptive sampling never ran on this accumulation");
    size_t n = (size_t)acc->width * acc->height * 3;
    if (len < n)
        return fail(VG_ERR_INVALID, "output too short");
    if (acc->precision == 32)
        return read_dev(acc, acc->stats, out, n * 4);
    std::vector<double> tmp(n);
    int st = read_dev(acc, acc->stats, tmp.data(), n * 8);
    if (st != VG_OK)
        return st;
    for (size_t i = 0; i < n; i++)
        out[i] = (float)tmp[i];
    return VG_OK;
}

int vg_accum_traversal_stats(const VgAccum* acc, uint64_t out[4])
{
    DevGuard device_guard(dev_of(acc));
    if (!acc || !out)
        return fail(VG_ERR_INVALID, "null argument");
    if (!acc->tstats.p)
        return fail(VG_ERR_INVALID, "no wavefront sample has run on this accumulation");
    return read_dev(acc, acc->tstats, out, 4 * 8);
}

int vg_accum_shadow_rays(const VgAccum* acc, uint64_t* out)
{
    DevGuard device_guard(dev_of(acc));
    if (!acc || !out)
        return fail(VG_ERR_INVALID, "null argument");
    if (!acc->tstats.p)
        return fail(VG_ERR_INVALID, "no wavefront sample has run on this accumulation");
    uint64_t words[5];
    int st = read_dev(acc, acc->tstats, words, sizeof(words));
    if (st == VG_OK)
        *out = words[4];
    return st;
}

int vg_accum_read_queue_counts(const VgAccum* acc, uint32_t* out, size_t len)
{
    DevGuard device_guard(dev_of(acc));
    if (!acc || !out)
        return fail(VG_ERR_INVALID, "null argument");
    if (!acc->counts.p || acc->samples == 0 || acc->last_depth == 0)
        return fail(VG_ERR_INVALID, "no wavefront sample has run on this accumulation");
    if (len < acc->last_depth + 1)
        return fail(VG_ERR_INVALID, "output too short");
    return read_dev(acc, acc->counts, out, (acc->last_depth + 1) * 4);
}

// pack.rs:97-108 View::camera_record
static void camera_record(const VgRenderer* r, uint32_t w, uint32_t h, float* rec)
{
    for (int i = 0; i < 16; i++)
        rec[i] = r->view.camera[i];
    rec[0] = (float)w;
    rec[1] = (float)h;
    rec[16] = r->view.shift[0];
    rec[17] = r->view.shift[1];
}

// One autotuner trial: a warm-up accumulate, then the device time of a second one on a scratch
// accumulation; camera paths per second in millions.
static double tune_trial(VgRenderer* r, uint32_t w, uint32_t h, uint32_t spp, int* st)
{
    VgAccum* a = nullptr;
    if ((*st = vg_accum_create(r, w, h, 0, &a)) != VG_OK)
        return 0.0;
    double m = 0.0;
    if ((*st = vg_accumulate(r, a, spp)) == VG_OK) {
        double g0 = a->gpu_seconds;
        if ((*st = vg_accumulate(r, a, spp)) == VG_OK)
            m = (double)w * h * spp / std::max(a->gpu_seconds - g0, 1e-9) / 1e6;
    }
    vg_accum_destroy(a);
    return m;
}

int vg_autotune(VgRenderer* r, const VgPacked* pk, uint32_t width, uint32_t height, uint32_t samples, VgTuneResult* out)
{
    DevGuard device_guard(dev_of(r));
    if (!r || !out || width == 0 || height == 0 || samples == 0)
        return fail(VG_ERR_INVALID, "null argument or empty trial");
    memset(out, 0, sizeof(*out));
    // Trials run the streaming wavefront without adaptive sampling or stage timing; the renderer is
    // left on the streaming wavefront with the best setting found.
    bool adaptive = r->adaptive, timing = r->stage_timing;
    r->adaptive = false;
    r->stage_timing = false;
    r->integrator = VG_WAVEFRONT;
    r->wavefront_mode = VG_WAVEFRONT_STREAMING;
    int st = VG_OK;
    uint32_t trials = 0;
    double best = tune_trial(r, width, height, samples, &st);
    trials++;
    out->mpaths_before = best;
    // Coordinate descent: one pass over the settings, a change kept when it gains over 1%.
    auto try_setting = [&](auto apply, auto values) {
        for (auto v : values) {
            if (st != VG_OK)
                return;
            auto keep = apply(v, true);
            double m = tune_trial(r, width, height, samples, &st);
            trials++;
            if (st == VG_OK && m > best * 1.01)
                best = m;
            else
                apply(keep, false);
        }
    };
    try_setting(
        [&](bool v, bool) {
            bool o = r->dynamic_fetch;
            r->dynamic_fetch = v;
            return o;
        },
        std::vector<bool>{!r->dynamic_fetch});
    try_setting(
        [&](bool v, bool) {
            bool o = r->defer_shadows;
            r->defer_shadows = v;
            return o;
        },
        std::vector<bool>{!r->defer_shadows});
    std::vector<uint32_t> tails;
    for (uint32_t t : {0u, 8192u, 32768u, 131072u})
        if (t != r->tail_threshold)
            tails.push_back(t);
    try_setting(
        [&](uint32_t v, bool) {
            uint32_t o = r->tail_threshold;
            r->tail_threshold = v;
            return o;
        },
        tails);
    try_setting(
        [&](uint32_t v, bool) {
            uint32_t o = r->graph_waves;
            r->graph_waves = v;
            return o;
        },
        std::vector<uint32_t>{r->graph_waves == 0 ? 8u : 0u});
    try_setting(
        [&](bool v, bool) {
            bool o = r->coop_tris;
            r->coop_tris = v;
            return o;
        },
        std::vector<bool>{!r->coop_tris});
    try_setting(
        [&](bool v, bool) {
            bool o = r->material_sort;
            r->material_sort = v;
            return o;
        },
        std::vector<bool>{!r->material_sort});
    std::vector<uint32_t> refills, steps;
    for (uint32_t v : {4u, 8u, 16u})
        if (v != r->fetch_refill)
            refills.push_back(v);
    try_setting(
        [&](uint32_t v, bool) {
            uint32_t o = r->fetch_refill;
            r->fetch_refill = r->shadow_fetch_refill = v;
            return o;
        },
        refills);
    for (uint32_t v : {2u, 4u, 8u})
        if (v != r->fetch_steps)
            steps.push_back(v);
    try_setting(
        [&](uint32_t v, bool) {
            uint32_t o = r->fetch_steps;
            r->fetch_steps = r->shadow_fetch_steps = v;
            return o;
        },
        steps);
    int most = vgx::wf_extend_blocks_per_sm();
    std::vector<int> extend_blocks;
    for (int b : {most, (3 * most) / 4, most / 2})
        if (b >= 1 && b != r->extend_blocks)
            extend_blocks.push_back(b);
    try_setting(
        [&](int v, bool) {
            int o = r->extend_blocks;
            r->extend_blocks = v;
            return o;
        },
        extend_blocks);
    if (pk && st == VG_OK) {
        std::vector<float> costs;
        for (float c : {0.25f, 0.5f, 2.0f})
            if (c != r->bvh_traversal_cost)
                costs.push_back(c);
        try_setting(
            [&](float v, bool) {
                float o = r->bvh_traversal_cost;
                int s2 = vg_set_bvh_traversal_cost(r, pk, v);
                if (s2 != VG_OK)
                    st = s2;
                return o;
            },
            costs);
    }
    r->adaptive = adaptive;
    r->stage_timing = timing;
    if (st != VG_OK)
        return st;
    out->dynamic_fetch = r->dynamic_fetch;
    out->deferred_shadows = r->defer_shadows;
    out->stream_tail = r->tail_threshold;
    out->graph_waves = r->graph_waves;
    out->bvh_traversal_cost = r->bvh_traversal_cost;
    out->extend_blocks_per_sm = r->extend_blocks;
    out->coop_triangles = r->coop_tris;
    out->material_sort = r->material_sort;
    out->fetch_refill = r->fetch_refill;
    out->fetch_steps = r->fetch_steps;
    out->mpaths_after = best;
    out->trials = trials;
    return VG_OK;
}

int vg_render_normals(VgRenderer* r, uint32_t width, uint32_t height, float* out)
{
    DevGuard device_guard(dev_of(r));
    if (!r || !out)
        return fail(VG_ERR_INVALID, "null argument");
    if (width == 0 || height == 0)
        return fail(VG_ERR_SCENE, "image size must be non-zero");
    size_t px = (size_t)width * height;
    cudaStream_t s = r->ctx->stream;
    DevBuf d;
    int st;
    if ((st = alloc(d, px * 12, s, false)) != VG_OK)
        return st;
    float rec[18];
    camera_record(r, width, height, rec);
    vgd::Ctx c = make_ctx(r, nullptr);
    VG_CHECK(cudaMemsetAsync(r->err.p, 0, 4, s), "error flag");
    VG_CHECK(vgx::launch_aov_normals(s, c, rec, (float*)d.p), "normals launch");
    VG_CHECK(cudaMemcpyAsync(out, d.p, px * 12, cudaMemcpyDeviceToHost, s), "readback");
    VG_CHECK(cudaStreamSynchronize(s), "normals");
    return read_err(r);
}

int vg_render_aovs(VgRenderer* r, uint32_t width, uint32_t height, float* albedo_depth, uint32_t* object_id,
                   uint32_t* material_id, float* coverage)
{
    DevGuard device_guard(dev_of(r));
    if (!r || !albedo_depth || !object_id || !material_id || !coverage)
        return fail(VG_ERR_INVALID, "null argument");
    if (width == 0 || height == 0)
        return fail(VG_ERR_SCENE, "image size must be non-zero");
    size_t px = (size_t)width * height;
    cudaStream_t s = r->ctx->stream;
    DevBuf ad, oi, mi, cv;
    int st;
    if ((st = alloc(ad, px * 16, s, false)) != VG_OK || (st = alloc(oi, px * 4, s, false)) != VG_OK ||
        (st = alloc(mi, px * 4, s, false)) != VG_OK || (st = alloc(cv, px * 4, s, false)) != VG_OK)
        return st;
    float rec[18];
    camera_record(r, width, height, rec);
    vgd::Ctx c = make_ctx(r, nullptr);
    VG_CHECK(cudaMemsetAsync(r->err.p, 0, 4, s), "error flag");
    VG_CHECK(vgx::launch_aov_main(s, c, rec, (float*)ad.p, (uint32_t*)oi.p, (uint32_t*)mi.p, (float*)cv.p),
             "aov launch");
    VG_CHECK(cudaMemcpyAsync(albedo_depth, ad.p, px * 16, cudaMemcpyDeviceToHost, s), "readback");
    VG_CHECK(cudaMemcpyAsync(object_id, oi.p, px * 4, cudaMemcpyDeviceToHost, s), "readback");
    VG_CHECK(cudaMemcpyAsync(material_id, mi.p, px * 4, cudaMemcpyDeviceToHost, s), "readback");
    VG_CHECK(cudaMemcpyAsync(coverage, cv.p, px * 4, cudaMemcpyDeviceToHost, s), "readback");
    VG_CHECK(cudaStreamSynchronize(s), "aovs");
    return read_err(r);
}

int vg_trace_closest_device(VgRenderer* r, const float* d_rays, size_t n, uint32_t* d_hits, double* seconds)
{
    DevGuard device_guard(dev_of(r));
    if (!r || (n > 0 && (!d_rays || !d_hits)))
        return fail(VG_ERR_INVALID, "null argument");
    if (n > 0xffffffffull)
        return fail(VG_ERR_INVALID, "too many rays");
    cudaStream_t s = r->ctx->stream;
    int st = VG_OK;
    if (!r->scratch.p && (st = alloc(r->scratch, 256, s, false)) != VG_OK)
        return st;
    vgd::Ctx c = make_ctx(r, nullptr);
    EventPool pool;
    cudaEvent_t a = pool.get(), b = pool.get();
    VG_CHECK(cudaMemsetAsync(r->err.p, 0, 4, s), "error flag");
    VG_CHECK(cudaMemsetAsync(r->scratch.p, 0, 4, s), "fetch counter");
    VG_CHECK(cudaEventRecord(a, s), "event");
    if (n > 0)
        VG_CHECK(vgx::launch_trace_rays(blocks_for(r, r->extend_blocks), s, c, d_rays, (uint4*)d_hits, (uint32_t)n,
                                        (uint32_t*)r->scratch.p),
                 "trace launch");
    VG_CHECK(cudaEventRecord(b, s), "event");
    if ((st = wait_event(b)) != VG_OK)
        return st;
    float ms = 0.0f;
    VG_CHECK(cudaEventElapsedTime(&ms, a, b), "event");
    if (seconds)
        *seconds = ms * 1e-3;
    return read_err(r);
}

int vg_trace_closest(VgRenderer* r, const float* rays, size_t n, uint32_t* hits)
{
    DevGuard device_guard(dev_of(r));
    if (!r || (n > 0 && (!rays || !hits)))
        return fail(VG_ERR_INVALID, "null argument");
    DevBuf dr, dh;
    cudaStream_t s = r->ctx->stream;
    int st;
    if ((st = alloc(dr, n * 24, s, false)) != VG_OK || (st = alloc(dh, n * 16, s, false)) != VG_OK)
        return st;
    if (n > 0)
        VG_CHECK(cudaMemcpyAsync(dr.p, rays, n * 24, cudaMemcpyHostToDevice, s), "ray upload");
    if ((st = vg_trace_closest_device(r, (const float*)dr.p, n, (uint32_t*)dh.p, nullptr)) != VG_OK)
        return st;
    if (n > 0) {
        VG_CHECK(cudaMemcpyAsync(hits, dh.p, n * 16, cudaMemcpyDeviceToHost, s), "hit readback");
        VG_CHECK(cudaStreamSynchronize(s), "hit readback");
    }
    return VG_OK;
}

} // extern "C"

// Static scratch of vg_trace_closest_noalloc: word 0 is the ray fetch counter, word 1 the error
// flag, then the staged rays (24 B each) and hits (16 B each) of at most VG_TRACE_NOALLOC_MAX_RAYS
// rays: 256 + 65536 * 40 bytes = 2.5 MiB of device memory in the module image.
namespace {
constexpr size_t NA_RAYS_OFF = 256;
constexpr size_t NA_HITS_OFF = NA_RAYS_OFF + (size_t)VG_TRACE_NOALLOC_MAX_RAYS * 24;
constexpr size_t NA_BYTES = NA_HITS_OFF + (size_t)VG_TRACE_NOALLOC_MAX_RAYS * 16;
constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mu;
unsigned char* g_na_addr[NA_MAX_DEVICES] = {};
} // namespace

static __device__ __align__(256) unsigned char g_trace_noalloc_scratch[NA_BYTES];

// Resolves the scratch array's address on `device` once (with that device current) and caches it.
static int noalloc_scratch(int device, unsigned char** out)
{
    if (device < 0 || device >= NA_MAX_DEVICES)
        return fail(VG_ERR_INVALID, "device ordinal out of range for the static scratch table");
    std::lock_guard<std::mutex> lock(g_na_mu);
    if (!g_na_addr[device]) {
        DevGuard on(device); // restores the caller's current device on return
        void* p = nullptr;
        VG_CHECK(cudaGetSymbolAddress(&p, g_trace_noalloc_scratch), "cudaGetSymbolAddress");
        g_na_addr[device] = (unsigned char*)p;
    }
    *out = g_na_addr[device];
    return VG_OK;
}

extern "C" {

int vg_trace_closest_noalloc(VgRenderer* r, const float* rays, size_t n, uint32_t* hits)
{
    DevGuard device_guard(dev_of(r));
    if (!r || (n > 0 && (!rays || !hits)))
        return fail(VG_ERR_INVALID, "null argument");
    if (n > VG_TRACE_NOALLOC_MAX_RAYS)
        return fail(VG_ERR_INVALID, "vg_trace_closest_noalloc: " + std::to_string(n) +
                                        " rays exceed its static scratch of " +
                                        std::to_string(VG_TRACE_NOALLOC_MAX_RAYS) +
                                        " rays; split the batch or call vg_trace_closest");
    unsigned char* base = nullptr;
    int st = noalloc_scratch(r->ctx->device, &base);
    if (st != VG_OK)
        return st;
    cudaStream_t s = r->ctx->stream;
    vgd::Ctx c = make_ctx(r, nullptr);
    c.err = (uint32_t*)(base + 4);
    // The fetch counter and the error flag must start at zero.
    VG_CHECK(cudaMemsetAsync(base, 0, 8, s), "scratch clear");
    if (n > 0) {
        VG_CHECK(cudaMemcpyAsync(base + NA_RAYS_OFF, rays, n * 24, cudaMemcpyHostToDevice, s), "ray upload");
        VG_CHECK(vgx::launch_trace_rays(blocks_for(r, r->extend_blocks), s, c, (const float*)(base + NA_RAYS_OFF),
                                        (uint4*)(base + NA_HITS_OFF), (uint32_t)n, (uint32_t*)base),
                 "trace launch");
        VG_CHECK(cudaMemcpyAsync(hits, base + NA_HITS_OFF, n * 16, cudaMemcpyDeviceToHost, s), "hit readback");
    }
    uint32_t e = 0;
    VG_CHECK(cudaMemcpyAsync(&e, base + 4, 4, cudaMemcpyDeviceToHost, s), "error flag");
    VG_CHECK(cudaStreamSynchronize(s), "trace");
    if (e & bvh8::ERR_STACK)
        return fail(VG_ERR_KERNEL, "BVH traversal stack overflow");
    if (e)
        return fail(VG_ERR_KERNEL, "kernel reported error status " + std::to_string(e));
    return VG_OK;
}

int vg_trace_occluded(VgRenderer* r, const float* rays, size_t n, uint32_t* out)
{
    DevGuard device_guard(dev_of(r));
    if (!r || (n > 0 && (!rays || !out)))
        return fail(VG_ERR_INVALID, "null argument");
    if (n > 0xffffffffull)
        return fail(VG_ERR_INVALID, "too many rays");
    DevBuf dr, dh;
    cudaStream_t s = r->ctx->stream;
    int st;
    if ((st = alloc(dr, n * 28, s, false)) != VG_OK || (st = alloc(dh, n * 4, s, false)) != VG_OK)
        return st;
    vgd::Ctx c = make_ctx(r, nullptr);
    VG_CHECK(cudaMemsetAsync(r->err.p, 0, 4, s), "error flag");
    if (n > 0) {
        VG_CHECK(cudaMemcpyAsync(dr.p, rays, n * 28, cudaMemcpyHostToDevice, s), "ray upload");
        VG_CHECK(vgx::launch_occlusion_rays(s, c, (const float*)dr.p, (uint32_t*)dh.p, (uint32_t)n), "occlusion launch");
        VG_CHECK(cudaMemcpyAsync(out, dh.p, n * 4, cudaMemcpyDeviceToHost, s), "readback");
    }
    VG_CHECK(cudaStreamSynchronize(s), "occlusion");
    return read_err(r);
}

} // extern "C"
