/* verion-gpu-cuda: C ABI of the GB300 (sm_103a) path-tracing backend.
 *
 * This is the surface a `verion-gpu-cuda` Rust crate binds to implement Verion's backend
 * contract: the `RayTracingBackend` trait (crates/verion-gpu/src/lib.rs:12-58) and the
 * `Accumulation` trait (crates/verion-gpu/src/lib.rs:74-93). Each entry point names the trait
 * method it replaces. Tables cross the boundary in exactly the layout of `pack::Packed`
 * (crates/verion-gpu/src/pack.rs:111-133), as pointer + length pairs, and are copied during the
 * call (the copy semantics of the Metal backend's newBufferWithBytes,
 * crates/verion-gpu-metal/src/renderer.rs:44-51).
 *
 * Handles are opaque and freed by the matching _destroy. A context and everything made from it
 * belong to the thread that made them (the reference's GPU objects are not Send,
 * crates/verion-render/src/session.rs:157-158). Every call returns a VgStatus; vg_last_error()
 * gives the thread's last message.
 */
#ifndef VGCUDA_H
#define VGCUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error kinds of the reference backends (crates/verion-gpu-metal/src/lib.rs:25-41,
 * crates/verion-gpu-vulkan/src/lib.rs:23-44), plus a timeout for bounded host waits. */
typedef enum VgStatus {
    VG_OK = 0,
    VG_ERR_NO_DEVICE = 1,   /* Error::NoDevice */
    VG_ERR_UNSUPPORTED = 2, /* Error::RaytracingUnsupported / Unsupported */
    VG_ERR_OOM = 3,         /* Error::OutOfMemory { needed, available } */
    VG_ERR_RESOURCE = 4,    /* Error::Resource */
    VG_ERR_KERNEL = 5,      /* Error::Shader: a kernel failed or reported an error status */
    VG_ERR_SCENE = 6,       /* Error::Scene */
    VG_ERR_TIMEOUT = 7,     /* the GPU did not finish within the host's deadline */
    VG_ERR_INVALID = 8      /* malformed call: null handle, bad size, bad table */
} VgStatus;

typedef struct VgContext VgContext;
typedef struct VgRenderer VgRenderer;
typedef struct VgAccum VgAccum;
typedef struct VgCache VgCache;

/* lib.rs:240-249 MemoryUsage */
typedef struct VgMemoryUsage {
    uint64_t budget;
    uint64_t allocated;
    uint64_t uploaded;
} VgMemoryUsage;

/* pack.rs:43-49 MeshRange */
typedef struct VgMeshRange {
    uint32_t vertex_offset;
    uint32_t vertex_count;
    uint32_t index_offset;
    uint32_t index_count;
} VgMeshRange;

/* pack.rs:54-69 SceneInfo */
typedef struct VgSceneInfo {
    uint32_t light_count;
    uint32_t emitter_count;
    uint32_t env_width;
    uint32_t env_height;
    float env_pdf_scale;
    float sky[3];
    uint32_t virtual_light;
    uint32_t transparent_background;
} VgSceneInfo;

/* pack.rs:72-81 View: camera[2] = tan(fov/2), camera[4..16] the camera-to-world rows. */
typedef struct VgView {
    float camera[16];
    float aperture;
    float focus;
    float shift[2];
} VgView;

/* pack.rs:111-133 Packed. `tlas_mesh` / `tlas_transform` are `Packed::tlas` (mesh index and 3x4
 * row-major object-to-world transform per instance, in instance-table order). */
typedef struct VgPacked {
    const float* positions;     size_t positions_len;
    const uint32_t* indices;    size_t indices_len;
    const float* uvs;           size_t uvs_len;
    const float* vnormals;      size_t vnormals_len;
    const uint32_t* instances;  size_t instances_len;
    const float* materials;     size_t materials_len;
    const uint32_t* lights;     size_t lights_len;
    const float* emitters;      size_t emitters_len;
    const float* emit_cdf;      size_t emit_cdf_len;
    const float* env_pixels;    size_t env_pixels_len;
    const float* env_marginal;  size_t env_marginal_len;
    const float* env_conditional; size_t env_conditional_len;
    const float* texels;        size_t texels_len;
    const uint32_t* tex_info;   size_t tex_info_len;
    const VgMeshRange* meshes;  size_t mesh_count;
    const uint32_t* tlas_mesh;
    const float* tlas_transform; size_t instance_count;
    VgSceneInfo info;
    VgView view;
} VgPacked;

/* lib.rs:98-104 Integrator */
typedef enum VgIntegrator { VG_MEGAKERNEL = 0, VG_WAVEFRONT = 1 } VgIntegrator;

/* Statistics of the acceleration structure a renderer built (no reference counterpart: the
 * reference's drivers build theirs). */
typedef struct VgBvhInfo {
    uint32_t triangles;
    uint32_t wide_nodes;
    uint32_t wide_depth;
    uint32_t binary_nodes;
    uint32_t binary_depth;
    uint64_t node_bytes;
    uint64_t triangle_bytes;
    double build_seconds;
} VgBvhInfo;

/* Copies the calling thread's last error message (NUL-terminated, truncated to len). Returns the
 * full message length. */
size_t vg_last_error(char* buf, size_t len);
/* OutOfMemory details of the thread's last VG_ERR_OOM. */
void vg_last_oom(uint64_t* needed, uint64_t* available);

/* RayTracingBackend::context (lib.rs:18-19): opens the calling thread's current CUDA device (device
 * 0 unless the caller selected another, e.g. one process per GPU under torchrun);
 * VG_ERR_NO_DEVICE without a GPU, VG_ERR_UNSUPPORTED unless it is an sm_103 device. Every object
 * made from a context belongs to its device: each call on it makes that device current for the
 * call's duration and restores the caller's current device afterwards. */
int vg_context_create(VgContext** out);
/* The same on device `device` (an ordinal below cudaGetDeviceCount; VG_ERR_INVALID otherwise).
 * The caller's current device is left as it was. No reference counterpart: the reference's
 * backends open the system default device. */
int vg_context_create_on(int device, VgContext** out);
void vg_context_destroy(VgContext* ctx);
/* RayTracingBackend::memory (lib.rs:20) */
int vg_memory(VgContext* ctx, VgMemoryUsage* out);

/* RayTracingBackend::new (lib.rs:22): uploads the tables and builds the BVH. An empty instance
 * table is VG_ERR_SCENE (pack.rs:727-729). */
int vg_renderer_create(VgContext* ctx, const VgPacked* packed, VgRenderer** out);
void vg_renderer_destroy(VgRenderer* r);

/* pack.rs:758-784 UpdatePlan: what a batch of scene edits makes the backend redo. `blases` lists
 * the meshes whose vertices were rewritten in place (same vertex counts). */
typedef struct VgUpdatePlan {
    int full;      /* meshes or instances added or re-pointed: rebuild everything */
    int materials; /* material and texture tables */
    int lights;    /* light table, sky, environment map */
    int emitters;  /* emitter table and CDF */
    int instances; /* instance table */
    int vertices;  /* vertex tables of the meshes in `blases` */
    const uint32_t* blases;
    size_t blas_count;
    int tlas;      /* instance transforms changed */
    int camera;
} VgUpdatePlan;

/* lib.rs:63-71 UpdateReport. */
typedef struct VgUpdateReport {
    uint64_t blases_built;
    int tlas_built;
    uint64_t bytes_uploaded;
} VgUpdateReport;

/* RayTracingBackend::update (lib.rs:23-27; Metal renderer.rs:226-349): applies the edits `plan`
 * names, taking the tables of the edited scene from `packed` (pack::pack of the edited scene) and
 * leaving everything else as it is. This backend's acceleration structure is one BVH8 over the
 * world-space triangles of all instances, rebuilt when instance transforms or vertices change
 * (`tlas_built`); `blases_built` counts the meshes whose vertex tables were rewritten (all meshes
 * on a full rebuild). `bytes_uploaded` counts table and BVH bytes written to the device. Settings
 * (integrator, adaptive, ReSTIR, depth, precision, cache) are kept. A deformation that changes a
 * mesh's vertex count is VG_ERR_SCENE: that is a geometry change (plan.full). Start a new
 * accumulation afterwards: samples from before the edit no longer match the scene. */
int vg_renderer_update(VgRenderer* r, const VgPacked* packed, const VgUpdatePlan* plan, VgUpdateReport* out);
int vg_renderer_bvh_info(const VgRenderer* r, VgBvhInfo* out);

/* RayTracingBackend::set_camera (lib.rs:31) */
int vg_set_camera(VgRenderer* r, const VgView* view);
/* RayTracingBackend::set_multiscatter (lib.rs:33) */
int vg_set_multiscatter(VgRenderer* r, int on);
/* RayTracingBackend::set_integrator / integrator (lib.rs:34-35) */
int vg_set_integrator(VgRenderer* r, int integrator);
int vg_integrator(const VgRenderer* r);
/* RayTracingBackend::set_stage_timing (lib.rs:37) */
int vg_set_stage_timing(VgRenderer* r, int on);
/* RayTracingBackend::set_adaptive (lib.rs:39): on = 0 is None. */
int vg_set_adaptive(VgRenderer* r, int on, float threshold, uint32_t min_spp);
/* RayTracingBackend::set_restir (lib.rs:42): on = 0 is None. `di` and `gi` select ReSTIR DI
 * (pt_core.slang:759-882) and ReSTIR GI (:897-981, :1566-1617); GI stays off with the lighting
 * split, as in the reference. */
int vg_set_restir(VgRenderer* r, int on, int di, int gi, uint32_t candidates, uint32_t history);

/* Extensions with no reference counterpart. */
/* Path length limit for accumulations (reference: the constant MAX_DEPTH = 8, pack.rs:13). */
int vg_set_max_depth(VgRenderer* r, uint32_t depth);
/* Wavefront scheduling. VG_WAVEFRONT_PER_SAMPLE is the reference's order: one sample at a time,
 * one extend and one shade launch per depth, with per-depth queue counts readable afterwards.
 * VG_WAVEFRONT_STREAMING (default) regenerates paths: each pixel's slot runs the call's samples
 * back to back, so a launch covers every live path whatever its depth; per pixel the samples are
 * still added in order, and the sums are identical. ReSTIR always runs per sample. */
typedef enum VgWavefrontMode { VG_WAVEFRONT_PER_SAMPLE = 0, VG_WAVEFRONT_STREAMING = 1 } VgWavefrontMode;
int vg_set_wavefront_mode(VgRenderer* r, int mode);
/* Streaming mode: when at most `threshold` slots are live after a wave, the rest of the batch
 * (those paths and their remaining samples) runs in one launch, trace and shade in a loop per slot,
 * instead of one wave per bounce. 0 disables it. Default 32768. */
int vg_set_stream_tail(VgRenderer* r, uint32_t threshold);
/* Streaming mode without the lighting split: trace the bounce's emitter / environment shadow ray
 * in a separate stage after shade (default on) or inline in shade (off). Same sums either way. */
int vg_set_deferred_shadows(VgRenderer* r, int on);
/* Streaming mode: the extend and shadow stages refill a warp's idle lanes with queued rays
 * (default on) or give each warp 32 rays at a time (off). Same results either way. */
int vg_set_dynamic_fetch(VgRenderer* r, int on);
/* Streaming mode with dynamic fetch: the extend and shadow stages test the triangles of the leaves
 * their warp's rays reached together, one (ray, triangle) pair per lane (on), or each lane its own
 * (off, the default: on the 1M-triangle workload the cooperative form's scan, shuffles and
 * shared-memory reductions cost more than the idle lanes they save). Same results either way. No
 * reference counterpart: the reference's hardware ray queries have no such choice. */
int vg_set_coop_triangles(VgRenderer* r, int on);
/* Streaming mode with deferred shadows: between the extend and shade stages each wave's slots are
 * regrouped by shading class (missed ray, diffuse, conductor, dielectric) so that the shade stage's
 * warps mostly run one BSDF's code (default on), or shaded in queue order (off). Same sums either
 * way. No reference counterpart. */
int vg_set_material_sort(VgRenderer* r, int on);
/* Streaming mode with dynamic fetch: a warp of the extend stage takes new rays once at least
 * `refill` of its 32 lanes are idle (1-32, default 8) and visits at most `steps` nodes per lane
 * between refills (1-64, default 4); shadow_refill and shadow_steps set the same for the shadow
 * stage. Same results for every setting. No reference counterpart. */
int vg_set_traversal_fetch(VgRenderer* r, uint32_t refill, uint32_t steps, uint32_t shadow_refill,
                           uint32_t shadow_steps);
/* Streaming mode: capture `waves` waves (an even count, 0 = off) of the bounce loop in a CUDA graph
 * once per call and replay it until the slots drain (without stage timing), instead of launching
 * every wave's kernels from the host. Same sums. */
int vg_set_wavefront_graph(VgRenderer* r, uint32_t waves);
/* Rebuilds the BVH8 with another SAH node-visit cost (relative to a triangle test; default 0.5):
 * smaller values give deeper trees with smaller leaves. `packed` must be the renderer's scene
 * tables (pack::pack of the same scene). Hits are the same with any BVH. */
int vg_set_bvh_traversal_cost(VgRenderer* r, const VgPacked* packed, float cost);

/* Autotuner of the streaming wavefront (no reference counterpart): on scratch accumulations of
 * width x height and `samples` per trial, a coordinate-descent pass over dynamic fetch, deferred
 * shadows, the tail threshold (0, 8192, 32768, 131072), the wave graph (0 or 8 waves), the CTAs
 * per SM of the persistent extend stage (the most that fit, 3/4 or 1/2 of it) and, when `packed` is
 * given, the BVH8's SAH traversal cost (0.25, 0.5, 1, 2); a change is kept when it is more than 1%
 * faster. Leaves the renderer on the streaming wavefront with the best setting. All of these
 * settings give the same sums. */
typedef struct VgTuneResult {
    int dynamic_fetch;
    int deferred_shadows;
    uint32_t stream_tail;
    uint32_t graph_waves;
    float bvh_traversal_cost;
    double mpaths_before, mpaths_after; /* camera paths per second, first and best trial */
    uint32_t trials;
    int extend_blocks_per_sm;
    int coop_triangles;                /* vg_set_coop_triangles */
    uint32_t fetch_refill, fetch_steps; /* vg_set_traversal_fetch, extend stage */
    int material_sort;                  /* vg_set_material_sort */
} VgTuneResult;
int vg_autotune(VgRenderer* r, const VgPacked* packed, uint32_t width, uint32_t height, uint32_t samples,
                VgTuneResult* out);
/* With stage timing: seconds of the last call's tail launch (0 if none ran). */
double vg_accum_tail_seconds(const VgAccum* acc);
/* Streaming mode: waves (extend + shade pairs) issued by the last vg_accumulate. */
uint32_t vg_accum_last_waves(const VgAccum* acc);
/* Streaming mode, last vg_accumulate: per wave, the live slots after it and (with stage timing)
 * the extend, shade and shadow-stage milliseconds (shadow 0 when shade traced inline), 4 floats
 * per wave for up to `waves` waves. Returns the number of waves recorded. */
size_t vg_accum_wave_profile(const VgAccum* acc, float* out, size_t waves);
/* Wavefront only: count rays, BVH nodes visited and triangles tested in the extend stage of
 * later accumulate calls (read with vg_accum_traversal_stats). */
int vg_set_traversal_stats(VgRenderer* r, int on);
/* Precision of the per-pixel sums of accumulations made afterwards: 32 (the reference's f32
 * sums) or 64 (double sums and double adaptive-sampling statistics, the default). */
int vg_set_accum_precision(VgRenderer* r, int bits);

/* RayTracingBackend::new_accumulation (lib.rs:45-51); zero size is VG_ERR_SCENE. */
int vg_accum_create(VgRenderer* r, uint32_t width, uint32_t height, int lighting, VgAccum** out);
void vg_accum_destroy(VgAccum* acc);
/* RayTracingBackend::accumulate (lib.rs:50-52): blocking. Switching adaptive sampling or ReSTIR
 * mid-accumulation is VG_ERR_SCENE (renderer.rs:800-828). */
int vg_accumulate(VgRenderer* r, VgAccum* acc, uint32_t samples);

/* Accumulation getters (lib.rs:76-92). */
uint32_t vg_accum_samples(const VgAccum* acc);
/* Per-pixel sample indices of this accumulation start at `first` (default 0) instead of 0: its
 * samples then share no random sequence with another accumulation's samples below `first` (each
 * sample's sequence is seeded from the pixel and the sample index, pt_core.slang:645-682), e.g.
 * for an independent reference image or for replicas that split one image's samples. Set before
 * the first sample; plain path tracing only (an accumulation with ReSTIR or the radiance cache
 * fails with VG_ERR_SCENE). No reference counterpart. */
int vg_accum_set_first_sample(VgAccum* acc, uint32_t first);
double vg_accum_gpu_seconds(const VgAccum* acc);
/* Stage seconds {extend, shade}; returns 0 when stage timing never ran (None). */
int vg_accum_stage_seconds(const VgAccum* acc, double out[2]);
size_t vg_accum_wavefront_bytes(const VgAccum* acc);
size_t vg_accum_restir_bytes(const VgAccum* acc);
/* Sum-precision of the accumulation in bits (32 or 64). */
int vg_accum_precision(const VgAccum* acc);
/* Raw sums for the shared readback arithmetic (readback.rs:18-137): 3 floats per pixel. A
 * 64-bit accumulation is rounded to float here; vg_accum_read_sums_f64 returns it whole. */
int vg_accum_read_sums(const VgAccum* acc, float* out, size_t len);
int vg_accum_read_sums_f64(const VgAccum* acc, double* out, size_t len);
/* Lighting split, LIGHTING_STRIDE = 65 floats per pixel (VG_ERR_INVALID without `lighting`). */
int vg_accum_read_lighting(const VgAccum* acc, float* out, size_t len);
/* Adaptive-sampling record, 3 floats per pixel: samples, luminance sum, square sum
 * (VG_ERR_INVALID when adaptive sampling never ran). */
int vg_accum_read_stats(const VgAccum* acc, float* out, size_t len);
/* Wavefront queue lengths of the last sample traced: live paths at depths 0..max depth
 * (max depth + 1 words; VG_ERR_INVALID before a wavefront accumulate). */
int vg_accum_read_queue_counts(const VgAccum* acc, uint32_t* out, size_t len);
/* Extend-stage counters since the accumulation began (with traversal stats on): rays, BVH nodes
 * visited, triangles tested, rays past depth 0. */
int vg_accum_traversal_stats(const VgAccum* acc, uint64_t out[4]);
/* Shadow rays traced by the streaming wavefront's any-hit stage since the accumulation began (with
 * traversal stats on; with the deferred shadow stage and dynamic fetch in opaque scenes). */
int vg_accum_shadow_rays(const VgAccum* acc, uint64_t* out);
/* Kernel launches made by vg_accumulate on this accumulation so far. */
uint64_t vg_accum_launches(const VgAccum* acc);
/* Average duration in seconds of one extend-kernel launch, from stage timing (0 if none). */
double vg_accum_extend_launch_seconds(const VgAccum* acc);

/* RayTracingBackend::render_normals (lib.rs:55): world-space normal of the first hit through each
 * pixel centre, facing the viewer, 3 floats per pixel into host memory; misses are zero. */
int vg_render_normals(VgRenderer* r, uint32_t width, uint32_t height, float* out);
/* RayTracingBackend::render_aovs (lib.rs:57, Aovs lib.rs:165-181), host arrays of width * height:
 * albedo (3 floats) and depth along the camera's forward axis (1 float) per pixel, instance + 1,
 * material + 1 (0 on a miss), and coverage of 16 stratified rays through translucent surfaces. */
int vg_render_aovs(VgRenderer* r, uint32_t width, uint32_t height, float* albedo_depth, uint32_t* object_id,
                   uint32_t* material_id, float* coverage);

/* Traversal entry points (no reference counterpart; the reference's traversal is the driver's).
 * Closest hits of n rays (6 floats each: origin xyz, direction xyz, host memory) into 4 words per
 * ray (hit flag, instance, primitive, t bits) as the wavefront's hit record (wf_extend.slang:26-29). */
int vg_trace_closest(VgRenderer* r, const float* rays, size_t n, uint32_t* hits);
/* Shadow-ray queries of n rays (7 floats each: origin, direction, tmax): 1 occluded, 0 free,
 * as pt_core.slang's occluded (:580-613). */
int vg_trace_occluded(VgRenderer* r, const float* rays, size_t n, uint32_t* out);
/* Device-resident form for timing: rays and hits are device pointers; returns the kernel time. */
int vg_trace_closest_device(VgRenderer* r, const float* d_rays, size_t n, uint32_t* d_hits, double* seconds);

/* vg_trace_closest without any device allocation (no reference counterpart). For callers that must
 * not allocate while they query the scene: a viewer's per-frame picking or a tool's probe rays run
 * beside other streams, and cudaMalloc / cudaFree (which vg_trace_closest does per call for its
 * ray and hit staging) synchronise the whole device or fail once the scene has taken the memory.
 * The staging, the fetch counter and the error flag live in one static device array of the
 * library module instead: at most VG_TRACE_NOALLOC_MAX_RAYS rays per call (2.5 MiB); larger n is
 * rejected with VG_ERR_INVALID. The first call on a device resolves that array's address (with
 * cudaGetSymbolAddress, the device made current) and caches it: make that first call before any
 * stream capture. All renderers on a device share the array, so calls that overlap on the GPU
 * (from several threads or contexts at once) race on it; the call synchronises its stream before
 * it returns. Results are identical to vg_trace_closest's. */
#define VG_TRACE_NOALLOC_MAX_RAYS 65536u
int vg_trace_closest_noalloc(VgRenderer* r, const float* rays, size_t n, uint32_t* hits);

/* Device allocations (cudaMalloc) and frees (cudaFree) this library has made since it was loaded,
 * for tests of the allocation-free entry point. No reference counterpart. */
void vg_debug_allocations(uint64_t* mallocs, uint64_t* frees);

/* ---- Batched rendering (no reference counterpart) -----------------------------------------------
 * Many render requests of uneven size, scene and sample count in shared launches, each captured in
 * a CUDA graph the first time and replayed while the batch keeps the same shape (same renderers,
 * accumulations, sample counts and caches in the same order):
 * - requests below a size threshold: one persistent tile launch. The work items (16 x 8 pixel tiles
 *   with all of a request's samples) are laid out shortest request first (or as given, or longest
 *   first) and taken by the CTAs of one kernel. A request with a cache ends its paths at the cache
 *   and evaluates the cache inside the same CTA (tensor cores); after the launch each cache takes
 *   its renderer's training steps (vg_set_cache) on the batch's training records.
 * - requests from the threshold up (by default every request): the batch wavefront, the streaming
 *   wavefront over the pixels of all of them (each path slot traces one pixel of one request with
 *   all its samples, then takes the next pixel in request order), its bounce loop running on the
 *   device inside the graph (a conditional WHILE node). A cached request's queries are answered
 *   after each wave by one kernel for all caches; the caches train after the loop.
 * - requests with a cache that the batch wavefront cannot tag (more than 2^22 pixels, or more than
 *   1024 requests in the batch): one at a time on the streaming cache integrator after the shared
 *   launches, shortest first.
 * The batch wavefront takes at most 2^31 pixels per batch (VG_ERR_INVALID beyond).
 * A plain request's samples are exactly what vg_accumulate's megakernel adds (same sums, either
 * shared launch); a cached request's exactly what the megakernel cache integrator adds with a fixed
 * cache. */
typedef enum VgBatchOrder { VG_BATCH_SHORTEST_FIRST = 0, VG_BATCH_AS_GIVEN = 1, VG_BATCH_LONGEST_FIRST = 2 } VgBatchOrder;

typedef struct VgBatchRequest {
    VgRenderer* renderer; /* scene and settings: megakernel paths without adaptive sampling, ReSTIR or the lighting split */
    VgAccum* accum;       /* the request's accumulation (its size is the frame size) */
    uint32_t samples;     /* samples per pixel to add */
    VgCache* cache;       /* null: plain path tracing; else the renderer's vg_set_cache settings apply */
} VgBatchRequest;

typedef struct VgBatchResult {
    double seconds; /* from the batch's start to this request's last tile or pixel, device clock */
} VgBatchResult;

/* Renders all requests (blocking). *total_seconds (optional) is the whole batch on the device
 * clock, training included; *graph_replayed (optional) tells whether the captured graph was reused. */
int vg_batch_render(VgContext* ctx, const VgBatchRequest* requests, size_t n, VgBatchResult* out,
                    double* total_seconds, int* graph_replayed);
/* The batch kernel's resident CTAs per SM, registers per thread, local bytes per thread, static
 * shared bytes, and the CUDA status of the occupancy query, in that order. */
int vg_batch_kernel_info(VgContext* ctx, int out[5]);
/* Batch kernel CTAs per SM (0: as many as fit), the item order, and the size (pixels) from which a
 * request leaves the tile launch for the batch wavefront (~0: never; default 0: every request on
 * the batch wavefront, the faster on both measured mixes). vg_batch_tune picks all three. */
int vg_set_batch_options(VgContext* ctx, int blocks_per_sm, int order, uint64_t wavefront_pixels);
/* Path slots of the batch wavefront (1024 to 2^26; default 2^21): at most this many pixels are in
 * flight at once. vg_batch_tune picks it. */
int vg_set_batch_wave_slots(VgContext* ctx, uint32_t slots);
/* Batch wavefront: run the bounce loop on the device inside the batch's graph (on, the default) or
 * from the host, one graph launch per two waves with the live count read back after each (off:
 * for tools that cannot look into graphs with conditional nodes, such as kernel profilers). Same
 * sums either way. */
int vg_set_batch_device_loop(VgContext* ctx, int on);
/* Autotuner: times the batch on scratch accumulations of the requests' sizes for each threshold
 * (0, 256^2, 512^2, 1024^2 pixels, never; one that splits the requests as an earlier one did is
 * skipped), shortest or longest first, the two largest CTA counts per SM that fit (when the tile
 * launch has requests) and 2^20 or 2^21 wavefront slots (when the batch wavefront has requests);
 * keeps the setting with the lowest objective (median plus 99th percentile request latency) and
 * reports it. The requests' own accumulations are not touched. */
typedef struct VgBatchTune {
    int blocks_per_sm;
    int order;
    uint64_t wavefront_pixels;
    double p50_seconds, p99_seconds, total_seconds; /* of the chosen setting */
    uint32_t trials;
    uint32_t wave_slots;
} VgBatchTune;
int vg_batch_tune(VgContext* ctx, const VgBatchRequest* requests, size_t n, VgBatchTune* out);

/* ---- EXR output (crates/verion-render-io/src/exr_out.rs) -----------------------------------------
 * Working and target colour spaces, tone map and transfer function (crates/verion-scene/src/color.rs). */
typedef enum VgColorSpace { VG_COLOR_LINEAR_REC709 = 0, VG_COLOR_ACESCG = 1 } VgColorSpace;
typedef enum VgToneMap { VG_TONEMAP_NONE = 0, VG_TONEMAP_REINHARD = 1 } VgToneMap;
typedef enum VgOetf { VG_OETF_LINEAR = 0, VG_OETF_SRGB = 1 } VgOetf;
/* color.rs:84-124 OutputTransform: {target, NONE, LINEAR} is OutputTransform::linear(target),
 * {LINEAR_REC709, REINHARD, SRGB} is OutputTransform::display(). */
typedef struct VgOutputTransform {
    int target;
    int tone_map;
    int oetf;
} VgOutputTransform;

/* exr_out.rs:8-79 ExrFrame + ExrAovs + RenderInfo. Pixels row-major from the top-left; 3 floats per
 * pixel for colour planes, 1 for depth and visibility. Optional planes are null when absent; the
 * lighting split needs all five parts and the visibility. */
typedef struct VgExrFrame {
    uint32_t width, height;
    int working_space;
    const float* beauty;
    const float* normal;
    const float* albedo;
    const float* depth;
    const uint32_t* object_id;
    const uint32_t* material_id;
    const uint32_t* sample_count;
    const float* lighting[5]; /* direct diffuse, indirect diffuse, specular, transmission, emission */
    const float* visibility;
    int physical;
    uint32_t samples;
    uint64_t stylization_revision;
    int has_grade;
    float exposure, saturation, white_balance[3];
    const char* denoiser; /* null: none */
    int has_adaptive_threshold;
    float adaptive_threshold;
    const char* restir;   /* null, "di" or "di+gi" */
} VgExrFrame;

/* write_exr (exr_out.rs:103-293): one OpenEXR file with the reference's channel names (R, G, B,
 * N.X.., Albedo.*, DirectDiffuse.* .. Emission.*, Visibility.V, Z, and the 32-bit integer channels
 * ObjectId, MaterialId, SampleCount), the target's chromaticities and the `verion/` metadata.
 * Uncompressed scanlines. VG_ERR_INVALID for a zero size or an incomplete lighting split;
 * VG_ERR_RESOURCE when the file cannot be written. */
int vg_write_exr(const char* path, const VgExrFrame* frame, const VgOutputTransform* transform);

/* ---- Radiance cache (no reference counterpart) -----------------------------------------------
 * A multi-resolution hash-grid encoding of the position (two fp16 features per level) feeding a
 * 64-wide MLP with 4 hidden ReLU layers (bf16 weights and activations, f32 accumulation on the
 * tensor cores) that predicts the radiance a surface point scatters toward a direction. Trained
 * online with Adam on the relative L2 loss sum_k (p_k - y_k)^2 / (p_k^2 + 0.01) (denominator held
 * constant).
 *
 * Records are VG_CACHE_RECORD_FLOATS floats: 0-2 world position, 3-5 direction toward the viewer
 * of the vertex, 6-8 shading normal, 9 roughness, 10-12 base colour, 13 metallic, 14 transmission,
 * 15 unused, 16-18 the training target (radiance), 19 unused.
 * Parameters (f32): the MLP as 4 matrices of 64 x 64 then one of 16 x 64 (rows 0-2 used), each
 * row-major (output, input), VG_CACHE_MLP_PARAMS floats; the grid as levels x 2^log2_entries x 2. */
#define VG_CACHE_RECORD_FLOATS 20u
#define VG_CACHE_MLP_PARAMS 17408u

typedef struct VgCacheConfig {
    uint32_t levels;          /* hash-grid levels, 1..16 (16) */
    uint32_t log2_entries;    /* table entries per level, log2, 8..24 (19) */
    uint32_t base_resolution; /* coarsest grid resolution over the box's largest side (16) */
    uint32_t max_resolution;  /* finest grid resolution (2048) */
    float learning_rate;      /* Adam step size (0.01; 0 keeps the parameters as they are) */
    float beta1, beta2, epsilon; /* Adam (0.9, 0.99, 1e-8) */
    uint32_t seed;            /* initialisation seed */
    float bounds_lo[3], bounds_hi[3]; /* scene box the grid spans (vg_renderer_bounds) */
} VgCacheConfig;

/* Fills the defaults above (bounds zero). */
void vg_cache_default_config(VgCacheConfig* out);
/* World-space box of the renderer's triangles. */
int vg_renderer_bounds(const VgRenderer* r, float lo[3], float hi[3]);
int vg_cache_create(VgContext* ctx, const VgCacheConfig* cfg, VgCache** out);
int vg_cache_destroy(VgCache* cache);
int vg_cache_param_counts(const VgCache* cache, size_t* mlp, size_t* grid);
/* f32 master parameters; either pointer may be null. */
int vg_cache_read_params(VgCache* cache, float* mlp, float* grid);
/* Replaces the parameters (either pointer may be null) and restarts the optimiser. */
int vg_cache_write_params(VgCache* cache, const float* mlp, const float* grid);
/* Predictions (3 floats per record) of n records. */
int vg_cache_infer(VgCache* cache, const float* records, size_t n, float* out);
/* Gradient sums over n records of the per-record loss, without applying them: mlp_grad has
 * VG_CACHE_MLP_PARAMS floats, grid_grad the grid's size (either may be null); *loss = loss sum. */
int vg_cache_gradients(VgCache* cache, const float* records, size_t n, float* mlp_grad, float* grid_grad,
                       double* loss);
/* Adam steps over consecutive batches of `batch` records (gradient = batch mean); *last_loss =
 * mean loss per channel of the last batch. */
int vg_cache_train(VgCache* cache, const float* records, size_t n, uint32_t batch, double* last_loss);
/* Device time per launch of the cache kernels on n records (one untimed round, then `reps`
 * launches of each back to back): out = {encode, inference, training pass (forward, backward and
 * weight gradients on the tensor cores), grid-gradient scatter} in seconds. Gradients are not
 * applied. For measurement. */
int vg_cache_time(VgCache* cache, const float* records, size_t n, uint32_t reps, double out[4]);
/* Radiance-cache integrator for this renderer's accumulations (cache null: off). Each sample
 * traces one path per pixel that ends at the first vertex past the primary one where the path
 * spread passes `spread` times the primary spread (Mueller et al. 2021), and adds the cache's
 * prediction there times the path throughput; about `train_paths` pixels per sample trace
 * training paths to full depth instead, whose vertices train the cache for `train_steps` Adam
 * steps of `train_batch` records after the sample. With the WAVEFRONT integrator the query paths
 * run on the streaming wavefront in frames of several samples (vg_set_cache_frame), with
 * MEGAKERNEL in one kernel per sample; training paths always run in a kernel of their own,
 * overlapping the query paths. For the same cache state both integrators find the same queries
 * and answers. The lighting split, adaptive sampling and ReSTIR are not available with it
 * (VG_ERR_UNSUPPORTED). The renderer does not own the cache: keep it alive while the renderer
 * uses it. */
int vg_set_cache(VgRenderer* r, VgCache* cache, float spread, uint32_t train_paths, uint32_t train_steps,
                 uint32_t train_batch);
/* WAVEFRONT integrator with a cache: samples per cache frame (1-16, default 4). The cache is fixed
 * within a frame and trained after it (vg_set_cache's steps), so a frame of k samples runs as one
 * streaming wavefront dispatch of k samples per pixel (the last waves of a dispatch are nearly
 * empty; k samples share them). The training pixels of a frame trace all its samples. */
int vg_set_cache_frame(VgRenderer* r, uint32_t samples_per_frame);
/* Radiance cache: training-only frames run before the first sample of each accumulation (default
 * 0). Each traces one sample of training paths (into a scratch buffer, not the image) and takes
 * the training steps, so the image does not average in the answers of a cache that has barely
 * been trained. Their device time counts in the accumulate call. */
int vg_set_cache_warmup(VgRenderer* r, uint32_t frames);
/* Of the last sample of the last accumulate call with the cache: query records, training
 * records (before the capacity clamp), and the last training step's mean loss per channel;
 * with stage timing, seconds spent in the path kernel, inference and training over that call. */
typedef struct VgCacheStats {
    uint32_t queries;
    uint32_t train_records;
    double loss;
    double path_seconds, infer_seconds, train_seconds;
} VgCacheStats;
int vg_accum_cache_stats(const VgAccum* acc, VgCacheStats* out);

#ifdef __cplusplus
}
#endif

#endif /* VGCUDA_H */
