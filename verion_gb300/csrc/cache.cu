// C ABI of the radiance cache (include/vgcuda.h, "Radiance cache"): the cache object, its
// parameters and optimiser state, the host-record entry points used by tests and tools, and the
// per-sample loop of the cache integrator. No reference counterpart.
#include <cmath>

#include "cache_host.h"

namespace vgc {

// Deterministic parameter initialisation: a PCG-hash stream of uniform numbers in [-1, 1).
float uniform_pm1(uint32_t seed, uint64_t i)
{
    auto pcg = [](uint32_t v) {
        uint32_t state = v * 747796405u + 2891336453u;
        uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
        return (word >> 22u) ^ word;
    };
    uint32_t h = pcg(pcg((uint32_t)i ^ seed) ^ (uint32_t)(i >> 32) ^ 0x9E3779B9u);
    return (float)((double)h / 4294967296.0 * 2.0 - 1.0);
}

int cache_check(const VgCache* k)
{
    uint32_t e = 0;
    VG_CHECK(cudaMemcpyAsync(&e, k->err.p, 4, cudaMemcpyDeviceToHost, k->ctx->stream), "error flag");
    VG_CHECK(cudaStreamSynchronize(k->ctx->stream), "cache");
    if (e & vgn::ERR_MMA_TIMEOUT)
        return fail(VG_ERR_KERNEL, "a tensor-core completion wait timed out");
    if (e)
        return fail(VG_ERR_KERNEL, "cache kernel reported error status " + std::to_string(e));
    return VG_OK;
}

// Regenerates the fp16 grid table and the bf16 weight image from the f32 parameters.
int cache_refresh(VgCache* k)
{
    cudaStream_t s = k->ctx->stream;
    VG_CHECK(vgx::nrc_launch_to_half(s, (const float*)k->grid.p, k->grid_h.p, k->grid_params), "grid copy");
    VG_CHECK(vgx::nrc_launch_pack(s, (const float*)k->mlp.p, (uint8_t*)k->img.p), "weight image");
    return VG_OK;
}

int cache_reset_optimiser(VgCache* k)
{
    cudaStream_t s = k->ctx->stream;
    VG_CHECK(cudaMemsetAsync(k->grid_grad.p, 0, k->grid_grad.bytes, s), "clear");
    VG_CHECK(cudaMemsetAsync(k->grid_m.p, 0, k->grid_m.bytes, s), "clear");
    VG_CHECK(cudaMemsetAsync(k->grid_v.p, 0, k->grid_v.bytes, s), "clear");
    VG_CHECK(cudaMemsetAsync(k->mlp_grad.p, 0, k->mlp_grad.bytes, s), "clear");
    VG_CHECK(cudaMemsetAsync(k->mlp_m.p, 0, k->mlp_m.bytes, s), "clear");
    VG_CHECK(cudaMemsetAsync(k->mlp_v.p, 0, k->mlp_v.bytes, s), "clear");
    VG_CHECK(cudaMemsetAsync(k->step.p, 0, 4, s), "clear");
    return VG_OK;
}

// Room for `rows` encoded records and input-gradient rows.
int ensure_work(VgCache* k, size_t rows)
{
    size_t xb = std::max<size_t>((rows + vgn::TILE - 1) / vgn::TILE, 1) * 16384;
    size_t gb = std::max<size_t>(rows, 1) * 32 * 4;
    int st;
    if (k->X.bytes < xb && (st = alloc(k->X, xb, k->ctx->stream, false)) != VG_OK)
        return st;
    if (k->GX.bytes < gb && (st = alloc(k->GX, gb, k->ctx->stream, false)) != VG_OK)
        return st;
    return VG_OK;
}

int encode_blocks(const VgCache* k) { return 8 * k->ctx->sms; }

// Gradient sums of the records [offset, offset + batch) of the first min(*count, cap) at `rec`:
// encode, the tensor-core pass, the grid scatter (ensure_work(batch) first).
int cache_gradient_pass(VgCache* k, const float* rec, const uint32_t* count, uint32_t cap, uint32_t offset,
                        uint32_t batch)
{
    cudaStream_t s = k->ctx->stream;
    vgn::CacheDev d = k->dev();
    VG_CHECK(vgx::nrc_launch_encode(encode_blocks(k), s, d, rec, count, cap, offset, batch, (uint8_t*)k->X.p),
             "encode launch");
    VG_CHECK(vgx::nrc_launch_train(k->ctx->sms, s, d, (const uint8_t*)k->X.p, rec, count, cap, offset, batch,
                                   (float*)k->GX.p),
             "train launch");
    VG_CHECK(vgx::nrc_launch_scatter(encode_blocks(k), s, d, rec, count, cap, offset, batch, (const float*)k->GX.p),
             "scatter launch");
    return VG_OK;
}

// One Adam step on the records [offset, offset + batch) of the first min(*count, cap) at `rec`.
int cache_train_step(VgCache* k, const float* rec, const uint32_t* count, uint32_t cap, uint32_t offset,
                     uint32_t batch)
{
    cudaStream_t s = k->ctx->stream;
    int st;
    VG_CHECK(cudaMemsetAsync(k->loss.p, 0, 8, s), "loss");
    if ((st = cache_gradient_pass(k, rec, count, cap, offset, batch)) != VG_OK)
        return st;
    VG_CHECK(vgx::nrc_launch_step(s, (uint32_t*)k->step.p), "step");
    NrcAdam a;
    a.lr = k->cfg.learning_rate;
    a.beta1 = k->cfg.beta1;
    a.beta2 = k->cfg.beta2;
    a.eps = k->cfg.epsilon;
    a.step = (const uint32_t*)k->step.p;
    VG_CHECK(vgx::nrc_launch_adam(s, (float*)k->mlp.p, (float*)k->mlp_grad.p, (float*)k->mlp_m.p, (float*)k->mlp_v.p,
                                  vgn::MLP_PARAMS, count, cap, offset, batch, a, nullptr, false),
             "adam");
    VG_CHECK(vgx::nrc_launch_pack(s, (const float*)k->mlp.p, (uint8_t*)k->img.p), "weight image");
    VG_CHECK(vgx::nrc_launch_adam(s, (float*)k->grid.p, (float*)k->grid_grad.p, (float*)k->grid_m.p,
                                  (float*)k->grid_v.p, k->grid_params, count, cap, offset, batch, a, k->grid_h.p,
                                  true),
             "adam");
    return VG_OK;
}

int stage_records(VgCache* k, DevBuf& b, const float* records, size_t n)
{
    int st;
    if ((st = alloc(b, n * vgn::REC_WORDS * 4, k->ctx->stream, false)) != VG_OK)
        return st;
    if (n > 0)
        VG_CHECK(cudaMemcpyAsync(b.p, records, n * vgn::REC_WORDS * 4, cudaMemcpyHostToDevice, k->ctx->stream),
                 "record upload");
    uint32_t n32 = (uint32_t)n;
    VG_CHECK(cudaMemcpyAsync(k->count.p, &n32, 4, cudaMemcpyHostToDevice, k->ctx->stream), "count");
    VG_CHECK(cudaStreamSynchronize(k->ctx->stream), "record upload");
    return VG_OK;
}

} // namespace vgc

using namespace vgc;

// The cache integrator's samples (called by vg_accumulate with the parameter block filled in), in
// frames: the query paths and training paths of a frame's samples, then the cache's answers for
// the queries (encode + inference, one launch pair per sample of the frame, in sample order), then
// the training steps on the frame's training records. With the streaming wavefront (`w`) a frame
// holds up to cache_frame samples (the cache is fixed within it); with the one-kernel query
// paths, one.
int cache_accumulate(VgRenderer* r, VgAccum* acc, vgd::Ctx& c, uint32_t samples, bool timed, const vgk::Wave* w)
{
    VgCache* k = r->cache;
    if (acc->lighting || acc->restir.on || acc->adaptive)
        return fail(VG_ERR_UNSUPPORTED,
                    "the radiance cache integrator runs without the lighting split, ReSTIR and adaptive sampling");
    cudaStream_t s = r->ctx->stream;
    size_t px = (size_t)acc->width * acc->height;
    uint32_t tcap = r->cache_steps * r->cache_batch;
    uint32_t frame = w ? std::max(1u, r->cache_frame) : 1u;
    int st;
    if (!acc->cache_q.p || acc->cache_q.bytes < frame * px * vgn::REC_WORDS * 4)
        if ((st = alloc(acc->cache_q, frame * px * vgn::REC_WORDS * 4, s, false)) != VG_OK)
            return st;
    if (!acc->cache_t.p || acc->cache_t.bytes < (size_t)std::max(tcap, 1u) * vgn::REC_WORDS * 4)
        if ((st = alloc(acc->cache_t, (size_t)std::max(tcap, 1u) * vgn::REC_WORDS * 4, s, false)) != VG_OK)
            return st;
    // Counters: [0] training records, [1 + j] queries of sample j of the frame.
    if (!acc->cache_ctr.p && (st = alloc(acc->cache_ctr, (1 + MAX_CACHE_FRAME) * 4, s, true)) != VG_OK)
        return st;
    if (w && !acc->cache_spread.p && (st = alloc(acc->cache_spread, px * 8, s, false)) != VG_OK)
        return st;
    if (!r->ctx->side) {
        VG_CHECK(cudaStreamCreateWithFlags(&r->ctx->side, cudaStreamNonBlocking), "side stream");
        VG_CHECK(cudaEventCreateWithFlags(&r->ctx->fork, cudaEventDisableTiming), "event");
        VG_CHECK(cudaEventCreateWithFlags(&r->ctx->join, cudaEventDisableTiming), "event");
    }
    VG_CHECK(cudaMemsetAsync(k->err.p, 0, 4, s), "error flag");
    uint32_t* ctr = (uint32_t*)acc->cache_ctr.p;
    NrcPathArgs a;
    a.spread = r->cache_spread;
    a.train_stride = (uint32_t)std::max<size_t>(1, r->cache_train_paths ? px / r->cache_train_paths : px + 1);
    a.qrec = (float*)acc->cache_q.p;
    a.qcount = ctr + 1;
    a.qcap = (uint32_t)px;
    a.trec = (float*)acc->cache_t.p;
    a.tcount = ctr;
    a.tcap = tcap;
    if ((st = ensure_work(k, std::max<size_t>(px, r->cache_batch))) != VG_OK)
        return st;
    vgk::CacheWave q;
    q.spread = a.spread;
    q.st = (float2*)acc->cache_spread.p;
    q.qrec = a.qrec;
    q.qcount = a.qcount;
    q.qcap = a.qcap;
    q.train_stride = a.train_stride;
    dim3 grid((acc->width + 15) / 16, (acc->height + 7) / 8);
    vgn::CacheDev d = k->dev();
    bool f64 = acc->precision == 64;
    vgx::Variant v = variant_of(r, acc);
    // Warm-up, before the first sample of an accumulation: training-only frames (one sample of
    // training paths into a scratch sum buffer, then the training steps) so that the image does
    // not average in the answers of an untrained cache. Their samples are numbered from
    // CACHE_WARMUP_SAMPLE, apart from the image's.
    if (acc->samples == 0 && r->cache_warmup > 0 && r->cache_steps > 0 && tcap > 0) {
        DevBuf scratch;
        if ((st = alloc(scratch, px * 3 * (acc->precision == 64 ? 8 : 4), s, false)) != VG_OK)
            return st;
        vgd::Ctx cw = c;
        cw.accum = scratch.p;
        for (uint32_t f = 0; f < r->cache_warmup; f++) {
            uint32_t sample = CACHE_WARMUP_SAMPLE + f;
            cw.p[P_SAMPLE] = sample;
            cw.p[P_SAMPLES_PER_DISPATCH] = 1; // one sample per training pixel: a quarter of the cost of a 4-sample frame
            a.train_offset = (sample * 2654435761u) % a.train_stride;
            VG_CHECK(cudaMemsetAsync(ctr, 0, 4, s), "counters");
            VG_CHECK(vgx::nrc_launch_train_paths(f64, s, cw, a), "cache training path launch");
            acc->launches++;
            for (uint32_t t = 0; t < r->cache_steps; t++) {
                if ((st = cache_train_step(k, a.trec, ctr, tcap, t * r->cache_batch, r->cache_batch)) != VG_OK)
                    return st;
                acc->launches += 7;
            }
        }
        VG_CHECK(cudaStreamSynchronize(s), "cache warm-up"); // the scratch buffer is freed next
    }
    EventPool pool;
    StageEvents stages;
    for (uint32_t i = 0; i < samples;) {
        uint32_t n = std::min(frame, samples - i);
        uint32_t sample = acc->samples + i;
        c.p[P_SAMPLE] = sample;
        c.p[P_SAMPLES_PER_DISPATCH] = n;
        a.train_offset = (sample * 2654435761u) % a.train_stride;
        q.train_offset = a.train_offset;
        cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr, e3 = nullptr;
        if (timed) {
            e0 = pool.get(), e1 = pool.get(), e2 = pool.get(), e3 = pool.get();
            VG_CHECK(cudaEventRecord(e0, s), "event");
        }
        VG_CHECK(cudaMemsetAsync(ctr, 0, (1 + n) * 4, s), "counters");
        // Training paths (full depth, few) on the side stream, overlapping the query paths and the
        // inference; joined before the training steps. They add to other pixels than the queries.
        uint32_t first;
        bool train = vgx::nrc_train_pixels(px, a.train_stride, a.train_offset, &first) > 0;
        if (train) {
            VG_CHECK(cudaEventRecord(r->ctx->fork, s), "fork");
            VG_CHECK(cudaStreamWaitEvent(r->ctx->side, r->ctx->fork, 0), "fork");
            VG_CHECK(vgx::nrc_launch_train_paths(f64, r->ctx->side, c, a), "cache training path launch");
            VG_CHECK(cudaEventRecord(r->ctx->join, r->ctx->side), "join");
            acc->launches++;
        }
        if (w) {
            if ((st = stream_samples(r, acc, c, v, *w, sample, n, false, pool, stages, &q)) != VG_OK)
                return st;
        } else {
            VG_CHECK(vgx::nrc_launch_query_paths(f64, grid, s, c, a), "cache path launch");
            acc->launches++;
        }
        if (timed)
            VG_CHECK(cudaEventRecord(e1, s), "event");
        for (uint32_t j = 0; j < n; j++) {
            const float* rj = a.qrec + (size_t)j * px * vgn::REC_WORDS;
            VG_CHECK(vgx::nrc_launch_encode(encode_blocks(k), s, d, rj, ctr + 1 + j, a.qcap, 0, a.qcap,
                                            (uint8_t*)k->X.p),
                     "cache encode launch");
            VG_CHECK(vgx::nrc_launch_infer(3 * r->ctx->sms, s, d, (const uint8_t*)k->X.p, rj, ctr + 1 + j, a.qcap,
                                           nullptr, c.accum, f64 ? 64 : 32),
                     "cache inference launch");
            acc->launches += 2;
        }
        if (timed)
            VG_CHECK(cudaEventRecord(e2, s), "event");
        if (train)
            VG_CHECK(cudaStreamWaitEvent(s, r->ctx->join, 0), "join");
        for (uint32_t t = 0; t < r->cache_steps; t++) {
            if ((st = cache_train_step(k, a.trec, ctr, tcap, t * r->cache_batch, r->cache_batch)) != VG_OK)
                return st;
            acc->launches += 7;
        }
        acc->cache_frame_last = n;
        if (timed) {
            VG_CHECK(cudaEventRecord(e3, s), "event");
            if ((st = wait_event(e3)) != VG_OK)
                return st;
            float ms[3] = {0, 0, 0};
            cudaEventElapsedTime(&ms[0], e0, e1);
            cudaEventElapsedTime(&ms[1], e1, e2);
            cudaEventElapsedTime(&ms[2], e2, e3);
            for (int m = 0; m < 3; m++)
                acc->cache_seconds[m] += ms[m] * 1e-3;
        }
        i += n;
    }
    return VG_OK;
}

int cache_status(VgRenderer* r)
{
    return r->cache ? cache_check(r->cache) : VG_OK;
}

extern "C" {

void vg_cache_default_config(VgCacheConfig* out)
{
    if (!out)
        return;
    memset(out, 0, sizeof(*out));
    out->levels = 16;
    out->log2_entries = 19;
    out->base_resolution = 16;
    out->max_resolution = 2048;
    out->learning_rate = 0.01f;
    out->beta1 = 0.9f;
    out->beta2 = 0.99f;
    out->epsilon = 1.0e-8f;
    out->seed = 0x5EED5EEDu;
}

int vg_renderer_bounds(const VgRenderer* r, float lo[3], float hi[3])
{
    if (!r || !lo || !hi)
        return fail(VG_ERR_INVALID, "null argument");
    for (int k = 0; k < 3; k++) {
        lo[k] = r->bounds_lo[k];
        hi[k] = r->bounds_hi[k];
    }
    return VG_OK;
}

int vg_cache_create(VgContext* ctx, const VgCacheConfig* cfg, VgCache** out)
{
    DevGuard device_guard(dev_of(ctx));
    if (!ctx || !cfg || !out)
        return fail(VG_ERR_INVALID, "null argument");
    *out = nullptr;
    const VgCacheConfig& c = *cfg;
    if (c.levels < 1 || c.levels > vgn::MAX_LEVELS || c.log2_entries < 8 || c.log2_entries > 24 ||
        c.base_resolution < 2 || c.max_resolution < c.base_resolution || c.max_resolution > 65536)
        return fail(VG_ERR_INVALID, "cache grid configuration out of range");
    if (!(c.learning_rate >= 0.0f) || !(c.beta1 >= 0.0f && c.beta1 < 1.0f) || !(c.beta2 >= 0.0f && c.beta2 < 1.0f) ||
        !(c.epsilon > 0.0f))
        return fail(VG_ERR_INVALID, "cache optimiser configuration out of range");
    for (int k = 0; k < 3; k++)
        if (!(c.bounds_hi[k] >= c.bounds_lo[k]) || !std::isfinite(c.bounds_lo[k]) || !std::isfinite(c.bounds_hi[k]))
            return fail(VG_ERR_INVALID, "cache bounds are not a box");
    if (!(std::max({c.bounds_hi[0] - c.bounds_lo[0], c.bounds_hi[1] - c.bounds_lo[1], c.bounds_hi[2] - c.bounds_lo[2]}) > 0.0f))
        return fail(VG_ERR_INVALID, "cache bounds are empty");
    vgx::nrc_prepare();
    VgCache* k = new VgCache();
    k->ctx = ctx;
    k->device = ctx->device;
    k->cfg = c;
    double growth = c.levels > 1 ? std::exp((std::log((double)c.max_resolution) - std::log((double)c.base_resolution)) /
                                            (double)(c.levels - 1))
                                 : 1.0;
    uint64_t entries = 1ull << c.log2_entries;
    for (uint32_t l = 0; l < c.levels; l++) {
        uint32_t res = (uint32_t)std::floor((double)c.base_resolution * std::pow(growth, (double)l) + 1e-9);
        k->res[l] = std::max(res, 2u);
        uint64_t side = (uint64_t)k->res[l] + 1;
        if (side * side * side <= entries)
            k->dense_mask |= 1u << l;
    }
    k->grid_params = (size_t)c.levels * entries * 2;
    cudaStream_t s = ctx->stream;
    int st;
    if ((st = alloc(k->grid, k->grid_params * 4, s, false)) != VG_OK ||
        (st = alloc(k->grid_h, k->grid_params * 2, s, false)) != VG_OK ||
        (st = alloc(k->grid_grad, k->grid_params * 4, s, true)) != VG_OK ||
        (st = alloc(k->grid_m, k->grid_params * 4, s, true)) != VG_OK ||
        (st = alloc(k->grid_v, k->grid_params * 4, s, true)) != VG_OK ||
        (st = alloc(k->mlp, vgn::MLP_PARAMS * 4, s, false)) != VG_OK ||
        (st = alloc(k->mlp_grad, vgn::MLP_PARAMS * 4, s, true)) != VG_OK ||
        (st = alloc(k->mlp_m, vgn::MLP_PARAMS * 4, s, true)) != VG_OK ||
        (st = alloc(k->mlp_v, vgn::MLP_PARAMS * 4, s, true)) != VG_OK ||
        (st = alloc(k->img, vgn::IMG_BYTES, s, true)) != VG_OK || (st = alloc(k->loss, 8, s, true)) != VG_OK ||
        (st = alloc(k->err, 4, s, true)) != VG_OK || (st = alloc(k->count, 4, s, true)) != VG_OK ||
        (st = alloc(k->step, 4, s, true)) != VG_OK) {
        delete k;
        return st;
    }
    // Glorot-uniform MLP weights (rows 3-15 of the output layer stay zero), grid features
    // uniform in [-1e-4, 1e-4].
    std::vector<float> w(vgn::MLP_PARAMS, 0.0f);
    for (uint32_t l = 0; l < 5; l++) {
        uint32_t rows = l < 4 ? vgn::WIDTH : 3;
        float lim = (float)std::sqrt(6.0 / (double)(vgn::WIDTH + rows));
        for (uint32_t o = 0; o < rows; o++)
            for (uint32_t i = 0; i < vgn::WIDTH; i++) {
                uint32_t idx = vgn::mlp_offset(l) + o * vgn::WIDTH + i;
                w[idx] = lim * uniform_pm1(c.seed, idx);
            }
    }
    std::vector<float> g(k->grid_params);
    for (size_t i = 0; i < g.size(); i++)
        g[i] = 1.0e-4f * uniform_pm1(c.seed ^ 0xA5A5A5A5u, i);
    if ((st = vg_cache_write_params(k, w.data(), g.data())) != VG_OK) {
        delete k;
        return st;
    }
    *out = k;
    return VG_OK;
}

int vg_cache_destroy(VgCache* cache)
{
    DevGuard device_guard(dev_of(cache));
    delete cache;
    return VG_OK;
}

int vg_cache_param_counts(const VgCache* k, size_t* mlp, size_t* grid)
{
    if (!k)
        return fail(VG_ERR_INVALID, "null cache");
    if (mlp)
        *mlp = vgn::MLP_PARAMS;
    if (grid)
        *grid = k->grid_params;
    return VG_OK;
}

int vg_cache_read_params(VgCache* k, float* mlp, float* grid)
{
    DevGuard device_guard(dev_of(k));
    if (!k)
        return fail(VG_ERR_INVALID, "null cache");
    cudaStream_t s = k->ctx->stream;
    if (mlp)
        VG_CHECK(cudaMemcpyAsync(mlp, k->mlp.p, vgn::MLP_PARAMS * 4, cudaMemcpyDeviceToHost, s), "readback");
    if (grid)
        VG_CHECK(cudaMemcpyAsync(grid, k->grid.p, k->grid_params * 4, cudaMemcpyDeviceToHost, s), "readback");
    VG_CHECK(cudaStreamSynchronize(s), "readback");
    return VG_OK;
}

int vg_cache_write_params(VgCache* k, const float* mlp, const float* grid)
{
    DevGuard device_guard(dev_of(k));
    if (!k)
        return fail(VG_ERR_INVALID, "null cache");
    cudaStream_t s = k->ctx->stream;
    if (mlp)
        VG_CHECK(cudaMemcpyAsync(k->mlp.p, mlp, vgn::MLP_PARAMS * 4, cudaMemcpyHostToDevice, s), "upload");
    if (grid)
        VG_CHECK(cudaMemcpyAsync(k->grid.p, grid, k->grid_params * 4, cudaMemcpyHostToDevice, s), "upload");
    int st;
    if ((st = cache_reset_optimiser(k)) != VG_OK || (st = cache_refresh(k)) != VG_OK)
        return st;
    VG_CHECK(cudaStreamSynchronize(s), "upload");
    return VG_OK;
}

int vg_cache_infer(VgCache* k, const float* records, size_t n, float* out)
{
    DevGuard device_guard(dev_of(k));
    if (!k || (n > 0 && (!records || !out)))
        return fail(VG_ERR_INVALID, "null argument");
    if (n > 0x7fffffffull)
        return fail(VG_ERR_INVALID, "too many records");
    if (n == 0)
        return VG_OK;
    DevBuf rec, o;
    int st;
    if ((st = stage_records(k, rec, records, n)) != VG_OK || (st = alloc(o, n * 12, k->ctx->stream, false)) != VG_OK ||
        (st = ensure_work(k, n)) != VG_OK)
        return st;
    cudaStream_t s = k->ctx->stream;
    vgn::CacheDev d = k->dev();
    const uint32_t* cnt = (const uint32_t*)k->count.p;
    VG_CHECK(cudaMemsetAsync(k->err.p, 0, 4, s), "error flag");
    VG_CHECK(vgx::nrc_launch_encode(encode_blocks(k), s, d, (const float*)rec.p, cnt, (uint32_t)n, 0, (uint32_t)n,
                                    (uint8_t*)k->X.p),
             "encode launch");
    VG_CHECK(vgx::nrc_launch_infer(3 * k->ctx->sms, s, d, (const uint8_t*)k->X.p, (const float*)rec.p, cnt,
                                   (uint32_t)n, (float*)o.p, nullptr, 32),
             "inference launch");
    VG_CHECK(cudaMemcpyAsync(out, o.p, n * 12, cudaMemcpyDeviceToHost, s), "readback");
    return cache_check(k);
}

int vg_cache_gradients(VgCache* k, const float* records, size_t n, float* mlp_grad, float* grid_grad, double* loss)
{
    DevGuard device_guard(dev_of(k));
    if (!k || (n > 0 && !records))
        return fail(VG_ERR_INVALID, "null argument");
    if (n > 0x7fffffffull)
        return fail(VG_ERR_INVALID, "too many records");
    DevBuf rec;
    int st;
    if ((st = stage_records(k, rec, records, n)) != VG_OK || (st = ensure_work(k, n)) != VG_OK)
        return st;
    cudaStream_t s = k->ctx->stream;
    VG_CHECK(cudaMemsetAsync(k->err.p, 0, 4, s), "error flag");
    VG_CHECK(cudaMemsetAsync(k->mlp_grad.p, 0, k->mlp_grad.bytes, s), "clear");
    VG_CHECK(cudaMemsetAsync(k->grid_grad.p, 0, k->grid_grad.bytes, s), "clear");
    VG_CHECK(cudaMemsetAsync(k->loss.p, 0, 8, s), "clear");
    if (n > 0 && (st = cache_gradient_pass(k, (const float*)rec.p, (const uint32_t*)k->count.p, (uint32_t)n, 0,
                                           (uint32_t)n)) != VG_OK)
        return st;
    if (mlp_grad)
        VG_CHECK(cudaMemcpyAsync(mlp_grad, k->mlp_grad.p, vgn::MLP_PARAMS * 4, cudaMemcpyDeviceToHost, s), "readback");
    if (grid_grad)
        VG_CHECK(cudaMemcpyAsync(grid_grad, k->grid_grad.p, k->grid_params * 4, cudaMemcpyDeviceToHost, s), "readback");
    double l = 0.0;
    VG_CHECK(cudaMemcpyAsync(&l, k->loss.p, 8, cudaMemcpyDeviceToHost, s), "readback");
    if ((st = cache_check(k)) != VG_OK)
        return st;
    VG_CHECK(cudaMemsetAsync(k->mlp_grad.p, 0, k->mlp_grad.bytes, s), "clear");
    VG_CHECK(cudaMemsetAsync(k->grid_grad.p, 0, k->grid_grad.bytes, s), "clear");
    VG_CHECK(cudaStreamSynchronize(s), "clear");
    if (loss)
        *loss = l;
    return VG_OK;
}

int vg_cache_train(VgCache* k, const float* records, size_t n, uint32_t batch, double* last_loss)
{
    DevGuard device_guard(dev_of(k));
    if (!k || (n > 0 && !records))
        return fail(VG_ERR_INVALID, "null argument");
    if (batch == 0 || n > 0x7fffffffull)
        return fail(VG_ERR_INVALID, "batch must be non-zero");
    DevBuf rec;
    int st;
    if ((st = stage_records(k, rec, records, n)) != VG_OK || (st = ensure_work(k, std::min<size_t>(n, batch))) != VG_OK)
        return st;
    cudaStream_t s = k->ctx->stream;
    VG_CHECK(cudaMemsetAsync(k->err.p, 0, 4, s), "error flag");
    uint32_t used = 0;
    for (size_t off = 0; off < n; off += batch) {
        if ((st = cache_train_step(k, (const float*)rec.p, (const uint32_t*)k->count.p, (uint32_t)n, (uint32_t)off,
                                   batch)) != VG_OK)
            return st;
        used = (uint32_t)std::min<size_t>(batch, n - off);
    }
    double l = 0.0;
    VG_CHECK(cudaMemcpyAsync(&l, k->loss.p, 8, cudaMemcpyDeviceToHost, s), "readback");
    if ((st = cache_check(k)) != VG_OK)
        return st;
    if (last_loss)
        *last_loss = used ? l / (3.0 * used) : 0.0;
    return VG_OK;
}

int vg_cache_time(VgCache* k, const float* records, size_t n, uint32_t reps, double out[4])
{
    DevGuard device_guard(dev_of(k));
    if (!k || !records || !out || n == 0 || reps == 0)
        return fail(VG_ERR_INVALID, "null argument or empty input");
    if (n > 0x7fffffffull)
        return fail(VG_ERR_INVALID, "too many records");
    DevBuf rec, o;
    int st;
    if ((st = stage_records(k, rec, records, n)) != VG_OK || (st = ensure_work(k, n)) != VG_OK ||
        (st = alloc(o, n * 12, k->ctx->stream, false)) != VG_OK)
        return st;
    cudaStream_t s = k->ctx->stream;
    vgn::CacheDev d = k->dev();
    const uint32_t* cnt = (const uint32_t*)k->count.p;
    const float* rp = (const float*)rec.p;
    uint32_t n32 = (uint32_t)n;
    VG_CHECK(cudaMemsetAsync(k->err.p, 0, 4, s), "error flag");
    EventPool pool;
    cudaEvent_t ev[5];
    for (int i = 0; i < 5; i++)
        ev[i] = pool.get();
    // One untimed round, then `reps` launches of each kernel back to back.
    for (uint32_t round = 0; round < 2; round++) {
        uint32_t m = round == 0 ? 1 : reps;
        if (round == 1)
            VG_CHECK(cudaEventRecord(ev[0], s), "event");
        for (uint32_t i = 0; i < m; i++)
            VG_CHECK(vgx::nrc_launch_encode(encode_blocks(k), s, d, rp, cnt, n32, 0, n32, (uint8_t*)k->X.p), "encode");
        if (round == 1)
            VG_CHECK(cudaEventRecord(ev[1], s), "event");
        for (uint32_t i = 0; i < m; i++)
            VG_CHECK(vgx::nrc_launch_infer(3 * k->ctx->sms, s, d, (const uint8_t*)k->X.p, rp, cnt, n32, (float*)o.p,
                                           nullptr, 32),
                     "infer");
        if (round == 1)
            VG_CHECK(cudaEventRecord(ev[2], s), "event");
        for (uint32_t i = 0; i < m; i++)
            VG_CHECK(vgx::nrc_launch_train(k->ctx->sms, s, d, (const uint8_t*)k->X.p, rp, cnt, n32, 0, n32,
                                           (float*)k->GX.p),
                     "train");
        if (round == 1)
            VG_CHECK(cudaEventRecord(ev[3], s), "event");
        for (uint32_t i = 0; i < m; i++)
            VG_CHECK(vgx::nrc_launch_scatter(encode_blocks(k), s, d, rp, cnt, n32, 0, n32, (const float*)k->GX.p),
                     "scatter");
        if (round == 1)
            VG_CHECK(cudaEventRecord(ev[4], s), "event");
    }
    if ((st = wait_event(ev[4])) != VG_OK)
        return st;
    for (int i = 0; i < 4; i++) {
        float ms = 0.0f;
        VG_CHECK(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]), "event");
        out[i] = ms * 1e-3 / reps;
    }
    if ((st = cache_check(k)) != VG_OK)
        return st;
    VG_CHECK(cudaMemsetAsync(k->mlp_grad.p, 0, k->mlp_grad.bytes, s), "clear");
    VG_CHECK(cudaMemsetAsync(k->grid_grad.p, 0, k->grid_grad.bytes, s), "clear");
    VG_CHECK(cudaStreamSynchronize(s), "clear");
    return VG_OK;
}

int vg_set_cache(VgRenderer* r, VgCache* cache, float spread, uint32_t train_paths, uint32_t train_steps,
                 uint32_t train_batch)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    if (cache && cache->ctx != r->ctx)
        return fail(VG_ERR_INVALID, "cache and renderer belong to different contexts");
    if (cache && (!(spread > 0.0f) || (train_steps > 0 && train_batch == 0) ||
                  (uint64_t)train_steps * train_batch > (1ull << 26)))
        return fail(VG_ERR_INVALID, "cache integrator settings out of range");
    r->cache = cache;
    r->cache_spread = spread;
    r->cache_train_paths = train_paths;
    r->cache_steps = train_steps;
    r->cache_batch = train_batch;
    return VG_OK;
}

int vg_set_cache_warmup(VgRenderer* r, uint32_t frames)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    if (frames > 4096)
        return fail(VG_ERR_INVALID, "cache warm-up out of range (0-4096 frames)");
    r->cache_warmup = frames;
    return VG_OK;
}

int vg_set_cache_frame(VgRenderer* r, uint32_t samples_per_frame)
{
    if (!r)
        return fail(VG_ERR_INVALID, "null renderer");
    if (samples_per_frame < 1 || samples_per_frame > MAX_CACHE_FRAME)
        return fail(VG_ERR_INVALID, "cache frame out of range (1-" + std::to_string(MAX_CACHE_FRAME) + " samples)");
    r->cache_frame = samples_per_frame;
    return VG_OK;
}

int vg_accum_cache_stats(const VgAccum* acc, VgCacheStats* out)
{
    if (!acc || !out)
        return fail(VG_ERR_INVALID, "null argument");
    memset(out, 0, sizeof(*out));
    out->path_seconds = acc->cache_seconds[0];
    out->infer_seconds = acc->cache_seconds[1];
    out->train_seconds = acc->cache_seconds[2];
    if (!acc->cache_ctr.p)
        return VG_OK;
    cudaStream_t s = acc->owner->ctx->stream;
    uint32_t ctr[1 + MAX_CACHE_FRAME] = {};
    uint32_t n = std::min<uint32_t>(acc->cache_frame_last, MAX_CACHE_FRAME);
    VG_CHECK(cudaMemcpyAsync(ctr, acc->cache_ctr.p, (1 + n) * 4, cudaMemcpyDeviceToHost, s), "readback");
    double l = 0.0;
    if (acc->owner->cache)
        VG_CHECK(cudaMemcpyAsync(&l, acc->owner->cache->loss.p, 8, cudaMemcpyDeviceToHost, s), "readback");
    VG_CHECK(cudaStreamSynchronize(s), "readback");
    for (uint32_t j = 0; j < n; j++)
        out->queries += ctr[1 + j];
    out->train_records = ctr[0];
    uint32_t tcap = acc->owner->cache_steps * acc->owner->cache_batch;
    uint32_t avail = std::min(ctr[0], tcap);
    uint32_t steps = acc->owner->cache_steps;
    if (steps > 0 && acc->owner->cache_batch > 0 && avail > 0) {
        uint32_t last_off = (steps - 1) * acc->owner->cache_batch;
        uint32_t used = avail > last_off ? std::min(acc->owner->cache_batch, avail - last_off) : 0;
        out->loss = used ? l / (3.0 * used) : 0.0;
    }
    return VG_OK;
}

} // extern "C"
