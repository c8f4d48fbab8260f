// Batched rendering (include/vgcuda.h, "Batched rendering"): the request table, the persistent
// batch launch (kern_batch.cu) and the caches' training steps, captured once in a CUDA graph and
// replayed while the batch keeps its shape; and the batch autotuner. No reference counterpart.
#include <numeric>

#include "cache_host.h"
#include "launch_batch.h"

struct BatchState {
    DevBuf reqs, done, next, err, t0;
    std::vector<vgb::BatchReq> host;
    std::vector<uint64_t> signature; // what the captured graph was made for
    cudaGraphExec_t graph = nullptr;
    ~BatchState()
    {
        if (graph)
            cudaGraphExecDestroy(graph);
    }
};

VgContext::~VgContext() { delete batch; }

namespace {

bool batch_compatible(const VgRenderer* r, const VgAccum* a)
{
    return !a->lighting && !r->restir.on && !r->adaptive && !(a->samples > 0 && (a->adaptive || a->restir.on));
}

// Appends the batch's launches to the stream (captured into the graph).
int batch_sequence(VgContext* ctx, BatchState* b, uint32_t nreq, uint32_t items, int blocks,
                   const std::vector<std::pair<VgCache*, VgRenderer*>>& caches)
{
    cudaStream_t s = ctx->stream;
    VG_CHECK(cudaMemsetAsync(b->next.p, 0, 4, s), "batch counter");
    VG_CHECK(vgx::launch_batch(blocks, s, (const vgb::BatchReq*)b->reqs.p, nreq, items, (uint32_t*)b->next.p,
                               (vgb::BatchDone*)b->done.p, (uint32_t*)b->err.p, (unsigned long long*)b->t0.p),
             "batch launch");
    for (auto& kc : caches) {
        VgCache* k = kc.first;
        VgRenderer* r = kc.second;
        uint32_t tcap = r->cache_steps * r->cache_batch;
        for (uint32_t t = 0; t < r->cache_steps; t++) {
            int st = vgc::cache_train_step(k, (const float*)k->batch_rec.p, (const uint32_t*)k->batch_count.p, tcap,
                                           t * r->cache_batch, r->cache_batch);
            if (st != VG_OK)
                return st;
        }
    }
    return VG_OK;
}

std::vector<size_t> order_of(const VgBatchRequest* reqs, size_t n, int order)
{
    std::vector<size_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    auto cost = [&](size_t i) {
        return (double)reqs[i].accum->width * reqs[i].accum->height * reqs[i].samples;
    };
    if (order == VG_BATCH_SHORTEST_FIRST)
        std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return cost(a) < cost(b); });
    else if (order == VG_BATCH_LONGEST_FIRST)
        std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return cost(a) > cost(b); });
    return idx;
}

int batch_kernel_run(VgContext* ctx, const VgBatchRequest* reqs, size_t n, int blocks_per_sm, int order,
                     VgBatchResult* out, double* total_seconds, int* replayed)
{
    if (!ctx || !reqs || n == 0 || n > 65536)
        return fail(VG_ERR_INVALID, "empty or oversized batch");
    for (size_t i = 0; i < n; i++) {
        const VgBatchRequest& q = reqs[i];
        if (!q.renderer || !q.accum || q.renderer->ctx != ctx || q.accum->owner != q.renderer || q.samples == 0)
            return fail(VG_ERR_INVALID, "batch request " + std::to_string(i) + " is malformed");
        if (!batch_compatible(q.renderer, q.accum))
            return fail(VG_ERR_UNSUPPORTED, "batch request " + std::to_string(i) +
                                                " uses adaptive sampling, ReSTIR or the lighting split");
        if (q.cache && q.cache->ctx != ctx)
            return fail(VG_ERR_INVALID, "batch request " + std::to_string(i) + " has a cache of another context");
    }
    if (!ctx->batch)
        ctx->batch = new BatchState();
    BatchState* b = ctx->batch;
    cudaStream_t s = ctx->stream;
    std::vector<size_t> idx = order_of(reqs, n, order);
    // Training buffers of the caches in the batch (first renderer using a cache sets its steps).
    std::vector<std::pair<VgCache*, VgRenderer*>> caches;
    int st;
    for (size_t i : idx) {
        VgCache* k = reqs[i].cache;
        if (!k)
            continue;
        bool seen = false;
        for (auto& kc : caches)
            seen |= kc.first == k;
        if (seen)
            continue;
        VgRenderer* r = reqs[i].renderer;
        size_t tcap = std::max<size_t>((size_t)r->cache_steps * r->cache_batch, 1);
        if (k->batch_rec.bytes < tcap * vgn::REC_WORDS * 4 &&
            (st = alloc(k->batch_rec, tcap * vgn::REC_WORDS * 4, s, false)) != VG_OK)
            return st;
        if (!k->batch_count.p && (st = alloc(k->batch_count, 16, s, true)) != VG_OK)
            return st;
        if ((st = vgc::ensure_work(k, std::max<size_t>(r->cache_batch, 1))) != VG_OK)
            return st;
        caches.push_back({k, r});
    }
    // The request table, in work order.
    b->host.resize(n);
    std::vector<uint64_t> sig;
    std::vector<vgb::BatchDone> done(n);
    uint32_t items = 0;
    for (size_t j = 0; j < n; j++) {
        const VgBatchRequest& q = reqs[idx[j]];
        VgRenderer* r = q.renderer;
        VgAccum* a = q.accum;
        if (a->samples == 0) {
            a->adaptive_fixed = true;
            a->adaptive = r->adaptive;
            a->restir = r->restir;
        }
        vgb::BatchReq& R = b->host[j];
        memset(&R, 0, sizeof(R));
        R.c = make_ctx(r, a);
        R.c.p[P_SAMPLE] = a->samples;
        R.c.p[P_SAMPLES_PER_DISPATCH] = q.samples;
        R.f64 = a->precision == 64;
        size_t px = (size_t)a->width * a->height;
        if (q.cache) {
            R.cached = 1;
            R.cd = q.cache->dev();
            R.spread = r->cache_spread;
            R.train_stride = (uint32_t)std::max<size_t>(1, r->cache_train_paths ? px / r->cache_train_paths : px + 1);
            R.trec = (float*)q.cache->batch_rec.p;
            R.tcount = (uint32_t*)q.cache->batch_count.p;
            for (auto& kc : caches)
                if (kc.first == q.cache)
                    R.tcap = kc.second->cache_steps * kc.second->cache_batch;
        }
        R.tiles_x = (a->width + 15) / 16;
        R.tiles = R.tiles_x * ((a->height + 7) / 8);
        R.item_begin = items;
        R.index = (uint32_t)idx[j];
        items += R.tiles;
        done[j].remaining = R.tiles;
        done[j].done_ns = 0;
        sig.insert(sig.end(), {(uint64_t)(uintptr_t)r, (uint64_t)(uintptr_t)a, q.samples, (uint64_t)(uintptr_t)q.cache,
                               q.cache ? ((uint64_t)r->cache_steps << 32 | r->cache_batch) : 0});
    }
    // A persistent kernel over a work counter: CTAs beyond what fits start when others leave, so a
    // larger request is safe.
    int bps = blocks_per_sm > 0 ? std::min(blocks_per_sm, 8) : vgx::batch_blocks_per_sm();
    sig.insert(sig.end(), {(uint64_t)bps, (uint64_t)order});
    if (b->reqs.bytes < n * sizeof(vgb::BatchReq) || b->done.bytes < n * sizeof(vgb::BatchDone)) {
        if ((st = alloc(b->reqs, n * sizeof(vgb::BatchReq), s, false)) != VG_OK ||
            (st = alloc(b->done, n * sizeof(vgb::BatchDone), s, false)) != VG_OK)
            return st;
        b->signature.clear(); // the graph points at the old buffers
    }
    if ((!b->next.p && (st = alloc(b->next, 16, s, true)) != VG_OK) ||
        (!b->err.p && (st = alloc(b->err, 16, s, true)) != VG_OK) ||
        (!b->t0.p && (st = alloc(b->t0, 16, s, true)) != VG_OK))
        return st;
    VG_CHECK(cudaMemcpyAsync(b->reqs.p, b->host.data(), n * sizeof(vgb::BatchReq), cudaMemcpyHostToDevice, s),
             "batch table");
    VG_CHECK(cudaMemcpyAsync(b->done.p, done.data(), n * sizeof(vgb::BatchDone), cudaMemcpyHostToDevice, s),
             "batch table");
    VG_CHECK(cudaMemsetAsync(b->err.p, 0, 4, s), "batch error flag");
    for (auto& kc : caches) {
        VG_CHECK(cudaMemsetAsync(kc.first->batch_count.p, 0, 4, s), "training count");
        VG_CHECK(cudaMemsetAsync(kc.first->err.p, 0, 4, s), "cache error flag");
    }
    for (size_t j = 0; j < n; j++)
        VG_CHECK(cudaMemsetAsync(b->host[j].c.err, 0, 4, s), "error flag");
    EventPool pool;
    cudaEvent_t e0 = pool.get(), e1 = pool.get();
    VG_CHECK(cudaEventRecord(e0, s), "event");
    bool reuse = b->graph && sig == b->signature;
    if (!reuse) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        b->signature.clear();
        VG_CHECK(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed), "graph capture");
        st = batch_sequence(ctx, b, (uint32_t)n, items, bps * ctx->sms, caches);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(s, &g);
        if (st != VG_OK) {
            if (g)
                cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess)
            return cuda_fail(e, "graph capture");
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->graph = nullptr;
            return cuda_fail(e, "graph instantiation");
        }
        b->signature = sig;
    }
    VG_CHECK(cudaGraphLaunch(b->graph, s), "graph launch");
    VG_CHECK(cudaEventRecord(e1, s), "event");
    if ((st = wait_event(e1)) != VG_OK)
        return st;
    uint32_t err = 0;
    unsigned long long t0 = 0;
    VG_CHECK(cudaMemcpy(&err, b->err.p, 4, cudaMemcpyDeviceToHost), "batch error flag");
    VG_CHECK(cudaMemcpy(&t0, b->t0.p, 8, cudaMemcpyDeviceToHost), "batch clock");
    VG_CHECK(cudaMemcpy(done.data(), b->done.p, n * sizeof(vgb::BatchDone), cudaMemcpyDeviceToHost), "batch times");
    if (err)
        return fail(VG_ERR_KERNEL, "a tensor-core completion wait timed out in the batch");
    for (size_t j = 0; j < n; j++) {
        if ((st = read_err(reqs[idx[j]].renderer)) != VG_OK)
            return st;
        if (done[j].remaining != 0)
            return fail(VG_ERR_KERNEL, "a batch request did not finish");
    }
    for (auto& kc : caches)
        if ((st = vgc::cache_check(kc.first)) != VG_OK)
            return st;
    float ms = 0.0f;
    VG_CHECK(cudaEventElapsedTime(&ms, e0, e1), "event");
    for (size_t j = 0; j < n; j++) {
        const VgBatchRequest& q = reqs[idx[j]];
        q.accum->samples += q.samples;
        q.accum->launches += 1;
        if (out)
            out[idx[j]].seconds = (double)(done[j].done_ns - t0) * 1e-9;
    }
    if (total_seconds)
        *total_seconds = ms * 1e-3;
    if (replayed)
        *replayed = reuse ? 1 : 0;
    return VG_OK;
}

// The hybrid schedule: requests below `big` pixels share the persistent launch; the rest follow
// one at a time on the streaming wavefront (or the cache integrator), shortest first.
int batch_run(VgContext* ctx, const VgBatchRequest* reqs, size_t n, int blocks_per_sm, int order, uint64_t big,
              VgBatchResult* out, double* total_seconds, int* replayed)
{
    if (!ctx || !reqs || n == 0 || n > 65536)
        return fail(VG_ERR_INVALID, "empty or oversized batch");
    std::vector<size_t> small, large;
    for (size_t i = 0; i < n; i++) {
        if (!reqs[i].renderer || !reqs[i].accum)
            return fail(VG_ERR_INVALID, "batch request " + std::to_string(i) + " is malformed");
        uint64_t px = (uint64_t)reqs[i].accum->width * reqs[i].accum->height;
        (px >= big ? large : small).push_back(i);
    }
    for (size_t i : large) {
        const VgBatchRequest& q = reqs[i];
        if (q.renderer->ctx != ctx || q.accum->owner != q.renderer || q.samples == 0)
            return fail(VG_ERR_INVALID, "batch request " + std::to_string(i) + " is malformed");
        if (!batch_compatible(q.renderer, q.accum))
            return fail(VG_ERR_UNSUPPORTED, "batch request " + std::to_string(i) +
                                                " uses adaptive sampling, ReSTIR or the lighting split");
        if (q.cache && q.cache->ctx != ctx)
            return fail(VG_ERR_INVALID, "batch request " + std::to_string(i) + " has a cache of another context");
    }
    double t = 0.0;
    int st, rep = 0;
    if (!small.empty()) {
        std::vector<VgBatchRequest> sr;
        for (size_t i : small)
            sr.push_back(reqs[i]);
        std::vector<VgBatchResult> so(sr.size());
        if ((st = batch_kernel_run(ctx, sr.data(), sr.size(), blocks_per_sm, order, so.data(), &t, &rep)) != VG_OK)
            return st;
        for (size_t j = 0; j < small.size(); j++)
            if (out)
                out[small[j]].seconds = so[j].seconds;
    }
    auto cost = [&](size_t i) { return (double)reqs[i].accum->width * reqs[i].accum->height * reqs[i].samples; };
    std::stable_sort(large.begin(), large.end(), [&](size_t a, size_t b) { return cost(a) < cost(b); });
    for (size_t i : large) {
        const VgBatchRequest& q = reqs[i];
        VgRenderer* r = q.renderer;
        int integ = r->integrator;
        VgCache* cache = r->cache;
        r->integrator = VG_WAVEFRONT;
        r->cache = q.cache;
        double g0 = q.accum->gpu_seconds;
        st = vg_accumulate(r, q.accum, q.samples);
        r->integrator = integ;
        r->cache = cache;
        if (st != VG_OK)
            return st;
        t += q.accum->gpu_seconds - g0;
        if (out)
            out[i].seconds = t;
    }
    if (total_seconds)
        *total_seconds = t;
    if (replayed)
        *replayed = rep;
    return VG_OK;
}

} // namespace

extern "C" {

int vg_batch_render(VgContext* ctx, const VgBatchRequest* requests, size_t n, VgBatchResult* out,
                    double* total_seconds, int* graph_replayed)
{
    DevGuard device_guard(dev_of(ctx));
    if (!ctx)
        return fail(VG_ERR_INVALID, "null context");
    return batch_run(ctx, requests, n, ctx->batch_blocks_per_sm, ctx->batch_order, ctx->batch_wavefront_pixels, out,
                     total_seconds, graph_replayed);
}

int vg_batch_kernel_info(VgContext* ctx, int out[5])
{
    DevGuard device_guard(dev_of(ctx));
    if (!ctx || !out)
        return fail(VG_ERR_INVALID, "null argument");
    out[0] = vgx::batch_kernel_info(&out[1], &out[2], &out[3], &out[4]);
    return VG_OK;
}

int vg_set_batch_options(VgContext* ctx, int blocks_per_sm, int order, uint64_t wavefront_pixels)
{
    if (!ctx || blocks_per_sm < 0 || order < VG_BATCH_SHORTEST_FIRST || order > VG_BATCH_LONGEST_FIRST)
        return fail(VG_ERR_INVALID, "batch options out of range");
    ctx->batch_blocks_per_sm = blocks_per_sm;
    ctx->batch_order = order;
    ctx->batch_wavefront_pixels = wavefront_pixels;
    return VG_OK;
}

int vg_batch_tune(VgContext* ctx, const VgBatchRequest* requests, size_t n, VgBatchTune* out)
{
    DevGuard device_guard(dev_of(ctx));
    if (!ctx || !requests || n == 0 || !out)
        return fail(VG_ERR_INVALID, "null argument");
    // Scratch accumulations of the requests' sizes and precision, so theirs stay untouched.
    std::vector<VgAccum*> scratch(n, nullptr);
    std::vector<VgBatchRequest> trial(requests, requests + n);
    int st = VG_OK;
    for (size_t i = 0; i < n && st == VG_OK; i++) {
        if (!requests[i].renderer || !requests[i].accum) {
            st = fail(VG_ERR_INVALID, "batch request is malformed");
            break;
        }
        VgAccum* a = requests[i].accum;
        if ((st = vg_accum_create(requests[i].renderer, a->width, a->height, 0, &scratch[i])) != VG_OK)
            break;
        scratch[i]->precision = a->precision;
        size_t px = (size_t)a->width * a->height * 3 * (a->precision == 64 ? 8 : 4);
        if ((st = alloc(scratch[i]->accum, px, ctx->stream, true)) != VG_OK)
            break;
        trial[i].accum = scratch[i];
    }
    int best_b = 0, best_o = 0;
    uint64_t best_px = ctx->batch_wavefront_pixels;
    double best = 1e300;
    const uint64_t thresholds[] = {256ull * 256, 512ull * 512, 1024ull * 1024, ~0ull};
    VgBatchTune res{};
    uint32_t trials = 0;
    std::vector<VgBatchResult> times(n);
    int max_b = vgx::batch_blocks_per_sm();
    // As given is the caller's order: left out. CTA counts: the two largest that fit.
    for (uint64_t big : thresholds)
    for (int o : {(int)VG_BATCH_SHORTEST_FIRST, (int)VG_BATCH_LONGEST_FIRST}) {
        for (int bps = std::max(1, max_b - 1); bps <= max_b && st == VG_OK; bps++) {
            double total = 0.0;
            // One run to capture the graph, one timed replay.
            for (int rep = 0; rep < 2 && st == VG_OK; rep++)
                st = batch_run(ctx, trial.data(), n, bps, o, big, times.data(), &total, nullptr);
            if (st != VG_OK)
                break;
            trials++;
            std::vector<double> lat(n);
            for (size_t i = 0; i < n; i++)
                lat[i] = times[i].seconds;
            std::sort(lat.begin(), lat.end());
            double p50 = lat[(n - 1) / 2], p99 = lat[std::min(n - 1, (size_t)std::ceil(0.99 * (double)n) - 1)];
            double objective = p50 + p99;
            if (objective < best) {
                best = objective;
                best_b = bps;
                best_o = o;
                best_px = big;
                res.p50_seconds = p50;
                res.p99_seconds = p99;
                res.total_seconds = total;
            }
        }
    }
    for (VgAccum* a : scratch)
        if (a)
            vg_accum_destroy(a);
    if (st != VG_OK)
        return st;
    ctx->batch_blocks_per_sm = best_b;
    ctx->batch_order = best_o;
    ctx->batch_wavefront_pixels = best_px;
    res.blocks_per_sm = best_b;
    res.order = best_o;
    res.wavefront_pixels = best_px;
    res.trials = trials;
    *out = res;
    return VG_OK;
}

} // extern "C"
