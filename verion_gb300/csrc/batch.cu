// Batched rendering (include/vgcuda.h, "Batched rendering"): the request table, the persistent
// batch launch (kern_batch.cu) and the caches' training steps, captured once in a CUDA graph and
// replayed while the batch keeps its shape; and the batch autotuner. No reference counterpart.
#include <functional>
#include <numeric>

#include "cache_host.h"
#include "launch_batch.h"

// The batch wavefront's graphs. Device loop: one graph of the prologue (counters, start kernel), a
// WHILE node whose body is two waves and the condition kernel, and the epilogue (the tail kernel
// for batches without caches, the caches' training steps). Host loop (for tools that cannot look
// into conditional graphs, such as profilers): the prologue, the two-wave body and the epilogue as
// three graphs, the host reading the live count after each body.
struct WaveGraphs {
    cudaGraphExec_t one = nullptr, pro = nullptr, body = nullptr, epi = nullptr;
    void release()
    {
        for (cudaGraphExec_t* g : {&one, &pro, &body, &epi})
            if (*g) {
                cudaGraphExecDestroy(*g);
                *g = nullptr;
            }
    }
};

// The batch wavefront's buffers: the wave planes of `slots` path slots, the request table and the
// completion state, and its captured graph.
struct WaveBufs {
    DevBuf state, hits, q0, q1, counts, fetch, sreq, meta, squeue, scount, slot_req, slot_pix;
    DevBuf reqs, done, next, err, loop, t0;
    DevBuf spread, tvert, tnv, caches, qrec, qcount; // cached requests
    uint32_t slots = 0, cache_slots = 0;
    size_t nreq = 0, ncache = 0;
    std::vector<vgb::WaveReq> host;
    std::vector<uint64_t> signature;
    WaveGraphs* graphs = nullptr;
};

struct BatchState {
    DevBuf reqs, done, next, err, t0;
    std::vector<vgb::BatchReq> host;
    std::vector<uint64_t> signature; // what the captured graph was made for
    cudaGraphExec_t graph = nullptr;
    WaveBufs wave;
    ~BatchState()
    {
        if (graph)
            cudaGraphExecDestroy(graph);
        if (wave.graphs) {
            wave.graphs->release();
            delete wave.graphs;
        }
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
    // The captured training steps use the caches' work buffers, which other calls may reallocate.
    for (auto& kc : caches)
        sig.insert(sig.end(), {(uint64_t)(uintptr_t)kc.first->X.p, (uint64_t)(uintptr_t)kc.first->GX.p,
                               (uint64_t)(uintptr_t)kc.first->batch_rec.p, (uint64_t)(uintptr_t)kc.first->batch_count.p});
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

namespace {

int capture_part(cudaStream_t s, cudaGraph_t* out, const std::function<int()>& launches, const char* what)
{
    *out = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess)
        return cuda_fail(e, what);
    int st = launches();
    e = cudaStreamEndCapture(s, out);
    if (st != VG_OK || e != cudaSuccess) {
        if (*out)
            cudaGraphDestroy(*out);
        *out = nullptr;
        return st != VG_OK ? st : cuda_fail(e, what);
    }
    return VG_OK;
}

int instantiate(cudaGraph_t g, cudaGraphExec_t* out)
{
    cudaError_t e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        *out = nullptr;
        return cuda_fail(e, "graph instantiation");
    }
    return VG_OK;
}

} // namespace

int bwave_graphs(VgContext* ctx, const vgb::WaveBatch& b, const vgk::Wave& w,
                 const std::vector<std::pair<VgCache*, VgRenderer*>>& caches, bool device_loop, WaveGraphs* out)
{
    cudaStream_t s = ctx->stream;
    int tb = 1, sb = 1;
    vgx::bwave_blocks_per_sm(&tb, &sb);
    auto pro = [&]() -> int {
        cudaError_t ce = cudaMemsetAsync(w.counts, 0, 2 * 4, s);
        if (ce == cudaSuccess)
            ce = cudaMemsetAsync(w.fetch, 0, 16 * 4, s);
        if (ce == cudaSuccess)
            ce = cudaMemsetAsync(w.scount, 0, 2 * 2 * vgk::SHADE_CLASSES * 4, s);
        if (ce == cudaSuccess)
            ce = cudaMemsetAsync(b.err, 0, 4, s);
        if (ce == cudaSuccess)
            ce = vgx::bwave_capture_start(s, b, w);
        return ce == cudaSuccess ? VG_OK : cuda_fail(ce, "graph capture (start)");
    };
    auto epi = [&]() -> int {
        if (caches.empty()) {
            cudaError_t ce = vgx::bwave_capture_tail(s, b, w);
            if (ce != cudaSuccess)
                return cuda_fail(ce, "graph capture (tail)");
        }
        for (auto& kc : caches) {
            VgCache* k = kc.first;
            VgRenderer* r = kc.second;
            uint32_t tcap = r->cache_steps * r->cache_batch;
            for (uint32_t t = 0; t < r->cache_steps; t++) {
                int st = vgc::cache_train_step(k, (const float*)k->batch_rec.p, (const uint32_t*)k->batch_count.p,
                                               tcap, t * r->cache_batch, r->cache_batch);
                if (st != VG_OK)
                    return st;
            }
        }
        return VG_OK;
    };
    cudaGraph_t gp = nullptr, ge = nullptr;
    int st;
    if ((st = capture_part(s, &gp, pro, "graph capture")) != VG_OK)
        return st;
    if ((st = capture_part(s, &ge, epi, "graph capture")) != VG_OK) {
        cudaGraphDestroy(gp);
        return st;
    }
    if (!device_loop) {
        cudaGraph_t gb = nullptr;
        auto body = [&]() -> int {
            cudaError_t ce = vgx::bwave_capture_body(s, tb * ctx->sms, sb * ctx->sms, ctx->sms, b, w, 0, false);
            return ce == cudaSuccess ? VG_OK : cuda_fail(ce, "graph capture (loop body)");
        };
        if ((st = capture_part(s, &gb, body, "graph capture")) != VG_OK) {
            cudaGraphDestroy(gp);
            cudaGraphDestroy(ge);
            return st;
        }
        if ((st = instantiate(gp, &out->pro)) != VG_OK) {
            cudaGraphDestroy(gb);
            cudaGraphDestroy(ge);
            return st;
        }
        if ((st = instantiate(gb, &out->body)) != VG_OK) {
            cudaGraphDestroy(ge);
            return st;
        }
        return instantiate(ge, &out->epi);
    }
    cudaGraph_t g = nullptr;
    cudaGraphNode_t n0 = nullptr, n1 = nullptr, n2 = nullptr;
    cudaGraphConditionalHandle loop = 0;
    auto done = [&](cudaError_t err, const char* what) -> int {
        if (gp)
            cudaGraphDestroy(gp);
        if (ge)
            cudaGraphDestroy(ge);
        if (g)
            cudaGraphDestroy(g);
        return cuda_fail(err, what);
    };
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess)
        return done(e, "graph creation");
    if ((e = cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess)
        return done(e, "graph condition");
    if ((e = cudaGraphAddChildGraphNode(&n0, g, nullptr, 0, gp)) != cudaSuccess)
        return done(e, "graph node");
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = loop;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    if ((e = cudaGraphAddNode(&n1, g, &n0, nullptr, 1, &cp)) != cudaSuccess)
        return done(e, "graph loop node");
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if ((e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) != cudaSuccess)
        return done(e, "graph capture");
    cudaError_t ce = vgx::bwave_capture_body(s, tb * ctx->sms, sb * ctx->sms, ctx->sms, b, w, loop, true);
    e = cudaStreamEndCapture(s, &body);
    if (ce != cudaSuccess || e != cudaSuccess)
        return done(ce != cudaSuccess ? ce : e, "graph capture (loop body)");
    if ((e = cudaGraphAddChildGraphNode(&n2, g, &n1, 1, ge)) != cudaSuccess)
        return done(e, "graph node");
    cudaGraphDestroy(gp);
    cudaGraphDestroy(ge);
    gp = ge = nullptr;
    return instantiate(g, &out->one);
}

// Requests on the batch wavefront (kern_bwave.cu), in `order`; the graph is captured the first time
// and replayed while the batch keeps its shape. Latencies from the start kernel.
int batch_wave_run(VgContext* ctx, const VgBatchRequest* reqs, size_t n, int order, VgBatchResult* out,
                   double* total_seconds, int* replayed)
{
    if (!ctx || !reqs || n == 0 || n > 65536)
        return fail(VG_ERR_INVALID, "empty or oversized batch");
    uint64_t items64 = 0, bounces = 0, chain = 0;
    for (size_t i = 0; i < n; i++) {
        const VgBatchRequest& q = reqs[i];
        if (!q.renderer || !q.accum || q.renderer->ctx != ctx || q.accum->owner != q.renderer || q.samples == 0)
            return fail(VG_ERR_INVALID, "batch request " + std::to_string(i) + " is malformed");
        if (!batch_compatible(q.renderer, q.accum))
            return fail(VG_ERR_UNSUPPORTED, "batch request " + std::to_string(i) +
                                                " uses adaptive sampling, ReSTIR or the lighting split");
        uint64_t px = (uint64_t)q.accum->width * q.accum->height;
        if (q.cache && (q.cache->ctx != ctx || px > (1u << 22) || n > 1024))
            return fail(VG_ERR_UNSUPPORTED, "batch request " + std::to_string(i) +
                                                ": a cached request on the batch wavefront needs the context's cache, "
                                                "at most 2^22 pixels and at most 1024 requests in the batch");
        uint64_t per = (uint64_t)q.samples * std::max<uint32_t>(q.renderer->max_depth, 1);
        items64 += px;
        bounces += px * per;
        chain = std::max(chain, per);
    }
    if (items64 >= (1ull << 31))
        return fail(VG_ERR_INVALID, "batch wavefront: more than 2^31 pixels in one batch");
    if (!ctx->batch)
        ctx->batch = new BatchState();
    WaveBufs& B = ctx->batch->wave;
    cudaStream_t s = ctx->stream;
    uint32_t items = (uint32_t)items64;
    uint32_t slots = (uint32_t)std::max<uint64_t>(std::min<uint64_t>(items64, std::max(ctx->batch_wave_slots, 1024u)), n);
    int st;
    if (B.slots < slots) {
        size_t S = slots;
        if ((st = alloc(B.state, S * 16 * vgk::BASE_PLANES, s, false)) != VG_OK ||
            (st = alloc(B.hits, S * 16, s, false)) != VG_OK || (st = alloc(B.q0, S * 4, s, false)) != VG_OK ||
            (st = alloc(B.q1, S * 4, s, false)) != VG_OK || (st = alloc(B.sreq, S * 16 * 3, s, false)) != VG_OK ||
            (st = alloc(B.meta, S * 4, s, false)) != VG_OK ||
            (st = alloc(B.squeue, S * 4 * 2 * vgk::SHADE_CLASSES, s, false)) != VG_OK ||
            (st = alloc(B.slot_req, S * 4, s, false)) != VG_OK || (st = alloc(B.slot_pix, S * 4, s, false)) != VG_OK) {
            B.slots = 0;
            return st;
        }
        B.slots = slots;
        B.signature.clear();
    }
    if (B.nreq < n) {
        if ((st = alloc(B.reqs, n * sizeof(vgb::WaveReq), s, false)) != VG_OK ||
            (st = alloc(B.done, n * sizeof(vgb::BatchDone), s, false)) != VG_OK) {
            B.nreq = 0;
            return st;
        }
        B.nreq = n;
        B.signature.clear();
    }
    if ((!B.counts.p && (st = alloc(B.counts, 16, s, true)) != VG_OK) ||
        (!B.fetch.p && (st = alloc(B.fetch, 64, s, true)) != VG_OK) ||
        (!B.scount.p && (st = alloc(B.scount, 64, s, true)) != VG_OK) ||
        (!B.next.p && (st = alloc(B.next, 16, s, true)) != VG_OK) ||
        (!B.err.p && (st = alloc(B.err, 16, s, true)) != VG_OK) ||
        (!B.loop.p && (st = alloc(B.loop, 16, s, true)) != VG_OK) ||
        (!B.t0.p && (st = alloc(B.t0, 16, s, true)) != VG_OK))
        return st;
    std::vector<size_t> idx = order_of(reqs, n, order);
    // The caches of the batch (the first renderer using a cache sets its training steps), their
    // training buffers and query buffers (one record per slot and wave).
    std::vector<std::pair<VgCache*, VgRenderer*>> caches;
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
    size_t nc = caches.size();
    if (nc && B.cache_slots < slots) {
        size_t S = slots;
        if ((st = alloc(B.spread, S * 8, s, false)) != VG_OK ||
            (st = alloc(B.tvert, S * vgb::WAVE_MAX_TRAIN_VERTICES * vgb::WAVE_VERTEX_VEC4 * 16, s, false)) != VG_OK ||
            (st = alloc(B.tnv, S * 4, s, false)) != VG_OK) {
            B.cache_slots = 0;
            return st;
        }
        B.cache_slots = slots;
        B.ncache = 0; // query buffers are per slot too
        B.signature.clear();
    }
    if (nc && B.ncache < nc) {
        if ((st = alloc(B.caches, nc * sizeof(vgb::WaveCache), s, false)) != VG_OK ||
            (st = alloc(B.qrec, nc * (size_t)B.cache_slots * vgn::REC_WORDS * 4, s, false)) != VG_OK ||
            (st = alloc(B.qcount, nc * 4, s, true)) != VG_OK) {
            B.ncache = 0;
            return st;
        }
        B.ncache = nc;
        B.signature.clear();
    }
    std::vector<vgb::WaveCache> ktab(nc);
    for (size_t j = 0; j < nc; j++) {
        VgCache* k = caches[j].first;
        VgRenderer* r = caches[j].second;
        vgb::WaveCache& K = ktab[j];
        memset(&K, 0, sizeof(K));
        K.cd = k->dev();
        K.qrec = (float*)B.qrec.p + j * (size_t)B.cache_slots * vgn::REC_WORDS;
        K.qcount = (uint32_t*)B.qcount.p + j;
        K.trec = (float*)k->batch_rec.p;
        K.tcount = (uint32_t*)k->batch_count.p;
        K.tcap = r->cache_steps * r->cache_batch;
    }
    B.host.resize(n);
    std::vector<uint64_t> sig;
    uint32_t begin = 0;
    for (size_t j = 0; j < n; j++) {
        const VgBatchRequest& q = reqs[idx[j]];
        VgRenderer* r = q.renderer;
        VgAccum* a = q.accum;
        if (a->samples == 0) {
            a->adaptive_fixed = true;
            a->adaptive = r->adaptive;
            a->restir = r->restir;
        }
        vgb::WaveReq& R = B.host[j];
        memset(&R, 0, sizeof(R));
        R.c = make_ctx(r, a);
        R.c.p[P_SAMPLE] = a->samples;
        R.c.p[P_SAMPLES_PER_DISPATCH] = q.samples;
        R.item_begin = begin;
        R.pixels = a->width * a->height;
        R.f64 = a->precision == 64;
        R.index = (uint32_t)idx[j];
        R.cache = vgb::NO_CACHE;
        if (q.cache) {
            for (size_t c = 0; c < nc; c++)
                if (caches[c].first == q.cache)
                    R.cache = (uint32_t)c;
            R.spread = r->cache_spread;
            R.train_stride = (uint32_t)std::max<size_t>(1, r->cache_train_paths ? R.pixels / r->cache_train_paths
                                                                                : (size_t)R.pixels + 1);
        }
        begin += R.pixels;
        sig.insert(sig.end(), {(uint64_t)(uintptr_t)r, (uint64_t)(uintptr_t)a, q.samples, (uint64_t)(uintptr_t)q.cache,
                               q.cache ? ((uint64_t)r->cache_steps << 32 | r->cache_batch) : 0});
    }
    VgRenderer* r0 = reqs[idx[0]].renderer;
    vgk::Wave w{};
    w.state = (float4*)B.state.p;
    w.hits = (uint4*)B.hits.p;
    w.queue[0] = (uint32_t*)B.q0.p;
    w.queue[1] = (uint32_t*)B.q1.p;
    w.counts = (uint32_t*)B.counts.p;
    w.fetch = (uint32_t*)B.fetch.p;
    w.tstats = nullptr;
    w.sreq = (float4*)B.sreq.p;
    w.meta = (uint32_t*)B.meta.p;
    w.n = slots;
    w.depth = 0;
    w.refill = r0->fetch_refill;
    w.steps = r0->fetch_steps;
    w.shadow_refill = r0->shadow_fetch_refill;
    w.shadow_steps = r0->shadow_fetch_steps;
    w.squeue = (uint32_t*)B.squeue.p;
    w.scount = (uint32_t*)B.scount.p;
    vgb::WaveBatch b{};
    b.reqs = (const vgb::WaveReq*)B.reqs.p;
    b.nreq = (uint32_t)n;
    b.items = items;
    b.slot_req = (uint32_t*)B.slot_req.p;
    b.slot_pix = (uint32_t*)B.slot_pix.p;
    b.next = (uint32_t*)B.next.p;
    b.done = (vgb::BatchDone*)B.done.p;
    b.err = (uint32_t*)B.err.p;
    b.loop = (uint32_t*)B.loop.p;
    b.t0 = (unsigned long long*)B.t0.p;
    b.tail = nc ? 0u : std::min(r0->tail_threshold, slots);
    b.caches = nc ? (const vgb::WaveCache*)B.caches.p : nullptr;
    b.ncache = (uint32_t)nc;
    b.spread = nc ? (float2*)B.spread.p : nullptr;
    b.tvert = nc ? (float4*)B.tvert.p : nullptr;
    b.tnv = nc ? (uint32_t*)B.tnv.p : nullptr;
    // Until the work items run out every slot is live, so each wave takes `slots` bounces; then at
    // most one pixel's samples remain per slot. Two waves per iteration.
    uint64_t waves = bounces / slots + chain + 4;
    b.max_iter = (uint32_t)std::min<uint64_t>(waves / 2 + 2, 1u << 30);
    sig.insert(sig.end(), {(uint64_t)slots, (uint64_t)items, (uint64_t)b.tail, (uint64_t)b.max_iter,
                           (uint64_t)w.refill << 32 | w.steps, (uint64_t)w.shadow_refill << 32 | w.shadow_steps});
    // The captured training steps use the caches' work buffers, which other calls may reallocate.
    for (auto& kc : caches)
        sig.insert(sig.end(), {(uint64_t)(uintptr_t)kc.first->X.p, (uint64_t)(uintptr_t)kc.first->GX.p,
                               (uint64_t)(uintptr_t)kc.first->batch_rec.p, (uint64_t)(uintptr_t)kc.first->batch_count.p});
    VG_CHECK(cudaMemcpyAsync(B.reqs.p, B.host.data(), n * sizeof(vgb::WaveReq), cudaMemcpyHostToDevice, s),
             "batch table");
    if (nc)
        VG_CHECK(cudaMemcpyAsync(B.caches.p, ktab.data(), nc * sizeof(vgb::WaveCache), cudaMemcpyHostToDevice, s),
                 "batch cache table");
    for (size_t j = 0; j < n; j++)
        VG_CHECK(cudaMemsetAsync(B.host[j].c.err, 0, 4, s), "error flag");
    for (auto& kc : caches) {
        VG_CHECK(cudaMemsetAsync(kc.first->batch_count.p, 0, 4, s), "training count");
        VG_CHECK(cudaMemsetAsync(kc.first->err.p, 0, 4, s), "cache error flag");
    }
    sig.push_back(ctx->batch_device_loop ? 1 : 0);
    if (!B.graphs)
        B.graphs = new WaveGraphs();
    bool reuse = (B.graphs->one || B.graphs->pro) && sig == B.signature;
    if (!reuse) {
        B.graphs->release();
        B.signature.clear();
        if ((st = bwave_graphs(ctx, b, w, caches, ctx->batch_device_loop, B.graphs)) != VG_OK) {
            B.graphs->release();
            return st;
        }
        B.signature = sig;
    }
    EventPool pool;
    cudaEvent_t e0 = pool.get(), e1 = pool.get();
    VG_CHECK(cudaEventRecord(e0, s), "event");
    if (ctx->batch_device_loop) {
        VG_CHECK(cudaGraphLaunch(B.graphs->one, s), "graph launch");
    } else {
        VG_CHECK(cudaGraphLaunch(B.graphs->pro, s), "graph launch");
        for (uint32_t it = 0; it < b.max_iter; it++) {
            VG_CHECK(cudaGraphLaunch(B.graphs->body, s), "graph launch");
            uint32_t live = 0;
            VG_CHECK(cudaMemcpyAsync(&live, w.counts, 4, cudaMemcpyDeviceToHost, s), "live count");
            VG_CHECK(cudaStreamSynchronize(s), "live count");
            if (live <= b.tail)
                break;
        }
        VG_CHECK(cudaGraphLaunch(B.graphs->epi, s), "graph launch");
    }
    VG_CHECK(cudaEventRecord(e1, s), "event");
    if ((st = wait_event(e1)) != VG_OK)
        return st;
    uint32_t err = 0;
    unsigned long long t0 = 0;
    std::vector<vgb::BatchDone> done(n);
    VG_CHECK(cudaMemcpy(&err, B.err.p, 4, cudaMemcpyDeviceToHost), "batch error flag");
    VG_CHECK(cudaMemcpy(&t0, B.t0.p, 8, cudaMemcpyDeviceToHost), "batch clock");
    VG_CHECK(cudaMemcpy(done.data(), B.done.p, n * sizeof(vgb::BatchDone), cudaMemcpyDeviceToHost), "batch times");
    if (err & vgn::ERR_MMA_TIMEOUT)
        return fail(VG_ERR_KERNEL, "batch wavefront: a tensor-core completion wait timed out");
    if (err)
        return fail(VG_ERR_KERNEL, "batch wavefront: a traversal stack overflowed");
    for (auto& kc : caches)
        if ((st = vgc::cache_check(kc.first)) != VG_OK)
            return st;
    for (size_t j = 0; j < n; j++) {
        if ((st = read_err(reqs[idx[j]].renderer)) != VG_OK)
            return st;
        if (done[j].remaining != 0)
            return fail(VG_ERR_KERNEL, "batch wavefront: a request did not finish");
    }
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

// The hybrid schedule: requests below `big` pixels share the persistent tile launch; the requests
// from `big` up share the batch wavefront after it, except cached ones the wavefront cannot tag
// (more than 2^22 pixels, or more than 1024 requests in the batch), which follow one at a time on
// the streaming cache integrator, shortest first. *replayed: every captured graph that ran was a
// replay.
int batch_run(VgContext* ctx, const VgBatchRequest* reqs, size_t n, int blocks_per_sm, int order, uint64_t big,
              VgBatchResult* out, double* total_seconds, int* replayed)
{
    if (!ctx || !reqs || n == 0 || n > 65536)
        return fail(VG_ERR_INVALID, "empty or oversized batch");
    std::vector<size_t> small, wave, large;
    for (size_t i = 0; i < n; i++) {
        if (!reqs[i].renderer || !reqs[i].accum)
            return fail(VG_ERR_INVALID, "batch request " + std::to_string(i) + " is malformed");
        uint64_t px = (uint64_t)reqs[i].accum->width * reqs[i].accum->height;
        (px < big ? small : reqs[i].cache && (px > (1u << 22) || n > 1024) ? large : wave).push_back(i);
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
    int st, graphs = 0, replays = 0;
    auto shared = [&](const std::vector<size_t>& part, bool tiles) -> int {
        std::vector<VgBatchRequest> sr;
        for (size_t i : part)
            sr.push_back(reqs[i]);
        std::vector<VgBatchResult> so(sr.size());
        double pt = 0.0;
        int rep = 0;
        int e = tiles ? batch_kernel_run(ctx, sr.data(), sr.size(), blocks_per_sm, order, so.data(), &pt, &rep)
                      : batch_wave_run(ctx, sr.data(), sr.size(), order, so.data(), &pt, &rep);
        if (e != VG_OK)
            return e;
        for (size_t j = 0; j < part.size(); j++)
            if (out)
                out[part[j]].seconds = t + so[j].seconds;
        t += pt;
        graphs++;
        replays += rep;
        return VG_OK;
    };
    if (!small.empty() && (st = shared(small, true)) != VG_OK)
        return st;
    if (!wave.empty() && (st = shared(wave, false)) != VG_OK)
        return st;
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
        *replayed = graphs > 0 && replays == graphs ? 1 : 0;
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

int vg_set_batch_device_loop(VgContext* ctx, int on)
{
    if (!ctx)
        return fail(VG_ERR_INVALID, "null context");
    ctx->batch_device_loop = on != 0;
    return VG_OK;
}

int vg_set_batch_wave_slots(VgContext* ctx, uint32_t slots)
{
    if (!ctx || slots < 1024 || slots > (1u << 26))
        return fail(VG_ERR_INVALID, "batch wavefront slots must be 1024 to 2^26");
    ctx->batch_wave_slots = slots;
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
    uint32_t best_slots = ctx->batch_wave_slots, slots0 = ctx->batch_wave_slots;
    double best = 1e300;
    const uint64_t thresholds[] = {0, 256ull * 256, 512ull * 512, 1024ull * 1024, ~0ull};
    VgBatchTune res{};
    uint32_t trials = 0;
    std::vector<VgBatchResult> times(n);
    int max_b = vgx::batch_blocks_per_sm();
    std::vector<std::pair<size_t, size_t>> tried;
    // As given is the caller's order: left out. CTA counts of the tile launch: the two largest
    // that fit; path slots of the batch wavefront: 2^20 and 2^21. A threshold that splits the
    // requests as an earlier one did is skipped.
    for (uint64_t big : thresholds) {
        size_t n_small = 0, n_wave = 0;
        for (size_t i = 0; i < n; i++) {
            uint64_t px = (uint64_t)requests[i].accum->width * requests[i].accum->height;
            n_small += px < big;
            n_wave += px >= big;
        }
        if (std::find(tried.begin(), tried.end(), std::make_pair(n_small, n_wave)) != tried.end())
            continue;
        tried.push_back({n_small, n_wave});
        std::vector<int> bpss, slotss;
        for (int bps = n_small ? std::max(1, max_b - 1) : max_b; bps <= max_b; bps++)
            bpss.push_back(bps);
        if (n_wave)
            slotss = {1 << 20, 1 << 21};
        else
            slotss = {(int)slots0};
        for (int o : {(int)VG_BATCH_SHORTEST_FIRST, (int)VG_BATCH_LONGEST_FIRST})
        for (int bps : bpss)
        for (int sl : slotss) {
            if (st != VG_OK)
                break;
            ctx->batch_wave_slots = (uint32_t)sl;
            double total = 0.0;
            // One run to capture the graphs, one timed replay.
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
                best_slots = (uint32_t)sl;
                res.p50_seconds = p50;
                res.p99_seconds = p99;
                res.total_seconds = total;
            }
        }
    }
    ctx->batch_wave_slots = best_slots;
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
    res.wave_slots = best_slots;
    res.trials = trials;
    *out = res;
    return VG_OK;
}

} // extern "C"
