// The radiance cache's host object and the helpers its C ABI (cache.cu) and the batch entry point
// (batch.cu) share.
#pragma once
#include <cmath>

#include "host.h"
#include "launch_nrc.h"

struct VgCache {
    VgContext* ctx = nullptr;
    int device = -1; // the context's device
    VgCacheConfig cfg{};
    uint32_t res[vgn::MAX_LEVELS] = {};
    uint32_t dense_mask = 0;
    size_t grid_params = 0; // levels x entries x 2
    DevBuf grid, grid_h, grid_grad, grid_m, grid_v;
    DevBuf mlp, mlp_grad, mlp_m, mlp_v, img;
    DevBuf loss, err, count;
    DevBuf X, GX; // encoded input tiles, input-gradient rows (grown on demand)
    DevBuf step;  // Adam step count (u32)
    DevBuf batch_rec, batch_count; // training records of batched requests (vg_batch_render)

    vgn::CacheDev dev() const
    {
        vgn::CacheDev d{};
        d.grid = (const uint32_t*)grid_h.p;
        d.grid_grad = (float*)grid_grad.p;
        d.img = (const uint8_t*)img.p;
        d.mlp_grad = (float*)mlp_grad.p;
        d.loss = (double*)loss.p;
        d.err = (uint32_t*)err.p;
        d.levels = cfg.levels;
        d.log2_t = cfg.log2_entries;
        d.dense_mask = dense_mask;
        for (uint32_t l = 0; l < vgn::MAX_LEVELS; l++)
            d.res[l] = res[l];
        float ext = 0.0f;
        for (int k = 0; k < 3; k++) {
            d.lo[k] = cfg.bounds_lo[k];
            ext = std::max(ext, cfg.bounds_hi[k] - cfg.bounds_lo[k]);
        }
        d.inv_extent = 1.0f / ext;
        return d;
    }
};

namespace {
int dev_of(const VgCache* k) { return k ? k->device : -1; }
} // namespace

namespace vgc {

int cache_check(const VgCache* k);
int ensure_work(VgCache* k, size_t rows);
// One Adam step on the records [offset, offset + batch) of the first min(*count, cap) at `rec`.
int cache_train_step(VgCache* k, const float* rec, const uint32_t* count, uint32_t cap, uint32_t offset,
                     uint32_t batch);

} // namespace vgc
