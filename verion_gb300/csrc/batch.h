// One request of a batched render (vg_batch_render): what the persistent batch kernel needs to run
// its work items. Host and device share this layout.
#pragma once
#include "ctx.h"
#include "nrc.cuh"

namespace vgb {

struct alignas(16) BatchReq {
    vgd::Ctx c;             // scene tables, parameter block (samples from P_SAMPLE, P_SAMPLES_PER_DISPATCH of them), sums
    vgn::CacheDev cd;       // the radiance cache of a cached request
    uint32_t cached;        // 1: paths end at the cache (fused inference), 0: plain paths
    uint32_t f64;           // sums in double precision
    float spread;           // cache: path-spread threshold
    uint32_t train_stride;  // cache: one pixel in train_stride traces a training path per sample
    float* trec;            // cache: training records (shared by the requests of one cache)
    uint32_t* tcount;
    uint32_t tcap;
    uint32_t item_begin;    // this request's work items: [item_begin, item_begin + tiles)
    uint32_t tiles;
    uint32_t tiles_x;       // 16 x 8 pixel tiles per row
    uint32_t index;         // position of the request in the caller's list
};

// Per-request completion, written by the CTA that finishes the request's last tile.
struct BatchDone {
    uint32_t remaining;           // tiles not finished yet
    uint32_t pad;
    unsigned long long done_ns;   // %globaltimer at completion
};

// One request of the batch wavefront (kern_bwave.cu): its pixels are the work items
// [item_begin, item_begin + pixels) of the batch, each traced with all of the request's samples.
struct alignas(16) WaveReq {
    vgd::Ctx c;          // scene tables, parameter block (samples from P_SAMPLE, P_SAMPLES_PER_DISPATCH of them), sums
    uint32_t item_begin;
    uint32_t pixels;
    uint32_t f64;        // sums in double precision
    uint32_t index;      // position of the request in the caller's list
    uint32_t cache;      // the request's radiance cache in the batch's cache table, NO_CACHE for a plain request
    float spread;        // cache: path-spread threshold
    uint32_t train_stride; // cache: one pixel in train_stride traces a training path per sample
    uint32_t pad;
};

constexpr uint32_t NO_CACHE = 0xffffffffu;
constexpr uint32_t WAVE_MAX_TRAIN_VERTICES = 16; // cache vertices recorded per training path
constexpr uint32_t WAVE_VERTEX_VEC4 = 6;         // per vertex: 16 features, throughput, radiance so far

// A radiance cache of the batch wavefront: its network and grid; the query records of the current
// wave (at most one per slot), each with its request and pixel ((request << 22) | pixel) in the
// last word; the batch's training records.
struct alignas(16) WaveCache {
    vgn::CacheDev cd;
    float* qrec;
    uint32_t* qcount;
    float* trec;
    uint32_t* tcount;
    uint32_t tcap;
    uint32_t pad[3];
};

// The batch wavefront's work and completion state besides the wave buffers (vgk::Wave, whose
// slots here hold any request's pixel).
struct WaveBatch {
    const WaveReq* reqs;
    uint32_t nreq;
    uint32_t items;             // pixels of all requests
    uint32_t* slot_req;         // per slot: request of the pixel it traces
    uint32_t* slot_pix;         // per slot: that pixel
    uint32_t* next;             // next work item
    BatchDone* done;            // per request: pixels not finished, completion time
    uint32_t* err;              // traversal error flags of the batch
    uint32_t* loop;             // iterations of the device-side bounce loop
    unsigned long long* t0;     // start time
    uint32_t tail;              // live slots at or below which the loop hands over to the tail kernel
    uint32_t max_iter;          // bound on the loop's iterations
    const WaveCache* caches;    // the radiance caches of the batch's cached requests
    uint32_t ncache;
    float2* spread;             // per slot: the path spread (a0, a) of a cached request's path
    float4* tvert;              // per slot: WAVE_MAX_TRAIN_VERTICES x WAVE_VERTEX_VEC4 (training paths)
    uint32_t* tnv;              // per slot: vertices recorded by its training path
};

} // namespace vgb
