// Plain data types shared by the kernels and the host code that launches them.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bvh8.h"
#include "vg_layout.h"

namespace vgd {

using namespace vgl;

// Guide tables of the CDF searches (the cutpoint method, cdf_guide.h): for a CDF of n entries and
// K buckets (K a power of two, so u K is exact), entry k is the search's answer for u = k / K,
// k = 0..K; every u with floor(u K) = k then has its answer between entries k and k + 1 (a bucket
// whose entries are reversed, lo > hi, means "search all n entries"). Environment layout: the
// marginal's K_M + 1 entries, then K_C + 1 entries per row of the conditional.
constexpr uint32_t ENV_GUIDE_M = 1024;
constexpr uint32_t ENV_GUIDE_C = 256;

// Device tables of one renderer.
struct DeviceScene {
    const float* positions;
    const uint32_t* indices;
    const uint32_t* instances;
    const float* materials;
    const uint32_t* lights;
    const float* emitters;
    const float* emit_cdf;
    const float* env_pixels;
    const float* env_marginal;
    const float* env_cond;
    const uint32_t* env_guide; // search ranges for env_marginal and env_cond (ENV_GUIDE_*)
    const uint32_t* emit_guide; // search ranges for emit_cdf: emit_guide_k + 1 entries
    uint32_t emit_guide_k;      // buckets of emit_guide (a power of two)
    const float* uvs;
    const float* texels;
    const uint32_t* tex_info;
    const float* vnormals;
    const uint4* nodes;
    const float4* tris;
    uint32_t shadow_any; // 1 when every surface is opaque: shadow rays stop at any hit
};

// ReSTIR DI reservoirs in structure-of-arrays form, one set per frame parity. The reference keeps
// 80 floats per pixel interleaved (pt_core.slang:55-63); here each field a neighbour reads is a
// 16-byte plane, so a reuse fetches three coalesced vectors.
struct Reservoirs {
    float4* g[2]; // shading point xyz, usable as a neighbour (bits, 1 or 0)   (words 8..10, 14)
    float4* n[2]; // shading normal xyz, emitter + 1 (bits, 0 = none)          (words 11..13, 0)
    float4* x[2]; // sample point xyz, contribution weight W                    (words 1..3, 4)
    float* m[2];  // sample count M                                             (word 5)
    // ReSTIR GI (pt_core.slang:897-981, 1566-1617), per frame parity:
    float4* gx[2]; // second-hit sample point xyz, contribution weight W        (words 16..18, 25)
    float4* gn[2]; // second-hit facing normal xyz, sample count M              (words 19..21, 26)
    float4* gl[2]; // radiance the sample point sent, usable (bits, 1 or 0)      (words 22..24, 27)
    // ...and the scratch of the current sample (words 56..78 of the reference's layout):
    float4* s[7]; // (wsum, M, p-hat, own bits), (c, qPrev), x, n, l, throughput of the first bounce, direct light
};

// Everything a launch reads: the tables, the parameter block and the accumulation buffers.
struct Ctx {
    DeviceScene s;
    uint32_t p[PARAM_WORDS];
    void* accum;     // 3 sums per pixel, float or double
    void* stats;     // adaptive sampling: samples, luminance sum, square sum per pixel
    float* lighting; // LIGHTING_STRIDE floats per pixel
    Reservoirs re;
    uint32_t* err;
};

} // namespace vgd

namespace vgk {

constexpr uint32_t BASE_PLANES = 4;  // 16-byte state planes per path
constexpr uint32_t SHADE_CLASSES = 4; // material-sorted shading: missed, diffuse, conductor, dielectric
constexpr uint32_t SPLIT_PLANES = 5; // more planes with the lighting split

// Wavefront buffers of one accumulation.
struct Wave {
    float4* state;
    uint4* hits;       // hit flag, instance, primitive, t bits (wf_extend.slang:26-29)
    uint32_t* queue[2];
    uint32_t* counts;  // live paths per depth, max depth + 1 entries
    uint32_t* fetch;   // work counters: extend of depth d at [d], shade at [(D + 1) + d]
    unsigned long long* tstats; // traversal counters: rays, nodes, triangle tests, rays past depth 0
    float4* sreq;      // streaming mode, deferred shadow requests: 3 planes of float4 per slot
    uint32_t* meta;    // streaming mode: per path slot, depth (bits 0-7) and sample within the batch (8+)
    uint32_t n;        // paths: one per pixel
    uint32_t depth;    // max depth
    uint32_t refill, steps;               // dynamic fetch of the extend stage: idle lanes per refill, visits between refills
    uint32_t shadow_refill, shadow_steps; // the same for the shadow stage
    // Material-sorted shading (streaming, deferred shadows): the wave's slots by shading class,
    // class k in squeue[k * n ...], counts scount[parity * 4 + k] (null when off).
    uint32_t* squeue;
    uint32_t* scount;
};

// Radiance-cache frames on the streaming wavefront: the path spread (a0, a) of every slot,
// carried between waves, and where a path that ends at the cache leaves its query record: sample
// k of the frame in range k (records qrec + k qcap ..., count qcount[k]), so that each range holds
// at most one query per pixel. Training pixels ((pixel + train_offset) % train_stride == 0) are
// traced by their own kernel.
struct CacheWave {
    float spread;          // threshold c of a^2 > c a0
    float2* st;            // per slot: a0, a
    float* qrec;           // query records (CACHE_REC_WORDS floats each)
    uint32_t* qcount;      // one count per sample of the frame
    uint32_t qcap;         // records per range (pixels)
    uint32_t train_stride, train_offset;
};

} // namespace vgk
