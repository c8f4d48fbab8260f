// Software ray traversal of the quantised 8-wide BVH (bvh8.h) on sm_103a, standing in for the
// hardware ray queries of Verion's kernels: `traceClosest` (shaders/include/pt_core.slang:684-700,
// closest opaque hit, TMin 0, TMax 1e30) and the shadow-ray query inside `occluded` (:580-613,
// accept the first hit and end the search).
//
// Hit rule, identical in the CPU oracle: a triangle is hit at distance t when the watertight test
// of Woop, Benthin and Wald ("Watertight Ray/Triangle Intersection", JCGT 2013) accepts it and
// 0 < t < tmax. The closest hit is the smallest t; equal distances go to the lower global triangle
// index, so the answer does not depend on the order the tree is walked in.
//
// Child boxes are tested in the node-local form of Ylitie, Karras and Laine (HPG 2017), one FMA per
// plane, with an explicit bound on its rounding error added outwards, so a box the ray touches is
// never rejected and the culling cannot change the answer.
#pragma once
#include "bvh8.h"
#include "vec3.h"

namespace vgt {

struct TRay {
    V3 o, d;
    float ix, iy, iz; // reciprocal direction for the slab test (tiny components clamped)
    uint32_t oct;     // sign octant of the direction
    int kx, ky, kz;   // watertight test axis permutation
    float sx, sy, sz; // watertight test shear
};

__device__ __forceinline__ float slab_rcp(float d)
{
    float a = fabsf(d);
    if (a < bvh8::MIN_DIR)
        d = copysignf(bvh8::MIN_DIR, d);
    return 1.0f / d;
}

__device__ __forceinline__ TRay make_ray(V3 o, V3 d)
{
    TRay r;
    r.o = o;
    r.d = d;
    r.ix = slab_rcp(d.x);
    r.iy = slab_rcp(d.y);
    r.iz = slab_rcp(d.z);
    r.oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    if (ay > ax)
        kz = 1;
    if (az > (kz == 0 ? ax : ay))
        kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    float dz = comp(d, kz);
    if (dz < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.sx = comp(d, kx) / dz;
    r.sy = comp(d, ky) / dz;
    r.sz = 1.0f / dz;
    return r;
}

// Watertight test. On success returns true with the distance t = T / det and the edge functions
// (U, V, W weigh vertices 0, 1, 2; divided by det they are the barycentrics). (Tried: a sign and
// magnitude test ahead of the division, rejecting where the quotient could only be rejected
// against the closest hit so far; it measured 1.5% slower per extend launch.)
__device__ __forceinline__ bool tri_test(const TRay& r, V3 v0, V3 v1, V3 v2, float& t, float& U, float& V, float& W,
                                         float& det)
{
    V3 A = v0 - r.o;
    V3 B = v1 - r.o;
    V3 C = v2 - r.o;
    float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
    float Ax = comp(A, r.kx) - r.sx * Akz;
    float Ay = comp(A, r.ky) - r.sy * Akz;
    float Bx = comp(B, r.kx) - r.sx * Bkz;
    float By = comp(B, r.ky) - r.sy * Bkz;
    float Cx = comp(C, r.kx) - r.sx * Ckz;
    float Cy = comp(C, r.ky) - r.sy * Ckz;
    U = Cx * By - Cy * Bx;
    V = Ax * Cy - Ay * Cx;
    W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        // Edge hit: redo the 2x2 determinants in double precision (the paper's fallback).
        double cxby = (double)Cx * (double)By, cybx = (double)Cy * (double)Bx;
        double axcy = (double)Ax * (double)Cy, aycx = (double)Ay * (double)Cx;
        double bxay = (double)Bx * (double)Ay, byax = (double)By * (double)Ax;
        U = (float)(cxby - cybx);
        V = (float)(axcy - aycx);
        W = (float)(bxay - byax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f))
        return false;
    det = U + V + W;
    if (det == 0.0f)
        return false;
    float Az = r.sz * Akz;
    float Bz = r.sz * Bkz;
    float Cz = r.sz * Ckz;
    float T = U * Az + V * Bz + W * Cz;
    t = T / det;
    return t > 0.0f;
}

struct TraceHit {
    bool hit;
    uint32_t inst, prim, gid;
    float t;
    float b1, b2;           // barycentric weights of vertices 1 and 2
    uint32_t nodes, tests;  // nodes visited and triangles tested (dropped by the compiler unless read)
};

__device__ __forceinline__ uint32_t byte_of(uint32_t lo, uint32_t hi, int i)
{
    uint32_t w = i < 4 ? lo : hi;
    return (w >> ((i & 3) * 8)) & 0xffu;
}

// The byte as a float, exactly: the byte placed in the mantissa of 2^23 (one byte permute), minus
// 2^23; equal to (float)byte_of(lo, hi, i) without an integer-to-float conversion.
__device__ __forceinline__ float byte_f(uint32_t lo, uint32_t hi, int i)
{
    uint32_t w = i < 4 ? lo : hi;
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7650u + (uint32_t)(i & 3))) - 8388608.0f;
}


// Child-box tests of one BVH8 node (words w0..w4, bvh8.h) for ray r with the closest hit so far at
// best_t: the hit internal children as bits (slot XOR octant, the visiting order) and the triangles
// of the hit leaf slots as bits from the node's triangle base.
//
// Node-local ray (Ylitie et al. 2017): t(q) = A + q S per axis with A = (p - o) / d and
// S = 2^e / d, one FMA per plane. The plane p + q 2^e is exact; A and S carry at most a few
// roundings, so every t is moved outwards by err = 2^-21 (|A| + 255 |S|), a bound on that error:
// the test never rejects a box the ray enters, and the hits stay those of brute force.
// (Tried: each axis's near and far planes through one packed f32x2 add and FMA, with three-input
// max / min for the slab bounds. Same values, 0.408 against 0.407 ms per extend launch on the
// 1M-triangle workload: the traversal is not limited by these instructions' count.)
__device__ __forceinline__ void node_test(const TRay& r, uint4 w0, uint4 w2, uint4 w3, uint4 w4, uint32_t imask,
                                          uint32_t meta_lo, uint32_t meta_hi, float best_t, uint32_t& inner_hits,
                                          uint32_t& tri_bits)
{
    float px = __uint_as_float(w0.x), py = __uint_as_float(w0.y), pz = __uint_as_float(w0.z);
    uint32_t em = w0.w;
    float scx = __uint_as_float((em & 0xffu) << 23);
    float scy = __uint_as_float(((em >> 8) & 0xffu) << 23);
    float scz = __uint_as_float(((em >> 16) & 0xffu) << 23);
    bool px_pos = r.ix >= 0.0f, py_pos = r.iy >= 0.0f, pz_pos = r.iz >= 0.0f;
    // Near and far quantised planes per axis (low words at w2.x .. high words at w4.w).
    uint32_t nxl = px_pos ? w2.x : w3.z, nxh = px_pos ? w2.y : w3.w;
    uint32_t fxl = px_pos ? w3.z : w2.x, fxh = px_pos ? w3.w : w2.y;
    uint32_t nyl = py_pos ? w2.z : w4.x, nyh = py_pos ? w2.w : w4.y;
    uint32_t fyl = py_pos ? w4.x : w2.z, fyh = py_pos ? w4.y : w2.w;
    uint32_t nzl = pz_pos ? w3.x : w4.z, nzh = pz_pos ? w3.y : w4.w;
    uint32_t fzl = pz_pos ? w4.z : w3.x, fzh = pz_pos ? w4.w : w3.y;
    float ax = (px - r.o.x) * r.ix, sx = scx * r.ix;
    float ay = (py - r.o.y) * r.iy, sy = scy * r.iy;
    float az = (pz - r.o.z) * r.iz, sz = scz * r.iz;
    float ex = 4.76837158e-7f * (fabsf(ax) + 255.0f * fabsf(sx));
    float ey = 4.76837158e-7f * (fabsf(ay) + 255.0f * fabsf(sy));
    float ez = 4.76837158e-7f * (fabsf(az) + 255.0f * fabsf(sz));
    float anx = ax - ex, afx = ax + ex, any_ = ay - ey, afy = ay + ey, anz = az - ez, afz = az + ez;
    inner_hits = 0;
    tri_bits = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        float tnx = fmaf(byte_f(nxl, nxh, i), sx, anx);
        float tny = fmaf(byte_f(nyl, nyh, i), sy, any_);
        float tnz = fmaf(byte_f(nzl, nzh, i), sz, anz);
        float tfx = fmaf(byte_f(fxl, fxh, i), sx, afx);
        float tfy = fmaf(byte_f(fyl, fyh, i), sy, afy);
        float tfz = fmaf(byte_f(fzl, fzh, i), sz, afz);
        float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.0f));
        float tf = fminf(fminf(tfx, tfy), fminf(tfz, best_t));
        if (tn <= tf) {
            if ((imask >> i) & 1u) {
                inner_hits |= 1u << (i ^ r.oct);
            } else {
                uint32_t m = byte_of(meta_lo, meta_hi, i);
                tri_bits |= ((1u << (m >> 5)) - 1u) << (m & 31u);
            }
        }
    }
}

// Closest hit (ANY = false) or any hit (ANY = true) with 0 < t < tmax.
template <bool ANY>
__device__ __forceinline__ TraceHit trace_bvh(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                              const TRay& r, float tmax, uint32_t* err)
{
    TraceHit h;
    h.hit = false;
    h.inst = h.prim = 0;
    h.gid = 0xffffffffu;
    h.t = tmax;
    h.b1 = h.b2 = 0.0f;
    h.nodes = h.tests = 0;
    float best_t = tmax;
    uint2 stack[bvh8::STACK_SIZE];
    int sp = 0;
    uint32_t node = 0;
    for (;;) {
        const uint4* np = nodes + (size_t)node * bvh8::NODE_VEC4;
        h.nodes++;
        uint4 w0 = __ldg(np);
        uint4 w1 = __ldg(np + 1);
        uint4 w2 = __ldg(np + 2);
        uint4 w3 = __ldg(np + 3);
        uint4 w4 = __ldg(np + 4);
        uint32_t imask = w0.w >> 24;
        uint32_t child_base = w1.x, tri_base = w1.y;
        uint32_t inner_hits, tri_bits;
        node_test(r, w0, w2, w3, w4, imask, w1.z, w1.w, best_t, inner_hits, tri_bits);
        // Triangles of this node's leaf slots.
        while (tri_bits) {
            uint32_t j = __ffs(tri_bits) - 1;
            tri_bits &= tri_bits - 1;
            const float4* tp = tris + (size_t)(tri_base + j) * bvh8::TRI_VEC4;
            float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
            float t, U, V, W, det;
            h.tests++;
            if (tri_test(r, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z), t, U, V, W, det)) {
                uint32_t gid = __float_as_uint(c.w);
                bool take = ANY ? t < tmax : (t < best_t || (h.hit && t == best_t && gid < h.gid));
                if (take) {
                    h.hit = true;
                    h.t = t;
                    best_t = t;
                    h.gid = gid;
                    h.inst = __float_as_uint(a.w);
                    h.prim = __float_as_uint(b.w);
                    h.b1 = V / det;
                    h.b2 = W / det;
                    if (ANY)
                        return h;
                }
            }
        }
        // Next node: from this node's hit children, else from the stack.
        uint32_t hits = inner_hits;
        uint32_t gbase = child_base, gmask = imask;
        if (hits == 0) {
            if (sp == 0)
                break;
            --sp;
            gbase = stack[sp].x;
            gmask = stack[sp].y & 0xffu;
            hits = stack[sp].y >> 8;
        }
        uint32_t b = __ffs(hits) - 1;
        hits &= hits - 1;
        uint32_t slot = b ^ r.oct;
        node = gbase + __popc(gmask & ((1u << slot) - 1u));
        if (hits) {
            if (sp >= (int)bvh8::STACK_SIZE) {
                atomicOr(err, bvh8::ERR_STACK);
                break;
            }
            stack[sp++] = make_uint2(gbase, gmask | (hits << 8));
        }
    }
    return h;
}

// ---------------------------------------------------------------------------------------------
// Queue traversal with dynamic ray fetch: a warp keeps one ray per lane and, whenever at least
// `refill` lanes have finished theirs, hands those lanes the next rays of the queue (one atomic per
// refill), so the warp does not idle on its longest ray (Aila and Laine, "Understanding the
// Efficiency of Ray Traversal on GPUs", HPG 2009). Each lane runs at most `steps` node visits
// between refills. Results are those of trace_bvh: the hit rule does not depend on the visiting order.
//
// get(i, r, tmax) loads queue item i into a ray and returns false when it has no ray (it then
// completes at once with a miss); put(i, hit) stores the result of item i.

struct Walk {
    TRay r;
    float tmax;
    uint32_t item;
    uint32_t node;
    int sp;
    TraceHit h;
};

// One node visit: box tests, the node's triangles, then the next node. Returns true when the walk
// has finished (stack empty, or any-hit found).
template <bool ANY>
__device__ __forceinline__ bool walk_step(const uint4* __restrict__ nodes, const float4* __restrict__ tris, Walk& w,
                                          uint2* stack, uint32_t* err)
{
    const TRay& r = w.r;
    const uint4* np = nodes + (size_t)w.node * bvh8::NODE_VEC4;
    uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
    w.h.nodes++;
    uint32_t imask = w0.w >> 24;
    uint32_t child_base = w1.x, tri_base = w1.y;
    uint32_t inner_hits, tri_bits;
    node_test(r, w0, w2, w3, w4, imask, w1.z, w1.w, w.tmax, inner_hits, tri_bits);
    while (tri_bits) {
        uint32_t j = __ffs(tri_bits) - 1;
        tri_bits &= tri_bits - 1;
        const float4* tp = tris + (size_t)(tri_base + j) * bvh8::TRI_VEC4;
        float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
        float t, U, V, W, det;
        w.h.tests++;
        if (tri_test(r, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z), t, U, V, W, det)) {
            uint32_t gid = __float_as_uint(c.w);
            bool take = ANY ? t < w.tmax : (t < w.tmax || (w.h.hit && t == w.tmax && gid < w.h.gid));
            if (take) {
                w.h.hit = true;
                w.h.t = t;
                w.tmax = ANY ? w.tmax : t;
                w.h.gid = gid;
                w.h.inst = __float_as_uint(a.w);
                w.h.prim = __float_as_uint(b.w);
                w.h.b1 = V / det;
                w.h.b2 = W / det;
                if (ANY)
                    return true;
            }
        }
    }
    uint32_t hits = inner_hits, gbase = child_base, gmask = imask;
    if (hits == 0) {
        if (w.sp == 0)
            return true;
        --w.sp;
        gbase = stack[w.sp].x;
        gmask = stack[w.sp].y & 0xffu;
        hits = stack[w.sp].y >> 8;
    }
    uint32_t b = __ffs(hits) - 1;
    hits &= hits - 1;
    w.node = gbase + __popc(gmask & ((1u << (b ^ r.oct)) - 1u));
    if (hits) {
        if (w.sp >= (int)bvh8::STACK_SIZE) {
            atomicOr(err, bvh8::ERR_STACK);
            return true;
        }
        stack[w.sp++] = make_uint2(gbase, gmask | (hits << 8));
    }
    return false;
}

// ---------------------------------------------------------------------------------------------
// Warp-cooperative leaf testing. In walk_step every lane tests its node's triangles itself, so a
// warp runs its triangle loop as often as its busiest lane needs while the other lanes idle: on the
// 1M-triangle workload about a third of the lanes are active per instruction. Here a step is split
// in three: every lane tests its node's child boxes (node_visit), then the warp tests all the
// (ray, triangle) pairs its lanes collected, one pair per lane (coop_tris), and then every lane
// picks its next node (next_node). The visiting order per ray is walk_step's, and the hit rule does
// not depend on which lane tests a triangle, so the results and the counters are the same.
// Measured on the 1M-triangle workload (1080p, depth 16): the extend stage takes 0.447 ms per launch
// this way against 0.407 ms with each lane testing its own triangles, so it is off by default: the
// per-step scan, owner search and shared-memory reductions cost more issue slots than the divergent
// triangle loop they replace.
//
// A pair lane reads the owner's ray from shared memory (written once per ray) and reports a hit
// with a 64-bit shared-memory atomicMin of (t bits << 32 | global triangle index) on the owner's
// slot: for t > 0 the float bits order like the floats, so the minimum is the closest hit with the
// lower index on ties, the rule of trace_bvh. The winning lane then leaves the hit's instance,
// primitive and barycentrics in the owner's slot. Any-hit rays only need a flag.

// Shared state of one warp (block size 128: four per block).
struct CoopWarp {
    float4 ra[32];               // owner ray: origin xyz, watertight axes kx | ky << 2 | kz << 4
    float4 rb[32];               // owner ray: shear sx, sy, sz; tmax (any-hit)
    unsigned long long key[32];  // closest-hit candidates, min-reduced
    uint4 info[32];              // the winner's instance, primitive, b1, b2 bits; any-hit: x = hit
};
constexpr uint32_t COOP_WARPS = 4; // warps per block of the cooperative kernels (128 threads)

__device__ __forceinline__ void coop_publish_ray(CoopWarp& cw, uint32_t lane, const TRay& r, float tmax)
{
    cw.ra[lane] = make_float4(r.o.x, r.o.y, r.o.z, __uint_as_float((uint32_t)(r.kx | (r.ky << 2) | (r.kz << 4))));
    cw.rb[lane] = make_float4(r.sx, r.sy, r.sz, tmax);
}

// Child-box tests of the walk's current node: the hit internal children (in ray-octant order, as
// walk_step) and the triangles of the hit leaf slots.
__device__ __forceinline__ void node_visit(const uint4* __restrict__ nodes, Walk& w, uint32_t& inner_hits,
                                           uint32_t& tri_bits, uint32_t& tri_base, uint32_t& child_base,
                                           uint32_t& imask)
{
    const TRay& r = w.r;
    const uint4* np = nodes + (size_t)w.node * bvh8::NODE_VEC4;
    uint4 w0 = __ldg(np), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
    w.h.nodes++;
    imask = w0.w >> 24;
    child_base = w1.x;
    tri_base = w1.y;
    node_test(r, w0, w2, w3, w4, imask, w1.z, w1.w, w.tmax, inner_hits, tri_bits);
}

// The next node of the walk after a visit (walk_step's tail). Returns true when the walk has
// finished (stack empty, or the stack overflowed: the error flag is then set).
__device__ __forceinline__ bool next_node(Walk& w, uint32_t inner_hits, uint32_t child_base, uint32_t imask,
                                          uint2* stack, uint32_t* err)
{
    uint32_t hits = inner_hits, gbase = child_base, gmask = imask;
    if (hits == 0) {
        if (w.sp == 0)
            return true;
        --w.sp;
        gbase = stack[w.sp].x;
        gmask = stack[w.sp].y & 0xffu;
        hits = stack[w.sp].y >> 8;
    }
    uint32_t b = __ffs(hits) - 1;
    hits &= hits - 1;
    w.node = gbase + __popc(gmask & ((1u << (b ^ w.r.oct)) - 1u));
    if (hits) {
        if (w.sp >= (int)bvh8::STACK_SIZE) {
            atomicOr(err, bvh8::ERR_STACK);
            return true;
        }
        stack[w.sp++] = make_uint2(gbase, gmask | (hits << 8));
    }
    return false;
}

// Tests every (ray, triangle) pair the warp's lanes collected in this step: lane i owns the
// triangles tri_base + bit of `bits` (its node's hit leaf slots). Called by all 32 lanes of a
// converged warp. Closest hit: the owner's walk takes the closest of them (or keeps its hit) and
// lowers its tmax. Any hit: returns true for an owner with a hit below its tmax (the walk then
// records the hit flag only).
template <bool ANY>
__device__ __forceinline__ bool coop_tris(CoopWarp& cw, uint32_t lane, uint32_t bits, uint32_t tri_base, Walk& w,
                                          const float4* __restrict__ tris)
{
    const uint32_t FULLM = 0xffffffffu;
    uint32_t cnt = __popc(bits);
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(FULLM, incl, o);
        if (lane >= (uint32_t)o)
            incl += v;
    }
    uint32_t total = __shfl_sync(FULLM, incl, 31);
    if (total == 0)
        return false;
    uint32_t excl = incl - cnt;
    unsigned long long init = 0;
    if (cnt) {
        w.h.tests += cnt;
        if (ANY) {
            cw.info[lane].x = 0u;
        } else {
            init = ((unsigned long long)__float_as_uint(w.tmax) << 32) | (w.h.hit ? w.h.gid : 0u);
            cw.key[lane] = init;
        }
    }
    __syncwarp();
    for (uint32_t q0 = 0; q0 < total; q0 += 32) {
        uint32_t q = q0 + lane;
        // Owner of pair q: the number of lanes whose inclusive count is <= q (a binary search over
        // the lanes' non-decreasing counts).
        uint32_t L = 0;
#pragma unroll
        for (uint32_t b = 16; b > 0; b >>= 1) {
            uint32_t v = __shfl_sync(FULLM, incl, L + b - 1);
            if (v <= q)
                L += b;
        }
        uint32_t obits = __shfl_sync(FULLM, bits, L);
        uint32_t oexcl = __shfl_sync(FULLM, excl, L);
        uint32_t obase = __shfl_sync(FULLM, tri_base, L);
        bool mine = false;
        unsigned long long key = 0;
        float V = 0.0f, Wb = 0.0f, det = 1.0f;
        uint32_t ainst = 0, bprim = 0;
        if (q < total) {
            for (uint32_t j = q - oexcl; j > 0; j--)
                obits &= obits - 1;
            const float4* tp = tris + (size_t)(obase + __ffs(obits) - 1) * bvh8::TRI_VEC4;
            float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
            float4 ra = cw.ra[L], rb = cw.rb[L];
            TRay r;
            r.o = v3(ra.x, ra.y, ra.z);
            uint32_t kk = __float_as_uint(ra.w);
            r.kx = (int)(kk & 3u);
            r.ky = (int)((kk >> 2) & 3u);
            r.kz = (int)((kk >> 4) & 3u);
            r.sx = rb.x;
            r.sy = rb.y;
            r.sz = rb.z;
            float t, U;
            if (tri_test(r, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), v3(c.x, c.y, c.z), t, U, V, Wb, det)) {
                if (ANY) {
                    if (t < rb.w)
                        cw.info[L].x = 1u;
                } else {
                    key = ((unsigned long long)__float_as_uint(t) << 32) | __float_as_uint(c.w);
                    atomicMin(&cw.key[L], key);
                    mine = true;
                    ainst = __float_as_uint(a.w);
                    bprim = __float_as_uint(b.w);
                }
            }
        }
        if (!ANY) {
            __syncwarp();
            // The lane whose candidate is the owner's minimum so far leaves its hit there.
            if (mine && cw.key[L] == key)
                cw.info[L] = make_uint4(ainst, bprim, __float_as_uint(V / det), __float_as_uint(Wb / det));
        }
        __syncwarp();
    }
    if (cnt == 0)
        return false;
    if (ANY)
        return cw.info[lane].x != 0u;
    unsigned long long best = cw.key[lane];
    if (best < init) {
        uint4 in = cw.info[lane];
        w.h.hit = true;
        w.h.t = __uint_as_float((uint32_t)(best >> 32));
        w.tmax = w.h.t;
        w.h.gid = (uint32_t)best;
        w.h.inst = in.x;
        w.h.prim = in.y;
        w.h.b1 = __uint_as_float(in.z);
        w.h.b2 = __uint_as_float(in.w);
    }
    return false;
}

// trace_queue with warp-cooperative leaf testing (same dynamic fetch, same results). `cw` is this
// warp's shared state.
template <bool ANY, typename GetRay, typename PutHit>
__device__ __forceinline__ void trace_queue_coop(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                                 uint32_t* fetch, uint32_t count, uint32_t* err, uint32_t refill,
                                                 uint32_t steps, CoopWarp& cw, GetRay get, PutHit put)
{
    const uint32_t FULLM = 0xffffffffu;
    uint32_t lane = threadIdx.x & 31u;
    uint32_t lt = (1u << lane) - 1u;
    uint2 stack[bvh8::STACK_SIZE];
    Walk w;
    bool active = false, exhausted = false;
    for (;;) {
        uint32_t need = __ballot_sync(FULLM, !active);
        if (!exhausted && (need == FULLM || (uint32_t)__popc(need) >= refill)) {
            uint32_t n = __popc(need);
            uint32_t base = 0;
            if (lane == 0)
                base = atomicAdd(fetch, n);
            base = __shfl_sync(FULLM, base, 0);
            exhausted = base + n >= count;
            if (!active) {
                uint32_t idx = base + __popc(need & lt);
                if (idx < count) {
                    V3 o, d;
                    float tmax;
                    w.item = idx;
                    w.h.hit = false;
                    w.h.inst = w.h.prim = 0;
                    w.h.gid = 0xffffffffu;
                    w.h.b1 = w.h.b2 = 0.0f;
                    w.h.nodes = w.h.tests = 0;
                    if (get(idx, o, d, tmax)) {
                        w.r = make_ray(o, d);
                        w.tmax = tmax;
                        w.h.t = tmax;
                        w.node = 0;
                        w.sp = 0;
                        active = true;
                        coop_publish_ray(cw, lane, w.r, tmax);
                    } else {
                        w.h.t = tmax;
                        put(idx, w.h);
                    }
                }
            }
        }
        if (__ballot_sync(FULLM, active) == 0) {
            if (exhausted)
                break;
            continue;
        }
        __syncwarp();
#pragma unroll 1
        for (uint32_t s = 0; s < steps; s++) {
            uint32_t inner = 0, bits = 0, tbase = 0, cbase = 0, imask = 0;
            if (active)
                node_visit(nodes, w, inner, bits, tbase, cbase, imask);
            bool hit = coop_tris<ANY>(cw, lane, bits, tbase, w, tris);
            if (active) {
                bool done = (ANY && hit) ? true : next_node(w, inner, cbase, imask, stack, err);
                if (ANY && hit) {
                    w.h.hit = true;
                }
                if (done) {
                    put(w.item, w.h);
                    active = false;
                }
            }
            if (__ballot_sync(FULLM, active) == 0)
                break;
        }
    }
}

// The body of trace_queue and trace_queue_scenes: with SCENES, `get` also names the BVH of each ray
// (its node and triangle arrays), which the lane keeps while it walks that ray.
template <bool ANY, bool SCENES, typename GetRay, typename PutHit>
__device__ __forceinline__ void trace_queue_impl(const uint4* __restrict__ nodes0, const float4* __restrict__ tris0,
                                                 uint32_t* fetch, uint32_t count, uint32_t* err, uint32_t refill,
                                                 uint32_t steps, GetRay get, PutHit put)
{
    const uint32_t FULLM = 0xffffffffu;
    const uint4* nodes = nodes0;
    const float4* tris = tris0;
    uint32_t lane = threadIdx.x & 31u;
    uint32_t lt = (1u << lane) - 1u;
    uint2 stack[bvh8::STACK_SIZE];
    Walk w;
    bool active = false, exhausted = false;
    for (;;) {
        uint32_t need = __ballot_sync(FULLM, !active);
        if (!exhausted && (need == FULLM || (uint32_t)__popc(need) >= refill)) {
            uint32_t n = __popc(need);
            uint32_t base = 0;
            if (lane == 0)
                base = atomicAdd(fetch, n);
            base = __shfl_sync(FULLM, base, 0);
            exhausted = base + n >= count;
            if (!active) {
                uint32_t idx = base + __popc(need & lt);
                if (idx < count) {
                    V3 o, d;
                    float tmax;
                    w.item = idx;
                    w.h.hit = false;
                    w.h.inst = w.h.prim = 0;
                    w.h.gid = 0xffffffffu;
                    w.h.b1 = w.h.b2 = 0.0f;
                    w.h.nodes = w.h.tests = 0;
                    bool ok;
                    if constexpr (SCENES)
                        ok = get(idx, o, d, tmax, nodes, tris);
                    else
                        ok = get(idx, o, d, tmax);
                    if (ok) {
                        w.r = make_ray(o, d);
                        w.tmax = tmax;
                        w.h.t = tmax;
                        w.node = 0;
                        w.sp = 0;
                        active = true;
                    } else {
                        w.h.t = tmax;
                        put(idx, w.h);
                    }
                }
            }
        }
        if (__ballot_sync(FULLM, active) == 0) {
            if (exhausted)
                break;
            continue;
        }
        if (active) {
#pragma unroll 1
            for (uint32_t s = 0; s < steps; s++) {
                if (walk_step<ANY>(nodes, tris, w, stack, err)) {
                    put(w.item, w.h);
                    active = false;
                    break;
                }
            }
        }
    }
}

template <bool ANY, typename GetRay, typename PutHit>
__device__ __forceinline__ void trace_queue(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                            uint32_t* fetch, uint32_t count, uint32_t* err, uint32_t refill,
                                            uint32_t steps, GetRay get, PutHit put)
{
    trace_queue_impl<ANY, false>(nodes, tris, fetch, count, err, refill, steps, get, put);
}

// trace_queue over the rays of several scenes: get(idx, o, d, tmax, nodes, tris) also sets the
// ray's BVH arrays.
template <bool ANY, typename GetRay, typename PutHit>
__device__ __forceinline__ void trace_queue_scenes(uint32_t* fetch, uint32_t count, uint32_t* err, uint32_t refill,
                                                   uint32_t steps, GetRay get, PutHit put)
{
    trace_queue_impl<ANY, true>(nullptr, nullptr, fetch, count, err, refill, steps, get, put);
}

} // namespace vgt
