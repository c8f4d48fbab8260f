// Device path core for sm_103a: one path split into generate, trace, shade and finish, shared by
// the megakernel and the wavefront kernels, as in Verion's shaders/include/pt_core.slang (the
// function comments name the Slang function each one follows, by line). It reads the same flat
// tables the reference packs (crates/verion-gpu/src/pack.rs) and consumes random numbers in the
// same order, so a path follows the reference's sequence for its pixel and sample.
//
// Traversal is this backend's own (traverse.cuh); everything else restates the reference's
// arithmetic operation by operation, in single precision, with the portable elementary
// functions of vg_math.h.
#pragma once
#include <stdint.h>

#include "ctx.h"
#include "traverse.cuh"
#include "vg_layout.h"

namespace vgd {

using namespace vgl;

constexpr float PI = 3.14159265358979f;

static __device__ __forceinline__ float pf(const Ctx& c, int i) { return __uint_as_float(c.p[i]); }

// pt_core.slang:69-84
static __device__ __forceinline__ uint32_t pcg(uint32_t v)
{
    uint32_t s = v * 747796405u + 2891336453u;
    uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}

struct Rng {
    uint32_t state;
    __device__ __forceinline__ float next()
    {
        state = pcg(state);
        return (float)(state >> 8) * (1.0f / 16777216.0f);
    }
};

static __device__ __forceinline__ float fget(const float* a, uint32_t i) { return __ldg(a + i); }
static __device__ __forceinline__ uint32_t uget(const uint32_t* a, uint32_t i) { return __ldg(a + i); }
static __device__ __forceinline__ float lw(const Ctx& c, uint32_t i) { return __uint_as_float(uget(c.s.lights, i)); }

static __device__ __forceinline__ V3 vertexPos(const Ctx& c, uint32_t v)
{
    return v3(fget(c.s.positions, 3 * v), fget(c.s.positions, 3 * v + 1), fget(c.s.positions, 3 * v + 2));
}

static __device__ __forceinline__ V3 vertexNormal(const Ctx& c, uint32_t v)
{
    return v3(fget(c.s.vnormals, 3 * v), fget(c.s.vnormals, 3 * v + 1), fget(c.s.vnormals, 3 * v + 2));
}

static __device__ __forceinline__ float iw(const Ctx& c, uint32_t i) { return __uint_as_float(uget(c.s.instances, i)); }

// pt_core.slang:90-99
static __device__ __forceinline__ V3 transformPoint(const Ctx& c, uint32_t base, V3 p)
{
    float r[3];
#pragma unroll
    for (uint32_t row = 0; row < 3; row++) {
        uint32_t o = base + 4 * row;
        r[row] = iw(c, o) * p.x + iw(c, o + 1) * p.y + iw(c, o + 2) * p.z + iw(c, o + 3);
    }
    return v3(r[0], r[1], r[2]);
}

// pt_core.slang:103-111
static __device__ __forceinline__ V3 transformNormal(const Ctx& c, uint32_t base, V3 n)
{
    V3 r0 = v3(iw(c, base), iw(c, base + 1), iw(c, base + 2));
    V3 r1 = v3(iw(c, base + 4), iw(c, base + 5), iw(c, base + 6));
    V3 r2 = v3(iw(c, base + 8), iw(c, base + 9), iw(c, base + 10));
    V3 c0 = cross(r1, r2);
    float s = dot(r0, c0) < 0.0f ? -1.0f : 1.0f;
    return s * v3(dot(c0, n), dot(cross(r2, r0), n), dot(cross(r0, r1), n));
}

// pt_core.slang:115-120
static __device__ __forceinline__ V3 cosineLocal(float u1, float u2)
{
    float r = sqrtf(u1);
    float phi = 2.0f * PI * u2;
    return v3(r * vgm::cosf_(phi), r * vgm::sinf_(phi), sqrtf(fmaxf(0.0f, 1.0f - u1)));
}

// pt_core.slang:122-127
static __device__ __forceinline__ float G1(float cosT, float alpha)
{
    float c2 = cosT * cosT;
    float tan2 = (1.0f - c2) / fmaxf(c2, 1.0e-8f);
    return 2.0f / (1.0f + sqrtf(1.0f + alpha * alpha * tan2));
}

// pt_core.slang:129-134
static __device__ __forceinline__ float Dggx(float hz, float alpha)
{
    float a2 = alpha * alpha;
    float d = hz * hz * (a2 - 1.0f) + 1.0f;
    return a2 / (PI * d * d);
}

// pt_core.slang:136-141
static __device__ __forceinline__ V3 schlick(V3 f0, float c)
{
    float m = 1.0f - saturatef(c);
    float m2 = m * m;
    return f0 + (1.0f - f0) * (m2 * m2 * m);
}

// pt_core.slang:144-153
static __device__ __forceinline__ float fresnelDielectric(float cosi, float eta)
{
    float s2 = (1.0f - cosi * cosi) / (eta * eta);
    if (s2 >= 1.0f)
        return 1.0f;
    float cost = sqrtf(1.0f - s2);
    float rs = (cosi - eta * cost) / (cosi + eta * cost);
    float rp = (eta * cosi - cost) / (eta * cosi + cost);
    return 0.5f * (rs * rs + rp * rp);
}

// pt_core.slang:155-160
static __device__ __forceinline__ void basis(V3 n, V3& t, V3& b)
{
    V3 a = fabsf(n.x) > 0.9f ? v3(0.0f, 1.0f, 0.0f) : v3(1.0f, 0.0f, 0.0f);
    b = normalize(cross(n, a));
    t = cross(b, n);
}

// pt_core.slang:163-177 (Heitz 2018 visible-normal sampling)
static __device__ __forceinline__ V3 sampleVndf(V3 wo, float alpha, float u1, float u2)
{
    V3 vh = normalize(v3(alpha * wo.x, alpha * wo.y, wo.z));
    float lensq = vh.x * vh.x + vh.y * vh.y;
    V3 t1 = lensq > 0.0f ? v3(-vh.y, vh.x, 0.0f) * (1.0f / sqrtf(lensq)) : v3(1.0f, 0.0f, 0.0f);
    V3 t2 = cross(vh, t1);
    float r = sqrtf(u1);
    float phi = 2.0f * PI * u2;
    float a = r * vgm::cosf_(phi);
    float b = r * vgm::sinf_(phi);
    float s = 0.5f * (1.0f + vh.z);
    b = (1.0f - s) * sqrtf(1.0f - a * a) + s * b;
    V3 nh = a * t1 + b * t2 + sqrtf(fmaxf(0.0f, 1.0f - a * a - b * b)) * vh;
    return normalize(v3(alpha * nh.x, alpha * nh.y, fmaxf(0.0f, nh.z)));
}

// pt_core.slang:181
static __device__ __forceinline__ float lum(V3 c) { return dot(c, v3(0.2126f, 0.7152f, 0.0722f)); }

// pt_core.slang:192-195
static __device__ __forceinline__ float albedoAt(const Ctx& c, uint32_t i) { return lw(c, c.p[P_LIGHT_COUNT] * 16 + i); }
static __device__ __forceinline__ uint32_t recvMask(const Ctx& c, uint32_t inst)
{
    return uget(c.s.lights, c.p[P_LIGHT_COUNT] * 16 + ALBEDO_WORDS + 2 * inst);
}
static __device__ __forceinline__ uint32_t emitMask(const Ctx& c, uint32_t inst)
{
    return uget(c.s.lights, c.p[P_LIGHT_COUNT] * 16 + ALBEDO_WORDS + 2 * inst + 1);
}

// pt_core.slang:199-216
static __device__ __noinline__ float iesFactor(const Ctx& c, uint32_t po, V3 d)
{
    V3 l = v3(dot(d, v3(lw(c, po), lw(c, po + 1), lw(c, po + 2))), dot(d, v3(lw(c, po + 3), lw(c, po + 4), lw(c, po + 5))),
              dot(d, v3(lw(c, po + 6), lw(c, po + 7), lw(c, po + 8))));
    float th = vgm::acosf_(clampf(-l.z, -1.0f, 1.0f)) * 57.29578f;
    float ph = vgm::atan2f_(l.y, l.x) * 57.29578f;
    if (ph < 0.0f)
        ph += 360.0f;
    uint32_t i = min((uint32_t)th, 179u);
    uint32_t j = min((uint32_t)ph, 359u);
    float ft = th - (float)i;
    float fp = ph - (float)j;
    uint32_t t = po + 9;
    float a0 = lerpf(lw(c, t + j * 181 + i), lw(c, t + j * 181 + i + 1), ft);
    float a1 = lerpf(lw(c, t + (j + 1) * 181 + i), lw(c, t + (j + 1) * 181 + i + 1), ft);
    return lerpf(a0, a1, fp);
}

// pt_core.slang:220-239
static __device__ __forceinline__ void addSlot(const Ctx& c, uint32_t pixel, uint32_t slot, V3 u, V3 s, V3 wi, float lit, float r)
{
    if (bad3(u) || bad3(s))
        return;
    float* o = c.lighting + (size_t)LIGHTING_STRIDE * pixel + 17 + SLOT_WORDS * slot;
    float w = lum(u);
    float wd = w + lum(s);
    o[0] += u.x;
    o[1] += u.y;
    o[2] += u.z;
    o[3] += w;
    o[4] += w * r;
    o[5] += s.x;
    o[6] += s.y;
    o[7] += s.z;
    o[8] += wd * wi.x;
    o[9] += wd * wi.y;
    o[10] += wd * wi.z;
    o[11] += wd * lit;
}

// pt_core.slang:241-245
static __device__ __forceinline__ V3 envTexel(const Ctx& c, uint32_t i, uint32_t j)
{
    uint32_t o = 3 * (j * c.p[P_ENV_W] + i);
    return v3(fget(c.s.env_pixels, o), fget(c.s.env_pixels, o + 1), fget(c.s.env_pixels, o + 2));
}

// pt_core.slang:248-256
static __device__ __forceinline__ void envCoords(const Ctx& c, V3 d, uint32_t& i, uint32_t& j)
{
    uint32_t w = c.p[P_ENV_W];
    uint32_t h = c.p[P_ENV_H];
    float u = vgm::atan2f_(d.x, -d.z) * (0.5f / PI) + 0.5f;
    float v = vgm::acosf_(clampf(d.y, -1.0f, 1.0f)) / PI;
    i = min((uint32_t)(u * (float)w), w - 1);
    j = min((uint32_t)(v * (float)h), h - 1);
}

static __device__ __forceinline__ V3 envRadiance(const Ctx& c, V3 d)
{
    uint32_t i, j;
    envCoords(c, d, i, j);
    return envTexel(c, i, j);
}

// pt_core.slang:267-272
static __device__ __forceinline__ float envPdf(const Ctx& c, V3 d)
{
    uint32_t i, j;
    envCoords(c, d, i, j);
    return lum(envTexel(c, i, j)) * pf(c, P_ENV_PDF_SCALE);
}

// The reference's inverse-CDF search (pt_core.slang:274-306, 1343-1352): the first of the n entries
// of `cdf` that is >= u, the last when none is. It starts from the guide table's range for u's
// bucket (K buckets, cdf_guide.h), which holds that entry, so it ends at the same one after a few
// steps instead of log2(n) dependent loads; a reversed range (lo > hi) marks a CDF that is not
// non-decreasing, searched over all n entries.
static __device__ __forceinline__ uint32_t guidedCdf(const float* cdf, uint32_t n, const uint32_t* guide, uint32_t K,
                                                     float u)
{
    uint32_t k = min((uint32_t)(u * (float)K), K - 1);
    uint32_t lo = __ldg(guide + k), hi = __ldg(guide + k + 1);
    if (lo > hi) {
        lo = 0;
        hi = n - 1;
    }
    while (lo < hi) {
        uint32_t mid = (lo + hi) / 2;
        if (fget(cdf, mid) >= u)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

// pt_core.slang:274-306, each CDF search through its guide table.
static __device__ __noinline__ V3 envSample(const Ctx& c, float u1, float u2, float u3, float u4, float& pdf, V3& le)
{
    uint32_t w = c.p[P_ENV_W];
    uint32_t h = c.p[P_ENV_H];
    const uint32_t* g = c.s.env_guide;
    uint32_t j = guidedCdf(c.s.env_marginal, h, g, ENV_GUIDE_M, u1);
    uint32_t i = guidedCdf(c.s.env_cond + (size_t)j * w, w, g + (ENV_GUIDE_M + 1) + j * (ENV_GUIDE_C + 1), ENV_GUIDE_C,
                           u2);
    float phi = (((float)i + u3) / (float)w - 0.5f) * 2.0f * PI;
    float theta = (((float)j + u4) / (float)h) * PI;
    float st = vgm::sinf_(theta);
    le = envTexel(c, i, j);
    pdf = lum(le) * pf(c, P_ENV_PDF_SCALE);
    return v3(st * vgm::sinf_(phi), vgm::cosf_(theta), -st * vgm::cosf_(phi));
}

// pt_core.slang:309-315
static __device__ __forceinline__ V3 texelAt(const Ctx& c, uint32_t base, uint32_t w, uint32_t h, int x, int y)
{
    uint32_t xi = (uint32_t)(((x % (int)w) + (int)w) % (int)w);
    uint32_t yi = (uint32_t)(((y % (int)h) + (int)h) % (int)h);
    uint32_t o = 3 * (base + yi * w + xi);
    return v3(fget(c.s.texels, o), fget(c.s.texels, o + 1), fget(c.s.texels, o + 2));
}

// pt_core.slang:317-328
static __device__ V3 bilinear(const Ctx& c, uint32_t base, uint32_t w, uint32_t h, float ux, float uy)
{
    float fx = ux * (float)w - 0.5f;
    float fy = uy * (float)h - 0.5f;
    int x0 = (int)floorf(fx);
    int y0 = (int)floorf(fy);
    float tx = fx - (float)x0;
    float ty = fy - (float)y0;
    V3 a = lerp3(texelAt(c, base, w, h, x0, y0), texelAt(c, base, w, h, x0 + 1, y0), tx);
    V3 b = lerp3(texelAt(c, base, w, h, x0, y0 + 1), texelAt(c, base, w, h, x0 + 1, y0 + 1), tx);
    return lerp3(a, b, ty);
}

// pt_core.slang:331-356
static __device__ __noinline__ V3 sampleTexture(const Ctx& c, uint32_t tex, float ux, float uy, float footprint)
{
    uint32_t ti = tex * 4;
    uint32_t base = uget(c.s.tex_info, ti);
    uint32_t w = uget(c.s.tex_info, ti + 1);
    uint32_t h = uget(c.s.tex_info, ti + 2);
    uint32_t levels = uget(c.s.tex_info, ti + 3);
    float lod = clampf(vgm::log2f_(fmaxf(footprint * (float)max(w, h), 1.0e-8f)), 0.0f, (float)(levels - 1));
    uint32_t l0 = (uint32_t)floorf(lod);
    float t = lod - (float)l0;
    uint32_t off = base, lwid = w, lhei = h;
    for (uint32_t k = 0; k < l0; k++) {
        off += lwid * lhei;
        lwid = max(lwid / 2, 1u);
        lhei = max(lhei / 2, 1u);
    }
    V3 a = bilinear(c, off, lwid, lhei, ux, uy);
    if (l0 + 1 >= levels || t <= 0.0f)
        return a;
    off += lwid * lhei;
    V3 b = bilinear(c, off, max(lwid / 2, 1u), max(lhei / 2, 1u), ux, uy);
    return lerp3(a, b, t);
}

// pt_core.slang:358-374
struct Surface {
    V3 albedo;
    float metallic, alpha, transmission, ior, eta, fSel, tComp;
    float coat, coatAlpha;
    V3 sheenColor;
    float sheenAlpha, sheenP, coatP;
};

struct Lobes {
    V3 diffuse, specular;
};

// pt_core.slang:384-395
static __device__ __noinline__ float ggxAlbedo(const Ctx& c, float cosO, float alpha)
{
    const uint32_t N = GGX_ALBEDO_N;
    float x = saturatef(cosO) * (float)(N - 1);
    float y = saturatef(sqrtf(alpha)) * (float)(N - 1);
    uint32_t x0 = min((uint32_t)x, N - 2);
    uint32_t y0 = min((uint32_t)y, N - 2);
    float fx = x - (float)x0;
    float fy = y - (float)y0;
    float a = lerpf(albedoAt(c, ALBEDO_GGX + y0 * N + x0), albedoAt(c, ALBEDO_GGX + y0 * N + x0 + 1), fx);
    float b = lerpf(albedoAt(c, ALBEDO_GGX + (y0 + 1) * N + x0), albedoAt(c, ALBEDO_GGX + (y0 + 1) * N + x0 + 1), fx);
    return lerpf(a, b, fy);
}

// pt_core.slang:401-406
static __device__ __forceinline__ V3 multiscatterFactor(const Ctx& c, const Surface& s, float cosO)
{
    if (c.p[P_MULTISCATTER] == 0)
        return v3(1.0f);
    return 1.0f + s.albedo * (1.0f / fmaxf(ggxAlbedo(c, cosO, s.alpha), 0.05f) - 1.0f);
}

// pt_core.slang:410-431
static __device__ __noinline__ float dielectricAlbedo(const Ctx& c, float cosO, float rough, float ior, bool outside)
{
    const uint32_t N = DIEL_ALBEDO_N;
    float x = saturatef(cosO) * (float)(N - 1);
    float y = saturatef(rough) * (float)(N - 1);
    float z = clampf((ior - 1.0f) * 4.0f, 0.0f, (float)(DIEL_ALBEDO_N_IOR - 1) - 1.0e-3f);
    uint32_t x0 = min((uint32_t)x, N - 2);
    uint32_t y0 = min((uint32_t)y, N - 2);
    uint32_t z0 = (uint32_t)z;
    float fx = x - (float)x0;
    float fy = y - (float)y0;
    float fz = z - (float)z0;
    uint32_t base = (outside ? 0 : DIEL_ALBEDO_N_IOR) * N * N;
    float cc[2];
#pragma unroll
    for (uint32_t k = 0; k < 2; k++) {
        uint32_t o = base + ((z0 + k) * N + y0) * N + x0;
        float a = lerpf(albedoAt(c, ALBEDO_DIEL + o), albedoAt(c, ALBEDO_DIEL + o + 1), fx);
        float b = lerpf(albedoAt(c, ALBEDO_DIEL + o + N), albedoAt(c, ALBEDO_DIEL + o + N + 1), fx);
        cc[k] = lerpf(a, b, fy);
    }
    return lerpf(cc[0], cc[1], fz);
}

// pt_core.slang:434-445
static __device__ __noinline__ float sheenAlbedo(const Ctx& c, float cosO, float r)
{
    const uint32_t N = SHEEN_ALBEDO_N;
    float x = saturatef(cosO) * (float)(N - 1);
    float y = saturatef(r) * (float)(N - 1);
    uint32_t x0 = min((uint32_t)x, N - 2);
    uint32_t y0 = min((uint32_t)y, N - 2);
    float fx = x - (float)x0;
    float fy = y - (float)y0;
    float a = lerpf(albedoAt(c, ALBEDO_SHEEN + y0 * N + x0), albedoAt(c, ALBEDO_SHEEN + y0 * N + x0 + 1), fx);
    float b = lerpf(albedoAt(c, ALBEDO_SHEEN + (y0 + 1) * N + x0), albedoAt(c, ALBEDO_SHEEN + (y0 + 1) * N + x0 + 1), fx);
    return lerpf(a, b, fy);
}

// pt_core.slang:449-455 (Charlie distribution, Neubelt visibility)
static __device__ __forceinline__ float sheenCore(float woz, float wiz, float hz, float alpha)
{
    float sinH = sqrtf(fmaxf(1.0f - hz * hz, 0.0f));
    float d = (2.0f + 1.0f / alpha) * vgm::powf_(sinH, 1.0f / alpha) / (2.0f * PI);
    float v = 1.0f / (4.0f * (wiz + woz - wiz * woz));
    return d * v * wiz;
}

// pt_core.slang:459-486
static __device__ __noinline__ Lobes evalLobes(const Ctx& c, const Surface& s, V3 woL, V3 wiL)
{
    V3 hh = normalize(woL + wiL);
    float woh = fmaxf(dot(woL, hh), 0.0f);
    float core = Dggx(hh.z, s.alpha) * G1(woL.z, s.alpha) * G1(wiL.z, s.alpha) / (4.0f * woL.z);
    float t = s.transmission;
    Lobes l;
    l.specular = s.metallic * schlick(s.albedo, woh) * multiscatterFactor(c, s, woL.z) * core +
                 (1.0f - s.metallic) *
                     (t * fresnelDielectric(woh, s.eta) * s.tComp + (1.0f - t) * fresnelDielectric(woh, s.ior)) * core;
    l.diffuse = (1.0f - s.metallic) * (1.0f - t) * (1.0f - s.fSel) * s.albedo * (wiL.z / PI);
    if (s.sheenP > 0.0f) {
        l.specular = (1.0f - s.sheenP) * l.specular + s.sheenColor * sheenCore(woL.z, wiL.z, hh.z, s.sheenAlpha);
        l.diffuse *= 1.0f - s.sheenP;
    }
    if (s.coat > 0.0f) {
        float coreC = Dggx(hh.z, s.coatAlpha) * G1(woL.z, s.coatAlpha) * G1(wiL.z, s.coatAlpha) / (4.0f * woL.z);
        l.specular = (1.0f - s.coatP) * l.specular + s.coat * fresnelDielectric(woh, 1.5f) * coreC;
        l.diffuse *= 1.0f - s.coatP;
    }
    return l;
}

static __device__ __forceinline__ V3 evalReflective(const Ctx& c, const Surface& s, V3 woL, V3 wiL)
{
    Lobes l = evalLobes(c, s, woL, wiL);
    return l.specular + l.diffuse;
}

// pt_core.slang:496-536. Only `total` is kept unless the lighting split is on.
template <bool LIGHT>
struct Parts {
    V3 total, directDiffuse, indirectDiffuse, specular, transmission, emission;
    __device__ __forceinline__ void zero()
    {
        total = directDiffuse = indirectDiffuse = specular = transmission = emission = v3(0.0f);
    }
    __device__ __forceinline__ void file(uint32_t depth, uint32_t cls, V3 c)
    {
        if (!LIGHT)
            return;
        if (depth == 0)
            emission += c;
        else if (cls == 0)
            indirectDiffuse += c;
        else if (cls == 1)
            specular += c;
        else
            transmission += c;
    }
    __device__ __forceinline__ void add(uint32_t depth, uint32_t cls, V3 c)
    {
        total += c;
        file(depth, cls, c);
    }
    __device__ __forceinline__ void addLight(uint32_t depth, uint32_t cls, V3 c, V3 cd, V3 cs)
    {
        total += c;
        if (!LIGHT)
            return;
        if (depth == 0) {
            directDiffuse += cd;
            specular += cs;
        } else
            file(depth, cls, cd + cs);
    }
};

// pt_core.slang:540-557
static __device__ __noinline__ float reflectivePdf(const Surface& s, V3 woL, V3 wiL)
{
    V3 hh = normalize(woL + wiL);
    float woh = fmaxf(dot(woL, hh), 0.0f);
    float spec = G1(woL.z, s.alpha) * Dggx(hh.z, s.alpha) / (4.0f * woL.z);
    float t = s.transmission;
    float pSpec = s.metallic + (1.0f - s.metallic) * (t * fresnelDielectric(woh, s.eta) + (1.0f - t) * s.fSel);
    float pDiff = (1.0f - s.metallic) * (1.0f - t) * (1.0f - s.fSel) * wiL.z / PI;
    float q = pSpec * spec + pDiff;
    if (s.sheenP > 0.0f)
        q = (1.0f - s.sheenP) * q + s.sheenP * wiL.z / PI;
    if (s.coat > 0.0f) {
        float specC = G1(woL.z, s.coatAlpha) * Dggx(hh.z, s.coatAlpha) / (4.0f * woL.z);
        q = (1.0f - s.coatP) * q + s.coatP * specC;
    }
    return q;
}

// pt_core.slang:561-576
static __device__ __noinline__ float opacityAt(const Ctx& c, uint32_t instIdx, uint32_t prim, float b1, float b2)
{
    uint32_t mi = uget(c.s.instances, instIdx * 16 + 2) * 24;
    float op = fget(c.s.materials, mi + 22);
    uint32_t tex = (uint32_t)fget(c.s.materials, mi + 23);
    if (tex > 0 && op > 0.0f) {
        uint32_t tri = uget(c.s.instances, instIdx * 16 + 1) + 3 * prim;
        uint32_t vo = uget(c.s.instances, instIdx * 16);
        uint32_t i0 = uget(c.s.indices, tri) + vo, i1 = uget(c.s.indices, tri + 1) + vo, i2 = uget(c.s.indices, tri + 2) + vo;
        float u0x = fget(c.s.uvs, 2 * i0), u0y = fget(c.s.uvs, 2 * i0 + 1);
        float u1x = fget(c.s.uvs, 2 * i1), u1y = fget(c.s.uvs, 2 * i1 + 1);
        float u2x = fget(c.s.uvs, 2 * i2), u2y = fget(c.s.uvs, 2 * i2 + 1);
        float ux = u0x + b1 * (u1x - u0x) + b2 * (u2x - u0x);
        float uy = u0y + b1 * (u1y - u0y) + b2 * (u2y - u0y);
        op *= sampleTexture(c, tex - 1, ux, uy, 0.0f).x;
    }
    return op;
}

static __device__ __forceinline__ vgt::TraceHit traceShadow(const Ctx& c, V3 o, V3 d, float tmax)
{
    vgt::TRay r = vgt::make_ray(o, d);
    if (c.s.shadow_any)
        return vgt::trace_bvh<true>(c.s.nodes, c.s.tris, r, tmax, c.err);
    return vgt::trace_bvh<false>(c.s.nodes, c.s.tris, r, tmax, c.err);
}

// pt_core.slang:580-613. A scene with translucent surfaces takes the closest occluder of each
// layer (the reference leaves "which hit" to the driver); a fully opaque one stops at any hit.
static __device__ __noinline__ bool occluded(const Ctx& c, V3 o, V3 d, float tmax)
{
    for (uint32_t layer = 0; layer < 8; layer++) {
        vgt::TraceHit q = traceShadow(c, o, d, tmax);
        if (!q.hit)
            return false;
        float opacity = opacityAt(c, q.inst, q.prim, q.b1, q.b2);
        if (opacity >= 1.0f)
            return true;
        uint32_t h = __float_as_uint(o.x) * 73856093u ^ __float_as_uint(o.y) * 19349663u ^
                     __float_as_uint(o.z) * 83492791u ^ __float_as_uint(d.x) * 2654435761u ^
                     __float_as_uint(d.y) * 40503u ^ __float_as_uint(d.z) * 2246822519u ^ layer * 3266489917u;
        h ^= h >> 16;
        h *= 0x7feb352du;
        h ^= h >> 15;
        h *= 0x846ca68bu;
        h ^= h >> 16;
        if ((float)(h >> 8) * (1.0f / 16777216.0f) < opacity)
            return true;
        float adv = q.t + 1.0e-4f;
        o += d * adv;
        tmax -= adv;
        if (tmax <= 0.0f)
            return false;
    }
    return true;
}

// pt_core.slang:616-633
template <bool LIGHT>
struct PathState {
    V3 org, dir, thr;
    uint32_t rng;
    uint32_t cls;
    int chan;
    float pathLen;
    bool misPrev, gi, restir;
    float qPrev;
    uint32_t prevInst;
    float visLit, visTotal;
    Parts<LIGHT> parts;
};

struct Hit {
    bool hit;
    uint32_t inst, prim;
    float t;
};

// pt_core.slang:645-682
template <bool LIGHT>
__device__ PathState<LIGHT> generatePathFor(const Ctx& c, uint32_t px, uint32_t py, uint32_t sample)
{
    uint32_t w = c.p[P_WIDTH];
    uint32_t h = c.p[P_HEIGHT];
    uint32_t pixel = py * w + px;
    Rng rng;
    rng.state = pcg(pixel ^ pcg(sample * 0x9E3779B9u + 0x7F4A7C15u));
    float t = pf(c, P_TAN_HALF_FOV);
    float aspect = (float)w / (float)h;
    float u = (2.0f * ((float)px + rng.next()) / (float)w - 1.0f + pf(c, P_SHIFT_X)) * aspect * t;
    float v = (1.0f - 2.0f * ((float)py + rng.next()) / (float)h + pf(c, P_SHIFT_Y)) * t;
    V3 focal = v3(u, v, -1.0f) * pf(c, P_FOCUS);
    float lensR = pf(c, P_APERTURE) * sqrtf(rng.next());
    float lensA = 2.0f * PI * rng.next();
    V3 lens = v3(lensR * vgm::cosf_(lensA), lensR * vgm::sinf_(lensA), 0.0f);
    V3 dc = normalize(focal - lens);
    PathState<LIGHT> s;
    float o[3], d[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        o[r] = pf(c, 8 + 4 * r) * lens.x + pf(c, 9 + 4 * r) * lens.y + pf(c, 10 + 4 * r) * lens.z + pf(c, 11 + 4 * r);
        d[r] = pf(c, 8 + 4 * r) * dc.x + pf(c, 9 + 4 * r) * dc.y + pf(c, 10 + 4 * r) * dc.z;
    }
    s.org = v3(o[0], o[1], o[2]);
    s.dir = normalize(v3(d[0], d[1], d[2]));
    s.thr = v3(1.0f);
    s.rng = rng.state;
    s.cls = 0;
    s.chan = -1;
    s.pathLen = 0.0f;
    s.misPrev = false;
    s.restir = false;
    s.gi = false;
    s.qPrev = 0.0f;
    s.prevInst = 0;
    s.visLit = 0.0f;
    s.visTotal = 0.0f;
    s.parts.zero();
    return s;
}

// pt_core.slang:684-700
static __device__ __forceinline__ Hit traceClosest(const Ctx& c, V3 org, V3 dir)
{
    vgt::TRay r = vgt::make_ray(org, dir);
    vgt::TraceHit q = vgt::trace_bvh<false>(c.s.nodes, c.s.tris, r, 1.0e30f, c.err);
    Hit h;
    h.hit = q.hit;
    h.inst = q.hit ? q.inst : 0;
    h.prim = q.hit ? q.prim : 0;
    h.t = q.hit ? q.t : 0.0f;
    return h;
}

// ---------------------------------------------------------------------------------------------
// ReSTIR DI (pt_core.slang:702-895), reservoirs in the structure-of-arrays form above.

// pt_core.slang:718-736
static __device__ bool restirLight(const Ctx& c, uint32_t e, uint32_t recv, V3 x, V3 p, V3 n, V3& wi, float& dist, float& cosi,
                            V3& g, float& plsa)
{
    uint32_t o = e * 16;
    const float* E = c.s.emitters;
    V3 a = v3(fget(E, o), fget(E, o + 1), fget(E, o + 2));
    V3 b = v3(fget(E, o + 3), fget(E, o + 4), fget(E, o + 5));
    V3 cc = v3(fget(E, o + 6), fget(E, o + 7), fget(E, o + 8));
    V3 toL = x - p;
    float d2 = dot(toL, toL);
    dist = sqrtf(d2);
    wi = toL / fmaxf(dist, 1.0e-6f);
    float cosl = fabsf(dot(normalize(cross(b - a, cc - a)), wi));
    cosi = dot(n, wi);
    g = v3(fget(E, o + 9), fget(E, o + 10), fget(E, o + 11)) * (cosl / fmaxf(d2, 1.0e-12f));
    plsa = fget(E, o + 13) * d2 / (fmaxf(fget(E, o + 12), 1.0e-30f) * fmaxf(cosl, 1.0e-5f));
    return cosi > 0.0f && cosl > 1.0e-5f && d2 > 1.0e-12f && (__float_as_uint(fget(E, o + 14)) & recv) != 0;
}

// pt_core.slang:739-743
static __device__ __forceinline__ float restirMis(const Surface& surf, V3 woL, V3 wiL, float plsa)
{
    float qb = reflectivePdf(surf, woL, wiL);
    return plsa * plsa / fmaxf(plsa * plsa + qb * qb, 1.0e-30f);
}

// The target function of a ReSTIR candidate, lum(evalReflective(...) * g) * restirMis(...), for many
// candidates at one shading point: the terms that depend on the outgoing direction alone
// (G1(wo), the multiple-scattering factor, 4 wo.z) are computed once per shading point, and the
// reflectance and the reflective pdf share their half vector, GGX density and Fresnel terms. Each
// value is computed by the same operations in the same order as in evalLobes and reflectivePdf,
// so the result is theirs bit for bit.
struct RestirTargetPoint {
    float g1o, g1oCoat, den;
    V3 msf;
};

static __device__ __forceinline__ RestirTargetPoint restirTargetPoint(const Ctx& c, const Surface& s, V3 woL)
{
    RestirTargetPoint e;
    e.g1o = G1(woL.z, s.alpha);
    e.g1oCoat = s.coat > 0.0f ? G1(woL.z, s.coatAlpha) : 0.0f;
    e.den = 4.0f * woL.z;
    e.msf = multiscatterFactor(c, s, woL.z);
    return e;
}

static __device__ __forceinline__ float restirTarget(const Surface& s, const RestirTargetPoint& e, V3 woL, V3 wiL, V3 g,
                                                     float plsa)
{
    V3 hh = normalize(woL + wiL);
    float woh = fmaxf(dot(woL, hh), 0.0f);
    float t = s.transmission;
    float dg = Dggx(hh.z, s.alpha) * e.g1o;
    float fEta = fresnelDielectric(woh, s.eta);
    // evalLobes
    float core = dg * G1(wiL.z, s.alpha) / e.den;
    V3 spec = s.metallic * schlick(s.albedo, woh) * e.msf * core +
              (1.0f - s.metallic) * (t * fEta * s.tComp + (1.0f - t) * fresnelDielectric(woh, s.ior)) * core;
    V3 diff = (1.0f - s.metallic) * (1.0f - t) * (1.0f - s.fSel) * s.albedo * (wiL.z / PI);
    // reflectivePdf
    float pSpec = s.metallic + (1.0f - s.metallic) * (t * fEta + (1.0f - t) * s.fSel);
    float pDiff = (1.0f - s.metallic) * (1.0f - t) * (1.0f - s.fSel) * wiL.z / PI;
    float q = pSpec * (dg / e.den) + pDiff;
    if (s.sheenP > 0.0f) {
        spec = (1.0f - s.sheenP) * spec + s.sheenColor * sheenCore(woL.z, wiL.z, hh.z, s.sheenAlpha);
        diff *= 1.0f - s.sheenP;
        q = (1.0f - s.sheenP) * q + s.sheenP * wiL.z / PI;
    }
    if (s.coat > 0.0f) {
        float dgC = Dggx(hh.z, s.coatAlpha) * e.g1oCoat;
        float coreC = dgC * G1(wiL.z, s.coatAlpha) / e.den;
        spec = (1.0f - s.coatP) * spec + s.coat * fresnelDielectric(woh, 1.5f) * coreC;
        diff *= 1.0f - s.coatP;
        q = (1.0f - s.coatP) * q + s.coatP * (dgC / e.den);
    }
    float mis = plsa * plsa / fmaxf(plsa * plsa + q * q, 1.0e-30f);
    return lum((spec + diff) * g) * mis;
}

struct RestirPick {
    bool valid;
    uint32_t e;
    V3 x;
    float W;
    bool occ;
};

// pt_core.slang:759-882
static __device__ __noinline__ RestirPick restirDI(const Ctx& c, uint32_t pixel, uint32_t recv, V3 p, V3 n, float pHitT, const Surface& surf,
                               V3 T, V3 B, V3 woL, Rng& rng)
{
    uint32_t w = c.p[P_WIDTH];
    uint32_t cur = c.p[P_SAMPLE] & 1u;
    uint32_t emitterCount = c.p[P_EMITTER_COUNT];
    float cap = (float)max(c.p[P_RESTIR_HISTORY], 1u);
    float wsum = 0.0f;
    float mTotal = 0.0f;
    uint32_t selE = 0;
    V3 selX = v3(0.0f);
    float selPhat = 0.0f;
    const float* E = c.s.emitters;
    RestirTargetPoint tp = restirTargetPoint(c, surf, woL);
    for (uint32_t k = 0; k < max(c.p[P_RESTIR_CANDIDATES], 1u); k++) {
        float ue = rng.next();
        float ua = rng.next();
        float ub = rng.next();
        uint32_t lo = guidedCdf(c.s.emit_cdf, emitterCount, c.s.emit_guide, c.s.emit_guide_k, ue);
        uint32_t o = lo * 16;
        V3 a = v3(fget(E, o), fget(E, o + 1), fget(E, o + 2));
        V3 b = v3(fget(E, o + 3), fget(E, o + 4), fget(E, o + 5));
        V3 cc = v3(fget(E, o + 6), fget(E, o + 7), fget(E, o + 8));
        float su = sqrtf(ua);
        V3 x = a * (1.0f - su) + b * (su * (1.0f - ub)) + cc * (su * ub);
        float area = fget(E, o + 12);
        float q = area > 0.0f ? fget(E, o + 13) / area : 0.0f;
        V3 wi, g;
        float dist, cosi, plsa;
        float phat = 0.0f;
        if (q > 0.0f && restirLight(c, lo, recv, x, p, n, wi, dist, cosi, g, plsa)) {
            V3 wiL = v3(dot(wi, T), dot(wi, B), cosi);
            phat = restirTarget(surf, tp, woL, wiL, g, plsa);
        }
        float wgt = phat / fmaxf(q, 1.0e-30f);
        mTotal += 1.0f;
        if (phat > 0.0f) {
            wsum += wgt;
            if (rng.next() * wsum < wgt) {
                selE = lo + 1;
                selX = x;
                selPhat = phat;
            }
        }
    }
    if (c.p[P_SAMPLE] > 0) {
        int px = (int)(pixel % w);
        int py = (int)(pixel / w);
        uint32_t prev = cur ^ 1u;
        for (uint32_t k = 0; k < 1 + RESTIR_NEIGHBOURS; k++) {
            int nx = px, ny = py;
            if (k > 0) {
                nx += (int)(rng.next() * (float)(2 * RESTIR_RADIUS + 1)) - RESTIR_RADIUS;
                ny += (int)(rng.next() * (float)(2 * RESTIR_RADIUS + 1)) - RESTIR_RADIUS;
                if (nx < 0 || ny < 0 || nx >= (int)w || ny >= (int)c.p[P_HEIGHT])
                    continue;
            }
            uint32_t q = (uint32_t)ny * w + (uint32_t)nx;
            float4 G = c.re.g[prev][q];
            float4 Nn = c.re.n[prev][q];
            uint32_t ei = __float_as_uint(Nn.w);
            if (__float_as_uint(G.w) == 0 || ei == 0)
                continue;
            V3 pn = v3(Nn.x, Nn.y, Nn.z);
            V3 pp = v3(G.x, G.y, G.z);
            if (dot(pn, n) < 0.9f || length(pp - p) > 0.05f * fmaxf(pHitT, 0.01f))
                continue;
            float4 X = c.re.x[prev][q];
            V3 xc = v3(X.x, X.y, X.z);
            float mc = fminf(c.re.m[prev][q], cap);
            V3 wi, g;
            float dist, cosi, plsa;
            float phat = 0.0f;
            if (restirLight(c, ei - 1, recv, xc, p, n, wi, dist, cosi, g, plsa)) {
                V3 wiL = v3(dot(wi, T), dot(wi, B), cosi);
                phat = restirTarget(surf, tp, woL, wiL, g, plsa);
            }
            float wgt = phat * X.w * mc;
            mTotal += mc;
            if (wgt > 0.0f) {
                wsum += wgt;
                if (rng.next() * wsum < wgt) {
                    selE = ei;
                    selX = xc;
                    selPhat = phat;
                }
            }
        }
    }
    RestirPick r;
    r.valid = selE != 0 && selPhat > 0.0f;
    r.e = selE;
    r.x = selX;
    r.W = r.valid ? wsum / (mTotal * selPhat) : 0.0f;
    r.occ = false;
    if (r.valid) {
        V3 wi, g;
        float dist, cosi, plsa;
        restirLight(c, selE - 1, recv, selX, p, n, wi, dist, cosi, g, plsa);
        r.occ = occluded(c, p, wi, dist * (1.0f - 1.0e-3f));
    }
    float4 nn = c.re.n[cur][pixel];
    nn.w = __uint_as_float(selE);
    c.re.n[cur][pixel] = nn;
    c.re.x[cur][pixel] = make_float4(selX.x, selX.y, selX.z, r.occ ? 0.0f : r.W);
    c.re.m[cur][pixel] = mTotal;
    return r;
}

// pt_core.slang:885-895
static __device__ __forceinline__ void restirGbuffer(const Ctx& c, uint32_t pixel, V3 p, V3 n)
{
    uint32_t cur = c.p[P_SAMPLE] & 1u;
    c.re.g[cur][pixel] = make_float4(p.x, p.y, p.z, __uint_as_float(1u));
    float4 nn = c.re.n[cur][pixel];
    c.re.n[cur][pixel] = make_float4(n.x, n.y, n.z, nn.w);
}

// pt_core.slang:983-988 (the GI validity word belongs to the GI reservoirs, not built here)
static __device__ __forceinline__ void restirClear(const Ctx& c, uint32_t pixel)
{
    uint32_t cur = c.p[P_SAMPLE] & 1u;
    float4 g = c.re.g[cur][pixel];
    g.w = __uint_as_float(0u);
    c.re.g[cur][pixel] = g;
    if (c.re.gl[cur]) {
        float4 l = c.re.gl[cur][pixel];
        l.w = __uint_as_float(0u);
        c.re.gl[cur][pixel] = l;
    }
}

// pt_core.slang:897-981 (ReSTIR GI, first half): the previous frame's second-hit samples of this
// pixel and its neighbours, reconnected to this shading point (the Jacobian of the solid-angle
// change, at most 10 either way), resampled by their reflected luminance; a candidate must see the
// point. The pick waits in the scratch planes for giFinish.
static __device__ __noinline__ void restirGIPrepare(const Ctx& c, uint32_t pixel, V3 p, V3 n, float pHitT,
                                                   const Surface& surf, V3 T, V3 B, V3 woL, Rng& rng)
{
    uint32_t w = c.p[P_WIDTH];
    uint32_t cur = c.p[P_SAMPLE] & 1u;
    float cap = (float)max(c.p[P_RESTIR_HISTORY], 1u);
    float wsum = 0.0f, mTotal = 0.0f, pSel = 0.0f;
    V3 cSel = v3(0.0f), xSel = v3(0.0f), nSel = v3(0.0f), lSel = v3(0.0f);
    if (c.p[P_SAMPLE] > 0) {
        int px = (int)(pixel % w);
        int py = (int)(pixel / w);
        uint32_t prev = cur ^ 1u;
        for (uint32_t k = 0; k < 1 + RESTIR_NEIGHBOURS; k++) {
            int nx = px, ny = py;
            if (k > 0) {
                nx += (int)(rng.next() * (float)(2 * RESTIR_RADIUS + 1)) - RESTIR_RADIUS;
                ny += (int)(rng.next() * (float)(2 * RESTIR_RADIUS + 1)) - RESTIR_RADIUS;
                if (nx < 0 || ny < 0 || nx >= (int)w || ny >= (int)c.p[P_HEIGHT])
                    continue;
            }
            uint32_t q = (uint32_t)ny * w + (uint32_t)nx;
            float4 G = c.re.g[prev][q];
            float4 L = c.re.gl[prev][q];
            if (__float_as_uint(G.w) == 0 || __float_as_uint(L.w) == 0)
                continue;
            float4 Nn = c.re.n[prev][q];
            V3 pq = v3(G.x, G.y, G.z);
            V3 nq = v3(Nn.x, Nn.y, Nn.z);
            if (dot(nq, n) < 0.9f || length(pq - p) > 0.05f * fmaxf(pHitT, 0.01f))
                continue;
            float4 X = c.re.gx[prev][q];
            float4 N2 = c.re.gn[prev][q];
            V3 x2 = v3(X.x, X.y, X.z);
            V3 n2 = v3(N2.x, N2.y, N2.z);
            V3 l2 = v3(L.x, L.y, L.z);
            float mq = fminf(N2.w, cap);
            mTotal += mq;
            V3 toX = x2 - p;
            float dR = length(toX);
            V3 wi = toX / fmaxf(dR, 1.0e-6f);
            float dQ = length(x2 - pq);
            float cosT = dot(n, wi);
            float cosR = fabsf(dot(n2, wi));
            float cosQ = fabsf(dot(n2, normalize(pq - x2)));
            if (cosT <= 0.0f || dR < 1.0e-3f || cosR < 1.0e-3f || cosQ < 1.0e-3f)
                continue;
            float jac = (cosR / cosQ) * (dQ * dQ) / (dR * dR);
            if (jac > 10.0f || jac < 1.0f / 10.0f)
                continue;
            V3 cc = evalReflective(c, surf, woL, v3(dot(wi, T), dot(wi, B), cosT)) * l2;
            float phat = lum(cc);
            if (phat <= 0.0f || occluded(c, p, wi, dR * (1.0f - 1.0e-3f)))
                continue;
            float wgt = phat * X.w * mq * jac;
            wsum += wgt;
            if (rng.next() * wsum < wgt) {
                pSel = phat;
                cSel = cc;
                xSel = x2;
                nSel = n2;
                lSel = l2;
            }
        }
    }
    c.re.s[0][pixel] = make_float4(wsum, mTotal, pSel, __uint_as_float(0u));
    c.re.s[1][pixel] = make_float4(cSel.x, cSel.y, cSel.z, 0.0f);
    c.re.s[2][pixel] = make_float4(xSel.x, xSel.y, xSel.z, 0.0f);
    c.re.s[3][pixel] = make_float4(nSel.x, nSel.y, nSel.z, 0.0f);
    c.re.s[4][pixel] = make_float4(lSel.x, lSel.y, lSel.z, 0.0f);
}

// pt_core.slang:1566-1617 (ReSTIR GI, second half): the path's own candidate (the surface its
// first bounce reached, with the radiance the rest of the path gathered there) joins the
// resampled ones; the pixel gets its direct light plus the indirect light of the pick, and the new
// reservoir goes to this frame's parity for the next frame.
static __device__ __noinline__ V3 giFinish(const Ctx& c, V3 pathTotal, uint32_t pixel)
{
    uint32_t cur = c.p[P_SAMPLE] & 1u;
    float4 s0 = c.re.s[0][pixel], s1 = c.re.s[1][pixel], s2 = c.re.s[2][pixel], s3 = c.re.s[3][pixel];
    float4 s4 = c.re.s[4][pixel], s5 = c.re.s[5][pixel], s6 = c.re.s[6][pixel];
    float wsum = s0.x;
    float m = s0.y + 1.0f;
    float pSel = s0.z;
    V3 cSel = v3(s1.x, s1.y, s1.z), xSel = v3(s2.x, s2.y, s2.z), nSel = v3(s3.x, s3.y, s3.z);
    V3 lSel = v3(s4.x, s4.y, s4.z), thr1 = v3(s5.x, s5.y, s5.z), d0 = v3(s6.x, s6.y, s6.z);
    float qPrev = s1.w;
    bool own = __float_as_uint(s0.w) != 0 && qPrev > 0.0f;
    V3 giTotal = pathTotal - d0;
    V3 result = d0;
    if (own) {
        V3 cOwn = giTotal * qPrev;
        float pOwn = lum(cOwn);
        if (pOwn > 0.0f) {
            float wOwn = pOwn / qPrev;
            wsum += wOwn;
            Rng r;
            r.state = pcg(pixel ^ pcg(c.p[P_SAMPLE] * 0x85EBCA6Bu + 0x1234u));
            if (r.next() * wsum < wOwn) {
                pSel = pOwn;
                cSel = cOwn;
                float4 X = c.re.gx[cur][pixel], N2 = c.re.gn[cur][pixel];
                xSel = v3(X.x, X.y, X.z);
                nSel = v3(N2.x, N2.y, N2.z);
                lSel = v3(thr1.x > 1.0e-6f ? giTotal.x / thr1.x : 0.0f, thr1.y > 1.0e-6f ? giTotal.y / thr1.y : 0.0f,
                          thr1.z > 1.0e-6f ? giTotal.z / thr1.z : 0.0f);
            }
        }
    } else
        result = result + giTotal;
    float W = pSel > 0.0f ? wsum / (m * pSel) : 0.0f;
    result = result + cSel * W;
    c.re.gx[cur][pixel] = make_float4(xSel.x, xSel.y, xSel.z, W);
    c.re.gn[cur][pixel] = make_float4(nSel.x, nSel.y, nSel.z, m);
    c.re.gl[cur][pixel] = make_float4(lSel.x, lSel.y, lSel.z, __uint_as_float(pSel > 0.0f ? 1u : 0u));
    return result;
}

// ---------------------------------------------------------------------------------------------

// The emitter / environment light sample of one bounce, whose visibility a later shadow stage
// tests: if the segment from o along d up to tmax is unoccluded, c is added to the path's radiance.
struct ShadowReq {
    bool valid;
    V3 o, d;
    float tmax;
    V3 c;
};

// pt_core.slang:992-1543: one bounce at `depth`. Returns false when the path ends here.
// DEFER (lighting split off only): the emitter / environment sample is not traced here but
// returned in *req; it is the last contribution of the bounce, so adding it afterwards keeps the
// order of the sums.
// Radiance-cache hook of shadePath (no reference counterpart). At every surface vertex the
// path reaches (after that vertex's emission is added, before its light sampling) the hook
// records the cache inputs, the throughput and the path radiance so far, and grows the path
// spread of Mueller et al. 2021 (Real-time Neural Radiance Caching, eq. 3):
// a = sum over vertices i >= 1 of sqrt(|x_{i-1} - x_i|^2 / (p(w_{i-1}) |cos theta_i|)), against
// a0 = |x_0 - x_1|^2 / (4 pi cos theta_1) at the primary vertex. A path that is not a training
// path ends at the first vertex past the primary one where a^2 > c a0 and is flagged as a query.
// Directions sampled without a finite solid-angle density (refraction) add nothing to a.
struct CacheHook {
    float c;        // spread threshold
    bool train;     // training path: never ends for a query
    float a0, a;    // spread state, carried across bounces
    bool vertex;    // a surface vertex was recorded at this bounce
    bool query;     // the path ended at this vertex for a cache query
    V3 pos, wo, n, albedo;
    float rough, metallic, transmission;
    V3 thr;         // throughput arriving at the vertex
    V3 L;           // path radiance after the vertex's emission
};

// Query / training record of a cache vertex: position, outgoing direction, normal, roughness,
// albedo, metallic, transmission, one spare word; then three words (throughput or target) and a
// fourth (pixel of a query).
constexpr uint32_t CACHE_REC_WORDS = 20;

__device__ __forceinline__ void cacheFeatures(float* d, const CacheHook& hk)
{
    d[0] = hk.pos.x, d[1] = hk.pos.y, d[2] = hk.pos.z;
    d[3] = hk.wo.x, d[4] = hk.wo.y, d[5] = hk.wo.z;
    d[6] = hk.n.x, d[7] = hk.n.y, d[8] = hk.n.z;
    d[9] = hk.rough;
    d[10] = hk.albedo.x, d[11] = hk.albedo.y, d[12] = hk.albedo.z;
    d[13] = hk.metallic;
    d[14] = hk.transmission;
    d[15] = 0.0f;
}

// The query record of a path that ended at the cache: features, the throughput arriving at the
// vertex, and the pixel the cache's answer is added to.
__device__ __forceinline__ void cacheQueryRecord(float* d, const CacheHook& hk, uint32_t pixel)
{
    cacheFeatures(d, hk);
    d[16] = hk.thr.x, d[17] = hk.thr.y, d[18] = hk.thr.z;
    d[19] = __uint_as_float(pixel);
}

template <bool LIGHT, bool RESTIR, bool DEFER = false, bool CACHE = false>
__device__ __forceinline__ bool shadePath(const Ctx& c, PathState<LIGHT>& st, Hit hq, uint32_t depth, uint32_t pixel,
                          ShadowReq* req = nullptr, CacheHook* hk = nullptr)
{
    static_assert(!(DEFER && LIGHT), "deferred shadow rays need the lighting split off");
    if (DEFER)
        req->valid = false;
    if (CACHE) {
        hk->vertex = false;
        hk->query = false;
    }
    V3 sky = v3(pf(c, P_SKY), pf(c, P_SKY + 1), pf(c, P_SKY + 2));
    bool lightingOn = LIGHT && c.p[P_LIGHTING] != 0;
    uint32_t lightCount = c.p[P_LIGHT_COUNT];
    uint32_t emitterCount = c.p[P_EMITTER_COUNT];
    bool hasEnv = c.p[P_ENV_W] > 0;
    float pEnv = hasEnv ? (emitterCount > 0 ? 0.5f : 1.0f) : 0.0f;
    Rng rng;
    rng.state = st.rng;
    V3 org = st.org;
    V3 dir = st.dir;
    V3 thr = st.thr;
    uint32_t cls = st.cls;
    int chan = st.chan;
    bool alive = true;
    const float* M = c.s.materials;
    do {
        if (!hq.hit) {
            if (RESTIR && depth == 0 && c.p[P_RESTIR] != 0)
                restirClear(c, pixel);
            if (depth == 0 && c.p[P_TRANSPARENT_BG] != 0) {
                alive = false;
                break;
            }
            st.parts.add(depth, cls, thr * sky);
            if (hasEnv) {
                float wB = 1.0f;
                if (st.misPrev) {
                    float pl = (st.restir && depth == 1 ? 1.0f : pEnv) * envPdf(c, dir);
                    float den = st.qPrev * st.qPrev + pl * pl;
                    wB = den > 0.0f ? st.qPrev * st.qPrev / den : 1.0f;
                }
                st.parts.add(depth, cls, thr * envRadiance(c, dir) * wB);
            }
            alive = false;
            break;
        }

        uint32_t inst = hq.inst * 16;
        uint32_t tri = uget(c.s.instances, inst + 1) + 3 * hq.prim;
        uint32_t vo = uget(c.s.instances, inst);
        uint32_t i0 = uget(c.s.indices, tri) + vo, i1 = uget(c.s.indices, tri + 1) + vo, i2 = uget(c.s.indices, tri + 2) + vo;
        V3 p0 = transformPoint(c, inst + 4, vertexPos(c, i0));
        V3 p1 = transformPoint(c, inst + 4, vertexPos(c, i1));
        V3 p2 = transformPoint(c, inst + 4, vertexPos(c, i2));
        V3 nOut = normalize(cross(p1 - p0, p2 - p0));
        V3 wo = -dir;
        bool outside = dot(nOut, wo) > 0.0f;
        V3 ng = outside ? nOut : -nOut;
        float pHitT = hq.t;
        st.pathLen += pHitT;
        V3 hit = org + dir * pHitT;
        V3 e1 = p1 - p0;
        V3 e2 = p2 - p0;
        V3 e3 = hit - p0;
        float d11 = dot(e1, e1);
        float d12 = dot(e1, e2);
        float d22 = dot(e2, e2);
        float den = fmaxf(d11 * d22 - d12 * d12, 1.0e-20f);
        float b1 = (d22 * dot(e3, e1) - d12 * dot(e3, e2)) / den;
        float b2 = (d11 * dot(e3, e2) - d12 * dot(e3, e1)) / den;

        float opacity = opacityAt(c, hq.inst, hq.prim, b1, b2);
        if (opacity < 1.0f && rng.next() >= opacity) {
            org = hit + dir * 1.0e-4f;
            break;
        }
        V3 p = hit + ng * 1.0e-4f;
        if (RESTIR && depth == 1 && st.gi) {
            // pt_core.slang:1072-1082: the first bounce's surface is ReSTIR GI's candidate.
            uint32_t cur = c.p[P_SAMPLE] & 1u;
            c.re.gx[cur][pixel] = make_float4(hit.x, hit.y, hit.z, 0.0f);
            c.re.gn[cur][pixel] = make_float4(ng.x, ng.y, ng.z, 0.0f);
            float4 s0 = c.re.s[0][pixel];
            s0.w = __uint_as_float(1u);
            c.re.s[0][pixel] = s0;
        }

        V3 nsObj = (1.0f - b1 - b2) * vertexNormal(c, i0) + b1 * vertexNormal(c, i1) + b2 * vertexNormal(c, i2);
        V3 ns = nOut;
        if (dot(nsObj, nsObj) > 1.0e-12f) {
            ns = normalize(transformNormal(c, inst + 4, nsObj));
            if (dot(ns, nOut) < 0.0f)
                ns = -ns;
        }
        V3 n = outside ? ns : -ns;

        uint32_t mi = uget(c.s.instances, inst + 2) * 24;
        V3 albedo = v3(fget(M, mi), fget(M, mi + 1), fget(M, mi + 2));
        uint32_t texBase = (uint32_t)fget(M, mi + 10);
        uint32_t texMR = (uint32_t)fget(M, mi + 11);
        uint32_t texEm = (uint32_t)fget(M, mi + 12);
        uint32_t texNm = (uint32_t)fget(M, mi + 13);
        float texRx = 1.0f, texRy = 1.0f; // x = roughness (green), y = metallic (blue)
        V3 texEmission = v3(1.0f);
        if (texBase + texMR + texEm + texNm > 0) {
            float u0x = fget(c.s.uvs, 2 * i0), u0y = fget(c.s.uvs, 2 * i0 + 1);
            float u1x = fget(c.s.uvs, 2 * i1), u1y = fget(c.s.uvs, 2 * i1 + 1);
            float u2x = fget(c.s.uvs, 2 * i2), u2y = fget(c.s.uvs, 2 * i2 + 1);
            float ux = u0x + b1 * (u1x - u0x) + b2 * (u2x - u0x);
            float uy = u0y + b1 * (u1y - u0y) + b2 * (u2y - u0y);
            float d1x = u1x - u0x, d1y = u1y - u0y;
            float d2x = u2x - u0x, d2y = u2y - u0y;
            float uvPerWorld = sqrtf(fabsf(d1x * d2y - d1y * d2x) / fmaxf(length(cross(e1, e2)), 1.0e-20f));
            float footprint = st.pathLen * pf(c, P_PIXEL_CONE) / fmaxf(fabsf(dot(nOut, dir)), 0.1f) * uvPerWorld;
            if (texBase > 0)
                albedo *= sampleTexture(c, texBase - 1, ux, uy, footprint);
            if (texMR > 0) {
                V3 t = sampleTexture(c, texMR - 1, ux, uy, footprint);
                texRx = t.y;
                texRy = t.z;
            }
            if (texEm > 0)
                texEmission = sampleTexture(c, texEm - 1, ux, uy, footprint);
            if (texNm > 0) {
                float det = d1x * d2y - d2x * d1y;
                V3 dPdu = (e1 * d2y - e2 * d1y) / det;
                V3 dPdv = (e2 * d1x - e1 * d2x) / det;
                V3 tg = dPdu - ns * dot(ns, dPdu);
                if (fabsf(det) > 1.0e-20f && dot(tg, tg) > 1.0e-20f) {
                    tg = normalize(tg);
                    V3 bt = cross(ns, tg);
                    if (dot(bt, dPdv) > 0.0f)
                        bt = -bt;
                    V3 nt = sampleTexture(c, texNm - 1, ux, uy, footprint) * 2.0f + -1.0f;
                    float scale = fget(M, mi + 14);
                    ns = normalize(nt.x * scale * tg + nt.y * scale * bt + nt.z * ns);
                    n = outside ? ns : -ns;
                }
            }
        }
        float woN = dot(n, wo);
        if (woN < 0.05f)
            n = normalize(n + wo * (0.05f - woN));

        V3 le = v3(fget(M, mi + 3), fget(M, mi + 4), fget(M, mi + 5)) * texEmission;
        if (st.prevInst != 0 && (emitMask(c, hq.inst) & recvMask(c, st.prevInst - 1)) == 0)
            le = v3(0.0f);
        if (le.x > 0.0f || le.y > 0.0f || le.z > 0.0f) {
            float wB = 1.0f;
            uint32_t eb = uget(c.s.instances, inst + 3);
            if (st.misPrev && eb != 0) {
                uint32_t e = (eb - 1 + hq.prim) * 16;
                float cosl = fmaxf(fabsf(dot(nOut, dir)), 1.0e-4f);
                float pl = (st.restir && depth == 1 ? 1.0f : 1.0f - pEnv) * fget(c.s.emitters, e + 13) * pHitT * pHitT /
                           (fget(c.s.emitters, e + 12) * cosl);
                wB = st.qPrev * st.qPrev / (st.qPrev * st.qPrev + pl * pl);
            }
            st.parts.add(depth, cls, thr * le * wB);
            if (RESTIR && depth == 1 && st.gi) {
                // pt_core.slang:1161-1168: counted with what the first hit gathered itself.
                V3 e = thr * le * wB;
                float4 d = c.re.s[6][pixel];
                c.re.s[6][pixel] = make_float4(d.x + e.x, d.y + e.y, d.z + e.z, d.w);
            }
        }
        float metallic = fget(M, mi + 6) * texRy;
        float rough = fget(M, mi + 7) * texRx;
        float transmission = fget(M, mi + 8);
        float ior = fget(M, mi + 9);
        float dispersion = fget(M, mi + 21);
        if (CACHE) {
            hk->vertex = true;
            hk->pos = p;
            hk->wo = wo;
            hk->n = n;
            hk->albedo = albedo;
            hk->rough = rough;
            hk->metallic = metallic;
            hk->transmission = transmission;
            hk->thr = thr;
            hk->L = st.parts.total;
            float cosT = fmaxf(fabsf(dot(nOut, dir)), 1.0e-4f);
            if (depth == 0) {
                hk->a0 = pHitT * pHitT / (4.0f * PI * cosT);
                hk->a = 0.0f;
            } else {
                if (st.misPrev && st.qPrev > 0.0f)
                    hk->a += sqrtf(pHitT * pHitT / (st.qPrev * cosT));
                if (!hk->train && hk->a * hk->a > hk->c * hk->a0) {
                    hk->query = true;
                    alive = false;
                    break;
                }
            }
        }
        if (dispersion > 0.0f && transmission > 0.0f) {
            if (chan < 0) {
                chan = min((int)(rng.next() * 3.0f), 2);
                thr *= 3.0f * v3(chan == 0 ? 1.0f : 0.0f, chan == 1 ? 1.0f : 0.0f, chan == 2 ? 1.0f : 0.0f);
            }
            ior = fmaxf(ior + (float)(chan - 1) * (ior - 1.0f) * 0.025f * dispersion, 1.0f);
        }
        if (RESTIR && depth == 1 && st.gi && transmission > 0.0f) {
            // pt_core.slang:1187-1190: a glass second hit cannot be reconnected to.
            float4 s0 = c.re.s[0][pixel];
            s0.w = __uint_as_float(0u);
            c.re.s[0][pixel] = s0;
        }
        float alpha = fmaxf(rough * rough, 1.0e-3f);
        float eta = outside ? ior : 1.0f / ior;

        V3 T, B;
        basis(n, T, B);
        V3 woL = v3(dot(wo, T), dot(wo, B), fmaxf(dot(wo, n), 1.0e-4f));
        float fSel = fresnelDielectric(woL.z, ior);
        Surface surf;
        surf.albedo = albedo;
        surf.metallic = metallic;
        surf.alpha = alpha;
        surf.transmission = transmission;
        surf.ior = ior;
        surf.eta = eta;
        surf.fSel = fSel;
        surf.tComp = 1.0f;
        if (c.p[P_MULTISCATTER] != 0 && transmission > 0.0f && rough > 0.0f)
            surf.tComp = 1.0f / fmaxf(dielectricAlbedo(c, woL.z, rough, ior, outside), 0.1f);
        surf.coat = outside ? fget(M, mi + 15) : 0.0f;
        surf.coatAlpha = fmaxf(fget(M, mi + 16) * fget(M, mi + 16), 1.0e-3f);
        float coatF = fresnelDielectric(woL.z, 1.5f);
        surf.coatP = surf.coat * coatF;
        surf.sheenColor = outside ? v3(fget(M, mi + 18), fget(M, mi + 19), fget(M, mi + 20)) : v3(0.0f);
        float sheenMax = fmaxf(surf.sheenColor.x, fmaxf(surf.sheenColor.y, surf.sheenColor.z));
        float sheenR = fmaxf(fget(M, mi + 17), 0.07f);
        surf.sheenAlpha = sheenR * sheenR;
        surf.sheenP = sheenMax > 0.0f ? sheenMax * sheenAlbedo(c, woL.z, sheenR) : 0.0f;

        // Delta lights (pt_core.slang:1224-1282).
        uint32_t recvHere = recvMask(c, hq.inst);
        for (uint32_t li = 0; li < lightCount; li++) {
            uint32_t o = li * 16;
            uint32_t kind = uget(c.s.lights, o);
            V3 col = v3(lw(c, o + 1), lw(c, o + 2), lw(c, o + 3)) * lw(c, o + 4);
            V3 vec = v3(lw(c, o + 5), lw(c, o + 6), lw(c, o + 7));
            bool virt = kind == 3;
            if (virt && !(lightingOn && depth == 0))
                continue;
            if ((uget(c.s.lights, o + 14) & recvHere) == 0)
                continue;
            V3 wi;
            float dist;
            V3 li_;
            if (kind == 1 || virt) {
                wi = -normalize(vec);
                dist = 1.0e30f;
                li_ = col;
            } else {
                V3 toL = vec - p;
                float d2 = dot(toL, toL);
                dist = sqrtf(d2);
                wi = toL / dist;
                li_ = col / d2;
                uint32_t ies = uget(c.s.lights, o + 15);
                if (ies != 0)
                    li_ *= iesFactor(c, ies - 1, -wi);
                if (kind == 2) {
                    V3 axis = v3(lw(c, o + 8), lw(c, o + 9), lw(c, o + 10));
                    float att = saturatef(dot(axis, -wi) * lw(c, o + 11) + lw(c, o + 12));
                    li_ *= att * att;
                }
            }
            float cc = dot(n, wi);
            if (cc > 0.0f) {
                bool occ = occluded(c, p, wi, dist - 1.0e-3f);
                bool track = lightingOn && depth == 0;
                if (!occ || track) {
                    Lobes l = evalLobes(c, surf, woL, v3(dot(wi, T), dot(wi, B), cc));
                    V3 cd = thr * l.diffuse * li_;
                    V3 cs = thr * l.specular * li_;
                    if (!occ && !virt)
                        st.parts.addLight(depth, cls, thr * (l.diffuse + l.specular) * li_, cd, cs);
                    if (LIGHT && track) {
                        float vv = virt ? 0.0f : lum(cd + cs);
                        st.visTotal += vv;
                        st.visLit += occ ? 0.0f : vv;
                        addSlot(c, pixel, uget(c.s.lights, o + 13), cd / cc, cs / cc, wi, occ ? 0.0f : 1.0f, occ ? 0.0f : cc);
                    }
                }
            }
        }

        // ReSTIR DI at the first hit (pt_core.slang:1284-1332).
        bool reDI = false;
        if (RESTIR && depth == 0 && c.p[P_RESTIR] != 0) {
            bool suits = pf(c, P_APERTURE) == 0.0f && transmission == 0.0f && surf.alpha >= RESTIR_MIN_ALPHA &&
                         (surf.coat == 0.0f || surf.coatAlpha >= RESTIR_MIN_ALPHA);
            reDI = suits && (c.p[P_RESTIR] & 1u) != 0 && emitterCount > 0;
            // ReSTIR GI replaces the path's own indirect light, which the lighting split cannot follow.
            bool reGI = suits && (c.p[P_RESTIR] & 2u) != 0 && !lightingOn;
            st.restir = reDI;
            st.gi = reGI;
            if (suits) {
                restirGbuffer(c, pixel, p, n);
                if (reGI)
                    restirGIPrepare(c, pixel, p, n, pHitT, surf, T, B, woL, rng);
            } else
                restirClear(c, pixel);
        }
        if (RESTIR && reDI) {
            RestirPick pick = restirDI(c, pixel, recvHere, p, n, pHitT, surf, T, B, woL, rng);
            if (pick.valid) {
                V3 wi, g;
                float dist, cosi, plsa;
                restirLight(c, pick.e - 1, recvHere, pick.x, p, n, wi, dist, cosi, g, plsa);
                bool track = lightingOn;
                if (!pick.occ || track) {
                    V3 wiL = v3(dot(wi, T), dot(wi, B), cosi);
                    float wl = restirMis(surf, woL, wiL, plsa);
                    Lobes l = evalLobes(c, surf, woL, wiL);
                    V3 cd = thr * l.diffuse * g * (wl * pick.W);
                    V3 cs = thr * l.specular * g * (wl * pick.W);
                    if (!pick.occ)
                        st.parts.addLight(depth, cls, cd + cs, cd, cs);
                    if (LIGHT && track) {
                        float vv = lum(cd + cs);
                        st.visTotal += vv;
                        st.visLit += pick.occ ? 0.0f : vv;
                        addSlot(c, pixel, 3u, cd / cosi, cs / cosi, wi, pick.occ ? 0.0f : 1.0f, pick.occ ? 0.0f : cosi);
                    }
                }
            }
        }

        // Emissive triangles with MIS (pt_core.slang:1334-1390).
        float chooseLight = rng.next();
        float pEnvHere = reDI ? (hasEnv ? 1.0f : 0.0f) : pEnv;
        bool chooseEnv = hasEnv && chooseLight < pEnvHere;
        if (emitterCount > 0 && !chooseEnv && !reDI) {
            float ue = rng.next();
            float ua = rng.next();
            float ub = rng.next();
            uint32_t lo = guidedCdf(c.s.emit_cdf, emitterCount, c.s.emit_guide, c.s.emit_guide_k, ue);
            uint32_t e = lo * 16;
            const float* E = c.s.emitters;
            V3 a = v3(fget(E, e), fget(E, e + 1), fget(E, e + 2));
            V3 b = v3(fget(E, e + 3), fget(E, e + 4), fget(E, e + 5));
            V3 cc = v3(fget(E, e + 6), fget(E, e + 7), fget(E, e + 8));
            float su = sqrtf(ua);
            V3 xl = a * (1.0f - su) + b * (su * (1.0f - ub)) + cc * (su * ub);
            V3 toL = xl - p;
            float d2 = dot(toL, toL);
            float dist = sqrtf(d2);
            V3 wi = toL / dist;
            float cosl = fabsf(dot(normalize(cross(b - a, cc - a)), wi));
            float cosi = dot(n, wi);
            if (DEFER && cosi > 0.0f && cosl > 1.0e-5f && (__float_as_uint(fget(E, e + 14)) & recvHere) != 0) {
                // Deferred: the shadow stage tests visibility and adds c, as the last add of this bounce.
                float pl = (1.0f - pEnv) * fget(E, e + 13) * d2 / (fget(E, e + 12) * cosl);
                V3 wiL = v3(dot(wi, T), dot(wi, B), cosi);
                float qb = reflectivePdf(surf, woL, wiL);
                float wl = pl * pl / (pl * pl + qb * qb);
                V3 lE = v3(fget(E, e + 9), fget(E, e + 10), fget(E, e + 11));
                Lobes l = evalLobes(c, surf, woL, wiL);
                req->valid = true;
                req->o = p;
                req->d = wi;
                req->tmax = dist * (1.0f - 1.0e-3f);
                req->c = thr * (l.specular + l.diffuse) * lE / pl * wl;
            } else if (cosi > 0.0f && cosl > 1.0e-5f && (__float_as_uint(fget(E, e + 14)) & recvHere) != 0) {
                bool occ = occluded(c, p, wi, dist * (1.0f - 1.0e-3f));
                bool track = lightingOn && depth == 0;
                if (!occ || track) {
                    float pl = (1.0f - pEnv) * fget(E, e + 13) * d2 / (fget(E, e + 12) * cosl);
                    V3 wiL = v3(dot(wi, T), dot(wi, B), cosi);
                    float qb = reflectivePdf(surf, woL, wiL);
                    float wl = pl * pl / (pl * pl + qb * qb);
                    V3 lE = v3(fget(E, e + 9), fget(E, e + 10), fget(E, e + 11));
                    Lobes l = evalLobes(c, surf, woL, wiL);
                    V3 cd = thr * l.diffuse * lE / pl * wl;
                    V3 cs = thr * l.specular * lE / pl * wl;
                    if (!occ)
                        st.parts.addLight(depth, cls, thr * (l.specular + l.diffuse) * lE / pl * wl, cd, cs);
                    if (LIGHT && track) {
                        float vv = lum(cd + cs);
                        st.visTotal += vv;
                        st.visLit += occ ? 0.0f : vv;
                        addSlot(c, pixel, 3u, cd / cosi, cs / cosi, wi, occ ? 0.0f : 1.0f, occ ? 0.0f : cosi);
                    }
                }
            }
        }

        // Environment map (pt_core.slang:1392-1427).
        if (chooseEnv) {
            float u1e = rng.next();
            float u2e = rng.next();
            float u3e = rng.next();
            float u4e = rng.next();
            float pdfE;
            V3 leE;
            V3 wi = envSample(c, u1e, u2e, u3e, u4e, pdfE, leE);
            float cosi = dot(n, wi);
            if (DEFER && pdfE > 0.0f && cosi > 0.0f) {
                float pl = pEnvHere * pdfE;
                V3 wiL = v3(dot(wi, T), dot(wi, B), cosi);
                float qb = reflectivePdf(surf, woL, wiL);
                float wl = pl * pl / (pl * pl + qb * qb);
                Lobes l = evalLobes(c, surf, woL, wiL);
                req->valid = true;
                req->o = p;
                req->d = wi;
                req->tmax = 1.0e30f;
                req->c = thr * (l.specular + l.diffuse) * leE / pl * wl;
            } else if (pdfE > 0.0f && cosi > 0.0f) {
                bool occ = occluded(c, p, wi, 1.0e30f);
                bool track = lightingOn && depth == 0;
                if (!occ || track) {
                    float pl = pEnvHere * pdfE;
                    V3 wiL = v3(dot(wi, T), dot(wi, B), cosi);
                    float qb = reflectivePdf(surf, woL, wiL);
                    float wl = pl * pl / (pl * pl + qb * qb);
                    Lobes l = evalLobes(c, surf, woL, wiL);
                    V3 cd = thr * l.diffuse * leE / pl * wl;
                    V3 cs = thr * l.specular * leE / pl * wl;
                    if (!occ)
                        st.parts.addLight(depth, cls, thr * (l.specular + l.diffuse) * leE / pl * wl, cd, cs);
                    if (LIGHT && track) {
                        float vv = lum(cd + cs);
                        st.visTotal += vv;
                        st.visLit += occ ? 0.0f : vv;
                        if (c.p[P_VIRTUAL_LIGHT] == 0)
                            addSlot(c, pixel, 3u, cd / cosi, cs / cosi, wi, occ ? 0.0f : 1.0f, occ ? 0.0f : cosi);
                    }
                }
            }
        }

        // Lobe choice and BSDF sampling (pt_core.slang:1429-1500).
        float lobe = rng.next();
        float u1 = rng.next();
        float u2 = rng.next();
        float u3 = rng.next();
        V3 wiL = v3(0.0f, 0.0f, 1.0f);
        V3 w = v3(1.0f);
        bool ok = true;
        bool refracted = false;
        uint32_t lobeCls = 1;
        float uc = surf.coat > 0.0f ? rng.next() : 1.0f;
        float us = surf.sheenP > 0.0f ? rng.next() : 1.0f;
        if (uc < surf.coatP) {
            V3 h = sampleVndf(woL, surf.coatAlpha, u1, u2);
            float woh = dot(woL, h);
            wiL = 2.0f * woh * h - woL;
            ok = wiL.z > 0.0f;
            w = v3(fresnelDielectric(woh, 1.5f) / coatF * G1(fmaxf(wiL.z, 0.0f), surf.coatAlpha));
        } else if (us < surf.sheenP) {
            wiL = cosineLocal(u1, u2);
            V3 hh = normalize(woL + wiL);
            w = surf.sheenColor * sheenCore(woL.z, wiL.z, hh.z, surf.sheenAlpha) * PI / (wiL.z * surf.sheenP);
        } else if (lobe < metallic) {
            V3 h = sampleVndf(woL, alpha, u1, u2);
            float woh = dot(woL, h);
            wiL = 2.0f * woh * h - woL;
            ok = wiL.z > 0.0f;
            w = schlick(albedo, woh) * multiscatterFactor(c, surf, woL.z) * G1(fmaxf(wiL.z, 0.0f), alpha);
        } else if (lobe < metallic + (1.0f - metallic) * transmission) {
            V3 h = sampleVndf(woL, alpha, u1, u2);
            float woh = dot(woL, h);
            if (u3 < fresnelDielectric(woh, eta)) {
                wiL = 2.0f * woh * h - woL;
                ok = wiL.z > 0.0f;
                w = v3(G1(fmaxf(wiL.z, 0.0f), alpha) * surf.tComp);
            } else {
                float r = 1.0f / eta;
                float k = 1.0f - r * r * (1.0f - woh * woh);
                wiL = -woL * r + (r * woh - sqrtf(fmaxf(k, 0.0f))) * h;
                ok = wiL.z < 0.0f && k > 0.0f;
                refracted = true;
                lobeCls = 2;
                w = albedo * G1(fmaxf(-wiL.z, 0.0f), alpha) * r * r * surf.tComp;
            }
        } else if (u3 < fSel) {
            V3 h = sampleVndf(woL, alpha, u1, u2);
            float woh = dot(woL, h);
            wiL = 2.0f * woh * h - woL;
            ok = wiL.z > 0.0f;
            w = v3(fresnelDielectric(woh, ior) / fSel * G1(fmaxf(wiL.z, 0.0f), alpha));
        } else {
            wiL = cosineLocal(u1, u2);
            w = albedo;
            lobeCls = 0;
        }
        if (!ok) {
            alive = false;
            break;
        }
        if (depth == 0)
            cls = lobeCls;
        st.misPrev = !refracted;
        st.qPrev = refracted ? 0.0f : reflectivePdf(surf, woL, wiL);
        st.prevInst = hq.inst + 1;

        dir = normalize(wiL.x * T + wiL.y * B + wiL.z * n);
        float side = dot(dir, ng);
        if (refracted ? side >= 0.0f : side <= 0.0f) {
            alive = false;
            break;
        }
        org = hit + ng * (side > 0.0f ? 1.0e-4f : -1.0e-4f);
        thr *= w;

        if (depth >= 2) {
            float pr = clampf(fmaxf(thr.x, fmaxf(thr.y, thr.z)), 0.05f, 0.95f);
            if (rng.next() > pr) {
                alive = false;
                break;
            }
            thr /= pr;
        }
    } while (false);
    st.rng = rng.state;
    st.org = org;
    st.dir = dir;
    st.thr = thr;
    st.cls = cls;
    st.chan = chan;
    if (RESTIR && depth == 0 && st.gi) {
        // pt_core.slang:1531-1541: what the first hit gathered and what the first bounce carries on.
        c.re.s[5][pixel] = make_float4(thr.x, thr.y, thr.z, 0.0f);
        c.re.s[6][pixel] = make_float4(st.parts.total.x, st.parts.total.y, st.parts.total.z, 0.0f);
        float4 s1 = c.re.s[1][pixel];
        s1.w = st.qPrev;
        c.re.s[1][pixel] = s1;
    }
    return alive;
}

// shadePath as one called function per instantiation, for the kernels that run whole paths per
// thread (megakernel, streaming tail, batch and cache path kernels): their warps soon sit in
// different parts of the path loop, and one out-of-line copy of the shading code keeps the
// instructions they fetch fewer. Measured on the megakernel (1M-triangle workload, 1080p): 70.2
// against 58.2 Mpaths/s inlined. The wavefront's shade stages call shadePath inline.
template <bool LIGHT, bool RESTIR, bool DEFER = false, bool CACHE = false>
__device__ __noinline__ bool shadePathCall(const Ctx& c, PathState<LIGHT>& st, Hit hq, uint32_t depth, uint32_t pixel,
                                           ShadowReq* req = nullptr, CacheHook* hk = nullptr)
{
    return shadePath<LIGHT, RESTIR, DEFER, CACHE>(c, st, hq, depth, pixel, req, hk);
}

// pt_core.slang:1551-1559 (mirrored by Adaptive::active, crates/verion-gpu/src/lib.rs:154-161).
// With double-precision statistics the same test runs in double.
template <typename A>
__device__ __forceinline__ bool pixelActive(const Ctx& c, uint32_t p)
{
    const A* st = (const A*)c.stats;
    A n = st[3 * p];
    if (n < (A)c.p[P_ADAPTIVE_MIN_SPP])
        return true;
    A mean = st[3 * p + 1] / n;
    A var = (st[3 * p + 2] / n - mean * mean);
    var = (var > (A)0 ? var : (A)0) * n / (n - (A)1);
    A m = mean > (A)0.05f ? mean : (A)0.05f;
    return sqrt(var / n) > (A)pf(c, P_ADAPTIVE_THRESHOLD) * m;
}

// pt_core.slang:1620-1667: adds a finished path to its pixel's sums. Only this path's thread
// writes the pixel during a sample, so plain read-modify-writes keep the reference's order.
template <bool LIGHT, typename A, bool GI = false>
__device__ void finishPath(const Ctx& c, const PathState<LIGHT>& st, uint32_t pixel)
{
    Parts<LIGHT> parts = st.parts;
    float visLit = st.visLit;
    float visTotal = st.visTotal;
    V3 radiance = parts.total;
    if (GI && st.gi) {
        // pt_core.slang:1627-1633: a dispersive path follows one channel and is not shared.
        if (st.chan >= 0) {
            float4 s0 = c.re.s[0][pixel];
            s0.w = __uint_as_float(0u);
            c.re.s[0][pixel] = s0;
        }
        radiance = giFinish(c, radiance, pixel);
    }
    if (bad3(radiance)) {
        radiance = v3(0.0f);
        parts.zero();
        visLit = 0.0f;
        visTotal = 0.0f;
    }
    A* acc = (A*)c.accum;
    size_t o = 3 * (size_t)pixel;
    acc[o] += (A)radiance.x;
    acc[o + 1] += (A)radiance.y;
    acc[o + 2] += (A)radiance.z;
    if (c.p[P_ADAPTIVE] != 0) {
        A* s = (A*)c.stats;
        float l = lum(radiance);
        s[o] += (A)1;
        s[o + 1] += (A)l;
        s[o + 2] += (A)l * (A)l;
    }
    if (LIGHT && c.p[P_LIGHTING] != 0) {
        float* lo = c.lighting + (size_t)LIGHTING_STRIDE * pixel;
        V3 split[5] = {parts.directDiffuse, parts.indirectDiffuse, parts.specular, parts.transmission, parts.emission};
#pragma unroll
        for (int k = 0; k < 5; k++) {
            lo[3 * k] += split[k].x;
            lo[3 * k + 1] += split[k].y;
            lo[3 * k + 2] += split[k].z;
        }
        lo[15] += visLit;
        lo[16] += visTotal;
    }
}

} // namespace vgd
