// Primary-hit AOV kernels: shaders/normals.slang:41-110 (interpolated normal facing the viewer) and
// shaders/aov.slang:86-188 (albedo, depth, object / material id through the pixel centre, and
// coverage of 16 stratified rays followed through translucent surfaces). One thread per pixel.
//
// The camera record is the reference's (crates/verion-gpu/src/pack.rs:97-108): width, height,
// tan(fov/2), pad, the camera-to-world 3x4 rows, lens shift x and y.
#pragma once
#include "pt_device.cuh"

namespace vga {

using namespace vgd;

struct CameraRecord {
    float v[18];
};

// aov.slang:79-86: camera-space unit direction through pixel position (px, py), world direction in dir.
__device__ __forceinline__ V3 pixelDir(const CameraRecord& cam, float px, float py, uint32_t w, uint32_t h, float t,
                                       float aspect, V3& dir)
{
    float u = (2.0f * px / (float)w - 1.0f + cam.v[16]) * aspect * t;
    float v = (1.0f - 2.0f * py / (float)h + cam.v[17]) * t;
    V3 d = normalize(v3(u, v, -1.0f));
    float r[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
        r[k] = cam.v[4 + 4 * k] * d.x + cam.v[5 + 4 * k] * d.y + cam.v[6 + 4 * k] * d.z;
    dir = v3(r[0], r[1], r[2]);
    return d;
}

// The hit triangle's world vertices and the barycentric weights of vertices 1 and 2 at distance t.
__device__ __forceinline__ void hitGeometry(const Ctx& c, Hit hq, V3 org, V3 dir, V3& p0, V3& p1, V3& p2, float& b1,
                                            float& b2, uint32_t& i0, uint32_t& i1, uint32_t& i2)
{
    uint32_t inst = hq.inst * 16;
    uint32_t tri = __ldg(c.s.instances + inst + 1) + 3 * hq.prim;
    uint32_t vo = __ldg(c.s.instances + inst);
    i0 = __ldg(c.s.indices + tri) + vo;
    i1 = __ldg(c.s.indices + tri + 1) + vo;
    i2 = __ldg(c.s.indices + tri + 2) + vo;
    p0 = transformPoint(c, inst + 4, vertexPos(c, i0));
    p1 = transformPoint(c, inst + 4, vertexPos(c, i1));
    p2 = transformPoint(c, inst + 4, vertexPos(c, i2));
    V3 e1 = p1 - p0, e2 = p2 - p0, e3 = org + dir * hq.t - p0;
    float d11 = dot(e1, e1), d12 = dot(e1, e2), d22 = dot(e2, e2);
    float den = fmaxf(d11 * d22 - d12 * d12, 1.0e-20f);
    b1 = (d22 * dot(e3, e1) - d12 * dot(e3, e2)) / den;
    b2 = (d11 * dot(e3, e2) - d12 * dot(e3, e1)) / den;
}

// normals.slang:41-110
static __global__ void __launch_bounds__(128) aov_normals(const __grid_constant__ Ctx c, CameraRecord cam, float* out)
{
    uint32_t w = (uint32_t)cam.v[0], h = (uint32_t)cam.v[1];
    uint32_t x = blockIdx.x * 16 + (threadIdx.x & 15u), y = blockIdx.y * 8 + (threadIdx.x >> 4);
    if (x >= w || y >= h)
        return;
    float t = cam.v[2];
    float aspect = cam.v[0] / cam.v[1];
    float u = (2.0f * ((float)x + 0.5f) / (float)w - 1.0f + cam.v[16]) * aspect * t;
    float v = (1.0f - 2.0f * ((float)y + 0.5f) / (float)h + cam.v[17]) * t;
    V3 d = normalize(v3(u, v, -1.0f));
    float dr[3], orr[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        dr[r] = cam.v[4 + 4 * r] * d.x + cam.v[5 + 4 * r] * d.y + cam.v[6 + 4 * r] * d.z;
        orr[r] = cam.v[7 + 4 * r];
    }
    V3 org = v3(orr[0], orr[1], orr[2]);
    V3 dir = normalize(v3(dr[0], dr[1], dr[2]));
    Hit hq = traceClosest(c, org, dir);
    V3 n = v3(0.0f);
    if (hq.hit) {
        V3 p0, p1, p2;
        float b1, b2;
        uint32_t i0, i1, i2;
        hitGeometry(c, hq, org, dir, p0, p1, p2, b1, b2, i0, i1, i2);
        V3 ng = normalize(cross(p1 - p0, p2 - p0));
        n = ng;
        V3 nsObj = (1.0f - b1 - b2) * vertexNormal(c, i0) + b1 * vertexNormal(c, i1) + b2 * vertexNormal(c, i2);
        if (dot(nsObj, nsObj) > 1.0e-12f) {
            n = normalize(transformNormal(c, hq.inst * 16 + 4, nsObj));
            if (dot(n, ng) < 0.0f)
                n = -n;
        }
        if (dot(ng, dir) > 0.0f)
            n = -n;
    }
    size_t o = 3 * ((size_t)y * w + x);
    out[o] = n.x;
    out[o + 1] = n.y;
    out[o + 2] = n.z;
}

// aov.slang:86-188
static __global__ void __launch_bounds__(128) aov_main(const __grid_constant__ Ctx c, CameraRecord cam,
                                                       float* albedo_depth, uint32_t* object_ids,
                                                       uint32_t* material_ids, float* coverage)
{
    uint32_t w = (uint32_t)cam.v[0], h = (uint32_t)cam.v[1];
    uint32_t x = blockIdx.x * 16 + (threadIdx.x & 15u), y = blockIdx.y * 8 + (threadIdx.x >> 4);
    if (x >= w || y >= h)
        return;
    float t = cam.v[2];
    float aspect = cam.v[0] / cam.v[1];
    V3 org = v3(cam.v[7], cam.v[11], cam.v[15]);
    V3 dir;
    V3 d = pixelDir(cam, (float)x + 0.5f, (float)y + 0.5f, w, h, t, aspect, dir);
    dir = normalize(dir);
    Hit hq = traceClosest(c, org, dir);
    V3 albedo = v3(0.0f);
    float depth = 0.0f;
    uint32_t id = 0, matId = 0;
    if (hq.hit) {
        uint32_t inst = hq.inst * 16;
        id = hq.inst + 1;
        uint32_t mat = __ldg(c.s.instances + inst + 2);
        matId = mat + 1;
        depth = hq.t * -d.z;
        uint32_t mi = mat * 24;
        albedo = v3(__ldg(c.s.materials + mi), __ldg(c.s.materials + mi + 1), __ldg(c.s.materials + mi + 2));
        uint32_t texBase = (uint32_t)__ldg(c.s.materials + mi + 10);
        if (texBase > 0) {
            V3 p0, p1, p2;
            float b1, b2;
            uint32_t i0, i1, i2;
            hitGeometry(c, hq, org, dir, p0, p1, p2, b1, b2, i0, i1, i2);
            float u0x = __ldg(c.s.uvs + 2 * i0), u0y = __ldg(c.s.uvs + 2 * i0 + 1);
            float u1x = __ldg(c.s.uvs + 2 * i1), u1y = __ldg(c.s.uvs + 2 * i1 + 1);
            float u2x = __ldg(c.s.uvs + 2 * i2), u2y = __ldg(c.s.uvs + 2 * i2 + 1);
            float ux = u0x + b1 * (u1x - u0x) + b2 * (u2x - u0x);
            float uy = u0y + b1 * (u1y - u0y) + b2 * (u2y - u0y);
            uint32_t ti = (texBase - 1) * 4;
            albedo *= bilinear(c, __ldg(c.s.tex_info + ti), __ldg(c.s.tex_info + ti + 1), __ldg(c.s.tex_info + ti + 2),
                               ux, uy);
        }
    }
    float cover = 0.0f;
    for (uint32_t k = 0; k < 16; k++) {
        V3 sdir;
        pixelDir(cam, (float)x + ((float)(k % 4) + 0.5f) / 4.0f, (float)y + ((float)(k / 4) + 0.5f) / 4.0f, w, h, t,
                 aspect, sdir);
        V3 so = org;
        V3 sd = normalize(sdir);
        float seen = 0.0f, through = 1.0f;
        for (uint32_t layer = 0; layer < 8 && through > 0.0f; layer++) {
            vgt::TRay r = vgt::make_ray(so, sd);
            vgt::TraceHit q = vgt::trace_bvh<false>(c.s.nodes, c.s.tris, r, 1.0e30f, c.err);
            if (!q.hit)
                break;
            float op = opacityAt(c, q.inst, q.prim, q.b1, q.b2);
            seen += through * op;
            through *= 1.0f - op;
            so = so + sd * (q.t + 1.0e-4f);
        }
        cover += seen;
    }
    size_t pixel = (size_t)y * w + x;
    coverage[pixel] = cover / 16.0f;
    albedo_depth[4 * pixel] = albedo.x;
    albedo_depth[4 * pixel + 1] = albedo.y;
    albedo_depth[4 * pixel + 2] = albedo.z;
    albedo_depth[4 * pixel + 3] = depth;
    object_ids[pixel] = id;
    material_ids[pixel] = matId;
}

} // namespace vga
