// Multi-channel OpenEXR output of a rendered frame (include/vgcuda.h vg_write_exr), restating the
// reference's writer (crates/verion-render-io/src/exr_out.rs:103-293): Beauty as R/G/B through
// the output transform, N.X/N.Y/N.Z, Albedo.*, the lighting parts, Visibility.V, Z, and the
// 32-bit integer channels ObjectId, MaterialId and SampleCount; render metadata as `verion/*`
// header attributes and the target's chromaticities. The colour conversions restate
// crates/verion-scene/src/color.rs:8-124 (the two matrices are that file's constants).
//
// The file is a single-part scanline image without compression (one scanline per chunk), little
// endian as the format prescribes; channels are stored in name order.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/vgcuda.h"

// The C ABI's error text (vg_last_error), kept by vgcuda.cu.
int vg_internal_fail(int status, const char* msg);

namespace {

// color.rs:18-28
const float REC709_TO_ACESCG[3][3] = {
    {0.613097f, 0.339523f, 0.047379f}, {0.070194f, 0.916354f, 0.013452f}, {0.020616f, 0.109570f, 0.869815f}};
const float ACESCG_TO_REC709[3][3] = {
    {1.705052f, -0.621792f, -0.083258f}, {-0.130257f, 1.140805f, -0.010548f}, {-0.024004f, -0.128969f, 1.152972f}};

void convert(int from, int to, const float* in, float* out)
{
    const float(*m)[3] = nullptr;
    if (from == VG_COLOR_LINEAR_REC709 && to == VG_COLOR_ACESCG)
        m = REC709_TO_ACESCG;
    else if (from == VG_COLOR_ACESCG && to == VG_COLOR_LINEAR_REC709)
        m = ACESCG_TO_REC709;
    if (!m) {
        out[0] = in[0], out[1] = in[1], out[2] = in[2];
        return;
    }
    for (int r = 0; r < 3; r++)
        out[r] = m[r][0] * in[0] + m[r][1] * in[1] + m[r][2] * in[2];
}

// color.rs:59-66
float luminance(int space, const float* c)
{
    if (space == VG_COLOR_ACESCG)
        return 0.272229f * c[0] + 0.674082f * c[1] + 0.053689f * c[2];
    return 0.2126f * c[0] + 0.7152f * c[1] + 0.0722f * c[2];
}

// color.rs:112-132: target primaries, then Reinhard on luminance, then the sRGB encoding.
void apply_transform(const VgOutputTransform& t, int working, const float* in, float* out)
{
    convert(working, t.target, in, out);
    if (t.tone_map == VG_TONEMAP_REINHARD) {
        float scale = 1.0f / (1.0f + std::max(luminance(t.target, out), 0.0f));
        for (int k = 0; k < 3; k++)
            out[k] *= scale;
    }
    if (t.oetf == VG_OETF_SRGB) {
        for (int k = 0; k < 3; k++) {
            float c = std::min(std::max(out[k], 0.0f), 1.0f);
            out[k] = c <= 0.0031308f ? c * 12.92f : 1.055f * std::pow(c, 1.0f / 2.4f) - 0.055f;
        }
    }
}

struct Writer {
    std::vector<unsigned char> b;
    void u8(unsigned v) { b.push_back((unsigned char)v); }
    void u32(uint32_t v)
    {
        for (int i = 0; i < 4; i++)
            u8((v >> (8 * i)) & 0xFF);
    }
    void i32(int32_t v) { u32((uint32_t)v); }
    void u64(uint64_t v)
    {
        for (int i = 0; i < 8; i++)
            u8((unsigned)((v >> (8 * i)) & 0xFF));
    }
    void f32(float f)
    {
        uint32_t u;
        memcpy(&u, &f, 4);
        u32(u);
    }
    void str0(const std::string& s)
    {
        b.insert(b.end(), s.begin(), s.end());
        u8(0);
    }
    // An attribute: name, type, byte size, then the value written by `body`.
    template <typename F>
    void attr(const std::string& name, const std::string& type, F body)
    {
        str0(name);
        str0(type);
        size_t at = b.size();
        u32(0);
        size_t start = b.size();
        body();
        uint32_t n = (uint32_t)(b.size() - start);
        for (int i = 0; i < 4; i++)
            b[at + i] = (unsigned char)((n >> (8 * i)) & 0xFF);
    }
};

struct Channel {
    std::string name;
    bool uint;
    std::vector<uint32_t> bits; // one 32-bit word per pixel
};

void add_plane(std::vector<Channel>& ch, const std::string& name, const float* v, size_t n, size_t stride,
               size_t comp)
{
    Channel c{name, false, std::vector<uint32_t>(n)};
    for (size_t i = 0; i < n; i++)
        memcpy(&c.bits[i], &v[i * stride + comp], 4);
    ch.push_back(std::move(c));
}

void add_uint(std::vector<Channel>& ch, const std::string& name, const uint32_t* v, size_t n)
{
    ch.push_back(Channel{name, true, std::vector<uint32_t>(v, v + n)});
}

const char* space_name(int s) { return s == VG_COLOR_ACESCG ? "AcesCg" : "LinearRec709"; }

} // namespace

extern "C" {

int vg_write_exr(const char* path, const VgExrFrame* f, const VgOutputTransform* t)
{
    if (!path || !f || !t)
        return vg_internal_fail(VG_ERR_INVALID, "null argument");
    size_t n = (size_t)f->width * f->height;
    if (n == 0 || !f->beauty)
        return vg_internal_fail(VG_ERR_INVALID, "invalid frame: size must be non-zero");
    int parts = 0;
    for (int k = 0; k < 5; k++)
        parts += f->lighting[k] ? 1 : 0;
    if ((parts != 0 && parts != 5) || ((parts == 5) != (f->visibility != nullptr)))
        return vg_internal_fail(VG_ERR_INVALID, "invalid frame: the lighting split needs all five parts and the visibility");
    if (t->target != VG_COLOR_LINEAR_REC709 && t->target != VG_COLOR_ACESCG)
        return vg_internal_fail(VG_ERR_INVALID, "unknown target colour space");
    std::vector<Channel> ch;
    std::vector<float> beauty(3 * n);
    for (size_t i = 0; i < n; i++)
        apply_transform(*t, f->working_space, &f->beauty[3 * i], &beauty[3 * i]);
    const char* rgb[3] = {"R", "G", "B"};
    for (int k = 0; k < 3; k++)
        add_plane(ch, rgb[k], beauty.data(), n, 3, k);
    if (f->normal) {
        const char* nn[3] = {"N.X", "N.Y", "N.Z"};
        for (int k = 0; k < 3; k++)
            add_plane(ch, nn[k], f->normal, n, 3, k);
    }
    VgOutputTransform prim = {t->target, VG_TONEMAP_NONE, VG_OETF_LINEAR};
    auto primaries = [&](const float* src) {
        std::vector<float> out(3 * n);
        for (size_t i = 0; i < n; i++)
            apply_transform(prim, f->working_space, &src[3 * i], &out[3 * i]);
        return out;
    };
    if (f->albedo) {
        std::vector<float> a = primaries(f->albedo);
        for (int k = 0; k < 3; k++)
            add_plane(ch, std::string("Albedo.") + rgb[k], a.data(), n, 3, k);
    }
    if (parts == 5) {
        const char* names[5] = {"DirectDiffuse", "IndirectDiffuse", "Specular", "Transmission", "Emission"};
        for (int p = 0; p < 5; p++) {
            std::vector<float> a = primaries(f->lighting[p]);
            for (int k = 0; k < 3; k++)
                add_plane(ch, std::string(names[p]) + "." + rgb[k], a.data(), n, 3, k);
        }
        add_plane(ch, "Visibility.V", f->visibility, n, 1, 0);
    }
    if (f->depth)
        add_plane(ch, "Z", f->depth, n, 1, 0);
    if (f->object_id)
        add_uint(ch, "ObjectId", f->object_id, n);
    if (f->material_id)
        add_uint(ch, "MaterialId", f->material_id, n);
    if (f->sample_count)
        add_uint(ch, "SampleCount", f->sample_count, n);
    std::sort(ch.begin(), ch.end(), [](const Channel& a, const Channel& b) { return a.name < b.name; });

    bool untouched = t->tone_map == VG_TONEMAP_NONE && t->oetf == VG_OETF_LINEAR;
    bool physical = f->physical && untouched && !f->denoiser && !f->has_adaptive_threshold && !f->restir;
    static const float CHROMA[2][8] = {{0.64f, 0.33f, 0.30f, 0.60f, 0.15f, 0.06f, 0.3127f, 0.3290f},
                                       {0.713f, 0.293f, 0.165f, 0.830f, 0.128f, 0.044f, 0.32168f, 0.33767f}};
    const char* tone = t->tone_map == VG_TONEMAP_REINHARD ? "Reinhard" : "None";
    const char* oetf = t->oetf == VG_OETF_SRGB ? "Srgb" : "Linear";
    std::string transform = std::string("OutputTransform { target: ") + space_name(t->target) + ", tone_map: " + tone +
                            ", oetf: " + oetf + " }";

    Writer w;
    w.u32(20000630u); // magic 76 2f 31 01
    w.u32(2);         // version 2, single-part scanline
    int32_t xmax = (int32_t)f->width - 1, ymax = (int32_t)f->height - 1;
    w.attr("channels", "chlist", [&] {
        for (auto& c : ch) {
            w.str0(c.name);
            w.i32(c.uint ? 0 : 2); // UINT or FLOAT
            w.u8(0);               // pLinear
            w.u8(0), w.u8(0), w.u8(0);
            w.i32(1), w.i32(1);    // sampling
        }
        w.u8(0);
    });
    w.attr("chromaticities", "chromaticities", [&] {
        for (int k = 0; k < 8; k++)
            w.f32(CHROMA[t->target == VG_COLOR_ACESCG ? 1 : 0][k]);
    });
    w.attr("compression", "compression", [&] { w.u8(0); });
    w.attr("dataWindow", "box2i", [&] { w.i32(0), w.i32(0), w.i32(xmax), w.i32(ymax); });
    w.attr("displayWindow", "box2i", [&] { w.i32(0), w.i32(0), w.i32(xmax), w.i32(ymax); });
    w.attr("lineOrder", "lineOrder", [&] { w.u8(0); });
    w.attr("pixelAspectRatio", "float", [&] { w.f32(1.0f); });
    w.attr("screenWindowCenter", "v2f", [&] { w.f32(0.0f), w.f32(0.0f); });
    w.attr("screenWindowWidth", "float", [&] { w.f32(1.0f); });
    auto text = [&](const std::string& name, const std::string& v) {
        w.attr(name, "string", [&] { w.b.insert(w.b.end(), v.begin(), v.end()); });
    };
    text("verion/physical", physical ? "true" : "false");
    w.attr("verion/samples", "int", [&] { w.i32((int32_t)std::min<uint32_t>(f->samples, 0x7fffffffu)); });
    text("verion/stylizationRevision", std::to_string((unsigned long long)f->stylization_revision));
    if (f->denoiser)
        text("verion/denoiser", f->denoiser);
    if (f->has_adaptive_threshold)
        w.attr("verion/adaptiveThreshold", "float", [&] { w.f32(f->adaptive_threshold); });
    if (f->restir)
        text("verion/restir", f->restir);
    if (f->has_grade) {
        w.attr("verion/exposure", "float", [&] { w.f32(f->exposure); });
        w.attr("verion/saturation", "float", [&] { w.f32(f->saturation); });
        w.attr("verion/whiteBalance", "v3f", [&] {
            for (int k = 0; k < 3; k++)
                w.f32(f->white_balance[k]);
        });
    }
    text("verion/workingSpace", space_name(f->working_space));
    text("verion/outputTransform", transform);
    w.u8(0); // end of header

    // Offset table, then one chunk per scanline: y, byte count, the channels' values in order.
    size_t line_bytes = (size_t)f->width * 4 * ch.size();
    size_t table = w.b.size();
    uint64_t first = table + 8 * (uint64_t)f->height;
    for (uint32_t y = 0; y < f->height; y++)
        w.u64(first + (uint64_t)y * (8 + line_bytes));
    w.b.reserve(w.b.size() + (size_t)f->height * (8 + line_bytes));
    for (uint32_t y = 0; y < f->height; y++) {
        w.i32((int32_t)y);
        w.u32((uint32_t)line_bytes);
        for (auto& c : ch)
            for (uint32_t x = 0; x < f->width; x++)
                w.u32(c.bits[(size_t)y * f->width + x]);
    }
    FILE* fp = fopen(path, "wb");
    if (!fp)
        return vg_internal_fail(VG_ERR_RESOURCE, (std::string("cannot open ") + path).c_str());
    size_t wrote = fwrite(w.b.data(), 1, w.b.size(), fp);
    int closed = fclose(fp);
    if (wrote != w.b.size() || closed != 0)
        return vg_internal_fail(VG_ERR_RESOURCE, (std::string("cannot write ") + path).c_str());
    return VG_OK;
}

} // extern "C"
