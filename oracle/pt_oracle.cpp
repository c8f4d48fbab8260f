// CPU ORACLE — test infrastructure only. Not product code: only the tests, the smoke check and
// the benchmark's CPU-baseline leg load it, and only as the checker.
//
// A restatement, in plain C++, of Verion's path-tracing integrator as its Slang kernels define it:
//   shaders/include/pt_core.slang   path core (every function below cites its lines)
//   shaders/include/wf_state.slang  wavefront path state (the reference's 16 + 17 word layout)
//   shaders/pathtrace.slang         megakernel loop
//   shaders/wf_select.slang, wf_args.slang, wf_extend.slang, wf_shade.slang  wavefront stages
//   crates/verion-gpu/src/lib.rs:151-162 adaptive predicate
// ReSTIR DI keeps the reference's interleaved 80-float reservoir layout (pt_core.slang:55-63).
//
// Two instantiations: R = float reproduces the single-precision arithmetic operation by operation
// (with the shared portable elementary functions, so results are bit-comparable with a GPU build
// that also avoids FMA contraction; this file must be compiled with -ffp-contract=off), and
// R = double evaluates the same estimator in double precision for converged reference images.
//
// Ray queries: the reference uses the driver's hardware ray tracing, which has no CPU form. The
// oracle answers them with its own binary BVH (median splits, robust slab test) or by brute force
// over all triangles, with the watertight ray/triangle test of Woop, Benthin and Wald (JCGT 2013)
// and the hit rule: 0 < t < tmax, smallest t, ties to the lower global triangle index.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>
#include <vector>

#include "../verion_gb300/csrc/vg_math.h"

namespace {

// ---------------------------------------------------------------------------------------------
// Scalar helpers per precision.
inline float msin(float x) { return vgm::sinf_(x); }
inline float mcos(float x) { return vgm::cosf_(x); }
inline float macos(float x) { return vgm::acosf_(x); }
inline float matan2(float y, float x) { return vgm::atan2f_(y, x); }
inline float mpow(float x, float y) { return vgm::powf_(x, y); }
inline float mlog2(float x) { return vgm::log2f_(x); }
inline double msin(double x) { return std::sin(x); }
inline double mcos(double x) { return std::cos(x); }
inline double macos(double x) { return std::acos(x); }
inline double matan2(double y, double x) { return std::atan2(y, x); }
inline double mpow(double x, double y) { return std::pow(x, y); }
inline double mlog2(double x) { return std::log2(x); }
inline float msqrt(float x) { return sqrtf(x); }
inline double msqrt(double x) { return std::sqrt(x); }
template <class R> inline R mmax(R a, R b) { return std::fmax(a, b); }
template <class R> inline R mmin(R a, R b) { return std::fmin(a, b); }
template <class R> inline R clampR(R x, R lo, R hi) { return mmin(mmax(x, lo), hi); }
template <class R> inline R sat(R x) { return mmin(mmax(x, R(0)), R(1)); }
template <class R> inline R lerpR(R a, R b, R t) { return a + t * (b - a); }
template <class R> inline R PI_() { return R(3.14159265358979); }

inline float bitsf(uint32_t u) { return vgm::as_float(u); }
inline uint32_t fbits(float f) { return vgm::as_uint(f); }

template <class R>
struct V {
    R x, y, z;
    V() : x(0), y(0), z(0) {}
    V(R a, R b, R c) : x(a), y(b), z(c) {}
    explicit V(R s) : x(s), y(s), z(s) {}
    R operator[](int k) const { return k == 0 ? x : (k == 1 ? y : z); }
};
template <class R> V<R> operator+(V<R> a, V<R> b) { return V<R>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> V<R> operator-(V<R> a, V<R> b) { return V<R>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> V<R> operator*(V<R> a, V<R> b) { return V<R>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class R> V<R> operator*(V<R> a, R s) { return V<R>(a.x * s, a.y * s, a.z * s); }
template <class R> V<R> operator*(R s, V<R> a) { return V<R>(s * a.x, s * a.y, s * a.z); }
template <class R> V<R> operator/(V<R> a, R s) { return V<R>(a.x / s, a.y / s, a.z / s); }
template <class R> V<R> operator+(V<R> a, R s) { return V<R>(a.x + s, a.y + s, a.z + s); }
template <class R> V<R> operator+(R s, V<R> a) { return V<R>(s + a.x, s + a.y, s + a.z); }
template <class R> V<R> operator-(R s, V<R> a) { return V<R>(s - a.x, s - a.y, s - a.z); }
template <class R> V<R> operator-(V<R> a) { return V<R>(-a.x, -a.y, -a.z); }
template <class R> R dot(V<R> a, V<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> V<R> cross(V<R> a, V<R> b)
{
    return V<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class R> R length(V<R> a) { return msqrt(dot(a, a)); }
template <class R> V<R> normalize(V<R> a)
{
    R inv = R(1) / msqrt(dot(a, a));
    return a * inv;
}
template <class R> V<R> lerpV(V<R> a, V<R> b, R t) { return a + t * (b - a); }
template <class R> bool badV(V<R> a)
{
    return std::isnan(a.x) || std::isnan(a.y) || std::isnan(a.z) || std::isinf(a.x) || std::isinf(a.y) ||
           std::isinf(a.z);
}

// ---------------------------------------------------------------------------------------------
// Scene tables (the packer's layouts) and the oracle's acceleration structure.

struct Tables {
    std::vector<float> positions, uvs, vnormals, materials, emitters, emit_cdf, env_pixels, env_marginal, env_cond,
        texels;
    std::vector<uint32_t> indices, instances, lights, tex_info;
    // World-space triangles (9 floats), instance, primitive; global index = position.
    std::vector<float> tv;
    std::vector<uint32_t> tinst, tprim;
    bool translucent = false;
    // Binary BVH: per node float box lo[3], hi[3]; left/right or first/count.
    struct Node {
        float lo[3], hi[3];
        uint32_t a, b, count;
    };
    std::vector<Node> nodes;
    std::vector<uint32_t> order;
};

void build_bvh(Tables& t)
{
    uint32_t n = (uint32_t)t.tinst.size();
    t.order.resize(n);
    std::vector<float> cent(3 * (size_t)n);
    std::vector<float> blo(3 * (size_t)n), bhi(3 * (size_t)n);
    for (uint32_t i = 0; i < n; i++) {
        t.order[i] = i;
        for (int k = 0; k < 3; k++) {
            float a = t.tv[9 * (size_t)i + k], b = t.tv[9 * (size_t)i + 3 + k], c = t.tv[9 * (size_t)i + 6 + k];
            blo[3 * (size_t)i + k] = std::min(a, std::min(b, c));
            bhi[3 * (size_t)i + k] = std::max(a, std::max(b, c));
            cent[3 * (size_t)i + k] = 0.5f * (blo[3 * (size_t)i + k] + bhi[3 * (size_t)i + k]);
        }
    }
    t.nodes.clear();
    t.nodes.push_back({});
    struct Task { uint32_t id, begin, end; };
    std::vector<Task> st{{0, 0, n}};
    while (!st.empty()) {
        Task k = st.back();
        st.pop_back();
        Tables::Node& nd = t.nodes[k.id];
        for (int a = 0; a < 3; a++) {
            nd.lo[a] = INFINITY;
            nd.hi[a] = -INFINITY;
        }
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t i = k.begin; i < k.end; i++) {
            uint32_t p = t.order[i];
            for (int a = 0; a < 3; a++) {
                nd.lo[a] = std::min(nd.lo[a], blo[3 * (size_t)p + a]);
                nd.hi[a] = std::max(nd.hi[a], bhi[3 * (size_t)p + a]);
                clo[a] = std::min(clo[a], cent[3 * (size_t)p + a]);
                chi[a] = std::max(chi[a], cent[3 * (size_t)p + a]);
            }
        }
        if (k.end - k.begin <= 4) {
            nd.a = k.begin;
            nd.count = k.end - k.begin;
            continue;
        }
        int axis = 0;
        for (int a = 1; a < 3; a++)
            if (chi[a] - clo[a] > chi[axis] - clo[axis])
                axis = a;
        uint32_t mid = (k.begin + k.end) / 2;
        std::nth_element(t.order.begin() + k.begin, t.order.begin() + mid, t.order.begin() + k.end,
                         [&](uint32_t x, uint32_t y) { return cent[3 * (size_t)x + axis] < cent[3 * (size_t)y + axis]; });
        uint32_t l = (uint32_t)t.nodes.size();
        t.nodes.push_back({});
        t.nodes.push_back({});
        t.nodes[k.id].a = l;
        t.nodes[k.id].b = l + 1;
        t.nodes[k.id].count = 0;
        st.push_back({l, k.begin, mid});
        st.push_back({l + 1, mid, k.end});
    }
}

template <class R>
struct Ray {
    V<R> o, d;
    R inv[3];
    int kx, ky, kz;
    R sx, sy, sz;
};

template <class R> R robust_far();
template <> float robust_far<float>() { return 1.00000048f; }
template <> double robust_far<double>() { return 1.0000000000000009; }

template <class R>
Ray<R> make_ray(V<R> o, V<R> d)
{
    Ray<R> r;
    r.o = o;
    r.d = d;
    for (int k = 0; k < 3; k++) {
        R c = d[k];
        if (std::fabs(c) < R(1e-20f))
            c = std::copysign(R(1e-20f), c);
        r.inv[k] = R(1) / c;
    }
    R ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int kz = 0;
    if (ay > ax)
        kz = 1;
    if (az > (kz == 0 ? ax : ay))
        kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    R dz = d[kz];
    if (dz < R(0))
        std::swap(kx, ky);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.sx = d[kx] / dz;
    r.sy = d[ky] / dz;
    r.sz = R(1) / dz;
    return r;
}

// Woop, Benthin, Wald 2013 watertight test; t = T / det.
template <class R>
bool tri_test(const Ray<R>& r, const float* tv, R& t, R& b1, R& b2)
{
    V<R> v0(tv[0], tv[1], tv[2]), v1(tv[3], tv[4], tv[5]), v2(tv[6], tv[7], tv[8]);
    V<R> A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    R Akz = A[r.kz], Bkz = B[r.kz], Ckz = C[r.kz];
    R Ax = A[r.kx] - r.sx * Akz;
    R Ay = A[r.ky] - r.sy * Akz;
    R Bx = B[r.kx] - r.sx * Bkz;
    R By = B[r.ky] - r.sy * Bkz;
    R Cx = C[r.kx] - r.sx * Ckz;
    R Cy = C[r.ky] - r.sy * Ckz;
    R U = Cx * By - Cy * Bx;
    R Vv = Ax * Cy - Ay * Cx;
    R W = Bx * Ay - By * Ax;
    if (U == R(0) || Vv == R(0) || W == R(0)) {
        double cxby = (double)Cx * (double)By, cybx = (double)Cy * (double)Bx;
        double axcy = (double)Ax * (double)Cy, aycx = (double)Ay * (double)Cx;
        double bxay = (double)Bx * (double)Ay, byax = (double)By * (double)Ax;
        U = (R)(cxby - cybx);
        Vv = (R)(axcy - aycx);
        W = (R)(bxay - byax);
    }
    if ((U < R(0) || Vv < R(0) || W < R(0)) && (U > R(0) || Vv > R(0) || W > R(0)))
        return false;
    R det = U + Vv + W;
    if (det == R(0))
        return false;
    R Az = r.sz * Akz, Bz = r.sz * Bkz, Cz = r.sz * Ckz;
    R T = U * Az + Vv * Bz + W * Cz;
    t = T / det;
    b1 = Vv / det;
    b2 = W / det;
    return t > R(0);
}

template <class R>
struct QHit {
    bool hit = false;
    uint32_t inst = 0, prim = 0, gid = 0xffffffffu;
    R t = 0, b1 = 0, b2 = 0;
};

// The far side is widened by the slab test's rounding bound (robust_far). The closest hit so far
// (tmax) is widened by 2^-18 relative as well: the triangle test computes its t with roundings of
// its own, so a triangle whose computed t is below the best one can sit in a box whose computed
// entry is a few ulps above it (a flat box in the plane of the hit, e.g. a floor made of many
// triangles). Culling is only a shortcut here, so the margin costs speed, never a hit.
template <class R>
bool box_hit(const Ray<R>& r, const float* lo, const float* hi, R tmax)
{
    R tn = R(0), tf = INFINITY;
    for (int k = 0; k < 3; k++) {
        R t0 = (R(lo[k]) - r.o[k]) * r.inv[k];
        R t1 = (R(hi[k]) - r.o[k]) * r.inv[k];
        if (t0 > t1)
            std::swap(t0, t1);
        tn = mmax(tn, t0);
        tf = mmin(tf, t1);
    }
    tf = mmin(tf * robust_far<R>(), tmax * R(1.0 + 1.0 / 262144.0));
    return tn <= tf;
}

template <class R>
inline bool better(const QHit<R>& h, R t, uint32_t gid, R best)
{
    return t < best || (h.hit && t == best && gid < h.gid);
}

// Closest (any = false) or first found (any = true) hit with 0 < t < tmax.
template <class R>
QHit<R> trace(const Tables& T, V<R> o, V<R> d, R tmax, bool any, bool brute)
{
    Ray<R> r = make_ray(o, d);
    QHit<R> h;
    R best = tmax;
    auto test = [&](uint32_t g) -> bool {
        R t, b1, b2;
        if (tri_test(r, &T.tv[9 * (size_t)g], t, b1, b2)) {
            if (any ? t < tmax : better(h, t, g, best)) {
                h.hit = true;
                h.t = t;
                best = t;
                h.gid = g;
                h.inst = T.tinst[g];
                h.prim = T.tprim[g];
                h.b1 = b1;
                h.b2 = b2;
                return any;
            }
        }
        return false;
    };
    if (brute || T.nodes.empty()) {
        for (uint32_t g = 0; g < T.tinst.size(); g++)
            if (test(g))
                return h;
        return h;
    }
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const Tables::Node& nd = T.nodes[stack[--sp]];
        if (!box_hit(r, nd.lo, nd.hi, best))
            continue;
        if (nd.count > 0) {
            for (uint32_t i = 0; i < nd.count; i++)
                if (test(T.order[nd.a + i]))
                    return h;
        } else {
            stack[sp++] = nd.b;
            stack[sp++] = nd.a;
        }
    }
    return h;
}

// ---------------------------------------------------------------------------------------------
// The integrator (pt_core.slang), parameterised by precision.

constexpr uint32_t LIGHTING_STRIDE = 65, SLOT_WORDS = 12;
constexpr uint32_t GGX_N = 32, SHEEN_N = 16, DIEL_N = 16, DIEL_N_IOR = 9;
constexpr uint32_t ALBEDO_GGX = 0, ALBEDO_SHEEN = GGX_N * GGX_N, ALBEDO_DIEL = ALBEDO_SHEEN + SHEEN_N * SHEEN_N;
constexpr uint32_t ALBEDO_WORDS = ALBEDO_DIEL + DIEL_N * DIEL_N * DIEL_N_IOR * 2;
constexpr uint32_t RESTIR_HALF = 28, RESTIR_STRIDE = 80;
constexpr int RESTIR_RADIUS = 6;
constexpr uint32_t RESTIR_NEIGHBOURS = 2;

// pt_core.slang:69-84
inline uint32_t pcg(uint32_t v)
{
    uint32_t s = v * 747796405u + 2891336453u;
    uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}

template <class R>
struct Rng {
    uint32_t state;
    R next()
    {
        state = pcg(state);
        return R((float)(state >> 8) * (1.0f / 16777216.0f));
    }
};

template <class R>
struct Parts {
    V<R> total, directDiffuse, indirectDiffuse, specular, transmission, emission;
    void file(uint32_t depth, uint32_t cls, V<R> c)
    {
        if (depth == 0)
            emission = emission + c;
        else if (cls == 0)
            indirectDiffuse = indirectDiffuse + c;
        else if (cls == 1)
            specular = specular + c;
        else
            transmission = transmission + c;
    }
    void add(uint32_t depth, uint32_t cls, V<R> c)
    {
        total = total + c;
        file(depth, cls, c);
    }
    void addLight(uint32_t depth, uint32_t cls, V<R> c, V<R> cd, V<R> cs)
    {
        total = total + c;
        if (depth == 0) {
            directDiffuse = directDiffuse + cd;
            specular = specular + cs;
        } else
            file(depth, cls, cd + cs);
    }
};

template <class R>
struct PathState {
    V<R> org, dir, thr;
    uint32_t rng = 0, cls = 0;
    int chan = -1;
    R pathLen = 0;
    bool misPrev = false, gi = false, restir = false;
    R qPrev = 0;
    uint32_t prevInst = 0;
    R visLit = 0, visTotal = 0;
    Parts<R> parts;
};

template <class R>
struct HitRec {
    bool hit;
    uint32_t inst, prim;
    R t;
};

template <class R>
struct Surface {
    V<R> albedo;
    R metallic, alpha, transmission, ior, eta, fSel, tComp, coat, coatAlpha;
    V<R> sheenColor;
    R sheenAlpha, sheenP, coatP;
};

template <class R>
struct Lobes {
    V<R> diffuse, specular;
};

template <class R>
struct Job {
    const Tables* T;
    const uint32_t* params;
    void* accum; // R-typed sums: float for parity, double for converged (see Acc)
    void* stats;
    float* lighting;
    float* restir;
    bool acc64;
    bool brute;
};

template <class R>
struct PT {
    const Tables& T;
    const uint32_t* P;
    const Job<R>& J;

    R pf(int i) const { return R(bitsf(P[i])); }
    R fm(uint32_t i) const { return R(T.materials[i]); }
    R lwf(uint32_t i) const { return R(bitsf(T.lights[i])); }
    R iwf(uint32_t i) const { return R(bitsf(T.instances[i])); }
    R em(uint32_t i) const { return R(T.emitters[i]); }

    V<R> vertexPos(uint32_t v) const { return V<R>(T.positions[3 * v], T.positions[3 * v + 1], T.positions[3 * v + 2]); }
    V<R> vertexNormal(uint32_t v) const { return V<R>(T.vnormals[3 * v], T.vnormals[3 * v + 1], T.vnormals[3 * v + 2]); }

    // pt_core.slang:90-99
    V<R> transformPoint(uint32_t base, V<R> p) const
    {
        R r[3];
        for (uint32_t row = 0; row < 3; row++) {
            uint32_t o = base + 4 * row;
            r[row] = iwf(o) * p.x + iwf(o + 1) * p.y + iwf(o + 2) * p.z + iwf(o + 3);
        }
        return V<R>(r[0], r[1], r[2]);
    }

    // pt_core.slang:103-111
    V<R> transformNormal(uint32_t base, V<R> n) const
    {
        V<R> r0(iwf(base), iwf(base + 1), iwf(base + 2));
        V<R> r1(iwf(base + 4), iwf(base + 5), iwf(base + 6));
        V<R> r2(iwf(base + 8), iwf(base + 9), iwf(base + 10));
        V<R> c0 = cross(r1, r2);
        R s = dot(r0, c0) < R(0) ? R(-1) : R(1);
        return s * V<R>(dot(c0, n), dot(cross(r2, r0), n), dot(cross(r0, r1), n));
    }

    // pt_core.slang:115-120
    static V<R> cosineLocal(R u1, R u2)
    {
        R r = msqrt(u1);
        R phi = R(2) * PI_<R>() * u2;
        return V<R>(r * mcos(phi), r * msin(phi), msqrt(mmax(R(0), R(1) - u1)));
    }

    // pt_core.slang:122-134
    static R G1(R cosT, R alpha)
    {
        R c2 = cosT * cosT;
        R tan2 = (R(1) - c2) / mmax(c2, R(1.0e-8f));
        return R(2) / (R(1) + msqrt(R(1) + alpha * alpha * tan2));
    }
    static R D(R hz, R alpha)
    {
        R a2 = alpha * alpha;
        R d = hz * hz * (a2 - R(1)) + R(1);
        return a2 / (PI_<R>() * d * d);
    }

    // pt_core.slang:136-153
    static V<R> schlick(V<R> f0, R c)
    {
        R m = R(1) - sat(c);
        R m2 = m * m;
        return f0 + (R(1) - f0) * (m2 * m2 * m);
    }
    static R fresnelDielectric(R cosi, R eta)
    {
        R s2 = (R(1) - cosi * cosi) / (eta * eta);
        if (s2 >= R(1))
            return R(1);
        R cost = msqrt(R(1) - s2);
        R rs = (cosi - eta * cost) / (cosi + eta * cost);
        R rp = (eta * cosi - cost) / (eta * cosi + cost);
        return R(0.5f) * (rs * rs + rp * rp);
    }

    // pt_core.slang:155-160
    static void basis(V<R> n, V<R>& t, V<R>& b)
    {
        V<R> a = std::fabs(n.x) > R(0.9f) ? V<R>(0, 1, 0) : V<R>(1, 0, 0);
        b = normalize(cross(n, a));
        t = cross(b, n);
    }

    // pt_core.slang:163-177
    static V<R> sampleVndf(V<R> wo, R alpha, R u1, R u2)
    {
        V<R> vh = normalize(V<R>(alpha * wo.x, alpha * wo.y, wo.z));
        R lensq = vh.x * vh.x + vh.y * vh.y;
        V<R> t1 = lensq > R(0) ? V<R>(-vh.y, vh.x, R(0)) * (R(1) / msqrt(lensq)) : V<R>(1, 0, 0);
        V<R> t2 = cross(vh, t1);
        R r = msqrt(u1);
        R phi = R(2) * PI_<R>() * u2;
        R a = r * mcos(phi);
        R b = r * msin(phi);
        R s = R(0.5f) * (R(1) + vh.z);
        b = (R(1) - s) * msqrt(R(1) - a * a) + s * b;
        V<R> nh = a * t1 + b * t2 + msqrt(mmax(R(0), R(1) - a * a - b * b)) * vh;
        return normalize(V<R>(alpha * nh.x, alpha * nh.y, mmax(R(0), nh.z)));
    }

    static R lum(V<R> c) { return dot(c, V<R>(R(0.2126f), R(0.7152f), R(0.0722f))); }

    // pt_core.slang:192-195
    R albedoAt(uint32_t i) const { return lwf(P[5] * 16 + i); }
    uint32_t recvMask(uint32_t inst) const { return T.lights[P[5] * 16 + ALBEDO_WORDS + 2 * inst]; }
    uint32_t emitMask(uint32_t inst) const { return T.lights[P[5] * 16 + ALBEDO_WORDS + 2 * inst + 1]; }

    // pt_core.slang:199-216
    R iesFactor(uint32_t po, V<R> d) const
    {
        V<R> l(dot(d, V<R>(lwf(po), lwf(po + 1), lwf(po + 2))), dot(d, V<R>(lwf(po + 3), lwf(po + 4), lwf(po + 5))),
               dot(d, V<R>(lwf(po + 6), lwf(po + 7), lwf(po + 8))));
        R th = macos(clampR(-l.z, R(-1), R(1))) * R(57.29578f);
        R ph = matan2(l.y, l.x) * R(57.29578f);
        if (ph < R(0))
            ph += R(360);
        uint32_t i = std::min((uint32_t)th, 179u);
        uint32_t j = std::min((uint32_t)ph, 359u);
        R ft = th - R(i);
        R fp = ph - R(j);
        uint32_t t = po + 9;
        R a0 = lerpR(lwf(t + j * 181 + i), lwf(t + j * 181 + i + 1), ft);
        R a1 = lerpR(lwf(t + (j + 1) * 181 + i), lwf(t + (j + 1) * 181 + i + 1), ft);
        return lerpR(a0, a1, fp);
    }

    // pt_core.slang:220-239
    void addSlot(uint32_t pixel, uint32_t slot, V<R> u, V<R> s, V<R> wi, R lit, R r) const
    {
        if (badV(u) || badV(s))
            return;
        float* L = J.lighting + (size_t)LIGHTING_STRIDE * pixel + 17 + SLOT_WORDS * slot;
        R w = lum(u);
        R wd = w + lum(s);
        R v[12] = {u.x, u.y, u.z, w, w * r, s.x, s.y, s.z, wd * wi.x, wd * wi.y, wd * wi.z, wd * lit};
        for (int k = 0; k < 12; k++)
            L[k] = (float)(R(L[k]) + v[k]);
    }

    // pt_core.slang:241-306
    V<R> envTexel(uint32_t i, uint32_t j) const
    {
        uint32_t o = 3 * (j * P[24] + i);
        return V<R>(T.env_pixels[o], T.env_pixels[o + 1], T.env_pixels[o + 2]);
    }
    void envCoords(V<R> d, uint32_t& i, uint32_t& j) const
    {
        uint32_t w = P[24], h = P[25];
        R u = matan2(d.x, -d.z) * (R(0.5f) / PI_<R>()) + R(0.5f);
        R v = macos(clampR(d.y, R(-1), R(1))) / PI_<R>();
        i = std::min((uint32_t)(u * R(w)), w - 1);
        j = std::min((uint32_t)(v * R(h)), h - 1);
    }
    V<R> envRadiance(V<R> d) const
    {
        uint32_t i, j;
        envCoords(d, i, j);
        return envTexel(i, j);
    }
    R envPdf(V<R> d) const
    {
        uint32_t i, j;
        envCoords(d, i, j);
        return lum(envTexel(i, j)) * pf(26);
    }
    V<R> envSample(R u1, R u2, R u3, R u4, R& pdf, V<R>& le) const
    {
        uint32_t w = P[24], h = P[25];
        uint32_t lo = 0, hi = h - 1;
        while (lo < hi) {
            uint32_t mid = (lo + hi) / 2;
            if (R(T.env_marginal[mid]) >= u1)
                hi = mid;
            else
                lo = mid + 1;
        }
        uint32_t j = lo;
        lo = 0;
        hi = w - 1;
        while (lo < hi) {
            uint32_t mid = (lo + hi) / 2;
            if (R(T.env_cond[j * w + mid]) >= u2)
                hi = mid;
            else
                lo = mid + 1;
        }
        uint32_t i = lo;
        R phi = ((R(i) + u3) / R(w) - R(0.5f)) * R(2) * PI_<R>();
        R theta = ((R(j) + u4) / R(h)) * PI_<R>();
        R st = msin(theta);
        le = envTexel(i, j);
        pdf = lum(le) * pf(26);
        return V<R>(st * msin(phi), mcos(theta), -st * mcos(phi));
    }

    // pt_core.slang:309-356
    V<R> texelAt(uint32_t base, uint32_t w, uint32_t h, int x, int y) const
    {
        uint32_t xi = (uint32_t)(((x % (int)w) + (int)w) % (int)w);
        uint32_t yi = (uint32_t)(((y % (int)h) + (int)h) % (int)h);
        uint32_t o = 3 * (base + yi * w + xi);
        return V<R>(T.texels[o], T.texels[o + 1], T.texels[o + 2]);
    }
    V<R> bilinear(uint32_t base, uint32_t w, uint32_t h, R ux, R uy) const
    {
        R fx = ux * R(w) - R(0.5f);
        R fy = uy * R(h) - R(0.5f);
        int x0 = (int)std::floor(fx);
        int y0 = (int)std::floor(fy);
        R tx = fx - R(x0);
        R ty = fy - R(y0);
        V<R> a = lerpV(texelAt(base, w, h, x0, y0), texelAt(base, w, h, x0 + 1, y0), tx);
        V<R> b = lerpV(texelAt(base, w, h, x0, y0 + 1), texelAt(base, w, h, x0 + 1, y0 + 1), tx);
        return lerpV(a, b, ty);
    }
    V<R> sampleTexture(uint32_t tex, R ux, R uy, R footprint) const
    {
        uint32_t ti = tex * 4;
        uint32_t base = T.tex_info[ti], w = T.tex_info[ti + 1], h = T.tex_info[ti + 2], levels = T.tex_info[ti + 3];
        R lod = clampR(mlog2(mmax(footprint * R(std::max(w, h)), R(1.0e-8f))), R(0), R(levels - 1));
        uint32_t l0 = (uint32_t)std::floor(lod);
        R t = lod - R(l0);
        uint32_t off = base, lw = w, lh = h;
        for (uint32_t k = 0; k < l0; k++) {
            off += lw * lh;
            lw = std::max(lw / 2, 1u);
            lh = std::max(lh / 2, 1u);
        }
        V<R> a = bilinear(off, lw, lh, ux, uy);
        if (l0 + 1 >= levels || t <= R(0))
            return a;
        off += lw * lh;
        V<R> b = bilinear(off, std::max(lw / 2, 1u), std::max(lh / 2, 1u), ux, uy);
        return lerpV(a, b, t);
    }

    // pt_core.slang:384-445
    R ggxAlbedo(R cosO, R alpha) const
    {
        R x = sat(cosO) * R(GGX_N - 1);
        R y = sat(msqrt(alpha)) * R(GGX_N - 1);
        uint32_t x0 = std::min((uint32_t)x, GGX_N - 2), y0 = std::min((uint32_t)y, GGX_N - 2);
        R fx = x - R(x0), fy = y - R(y0);
        R a = lerpR(albedoAt(ALBEDO_GGX + y0 * GGX_N + x0), albedoAt(ALBEDO_GGX + y0 * GGX_N + x0 + 1), fx);
        R b = lerpR(albedoAt(ALBEDO_GGX + (y0 + 1) * GGX_N + x0), albedoAt(ALBEDO_GGX + (y0 + 1) * GGX_N + x0 + 1), fx);
        return lerpR(a, b, fy);
    }
    V<R> multiscatterFactor(const Surface<R>& s, R cosO) const
    {
        if (P[29] == 0)
            return V<R>(R(1));
        return R(1) + s.albedo * (R(1) / mmax(ggxAlbedo(cosO, s.alpha), R(0.05f)) - R(1));
    }
    R dielectricAlbedo(R cosO, R rough, R ior, bool outside) const
    {
        R x = sat(cosO) * R(DIEL_N - 1);
        R y = sat(rough) * R(DIEL_N - 1);
        R z = clampR((ior - R(1)) * R(4), R(0), R(DIEL_N_IOR - 1) - R(1.0e-3f));
        uint32_t x0 = std::min((uint32_t)x, DIEL_N - 2), y0 = std::min((uint32_t)y, DIEL_N - 2), z0 = (uint32_t)z;
        R fx = x - R(x0), fy = y - R(y0), fz = z - R(z0);
        uint32_t base = (outside ? 0 : DIEL_N_IOR) * DIEL_N * DIEL_N;
        R c[2];
        for (uint32_t k = 0; k < 2; k++) {
            uint32_t o = base + ((z0 + k) * DIEL_N + y0) * DIEL_N + x0;
            R a = lerpR(albedoAt(ALBEDO_DIEL + o), albedoAt(ALBEDO_DIEL + o + 1), fx);
            R b = lerpR(albedoAt(ALBEDO_DIEL + o + DIEL_N), albedoAt(ALBEDO_DIEL + o + DIEL_N + 1), fx);
            c[k] = lerpR(a, b, fy);
        }
        return lerpR(c[0], c[1], fz);
    }
    R sheenAlbedo(R cosO, R r) const
    {
        R x = sat(cosO) * R(SHEEN_N - 1);
        R y = sat(r) * R(SHEEN_N - 1);
        uint32_t x0 = std::min((uint32_t)x, SHEEN_N - 2), y0 = std::min((uint32_t)y, SHEEN_N - 2);
        R fx = x - R(x0), fy = y - R(y0);
        R a = lerpR(albedoAt(ALBEDO_SHEEN + y0 * SHEEN_N + x0), albedoAt(ALBEDO_SHEEN + y0 * SHEEN_N + x0 + 1), fx);
        R b = lerpR(albedoAt(ALBEDO_SHEEN + (y0 + 1) * SHEEN_N + x0),
                    albedoAt(ALBEDO_SHEEN + (y0 + 1) * SHEEN_N + x0 + 1), fx);
        return lerpR(a, b, fy);
    }

    // pt_core.slang:449-455
    static R sheenCore(R woz, R wiz, R hz, R alpha)
    {
        R sinH = msqrt(mmax(R(1) - hz * hz, R(0)));
        R d = (R(2) + R(1) / alpha) * mpow(sinH, R(1) / alpha) / (R(2) * PI_<R>());
        R v = R(1) / (R(4) * (wiz + woz - wiz * woz));
        return d * v * wiz;
    }

    // pt_core.slang:459-492
    Lobes<R> evalLobes(const Surface<R>& s, V<R> woL, V<R> wiL) const
    {
        V<R> hh = normalize(woL + wiL);
        R woh = mmax(dot(woL, hh), R(0));
        R core = D(hh.z, s.alpha) * G1(woL.z, s.alpha) * G1(wiL.z, s.alpha) / (R(4) * woL.z);
        R t = s.transmission;
        Lobes<R> l;
        l.specular = s.metallic * schlick(s.albedo, woh) * multiscatterFactor(s, woL.z) * core +
                     (R(1) - s.metallic) *
                         (t * fresnelDielectric(woh, s.eta) * s.tComp + (R(1) - t) * fresnelDielectric(woh, s.ior)) * core;
        l.diffuse = (R(1) - s.metallic) * (R(1) - t) * (R(1) - s.fSel) * s.albedo * (wiL.z / PI_<R>());
        if (s.sheenP > R(0)) {
            l.specular = (R(1) - s.sheenP) * l.specular + s.sheenColor * sheenCore(woL.z, wiL.z, hh.z, s.sheenAlpha);
            l.diffuse = l.diffuse * (R(1) - s.sheenP);
        }
        if (s.coat > R(0)) {
            R coreC = D(hh.z, s.coatAlpha) * G1(woL.z, s.coatAlpha) * G1(wiL.z, s.coatAlpha) / (R(4) * woL.z);
            l.specular = (R(1) - s.coatP) * l.specular + s.coat * fresnelDielectric(woh, R(1.5f)) * coreC;
            l.diffuse = l.diffuse * (R(1) - s.coatP);
        }
        return l;
    }
    V<R> evalReflective(const Surface<R>& s, V<R> woL, V<R> wiL) const
    {
        Lobes<R> l = evalLobes(s, woL, wiL);
        return l.specular + l.diffuse;
    }

    // pt_core.slang:540-557
    static R reflectivePdf(const Surface<R>& s, V<R> woL, V<R> wiL)
    {
        V<R> hh = normalize(woL + wiL);
        R woh = mmax(dot(woL, hh), R(0));
        R spec = G1(woL.z, s.alpha) * D(hh.z, s.alpha) / (R(4) * woL.z);
        R t = s.transmission;
        R pSpec = s.metallic + (R(1) - s.metallic) * (t * fresnelDielectric(woh, s.eta) + (R(1) - t) * s.fSel);
        R pDiff = (R(1) - s.metallic) * (R(1) - t) * (R(1) - s.fSel) * wiL.z / PI_<R>();
        R q = pSpec * spec + pDiff;
        if (s.sheenP > R(0))
            q = (R(1) - s.sheenP) * q + s.sheenP * wiL.z / PI_<R>();
        if (s.coat > R(0)) {
            R specC = G1(woL.z, s.coatAlpha) * D(hh.z, s.coatAlpha) / (R(4) * woL.z);
            q = (R(1) - s.coatP) * q + s.coatP * specC;
        }
        return q;
    }

    // pt_core.slang:561-576
    R opacityAt(uint32_t instIdx, uint32_t prim, R b1, R b2) const
    {
        uint32_t mi = T.instances[instIdx * 16 + 2] * 24;
        R op = fm(mi + 22);
        uint32_t tex = (uint32_t)T.materials[mi + 23];
        if (tex > 0 && op > R(0)) {
            uint32_t tri = T.instances[instIdx * 16 + 1] + 3 * prim;
            uint32_t vo = T.instances[instIdx * 16];
            uint32_t i0 = T.indices[tri] + vo, i1 = T.indices[tri + 1] + vo, i2 = T.indices[tri + 2] + vo;
            R u0x = T.uvs[2 * i0], u0y = T.uvs[2 * i0 + 1], u1x = T.uvs[2 * i1], u1y = T.uvs[2 * i1 + 1];
            R u2x = T.uvs[2 * i2], u2y = T.uvs[2 * i2 + 1];
            R ux = u0x + b1 * (u1x - u0x) + b2 * (u2x - u0x);
            R uy = u0y + b1 * (u1y - u0y) + b2 * (u2y - u0y);
            op = op * sampleTexture(tex - 1, ux, uy, R(0)).x;
        }
        return op;
    }

    // pt_core.slang:580-613
    bool occluded(V<R> o, V<R> d, R tmax) const
    {
        for (uint32_t layer = 0; layer < 8; layer++) {
            QHit<R> q = trace<R>(T, o, d, tmax, !T.translucent, J.brute);
            if (!q.hit)
                return false;
            R opacity = opacityAt(q.inst, q.prim, q.b1, q.b2);
            if (opacity >= R(1))
                return true;
            uint32_t h = fbits((float)o.x) * 73856093u ^ fbits((float)o.y) * 19349663u ^ fbits((float)o.z) * 83492791u ^
                         fbits((float)d.x) * 2654435761u ^ fbits((float)d.y) * 40503u ^
                         fbits((float)d.z) * 2246822519u ^ layer * 3266489917u;
            h ^= h >> 16;
            h *= 0x7feb352du;
            h ^= h >> 15;
            h *= 0x846ca68bu;
            h ^= h >> 16;
            if (R((float)(h >> 8) * (1.0f / 16777216.0f)) < opacity)
                return true;
            R adv = q.t + R(1.0e-4f);
            o = o + d * adv;
            tmax -= adv;
            if (tmax <= R(0))
                return false;
        }
        return true;
    }

    // pt_core.slang:645-682
    PathState<R> generatePathFor(uint32_t px, uint32_t py, uint32_t sample) const
    {
        uint32_t w = P[0], h = P[1];
        uint32_t pixel = py * w + px;
        Rng<R> rng;
        rng.state = pcg(pixel ^ pcg(sample * 0x9E3779B9u + 0x7F4A7C15u));
        R t = pf(2);
        R aspect = R(w) / R(h);
        R u = (R(2) * (R(px) + rng.next()) / R(w) - R(1) + pf(39)) * aspect * t;
        R v = (R(1) - R(2) * (R(py) + rng.next()) / R(h) + pf(40)) * t;
        V<R> focal = V<R>(u, v, R(-1)) * pf(4);
        R lensR = pf(3) * msqrt(rng.next());
        R lensA = R(2) * PI_<R>() * rng.next();
        V<R> lens(lensR * mcos(lensA), lensR * msin(lensA), R(0));
        V<R> dc = normalize(focal - lens);
        PathState<R> s;
        R o[3], d[3];
        for (int r = 0; r < 3; r++) {
            o[r] = pf(8 + 4 * r) * lens.x + pf(9 + 4 * r) * lens.y + pf(10 + 4 * r) * lens.z + pf(11 + 4 * r);
            d[r] = pf(8 + 4 * r) * dc.x + pf(9 + 4 * r) * dc.y + pf(10 + 4 * r) * dc.z;
        }
        s.org = V<R>(o[0], o[1], o[2]);
        s.dir = normalize(V<R>(d[0], d[1], d[2]));
        s.thr = V<R>(R(1));
        s.rng = rng.state;
        return s;
    }

    // pt_core.slang:684-700
    HitRec<R> traceClosest(V<R> org, V<R> dir) const
    {
        QHit<R> q = trace<R>(T, org, dir, R(1.0e30f), false, J.brute);
        HitRec<R> h;
        h.hit = q.hit;
        h.inst = q.hit ? q.inst : 0;
        h.prim = q.hit ? q.prim : 0;
        h.t = q.hit ? q.t : R(0);
        return h;
    }

    // ReSTIR DI (pt_core.slang:702-895), reservoirs in the reference's AoS layout.
    static uint32_t restirBase(uint32_t pixel, uint32_t which) { return pixel * RESTIR_STRIDE + which * RESTIR_HALF; }
    R rr(uint32_t i) const { return R(J.restir[i]); }
    uint32_t ru(uint32_t i) const { return fbits(J.restir[i]); }
    void rw(uint32_t i, R v) const { J.restir[i] = (float)v; }
    void rwu(uint32_t i, uint32_t v) const { J.restir[i] = bitsf(v); }

    bool restirLight(uint32_t e, uint32_t recv, V<R> x, V<R> p, V<R> n, V<R>& wi, R& dist, R& cosi, V<R>& g,
                     R& plsa) const
    {
        uint32_t o = e * 16;
        V<R> a(em(o), em(o + 1), em(o + 2)), b(em(o + 3), em(o + 4), em(o + 5)), c(em(o + 6), em(o + 7), em(o + 8));
        V<R> toL = x - p;
        R d2 = dot(toL, toL);
        dist = msqrt(d2);
        wi = toL / mmax(dist, R(1.0e-6f));
        R cosl = std::fabs(dot(normalize(cross(b - a, c - a)), wi));
        cosi = dot(n, wi);
        g = V<R>(em(o + 9), em(o + 10), em(o + 11)) * (cosl / mmax(d2, R(1.0e-12f)));
        plsa = em(o + 13) * d2 / (mmax(em(o + 12), R(1.0e-30f)) * mmax(cosl, R(1.0e-5f)));
        return cosi > R(0) && cosl > R(1.0e-5f) && d2 > R(1.0e-12f) && (fbits(T.emitters[o + 14]) & recv) != 0;
    }
    static R restirMis(const Surface<R>& s, V<R> woL, V<R> wiL, R plsa)
    {
        R qb = reflectivePdf(s, woL, wiL);
        return plsa * plsa / mmax(plsa * plsa + qb * qb, R(1.0e-30f));
    }
    struct Pick {
        bool valid;
        uint32_t e;
        V<R> x;
        R W;
        bool occ;
    };
    Pick restirDI(uint32_t pixel, uint32_t recv, V<R> p, V<R> n, R pHitT, const Surface<R>& surf, V<R> Tt, V<R> B,
                  V<R> woL, Rng<R>& rng) const
    {
        uint32_t w = P[0];
        uint32_t cur = P[6] & 1u;
        uint32_t emitterCount = P[23];
        R cap = R(std::max(P[38], 1u));
        R wsum = 0, mTotal = 0;
        uint32_t selE = 0;
        V<R> selX;
        R selPhat = 0;
        for (uint32_t k = 0; k < std::max(P[37], 1u); k++) {
            R ue = rng.next(), ua = rng.next(), ub = rng.next();
            uint32_t lo = 0, hi = emitterCount - 1;
            while (lo < hi) {
                uint32_t mid = (lo + hi) / 2;
                if (R(T.emit_cdf[mid]) >= ue)
                    hi = mid;
                else
                    lo = mid + 1;
            }
            uint32_t o = lo * 16;
            V<R> a(em(o), em(o + 1), em(o + 2)), b(em(o + 3), em(o + 4), em(o + 5)), c(em(o + 6), em(o + 7), em(o + 8));
            R su = msqrt(ua);
            V<R> x = a * (R(1) - su) + b * (su * (R(1) - ub)) + c * (su * ub);
            R area = em(o + 12);
            R q = area > R(0) ? em(o + 13) / area : R(0);
            V<R> wi, g;
            R dist, cosi, plsa;
            R phat = 0;
            if (q > R(0) && restirLight(lo, recv, x, p, n, wi, dist, cosi, g, plsa)) {
                V<R> wiL(dot(wi, Tt), dot(wi, B), cosi);
                phat = lum(evalReflective(surf, woL, wiL) * g) * restirMis(surf, woL, wiL, plsa);
            }
            R wgt = phat / mmax(q, R(1.0e-30f));
            mTotal += R(1);
            if (phat > R(0)) {
                wsum += wgt;
                if (rng.next() * wsum < wgt) {
                    selE = lo + 1;
                    selX = x;
                    selPhat = phat;
                }
            }
        }
        if (P[6] > 0) {
            int px = (int)(pixel % w), py = (int)(pixel / w);
            for (uint32_t k = 0; k < 1 + RESTIR_NEIGHBOURS; k++) {
                int nx = px, ny = py;
                if (k > 0) {
                    nx += (int)(rng.next() * R(2 * RESTIR_RADIUS + 1)) - RESTIR_RADIUS;
                    ny += (int)(rng.next() * R(2 * RESTIR_RADIUS + 1)) - RESTIR_RADIUS;
                    if (nx < 0 || ny < 0 || nx >= (int)w || ny >= (int)P[1])
                        continue;
                }
                uint32_t ro = restirBase((uint32_t)ny * w + (uint32_t)nx, cur ^ 1u);
                uint32_t ei = ru(ro);
                if (ru(ro + 14) == 0 || ei == 0)
                    continue;
                V<R> pn(rr(ro + 11), rr(ro + 12), rr(ro + 13));
                V<R> pp(rr(ro + 8), rr(ro + 9), rr(ro + 10));
                if (dot(pn, n) < R(0.9f) || length(pp - p) > R(0.05f) * mmax(pHitT, R(0.01f)))
                    continue;
                V<R> xc(rr(ro + 1), rr(ro + 2), rr(ro + 3));
                R mc = mmin(rr(ro + 5), cap);
                V<R> wi, g;
                R dist, cosi, plsa;
                R phat = 0;
                if (restirLight(ei - 1, recv, xc, p, n, wi, dist, cosi, g, plsa)) {
                    V<R> wiL(dot(wi, Tt), dot(wi, B), cosi);
                    phat = lum(evalReflective(surf, woL, wiL) * g) * restirMis(surf, woL, wiL, plsa);
                }
                R wgt = phat * rr(ro + 4) * mc;
                mTotal += mc;
                if (wgt > R(0)) {
                    wsum += wgt;
                    if (rng.next() * wsum < wgt) {
                        selE = ei;
                        selX = xc;
                        selPhat = phat;
                    }
                }
            }
        }
        Pick r;
        r.valid = selE != 0 && selPhat > R(0);
        r.e = selE;
        r.x = selX;
        r.W = r.valid ? wsum / (mTotal * selPhat) : R(0);
        r.occ = false;
        if (r.valid) {
            V<R> wi, g;
            R dist, cosi, plsa;
            restirLight(selE - 1, recv, selX, p, n, wi, dist, cosi, g, plsa);
            r.occ = occluded(p, wi, dist * (R(1) - R(1.0e-3f)));
        }
        uint32_t co = restirBase(pixel, cur);
        rwu(co, selE);
        rw(co + 1, selX.x);
        rw(co + 2, selX.y);
        rw(co + 3, selX.z);
        rw(co + 4, r.occ ? R(0) : r.W);
        rw(co + 5, mTotal);
        return r;
    }
    void restirGbuffer(uint32_t pixel, V<R> p, V<R> n) const
    {
        uint32_t co = restirBase(pixel, P[6] & 1u);
        rw(co + 8, p.x);
        rw(co + 9, p.y);
        rw(co + 10, p.z);
        rw(co + 11, n.x);
        rw(co + 12, n.y);
        rw(co + 13, n.z);
        rwu(co + 14, 1u);
    }
    void restirClear(uint32_t pixel) const
    {
        uint32_t co = restirBase(pixel, P[6] & 1u);
        rwu(co + 14, 0u);
        rwu(co + 27, 0u);
    }

    // pt_core.slang:713
    static uint32_t restirScratch(uint32_t pixel) { return pixel * RESTIR_STRIDE + 2 * RESTIR_HALF; }

    // pt_core.slang:897-981: the previous frame's second-hit samples of this pixel and its
    // neighbours, reconnected to this shading point (Jacobian of the solid-angle change), RIS over
    // them; the pick goes to the scratch words for giFinish.
    void restirGIPrepare(uint32_t pixel, V<R> p, V<R> n, R pHitT, const Surface<R>& surf, V<R> Tt, V<R> B, V<R> woL,
                         Rng<R>& rng) const
    {
        uint32_t w = P[0];
        uint32_t cur = P[6] & 1u;
        R cap = R((float)std::max(P[38], 1u));
        R wsum = 0, mTotal = 0, pSel = 0;
        V<R> cSel(R(0)), xSel(R(0)), nSel(R(0)), lSel(R(0));
        if (P[6] > 0) {
            int px = (int)(pixel % w);
            int py = (int)(pixel / w);
            for (uint32_t k = 0; k < 1 + RESTIR_NEIGHBOURS; k++) {
                int nx = px, ny = py;
                if (k > 0) {
                    nx += (int)(rng.next() * R(2 * RESTIR_RADIUS + 1)) - RESTIR_RADIUS;
                    ny += (int)(rng.next() * R(2 * RESTIR_RADIUS + 1)) - RESTIR_RADIUS;
                    if (nx < 0 || ny < 0 || nx >= (int)w || ny >= (int)P[1])
                        continue;
                }
                uint32_t ro = restirBase((uint32_t)ny * w + (uint32_t)nx, cur ^ 1u);
                if (ru(ro + 14) == 0 || ru(ro + 27) == 0)
                    continue;
                V<R> pq(rr(ro + 8), rr(ro + 9), rr(ro + 10));
                V<R> nq(rr(ro + 11), rr(ro + 12), rr(ro + 13));
                if (dot(nq, n) < R(0.9f) || length(pq - p) > R(0.05f) * mmax(pHitT, R(0.01f)))
                    continue;
                V<R> x2(rr(ro + 16), rr(ro + 17), rr(ro + 18));
                V<R> n2(rr(ro + 19), rr(ro + 20), rr(ro + 21));
                V<R> l2(rr(ro + 22), rr(ro + 23), rr(ro + 24));
                R mq = mmin(rr(ro + 26), cap);
                mTotal += mq;
                V<R> toX = x2 - p;
                R dR = length(toX);
                V<R> wi = toX / mmax(dR, R(1.0e-6f));
                R dQ = length(x2 - pq);
                R cosT = dot(n, wi);
                R cosR = std::fabs(dot(n2, wi));
                R cosQ = std::fabs(dot(n2, normalize(pq - x2)));
                if (cosT <= R(0) || dR < R(1.0e-3f) || cosR < R(1.0e-3f) || cosQ < R(1.0e-3f))
                    continue;
                R jac = (cosR / cosQ) * (dQ * dQ) / (dR * dR);
                if (jac > R(10) || jac < R(1) / R(10))
                    continue;
                V<R> c = evalReflective(surf, woL, V<R>(dot(wi, Tt), dot(wi, B), cosT)) * l2;
                R phat = lum(c);
                if (phat <= R(0) || occluded(p, wi, dR * (R(1) - R(1.0e-3f))))
                    continue;
                R wgt = phat * rr(ro + 25) * mq * jac;
                wsum += wgt;
                if (rng.next() * wsum < wgt) {
                    pSel = phat;
                    cSel = c;
                    xSel = x2;
                    nSel = n2;
                    lSel = l2;
                }
            }
        }
        uint32_t so = restirScratch(pixel);
        rw(so, wsum);
        rw(so + 1, mTotal);
        rw(so + 2, pSel);
        V<R> vs[4] = {cSel, xSel, nSel, lSel};
        for (int q = 0; q < 4; q++) {
            rw(so + 3 + 3 * q, vs[q].x);
            rw(so + 4 + 3 * q, vs[q].y);
            rw(so + 5 + 3 * q, vs[q].z);
        }
        rwu(so + 22, 0u);
    }

    // pt_core.slang:1566-1617: the path's own candidate joins the resampled ones; the pixel gets
    // its direct light plus the indirect light of the pick; the new reservoir goes to this frame's
    // half.
    V<R> giFinish(V<R> pathTotal, uint32_t pixel) const
    {
        uint32_t co = restirBase(pixel, P[6] & 1u);
        uint32_t so = restirScratch(pixel);
        R wsum = rr(so);
        R m = rr(so + 1) + R(1);
        R pSel = rr(so + 2);
        V<R> cSel(rr(so + 3), rr(so + 4), rr(so + 5));
        V<R> xSel(rr(so + 6), rr(so + 7), rr(so + 8));
        V<R> nSel(rr(so + 9), rr(so + 10), rr(so + 11));
        V<R> lSel(rr(so + 12), rr(so + 13), rr(so + 14));
        V<R> thr1(rr(so + 15), rr(so + 16), rr(so + 17));
        V<R> d0(rr(so + 18), rr(so + 19), rr(so + 20));
        R qPrev = rr(so + 21);
        bool own = ru(so + 22) != 0 && qPrev > R(0);
        V<R> giTotal = pathTotal - d0;
        V<R> result = d0;
        if (own) {
            V<R> cOwn = giTotal * qPrev;
            R pOwn = lum(cOwn);
            if (pOwn > R(0)) {
                R wOwn = pOwn / qPrev;
                wsum += wOwn;
                Rng<R> r;
                r.state = pcg(pixel ^ pcg(P[6] * 0x85EBCA6Bu + 0x1234u));
                if (r.next() * wsum < wOwn) {
                    pSel = pOwn;
                    cSel = cOwn;
                    xSel = V<R>(rr(co + 16), rr(co + 17), rr(co + 18));
                    nSel = V<R>(rr(co + 19), rr(co + 20), rr(co + 21));
                    lSel = V<R>(thr1.x > R(1.0e-6f) ? giTotal.x / thr1.x : R(0),
                                thr1.y > R(1.0e-6f) ? giTotal.y / thr1.y : R(0),
                                thr1.z > R(1.0e-6f) ? giTotal.z / thr1.z : R(0));
                }
            }
        } else
            result = result + giTotal;
        R W = pSel > R(0) ? wsum / (m * pSel) : R(0);
        result = result + cSel * W;
        V<R> vs[3] = {xSel, nSel, lSel};
        for (int q = 0; q < 3; q++) {
            rw(co + 16 + 3 * q, vs[q].x);
            rw(co + 17 + 3 * q, vs[q].y);
            rw(co + 18 + 3 * q, vs[q].z);
        }
        rw(co + 25, W);
        rw(co + 26, m);
        rwu(co + 27, pSel > R(0) ? 1u : 0u);
        return result;
    }

    // pt_core.slang:992-1543
    bool shadePath(PathState<R>& st, HitRec<R> hq, uint32_t depth, uint32_t pixel) const
    {
        const R PI = PI_<R>();
        V<R> sky(pf(20), pf(21), pf(22));
        bool lightingOn = P[28] != 0;
        uint32_t lightCount = P[5], emitterCount = P[23];
        bool hasEnv = P[24] > 0;
        R pEnv = hasEnv ? (emitterCount > 0 ? R(0.5f) : R(1)) : R(0);
        Rng<R> rng;
        rng.state = st.rng;
        V<R> org = st.org, dir = st.dir, thr = st.thr;
        uint32_t cls = st.cls;
        int chan = st.chan;
        bool alive = true;
        for (uint32_t once = 0; once < 1; once++) {
            if (!hq.hit) {
                if (depth == 0 && P[36] != 0)
                    restirClear(pixel);
                if (depth == 0 && P[42] != 0) {
                    alive = false;
                    break;
                }
                st.parts.add(depth, cls, thr * sky);
                if (hasEnv) {
                    R wB = 1;
                    if (st.misPrev) {
                        R pl = (st.restir && depth == 1 ? R(1) : pEnv) * envPdf(dir);
                        R den = st.qPrev * st.qPrev + pl * pl;
                        wB = den > R(0) ? st.qPrev * st.qPrev / den : R(1);
                    }
                    st.parts.add(depth, cls, thr * envRadiance(dir) * wB);
                }
                alive = false;
                break;
            }
            uint32_t inst = hq.inst * 16;
            uint32_t tri = T.instances[inst + 1] + 3 * hq.prim;
            uint32_t vo = T.instances[inst];
            uint32_t i0 = T.indices[tri] + vo, i1 = T.indices[tri + 1] + vo, i2 = T.indices[tri + 2] + vo;
            V<R> p0 = transformPoint(inst + 4, vertexPos(i0));
            V<R> p1 = transformPoint(inst + 4, vertexPos(i1));
            V<R> p2 = transformPoint(inst + 4, vertexPos(i2));
            V<R> nOut = normalize(cross(p1 - p0, p2 - p0));
            V<R> wo = -dir;
            bool outside = dot(nOut, wo) > R(0);
            V<R> ng = outside ? nOut : -nOut;
            R pHitT = hq.t;
            st.pathLen += pHitT;
            V<R> hit = org + dir * pHitT;
            V<R> e1 = p1 - p0, e2 = p2 - p0, e3 = hit - p0;
            R d11 = dot(e1, e1), d12 = dot(e1, e2), d22 = dot(e2, e2);
            R den = mmax(d11 * d22 - d12 * d12, R(1.0e-20f));
            R b1 = (d22 * dot(e3, e1) - d12 * dot(e3, e2)) / den;
            R b2 = (d11 * dot(e3, e2) - d12 * dot(e3, e1)) / den;
            R opacity = opacityAt(hq.inst, hq.prim, b1, b2);
            if (opacity < R(1) && rng.next() >= opacity) {
                org = hit + dir * R(1.0e-4f);
                break;
            }
            V<R> p = hit + ng * R(1.0e-4f);
            if (depth == 1 && st.gi) {
                // pt_core.slang:1072-1082: the first bounce's surface is ReSTIR GI's candidate.
                uint32_t co = restirBase(pixel, P[6] & 1u);
                rw(co + 16, hit.x), rw(co + 17, hit.y), rw(co + 18, hit.z);
                rw(co + 19, ng.x), rw(co + 20, ng.y), rw(co + 21, ng.z);
                rwu(restirScratch(pixel) + 22, 1u);
            }
            V<R> nsObj = (R(1) - b1 - b2) * vertexNormal(i0) + b1 * vertexNormal(i1) + b2 * vertexNormal(i2);
            V<R> ns = nOut;
            if (dot(nsObj, nsObj) > R(1.0e-12f)) {
                ns = normalize(transformNormal(inst + 4, nsObj));
                if (dot(ns, nOut) < R(0))
                    ns = -ns;
            }
            V<R> n = outside ? ns : -ns;
            uint32_t mi = T.instances[inst + 2] * 24;
            V<R> albedo(fm(mi), fm(mi + 1), fm(mi + 2));
            uint32_t texBase = (uint32_t)T.materials[mi + 10], texMR = (uint32_t)T.materials[mi + 11];
            uint32_t texEm = (uint32_t)T.materials[mi + 12], texNm = (uint32_t)T.materials[mi + 13];
            R texRx = 1, texRy = 1;
            V<R> texEmission(R(1));
            if (texBase + texMR + texEm + texNm > 0) {
                R u0x = T.uvs[2 * i0], u0y = T.uvs[2 * i0 + 1], u1x = T.uvs[2 * i1], u1y = T.uvs[2 * i1 + 1];
                R u2x = T.uvs[2 * i2], u2y = T.uvs[2 * i2 + 1];
                R ux = u0x + b1 * (u1x - u0x) + b2 * (u2x - u0x);
                R uy = u0y + b1 * (u1y - u0y) + b2 * (u2y - u0y);
                R d1x = u1x - u0x, d1y = u1y - u0y, d2x = u2x - u0x, d2y = u2y - u0y;
                R uvPerWorld = msqrt(std::fabs(d1x * d2y - d1y * d2x) / mmax(length(cross(e1, e2)), R(1.0e-20f)));
                R footprint = st.pathLen * pf(27) / mmax(std::fabs(dot(nOut, dir)), R(0.1f)) * uvPerWorld;
                if (texBase > 0)
                    albedo = albedo * sampleTexture(texBase - 1, ux, uy, footprint);
                if (texMR > 0) {
                    V<R> t = sampleTexture(texMR - 1, ux, uy, footprint);
                    texRx = t.y;
                    texRy = t.z;
                }
                if (texEm > 0)
                    texEmission = sampleTexture(texEm - 1, ux, uy, footprint);
                if (texNm > 0) {
                    R det = d1x * d2y - d2x * d1y;
                    V<R> dPdu = (e1 * d2y - e2 * d1y) / det;
                    V<R> dPdv = (e2 * d1x - e1 * d2x) / det;
                    V<R> tg = dPdu - ns * dot(ns, dPdu);
                    if (std::fabs(det) > R(1.0e-20f) && dot(tg, tg) > R(1.0e-20f)) {
                        tg = normalize(tg);
                        V<R> bt = cross(ns, tg);
                        if (dot(bt, dPdv) > R(0))
                            bt = -bt;
                        V<R> nt = sampleTexture(texNm - 1, ux, uy, footprint) * R(2) + R(-1);
                        R scale = fm(mi + 14);
                        ns = normalize(nt.x * scale * tg + nt.y * scale * bt + nt.z * ns);
                        n = outside ? ns : -ns;
                    }
                }
            }
            R woN = dot(n, wo);
            if (woN < R(0.05f))
                n = normalize(n + wo * (R(0.05f) - woN));
            V<R> le = V<R>(fm(mi + 3), fm(mi + 4), fm(mi + 5)) * texEmission;
            if (st.prevInst != 0 && (emitMask(hq.inst) & recvMask(st.prevInst - 1)) == 0)
                le = V<R>(R(0));
            if (le.x > R(0) || le.y > R(0) || le.z > R(0)) {
                R wB = 1;
                uint32_t eb = T.instances[inst + 3];
                if (st.misPrev && eb != 0) {
                    uint32_t e = (eb - 1 + hq.prim) * 16;
                    R cosl = mmax(std::fabs(dot(nOut, dir)), R(1.0e-4f));
                    R pl = (st.restir && depth == 1 ? R(1) : R(1) - pEnv) * em(e + 13) * pHitT * pHitT / (em(e + 12) * cosl);
                    wB = st.qPrev * st.qPrev / (st.qPrev * st.qPrev + pl * pl);
                }
                st.parts.add(depth, cls, thr * le * wB);
                if (depth == 1 && st.gi) {
                    // pt_core.slang:1161-1168: counted with what the first hit gathered itself.
                    uint32_t so = restirScratch(pixel) + 18;
                    V<R> e = thr * le * wB;
                    rw(so, rr(so) + e.x);
                    rw(so + 1, rr(so + 1) + e.y);
                    rw(so + 2, rr(so + 2) + e.z);
                }
            }
            R metallic = fm(mi + 6) * texRy, rough = fm(mi + 7) * texRx, transmission = fm(mi + 8), ior = fm(mi + 9);
            R dispersion = fm(mi + 21);
            if (dispersion > R(0) && transmission > R(0)) {
                if (chan < 0) {
                    chan = std::min((int)(rng.next() * R(3)), 2);
                    thr = thr * (R(3) * V<R>(chan == 0 ? R(1) : R(0), chan == 1 ? R(1) : R(0), chan == 2 ? R(1) : R(0)));
                }
                ior = mmax(ior + R(chan - 1) * (ior - R(1)) * R(0.025f) * dispersion, R(1));
            }
            // pt_core.slang:1187-1190: a glass second hit cannot be reconnected to.
            if (depth == 1 && st.gi && transmission > R(0))
                rwu(restirScratch(pixel) + 22, 0u);
            R alpha = mmax(rough * rough, R(1.0e-3f));
            R eta = outside ? ior : R(1) / ior;
            V<R> Tt, B;
            basis(n, Tt, B);
            V<R> woL(dot(wo, Tt), dot(wo, B), mmax(dot(wo, n), R(1.0e-4f)));
            R fSel = fresnelDielectric(woL.z, ior);
            Surface<R> surf;
            surf.albedo = albedo;
            surf.metallic = metallic;
            surf.alpha = alpha;
            surf.transmission = transmission;
            surf.ior = ior;
            surf.eta = eta;
            surf.fSel = fSel;
            surf.tComp = R(1);
            if (P[29] != 0 && transmission > R(0) && rough > R(0))
                surf.tComp = R(1) / mmax(dielectricAlbedo(woL.z, rough, ior, outside), R(0.1f));
            surf.coat = outside ? fm(mi + 15) : R(0);
            surf.coatAlpha = mmax(fm(mi + 16) * fm(mi + 16), R(1.0e-3f));
            R coatF = fresnelDielectric(woL.z, R(1.5f));
            surf.coatP = surf.coat * coatF;
            surf.sheenColor = outside ? V<R>(fm(mi + 18), fm(mi + 19), fm(mi + 20)) : V<R>(R(0));
            R sheenMax = mmax(surf.sheenColor.x, mmax(surf.sheenColor.y, surf.sheenColor.z));
            R sheenR = mmax(fm(mi + 17), R(0.07f));
            surf.sheenAlpha = sheenR * sheenR;
            surf.sheenP = sheenMax > R(0) ? sheenMax * sheenAlbedo(woL.z, sheenR) : R(0);

            // pt_core.slang:1224-1282
            for (uint32_t li = 0; li < lightCount; li++) {
                uint32_t o = li * 16;
                V<R> col = V<R>(lwf(o + 1), lwf(o + 2), lwf(o + 3)) * lwf(o + 4);
                V<R> vec(lwf(o + 5), lwf(o + 6), lwf(o + 7));
                bool virt = T.lights[o] == 3;
                if (virt && !(lightingOn && depth == 0))
                    continue;
                if ((T.lights[o + 14] & recvMask(hq.inst)) == 0)
                    continue;
                V<R> wi;
                R dist;
                V<R> li_;
                if (T.lights[o] == 1 || virt) {
                    wi = -normalize(vec);
                    dist = R(1.0e30f);
                    li_ = col;
                } else {
                    V<R> toL = vec - p;
                    R d2 = dot(toL, toL);
                    dist = msqrt(d2);
                    wi = toL / dist;
                    li_ = col / d2;
                    if (T.lights[o + 15] != 0)
                        li_ = li_ * iesFactor(T.lights[o + 15] - 1, -wi);
                    if (T.lights[o] == 2) {
                        V<R> axis(lwf(o + 8), lwf(o + 9), lwf(o + 10));
                        R att = sat(dot(axis, -wi) * lwf(o + 11) + lwf(o + 12));
                        li_ = li_ * (att * att);
                    }
                }
                R c = dot(n, wi);
                if (c > R(0)) {
                    bool occ = occluded(p, wi, dist - R(1.0e-3f));
                    bool track = lightingOn && depth == 0;
                    if (!occ || track) {
                        Lobes<R> l = evalLobes(surf, woL, V<R>(dot(wi, Tt), dot(wi, B), c));
                        V<R> cd = thr * l.diffuse * li_;
                        V<R> cs = thr * l.specular * li_;
                        if (!occ && !virt)
                            st.parts.addLight(depth, cls, thr * (l.diffuse + l.specular) * li_, cd, cs);
                        if (track) {
                            R vv = virt ? R(0) : lum(cd + cs);
                            st.visTotal += vv;
                            st.visLit += occ ? R(0) : vv;
                            addSlot(pixel, T.lights[o + 13], cd / c, cs / c, wi, occ ? R(0) : R(1), occ ? R(0) : c);
                        }
                    }
                }
            }

            // pt_core.slang:1284-1332
            bool reDI = false;
            if (depth == 0 && P[36] != 0) {
                bool suits = pf(3) == R(0) && transmission == R(0) && surf.alpha >= R(0.15f) &&
                             (surf.coat == R(0) || surf.coatAlpha >= R(0.15f));
                reDI = suits && (P[36] & 1u) != 0 && emitterCount > 0;
                bool reGI = suits && (P[36] & 2u) != 0 && !lightingOn;
                st.restir = reDI;
                st.gi = reGI;
                if (suits) {
                    restirGbuffer(pixel, p, n);
                    if (reGI)
                        restirGIPrepare(pixel, p, n, pHitT, surf, Tt, B, woL, rng);
                } else
                    restirClear(pixel);
            }
            if (reDI) {
                Pick pick = restirDI(pixel, recvMask(hq.inst), p, n, pHitT, surf, Tt, B, woL, rng);
                if (pick.valid) {
                    V<R> wi, g;
                    R dist, cosi, plsa;
                    restirLight(pick.e - 1, recvMask(hq.inst), pick.x, p, n, wi, dist, cosi, g, plsa);
                    bool track = lightingOn;
                    if (!pick.occ || track) {
                        V<R> wiL(dot(wi, Tt), dot(wi, B), cosi);
                        R wl = restirMis(surf, woL, wiL, plsa);
                        Lobes<R> l = evalLobes(surf, woL, wiL);
                        V<R> cd = thr * l.diffuse * g * (wl * pick.W);
                        V<R> cs = thr * l.specular * g * (wl * pick.W);
                        if (!pick.occ)
                            st.parts.addLight(depth, cls, cd + cs, cd, cs);
                        if (track) {
                            R vv = lum(cd + cs);
                            st.visTotal += vv;
                            st.visLit += pick.occ ? R(0) : vv;
                            addSlot(pixel, 3u, cd / cosi, cs / cosi, wi, pick.occ ? R(0) : R(1), pick.occ ? R(0) : cosi);
                        }
                    }
                }
            }

            // pt_core.slang:1334-1390
            R chooseLight = rng.next();
            R pEnvHere = reDI ? (hasEnv ? R(1) : R(0)) : pEnv;
            bool chooseEnv = hasEnv && chooseLight < pEnvHere;
            if (emitterCount > 0 && !chooseEnv && !reDI) {
                R ue = rng.next(), ua = rng.next(), ub = rng.next();
                uint32_t lo = 0, hi = emitterCount - 1;
                while (lo < hi) {
                    uint32_t mid = (lo + hi) / 2;
                    if (R(T.emit_cdf[mid]) >= ue)
                        hi = mid;
                    else
                        lo = mid + 1;
                }
                uint32_t e = lo * 16;
                V<R> a(em(e), em(e + 1), em(e + 2)), b(em(e + 3), em(e + 4), em(e + 5)), c(em(e + 6), em(e + 7), em(e + 8));
                R su = msqrt(ua);
                V<R> xl = a * (R(1) - su) + b * (su * (R(1) - ub)) + c * (su * ub);
                V<R> toL = xl - p;
                R d2 = dot(toL, toL);
                R dist = msqrt(d2);
                V<R> wi = toL / dist;
                R cosl = std::fabs(dot(normalize(cross(b - a, c - a)), wi));
                R cosi = dot(n, wi);
                if (cosi > R(0) && cosl > R(1.0e-5f) && (fbits(T.emitters[e + 14]) & recvMask(hq.inst)) != 0) {
                    bool occ = occluded(p, wi, dist * (R(1) - R(1.0e-3f)));
                    bool track = lightingOn && depth == 0;
                    if (!occ || track) {
                        R pl = (R(1) - pEnv) * em(e + 13) * d2 / (em(e + 12) * cosl);
                        V<R> wiL(dot(wi, Tt), dot(wi, B), cosi);
                        R qb = reflectivePdf(surf, woL, wiL);
                        R wl = pl * pl / (pl * pl + qb * qb);
                        V<R> lE(em(e + 9), em(e + 10), em(e + 11));
                        Lobes<R> l = evalLobes(surf, woL, wiL);
                        V<R> cd = thr * l.diffuse * lE / pl * wl;
                        V<R> cs = thr * l.specular * lE / pl * wl;
                        if (!occ)
                            st.parts.addLight(depth, cls, thr * evalReflective(surf, woL, wiL) * lE / pl * wl, cd, cs);
                        if (track) {
                            R vv = lum(cd + cs);
                            st.visTotal += vv;
                            st.visLit += occ ? R(0) : vv;
                            addSlot(pixel, 3u, cd / cosi, cs / cosi, wi, occ ? R(0) : R(1), occ ? R(0) : cosi);
                        }
                    }
                }
            }

            // pt_core.slang:1392-1427
            if (chooseEnv) {
                R a1 = rng.next(), a2 = rng.next(), a3 = rng.next(), a4 = rng.next();
                R pdfE;
                V<R> leE;
                V<R> wi = envSample(a1, a2, a3, a4, pdfE, leE);
                R cosi = dot(n, wi);
                if (pdfE > R(0) && cosi > R(0)) {
                    bool occ = occluded(p, wi, R(1.0e30f));
                    bool track = lightingOn && depth == 0;
                    if (!occ || track) {
                        R pl = pEnvHere * pdfE;
                        V<R> wiL(dot(wi, Tt), dot(wi, B), cosi);
                        R qb = reflectivePdf(surf, woL, wiL);
                        R wl = pl * pl / (pl * pl + qb * qb);
                        Lobes<R> l = evalLobes(surf, woL, wiL);
                        V<R> cd = thr * l.diffuse * leE / pl * wl;
                        V<R> cs = thr * l.specular * leE / pl * wl;
                        if (!occ)
                            st.parts.addLight(depth, cls, thr * evalReflective(surf, woL, wiL) * leE / pl * wl, cd, cs);
                        if (track) {
                            R vv = lum(cd + cs);
                            st.visTotal += vv;
                            st.visLit += occ ? R(0) : vv;
                            if (P[41] == 0)
                                addSlot(pixel, 3u, cd / cosi, cs / cosi, wi, occ ? R(0) : R(1), occ ? R(0) : cosi);
                        }
                    }
                }
            }

            // pt_core.slang:1429-1500
            R lobe = rng.next(), u1 = rng.next(), u2 = rng.next(), u3 = rng.next();
            V<R> wiL(0, 0, 1);
            V<R> w(R(1));
            bool ok = true, refracted = false;
            uint32_t lobeCls = 1;
            R uc = surf.coat > R(0) ? rng.next() : R(1);
            R us = surf.sheenP > R(0) ? rng.next() : R(1);
            if (uc < surf.coatP) {
                V<R> h = sampleVndf(woL, surf.coatAlpha, u1, u2);
                R woh = dot(woL, h);
                wiL = R(2) * woh * h - woL;
                ok = wiL.z > R(0);
                w = V<R>(fresnelDielectric(woh, R(1.5f)) / coatF * G1(mmax(wiL.z, R(0)), surf.coatAlpha));
            } else if (us < surf.sheenP) {
                wiL = cosineLocal(u1, u2);
                V<R> hh = normalize(woL + wiL);
                w = surf.sheenColor * sheenCore(woL.z, wiL.z, hh.z, surf.sheenAlpha) * PI / (wiL.z * surf.sheenP);
            } else if (lobe < metallic) {
                V<R> h = sampleVndf(woL, alpha, u1, u2);
                R woh = dot(woL, h);
                wiL = R(2) * woh * h - woL;
                ok = wiL.z > R(0);
                w = schlick(albedo, woh) * multiscatterFactor(surf, woL.z) * G1(mmax(wiL.z, R(0)), alpha);
            } else if (lobe < metallic + (R(1) - metallic) * transmission) {
                V<R> h = sampleVndf(woL, alpha, u1, u2);
                R woh = dot(woL, h);
                if (u3 < fresnelDielectric(woh, eta)) {
                    wiL = R(2) * woh * h - woL;
                    ok = wiL.z > R(0);
                    w = V<R>(G1(mmax(wiL.z, R(0)), alpha) * surf.tComp);
                } else {
                    R r = R(1) / eta;
                    R k = R(1) - r * r * (R(1) - woh * woh);
                    wiL = -woL * r + (r * woh - msqrt(mmax(k, R(0)))) * h;
                    ok = wiL.z < R(0) && k > R(0);
                    refracted = true;
                    lobeCls = 2;
                    w = albedo * G1(mmax(-wiL.z, R(0)), alpha) * r * r * surf.tComp;
                }
            } else if (u3 < fSel) {
                V<R> h = sampleVndf(woL, alpha, u1, u2);
                R woh = dot(woL, h);
                wiL = R(2) * woh * h - woL;
                ok = wiL.z > R(0);
                w = V<R>(fresnelDielectric(woh, ior) / fSel * G1(mmax(wiL.z, R(0)), alpha));
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
            st.qPrev = refracted ? R(0) : reflectivePdf(surf, woL, wiL);
            st.prevInst = hq.inst + 1;
            dir = normalize(wiL.x * Tt + wiL.y * B + wiL.z * n);
            R side = dot(dir, ng);
            if (refracted ? side >= R(0) : side <= R(0)) {
                alive = false;
                break;
            }
            org = hit + ng * (side > R(0) ? R(1.0e-4f) : R(-1.0e-4f));
            thr = thr * w;
            if (depth >= 2) {
                R pr = clampR(mmax(thr.x, mmax(thr.y, thr.z)), R(0.05f), R(0.95f));
                if (rng.next() > pr) {
                    alive = false;
                    break;
                }
                thr = thr / pr;
            }
        }
        st.rng = rng.state;
        st.org = org;
        st.dir = dir;
        st.thr = thr;
        st.cls = cls;
        st.chan = chan;
        if (depth == 0 && st.gi) {
            // pt_core.slang:1531-1541: what the first hit gathered and what the first bounce carries.
            uint32_t so = restirScratch(pixel);
            rw(so + 15, thr.x), rw(so + 16, thr.y), rw(so + 17, thr.z);
            rw(so + 18, st.parts.total.x), rw(so + 19, st.parts.total.y), rw(so + 20, st.parts.total.z);
            rw(so + 21, st.qPrev);
        }
        return alive;
    }

    // pt_core.slang:1551-1559; statistics in the sums' precision.
    template <class A>
    bool pixelActiveT(uint32_t p) const
    {
        const A* s = (const A*)J.stats;
        A n = s[3 * p];
        if (n < A(P[34]))
            return true;
        A mean = s[3 * p + 1] / n;
        A var = std::fmax(s[3 * p + 2] / n - mean * mean, A(0)) * n / (n - A(1));
        return std::sqrt(var / n) > A(bitsf(P[33])) * std::fmax(mean, A(0.05f));
    }
    bool pixelActive(uint32_t p) const { return J.acc64 ? pixelActiveT<double>(p) : pixelActiveT<float>(p); }

    // pt_core.slang:1620-1667
    template <class A>
    void finishT(const PathState<R>& st, uint32_t pixel) const
    {
        Parts<R> parts = st.parts;
        R visLit = st.visLit, visTotal = st.visTotal;
        V<R> radiance = parts.total;
        if (st.gi) {
            // pt_core.slang:1627-1633: a dispersive path follows one channel and is not shared.
            if (st.chan >= 0)
                rwu(restirScratch(pixel) + 22, 0u);
            radiance = giFinish(radiance, pixel);
        }
        if (badV(radiance)) {
            radiance = V<R>();
            parts = Parts<R>();
            visLit = visTotal = 0;
        }
        A* acc = (A*)J.accum;
        size_t o = 3 * (size_t)pixel;
        acc[o] += A(radiance.x);
        acc[o + 1] += A(radiance.y);
        acc[o + 2] += A(radiance.z);
        if (P[32] != 0) {
            A* s = (A*)J.stats;
            R l = lum(radiance);
            s[o] += A(1);
            s[o + 1] += A(l);
            s[o + 2] += A(l) * A(l);
        }
        if (P[28] != 0) {
            float* L = J.lighting + (size_t)LIGHTING_STRIDE * pixel;
            V<R> split[5] = {parts.directDiffuse, parts.indirectDiffuse, parts.specular, parts.transmission, parts.emission};
            for (int k = 0; k < 5; k++) {
                L[3 * k] = (float)(R(L[3 * k]) + split[k].x);
                L[3 * k + 1] = (float)(R(L[3 * k + 1]) + split[k].y);
                L[3 * k + 2] = (float)(R(L[3 * k + 2]) + split[k].z);
            }
            L[15] = (float)(R(L[15]) + visLit);
            L[16] = (float)(R(L[16]) + visTotal);
        }
    }
    void finishPath(const PathState<R>& st, uint32_t pixel) const
    {
        if (J.acc64)
            finishT<double>(st, pixel);
        else
            finishT<float>(st, pixel);
    }
};

template <class F>
void parallel_for(uint32_t n, int threads, F f)
{
    if (threads <= 1 || n < 64) {
        for (uint32_t i = 0; i < n; i++)
            f(i);
        return;
    }
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++)
        pool.emplace_back([&] {
            for (;;) {
                uint32_t b = next.fetch_add(64);
                if (b >= n)
                    break;
                uint32_t e = std::min(n, b + 64);
                for (uint32_t i = b; i < e; i++)
                    f(i);
            }
        });
    for (auto& th : pool)
        th.join();
}

} // namespace

// ---------------------------------------------------------------------------------------------
// C interface for the tests (ctypes).

extern "C" {

struct OrTables {
    const float* positions; size_t positions_len;
    const uint32_t* indices; size_t indices_len;
    const float* uvs; size_t uvs_len;
    const float* vnormals; size_t vnormals_len;
    const uint32_t* instances; size_t instances_len;
    const float* materials; size_t materials_len;
    const uint32_t* lights; size_t lights_len;
    const float* emitters; size_t emitters_len;
    const float* emit_cdf; size_t emit_cdf_len;
    const float* env_pixels; size_t env_pixels_len;
    const float* env_marginal; size_t env_marginal_len;
    const float* env_cond; size_t env_cond_len;
    const float* texels; size_t texels_len;
    const uint32_t* tex_info; size_t tex_info_len;
    const uint32_t* tri_counts; // triangles per instance (its mesh's index count / 3)
    size_t instance_count;
};

void* or_scene_create(const OrTables* t)
{
    Tables* T = new Tables();
    auto cpf = [](std::vector<float>& v, const float* p, size_t n) { v.assign(p, p + n); };
    auto cpu = [](std::vector<uint32_t>& v, const uint32_t* p, size_t n) { v.assign(p, p + n); };
    cpf(T->positions, t->positions, t->positions_len);
    cpu(T->indices, t->indices, t->indices_len);
    cpf(T->uvs, t->uvs, t->uvs_len);
    cpf(T->vnormals, t->vnormals, t->vnormals_len);
    cpu(T->instances, t->instances, t->instances_len);
    cpf(T->materials, t->materials, t->materials_len);
    cpu(T->lights, t->lights, t->lights_len);
    cpf(T->emitters, t->emitters, t->emitters_len);
    cpf(T->emit_cdf, t->emit_cdf, t->emit_cdf_len);
    cpf(T->env_pixels, t->env_pixels, t->env_pixels_len);
    cpf(T->env_marginal, t->env_marginal, t->env_marginal_len);
    cpf(T->env_cond, t->env_cond, t->env_cond_len);
    cpf(T->texels, t->texels, t->texels_len);
    cpu(T->tex_info, t->tex_info, t->tex_info_len);
    // World-space triangles with transformPoint's single-precision arithmetic (pt_core.slang:90-99).
    for (size_t i = 0; i < t->instance_count; i++) {
        const uint32_t* rec = &T->instances[16 * i];
        float m[12];
        for (int k = 0; k < 12; k++)
            m[k] = bitsf(rec[4 + k]);
        for (uint32_t p = 0; p < t->tri_counts[i]; p++) {
            for (int v = 0; v < 3; v++) {
                uint32_t vi = T->indices[rec[1] + 3 * p + v] + rec[0];
                float x = T->positions[3 * vi], y = T->positions[3 * vi + 1], z = T->positions[3 * vi + 2];
                for (int r = 0; r < 3; r++)
                    T->tv.push_back(m[4 * r] * x + m[4 * r + 1] * y + m[4 * r + 2] * z + m[4 * r + 3]);
            }
            T->tinst.push_back((uint32_t)i);
            T->tprim.push_back(p);
        }
    }
    for (size_t m = 0; m < T->materials.size() / 24; m++)
        if (T->materials[24 * m + 22] < 1.0f || T->materials[24 * m + 23] > 0.0f)
            T->translucent = true;
    build_bvh(*T);
    return T;
}

void or_scene_destroy(void* s) { delete (Tables*)s; }

uint32_t or_scene_triangles(void* s) { return (uint32_t)((Tables*)s)->tinst.size(); }

// Closest hits: rays 6 floats; hits 4 words (flag, inst, prim, t bits). brute != 0 tests every triangle.
void or_trace_closest(void* s, const float* rays, size_t n, uint32_t* hits, int brute, int threads)
{
    const Tables& T = *(const Tables*)s;
    parallel_for((uint32_t)n, threads, [&](uint32_t i) {
        const float* r = rays + 6 * (size_t)i;
        QHit<float> h = trace<float>(T, V<float>(r[0], r[1], r[2]), V<float>(r[3], r[4], r[5]), 1.0e30f, false, brute != 0);
        hits[4 * i] = h.hit ? 1u : 0u;
        hits[4 * i + 1] = h.hit ? h.inst : 0u;
        hits[4 * i + 2] = h.hit ? h.prim : 0u;
        hits[4 * i + 3] = h.hit ? fbits(h.t) : 0u;
    });
}

// Shadow-ray queries (pt_core.slang occluded): rays 7 floats (origin, direction, tmax).
void or_trace_occluded(void* s, const float* rays, size_t n, uint32_t* out, int threads)
{
    const Tables& T = *(const Tables*)s;
    uint32_t params[43] = {};
    Job<float> J{&T, params, nullptr, nullptr, nullptr, nullptr, false, false};
    PT<float> pt{T, params, J};
    parallel_for((uint32_t)n, threads, [&](uint32_t i) {
        const float* r = rays + 7 * (size_t)i;
        out[i] = pt.occluded(V<float>(r[0], r[1], r[2]), V<float>(r[3], r[4], r[5]), r[6]) ? 1u : 0u;
    });
}

// Renders `samples` samples from `sample_base` into caller-owned sums.
//   params: the 43-word block (words 6 and 35 are set here); precision 0 = single (bit parity),
//   1 = double (converged reference). acc64: sums and adaptive statistics are doubles.
//   wavefront != 0 runs the wavefront stages (queues and the reference's state layout) and writes
//   the depth-queue lengths of every sample into queue_counts[(sample) * (depth + 1) + d].
//   restir: 80 floats per pixel (zeroed by the caller before the first sample), or null.
//   rows: if non-null, only pixels whose row is listed are traced (a bounded sample).
int or_render(void* s, const uint32_t* params_in, uint32_t sample_base, uint32_t samples, int precision, int acc64,
              void* accum, void* stats, float* lighting, float* restir, int wavefront, uint32_t* queue_counts,
              int threads, int brute, const uint32_t* rows, uint32_t row_count)
{
    const Tables& T = *(const Tables*)s;
    uint32_t P[43];
    memcpy(P, params_in, sizeof(P));
    uint32_t w = P[0], h = P[1], depth = P[7];
    uint32_t npx = w * h;
    std::vector<uint32_t> pixels;
    if (rows) {
        for (uint32_t r = 0; r < row_count; r++)
            for (uint32_t x = 0; x < w; x++)
                pixels.push_back(rows[r] * w + x);
    } else {
        pixels.resize(npx);
        for (uint32_t p = 0; p < npx; p++)
            pixels[p] = p;
    }
    auto run = [&](auto tag) {
        using R = decltype(tag);
        Job<R> J{&T, P, accum, stats, lighting, restir, acc64 != 0, brute != 0};
        PT<R> pt{T, P, J};
        bool per_sample = wavefront || P[36] != 0;
        if (!per_sample) {
            // Megakernel (pathtrace.slang:9-26): one pixel runs all its samples.
            P[35] = samples;
            P[6] = sample_base;
            parallel_for((uint32_t)pixels.size(), threads, [&](uint32_t i) {
                uint32_t pixel = pixels[i];
                for (uint32_t k = 0; k < samples; k++) {
                    if (P[32] != 0 && !pt.pixelActive(pixel))
                        return;
                    PathState<R> st = pt.generatePathFor(pixel % w, pixel / w, P[6] + k);
                    for (uint32_t d = 0; d < depth; d++)
                        if (!pt.shadePath(st, pt.traceClosest(st.org, st.dir), d, pixel))
                            break;
                    pt.finishPath(st, pixel);
                }
            });
            return;
        }
        if (!wavefront) {
            // Megakernel under ReSTIR: one sample per dispatch (renderer.rs:459-463).
            for (uint32_t k = 0; k < samples; k++) {
                P[6] = sample_base + k;
                P[35] = 1;
                parallel_for((uint32_t)pixels.size(), threads, [&](uint32_t i) {
                    uint32_t pixel = pixels[i];
                    if (P[32] != 0 && !pt.pixelActive(pixel))
                        return;
                    PathState<R> st = pt.generatePathFor(pixel % w, pixel / w, P[6]);
                    for (uint32_t d = 0; d < depth; d++)
                        if (!pt.shadePath(st, pt.traceClosest(st.org, st.dir), d, pixel))
                            break;
                    pt.finishPath(st, pixel);
                });
            }
            return;
        }
        // Wavefront (wf_select / wf_args / wf_extend / wf_shade with wf_state.slang's layout).
        uint32_t N = npx;
        uint32_t words = 16 + (P[28] != 0 ? 17 : 0);
        std::vector<uint32_t> state((size_t)words * N), hits(4 * (size_t)N), q0(N), q1(N);
        std::vector<uint32_t> counts(depth + 1);
        auto put = [&](uint32_t f, uint32_t p, R v) { state[(size_t)f * N + p] = fbits((float)v); };
        auto get = [&](uint32_t f, uint32_t p) { return R(bitsf(state[(size_t)f * N + p])); };
        std::vector<uint8_t> selected(N, rows ? 0 : 1);
        if (rows)
            for (uint32_t p : pixels)
                selected[p] = 1;
        for (uint32_t k = 0; k < samples; k++) {
            P[6] = sample_base + k;
            P[31] = N;
            // wf_args at depth 0 / wf_select.
            std::fill(counts.begin(), counts.end(), 0u);
            std::vector<uint32_t>* qs[2] = {&q0, &q1};
            uint32_t c0 = 0;
            for (uint32_t p = 0; p < N; p++)
                if (selected[p] && (P[32] == 0 || pt.pixelActive(p)))
                    q0[c0++] = p;
            counts[0] = c0;
            for (uint32_t d = 0; d < depth; d++) {
                std::vector<uint32_t>& qin = *qs[d & 1];
                std::vector<uint32_t>& qout = *qs[(d + 1) & 1];
                uint32_t cnt = counts[d];
                // wf_extend
                parallel_for(cnt, threads, [&](uint32_t i) {
                    uint32_t p = qin[i];
                    V<R> org, dir;
                    if (d == 0) {
                        PathState<R> st = pt.generatePathFor(p % w, p / w, P[6]);
                        org = st.org;
                        dir = st.dir;
                    } else {
                        org = V<R>(get(0, p), get(1, p), get(2, p));
                        dir = V<R>(get(3, p), get(4, p), get(5, p));
                    }
                    HitRec<R> hr = pt.traceClosest(org, dir);
                    hits[4 * (size_t)p] = hr.hit ? 1u : 0u;
                    hits[4 * (size_t)p + 1] = hr.inst;
                    hits[4 * (size_t)p + 2] = hr.prim;
                    hits[4 * (size_t)p + 3] = fbits((float)hr.t);
                });
                // wf_shade (sequential append keeps the queue order deterministic; order does not
                // change any result)
                std::vector<uint8_t> live(cnt);
                parallel_for(cnt, threads, [&](uint32_t i) {
                    uint32_t p = qin[i];
                    PathState<R> st;
                    if (d == 0)
                        st = pt.generatePathFor(p % w, p / w, P[6]);
                    else {
                        st.org = V<R>(get(0, p), get(1, p), get(2, p));
                        st.dir = V<R>(get(3, p), get(4, p), get(5, p));
                        st.thr = V<R>(get(6, p), get(7, p), get(8, p));
                        st.rng = state[9 * (size_t)N + p];
                        uint32_t flags = state[10 * (size_t)N + p];
                        st.cls = flags & 3u;
                        st.chan = (int)((flags >> 2) & 3u) - 1;
                        st.misPrev = (flags & 16u) != 0;
                        st.restir = (flags & 32u) != 0;
                        st.gi = (flags & 64u) != 0;
                        st.prevInst = flags >> 8;
                        st.pathLen = get(11, p);
                        st.qPrev = get(12, p);
                        st.parts = Parts<R>();
                        st.parts.total = V<R>(get(13, p), get(14, p), get(15, p));
                        if (P[28] != 0) {
                            st.parts.directDiffuse = V<R>(get(16, p), get(17, p), get(18, p));
                            st.parts.indirectDiffuse = V<R>(get(19, p), get(20, p), get(21, p));
                            st.parts.specular = V<R>(get(22, p), get(23, p), get(24, p));
                            st.parts.transmission = V<R>(get(25, p), get(26, p), get(27, p));
                            st.parts.emission = V<R>(get(28, p), get(29, p), get(30, p));
                            st.visLit = get(31, p);
                            st.visTotal = get(32, p);
                        }
                    }
                    HitRec<R> hr;
                    hr.hit = hits[4 * (size_t)p] != 0;
                    hr.inst = hits[4 * (size_t)p + 1];
                    hr.prim = hits[4 * (size_t)p + 2];
                    hr.t = R(bitsf(hits[4 * (size_t)p + 3]));
                    if (pt.shadePath(st, hr, d, p) && d + 1 < depth) {
                        put(0, p, st.org.x); put(1, p, st.org.y); put(2, p, st.org.z);
                        put(3, p, st.dir.x); put(4, p, st.dir.y); put(5, p, st.dir.z);
                        put(6, p, st.thr.x); put(7, p, st.thr.y); put(8, p, st.thr.z);
                        state[9 * (size_t)N + p] = st.rng;
                        state[10 * (size_t)N + p] = st.cls | ((uint32_t)(st.chan + 1) << 2) | (st.misPrev ? 16u : 0u) |
                                                    (st.restir ? 32u : 0u) | (st.gi ? 64u : 0u) | (st.prevInst << 8);
                        put(11, p, st.pathLen);
                        put(12, p, st.qPrev);
                        put(13, p, st.parts.total.x); put(14, p, st.parts.total.y); put(15, p, st.parts.total.z);
                        if (P[28] != 0) {
                            V<R> v5[5] = {st.parts.directDiffuse, st.parts.indirectDiffuse, st.parts.specular,
                                          st.parts.transmission, st.parts.emission};
                            for (int q = 0; q < 5; q++) {
                                put(16 + 3 * q, p, v5[q].x);
                                put(17 + 3 * q, p, v5[q].y);
                                put(18 + 3 * q, p, v5[q].z);
                            }
                            put(31, p, st.visLit);
                            put(32, p, st.visTotal);
                        }
                        live[i] = 1;
                    } else {
                        pt.finishPath(st, p);
                        live[i] = 0;
                    }
                });
                uint32_t c = 0;
                for (uint32_t i = 0; i < cnt; i++)
                    if (live[i])
                        qout[c++] = qin[i];
                counts[d + 1] = c;
            }
            if (queue_counts)
                for (uint32_t d = 0; d <= depth; d++)
                    queue_counts[(size_t)k * (depth + 1) + d] = counts[d];
        }
    };
    if (precision == 0)
        run(float());
    else
        run(double());
    return 0;
}

// shaders/normals.slang:41-110: camera18 is the camera record (pack.rs:97-108).
void or_render_normals(void* s, const float* cam, float* out, int threads)
{
    const Tables& T = *(const Tables*)s;
    uint32_t params[43] = {};
    Job<float> J{&T, params, nullptr, nullptr, nullptr, nullptr, false, false};
    PT<float> pt{T, params, J};
    uint32_t w = (uint32_t)cam[0], h = (uint32_t)cam[1];
    parallel_for(w * h, threads, [&](uint32_t pix) {
        uint32_t x = pix % w, y = pix / w;
        float t = cam[2];
        float aspect = cam[0] / cam[1];
        float u = (2.0f * ((float)x + 0.5f) / (float)w - 1.0f + cam[16]) * aspect * t;
        float v = (1.0f - 2.0f * ((float)y + 0.5f) / (float)h + cam[17]) * t;
        V<float> d = normalize(V<float>(u, v, -1.0f));
        float dr[3], orr[3];
        for (int r = 0; r < 3; r++) {
            dr[r] = cam[4 + 4 * r] * d.x + cam[5 + 4 * r] * d.y + cam[6 + 4 * r] * d.z;
            orr[r] = cam[7 + 4 * r];
        }
        V<float> org(orr[0], orr[1], orr[2]);
        V<float> dir = normalize(V<float>(dr[0], dr[1], dr[2]));
        HitRec<float> q = pt.traceClosest(org, dir);
        V<float> n;
        if (q.hit) {
            uint32_t inst = q.inst * 16;
            uint32_t tri = T.instances[inst + 1] + 3 * q.prim;
            uint32_t vo = T.instances[inst];
            uint32_t i0 = T.indices[tri] + vo, i1 = T.indices[tri + 1] + vo, i2 = T.indices[tri + 2] + vo;
            V<float> p0 = pt.transformPoint(inst + 4, pt.vertexPos(i0));
            V<float> p1 = pt.transformPoint(inst + 4, pt.vertexPos(i1));
            V<float> p2 = pt.transformPoint(inst + 4, pt.vertexPos(i2));
            V<float> ng = normalize(cross(p1 - p0, p2 - p0));
            n = ng;
            V<float> e1 = p1 - p0, e2 = p2 - p0, e3 = org + dir * q.t - p0;
            float d11 = dot(e1, e1), d12 = dot(e1, e2), d22 = dot(e2, e2);
            float den = std::fmax(d11 * d22 - d12 * d12, 1.0e-20f);
            float b1 = (d22 * dot(e3, e1) - d12 * dot(e3, e2)) / den;
            float b2 = (d11 * dot(e3, e2) - d12 * dot(e3, e1)) / den;
            V<float> nsObj = (1.0f - b1 - b2) * pt.vertexNormal(i0) + b1 * pt.vertexNormal(i1) + b2 * pt.vertexNormal(i2);
            if (dot(nsObj, nsObj) > 1.0e-12f) {
                n = normalize(pt.transformNormal(inst + 4, nsObj));
                if (dot(n, ng) < 0.0f)
                    n = -n;
            }
            if (dot(ng, dir) > 0.0f)
                n = -n;
        }
        out[3 * pix] = n.x;
        out[3 * pix + 1] = n.y;
        out[3 * pix + 2] = n.z;
    });
}

// shaders/aov.slang:86-188
void or_render_aovs(void* s, const float* cam, float* albedo_depth, uint32_t* object_ids, uint32_t* material_ids,
                    float* coverage, int threads)
{
    const Tables& T = *(const Tables*)s;
    uint32_t params[43] = {};
    Job<float> J{&T, params, nullptr, nullptr, nullptr, nullptr, false, false};
    PT<float> pt{T, params, J};
    uint32_t w = (uint32_t)cam[0], h = (uint32_t)cam[1];
    float t = cam[2];
    float aspect = cam[0] / cam[1];
    auto pixelDir = [&](float px, float py, V<float>& dir) {
        float u = (2.0f * px / (float)w - 1.0f + cam[16]) * aspect * t;
        float v = (1.0f - 2.0f * py / (float)h + cam[17]) * t;
        V<float> d = normalize(V<float>(u, v, -1.0f));
        float r[3];
        for (int k = 0; k < 3; k++)
            r[k] = cam[4 + 4 * k] * d.x + cam[5 + 4 * k] * d.y + cam[6 + 4 * k] * d.z;
        dir = V<float>(r[0], r[1], r[2]);
        return d;
    };
    parallel_for(w * h, threads, [&](uint32_t pix) {
        uint32_t x = pix % w, y = pix / w;
        V<float> org(cam[7], cam[11], cam[15]);
        V<float> dir;
        V<float> d = pixelDir((float)x + 0.5f, (float)y + 0.5f, dir);
        dir = normalize(dir);
        HitRec<float> q = pt.traceClosest(org, dir);
        V<float> albedo;
        float depth = 0.0f;
        uint32_t id = 0, matId = 0;
        if (q.hit) {
            uint32_t inst = q.inst * 16;
            uint32_t tri = T.instances[inst + 1] + 3 * q.prim;
            uint32_t vo = T.instances[inst];
            id = q.inst + 1;
            matId = T.instances[inst + 2] + 1;
            depth = q.t * -d.z;
            uint32_t mi = T.instances[inst + 2] * 24;
            albedo = V<float>(T.materials[mi], T.materials[mi + 1], T.materials[mi + 2]);
            uint32_t texBase = (uint32_t)T.materials[mi + 10];
            if (texBase > 0) {
                uint32_t i0 = T.indices[tri] + vo, i1 = T.indices[tri + 1] + vo, i2 = T.indices[tri + 2] + vo;
                V<float> p0 = pt.transformPoint(inst + 4, pt.vertexPos(i0));
                V<float> p1 = pt.transformPoint(inst + 4, pt.vertexPos(i1));
                V<float> p2 = pt.transformPoint(inst + 4, pt.vertexPos(i2));
                V<float> e1 = p1 - p0, e2 = p2 - p0, e3 = org + dir * q.t - p0;
                float d11 = dot(e1, e1), d12 = dot(e1, e2), d22 = dot(e2, e2);
                float den = std::fmax(d11 * d22 - d12 * d12, 1.0e-20f);
                float b1 = (d22 * dot(e3, e1) - d12 * dot(e3, e2)) / den;
                float b2 = (d11 * dot(e3, e2) - d12 * dot(e3, e1)) / den;
                float u0x = T.uvs[2 * i0], u0y = T.uvs[2 * i0 + 1], u1x = T.uvs[2 * i1], u1y = T.uvs[2 * i1 + 1];
                float u2x = T.uvs[2 * i2], u2y = T.uvs[2 * i2 + 1];
                float ux = u0x + b1 * (u1x - u0x) + b2 * (u2x - u0x);
                float uy = u0y + b1 * (u1y - u0y) + b2 * (u2y - u0y);
                uint32_t ti = (texBase - 1) * 4;
                albedo = albedo * pt.bilinear(T.tex_info[ti], T.tex_info[ti + 1], T.tex_info[ti + 2], ux, uy);
            }
        }
        float cover = 0.0f;
        for (uint32_t k = 0; k < 16; k++) {
            V<float> sdir;
            pixelDir((float)x + ((float)(k % 4) + 0.5f) / 4.0f, (float)y + ((float)(k / 4) + 0.5f) / 4.0f, sdir);
            V<float> so = org, sd = normalize(sdir);
            float seen = 0.0f, through = 1.0f;
            for (uint32_t layer = 0; layer < 8 && through > 0.0f; layer++) {
                QHit<float> sq = trace<float>(T, so, sd, 1.0e30f, false, false);
                if (!sq.hit)
                    break;
                float op = pt.opacityAt(sq.inst, sq.prim, sq.b1, sq.b2);
                seen += through * op;
                through *= 1.0f - op;
                so = so + sd * (sq.t + 1.0e-4f);
            }
            cover += seen;
        }
        coverage[pix] = cover / 16.0f;
        albedo_depth[4 * pix] = albedo.x;
        albedo_depth[4 * pix + 1] = albedo.y;
        albedo_depth[4 * pix + 2] = albedo.z;
        albedo_depth[4 * pix + 3] = depth;
        object_ids[pix] = id;
        material_ids[pix] = matId;
    });
}

// Elementary functions, exported so the tests can bound their error against double precision.
float or_sinf(float x) { return vgm::sinf_(x); }
float or_cosf(float x) { return vgm::cosf_(x); }
float or_acosf(float x) { return vgm::acosf_(x); }
float or_atan2f(float y, float x) { return vgm::atan2f_(y, x); }
float or_log2f(float x) { return vgm::log2f_(x); }
float or_exp2f(float x) { return vgm::exp2f_(x); }
float or_powf(float x, float y) { return vgm::powf_(x, y); }
uint32_t or_pcg(uint32_t v) { return pcg(v); }

} // extern "C"
