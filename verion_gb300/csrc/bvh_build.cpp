// Host builder of the quantised 8-wide BVH (format in bvh8.h).
//
// Verion has no builder of its own: its backends hand the triangles to the graphics driver
// (crates/verion-gpu-metal/src/accel.rs:68-106, crates/verion-gpu-vulkan/src/accel.rs:153-233).
// This one works in two passes:
//   1. a binary BVH by the binned surface-area heuristic (32 bins per axis, leaves of at most
//      three triangles), with an object-median fallback below a depth limit so the tree depth is
//      bounded for any input;
//   2. a collapse into 8-wide nodes that repeatedly opens the internal child of largest surface
//      area, slot assignment by ray octant, and 8-bit quantisation of the child boxes against a
//      per-node power-of-two grid, checked in float so every decoded box contains its child.
// Must be compiled without floating-point contraction (-ffp-contract=off): the decoded planes
// are recomputed on the GPU and the containment check relies on the same rounding.
#include "bvh_build.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>

#include "bvh8.h"

namespace {

struct Box {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const float* p)
    {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    void grow(const Box& b)
    {
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    float area() const
    {
        float d[3];
        for (int k = 0; k < 3; k++)
            d[k] = std::max(hi[k] - lo[k], 0.0f);
        return 2.0f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
    bool empty() const { return lo[0] > hi[0]; }
};

struct BNode {
    Box box;
    uint32_t a = 0;     // leaf: first index into `order`; internal: left child
    uint32_t b = 0;     // internal: right child
    uint32_t count = 0; // triangles in a leaf, 0 for an internal node
};

constexpr int BINS = 32;
constexpr int MEDIAN_DEPTH = 40;   // below this depth splits fall back to the object median
struct Builder {
    const float* verts;
    uint32_t n;
    float c_trav = 1.0f; // SAH cost of one node visit, relative to one triangle test
    std::vector<Box> tbox;
    std::vector<float> cent; // 3 per triangle
    std::vector<uint32_t> order;
    std::vector<BNode> nodes;
    uint32_t max_depth = 0;

    void leaf(uint32_t id, uint32_t begin, uint32_t end)
    {
        nodes[id].a = begin;
        nodes[id].count = end - begin;
    }

    // Splits [begin, end) in place; returns the split index, or begin/end when no split helps.
    uint32_t split(const Box& box, uint32_t begin, uint32_t end, uint32_t depth)
    {
        uint32_t cnt = end - begin;
        Box cb;
        for (uint32_t i = begin; i < end; i++)
            cb.grow(&cent[3 * order[i]]);
        int axis = 0;
        float ext[3];
        for (int k = 0; k < 3; k++)
            ext[k] = cb.hi[k] - cb.lo[k];
        if (ext[1] > ext[axis])
            axis = 1;
        if (ext[2] > ext[axis])
            axis = 2;
        if (ext[axis] <= 0.0f) {
            // All centroids coincide: split by position in the list.
            return cnt <= bvh8::MAX_LEAF_TRIS ? begin : begin + cnt / 2;
        }
        if (depth >= MEDIAN_DEPTH) {
            uint32_t mid = begin + cnt / 2;
            std::nth_element(order.begin() + begin, order.begin() + mid, order.begin() + end,
                             [&](uint32_t x, uint32_t y) { return cent[3 * x + axis] < cent[3 * y + axis]; });
            return mid;
        }
        float best_cost = INFINITY;
        int best_axis = -1;
        int best_bin = 0;
        for (int k = 0; k < 3; k++) {
            if (ext[k] <= 0.0f)
                continue;
            Box bb[BINS];
            uint32_t bc[BINS] = {};
            float scale = BINS / ext[k];
            for (uint32_t i = begin; i < end; i++) {
                uint32_t t = order[i];
                int bi = std::min(BINS - 1, (int)((cent[3 * t + k] - cb.lo[k]) * scale));
                bb[bi].grow(tbox[t]);
                bc[bi]++;
            }
            float right_area[BINS];
            uint32_t right_cnt[BINS];
            Box acc;
            uint32_t c = 0;
            for (int i = BINS - 1; i > 0; i--) {
                acc.grow(bb[i]);
                c += bc[i];
                right_area[i] = acc.empty() ? 0.0f : acc.area();
                right_cnt[i] = c;
            }
            acc = Box();
            c = 0;
            for (int i = 0; i < BINS - 1; i++) {
                acc.grow(bb[i]);
                c += bc[i];
                if (c == 0 || right_cnt[i + 1] == 0)
                    continue;
                float cost = acc.area() * (float)c + right_area[i + 1] * (float)right_cnt[i + 1];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = k;
                    best_bin = i;
                }
            }
        }
        float pa = box.area();
        float leaf_cost = (float)cnt;
        float split_cost = pa > 0.0f ? c_trav + best_cost / pa : INFINITY;
        if (cnt <= bvh8::MAX_LEAF_TRIS && (best_axis < 0 || leaf_cost <= split_cost))
            return begin;
        if (best_axis < 0)
            return begin + cnt / 2;
        float scale = BINS / ext[best_axis];
        auto mid = std::partition(order.begin() + begin, order.begin() + end, [&](uint32_t t) {
            int bi = std::min(BINS - 1, (int)((cent[3 * t + best_axis] - cb.lo[best_axis]) * scale));
            return bi <= best_bin;
        });
        uint32_t m = (uint32_t)(mid - order.begin());
        if (m == begin || m == end)
            m = begin + cnt / 2;
        return m;
    }

    void build()
    {
        tbox.resize(n);
        cent.resize(3 * (size_t)n);
        order.resize(n);
        for (uint32_t t = 0; t < n; t++) {
            Box b;
            for (int v = 0; v < 3; v++)
                b.grow(&verts[9 * (size_t)t + 3 * v]);
            tbox[t] = b;
            for (int k = 0; k < 3; k++)
                cent[3 * (size_t)t + k] = 0.5f * (b.lo[k] + b.hi[k]);
            order[t] = t;
        }
        nodes.reserve(n > 0 ? 2 * (size_t)n : 1);
        nodes.emplace_back();
        struct Task { uint32_t id, begin, end, depth; };
        std::vector<Task> stack;
        stack.push_back({0, 0, n, 0});
        while (!stack.empty()) {
            Task t = stack.back();
            stack.pop_back();
            max_depth = std::max(max_depth, t.depth);
            Box box;
            for (uint32_t i = t.begin; i < t.end; i++)
                box.grow(tbox[order[i]]);
            nodes[t.id].box = box;
            uint32_t cnt = t.end - t.begin;
            if (cnt <= 1) {
                leaf(t.id, t.begin, t.end);
                continue;
            }
            uint32_t m = split(box, t.begin, t.end, t.depth);
            if (m == t.begin || m == t.end) {
                leaf(t.id, t.begin, t.end);
                continue;
            }
            uint32_t l = (uint32_t)nodes.size();
            nodes.emplace_back();
            nodes.emplace_back();
            nodes[t.id].a = l;
            nodes[t.id].b = l + 1;
            nodes[t.id].count = 0;
            stack.push_back({l + 1, m, t.end, t.depth + 1});
            stack.push_back({l, t.begin, m, t.depth + 1});
        }
    }
};

uint32_t f2u(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

float u2f(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}

float pow2(int e) { return u2f((uint32_t)(e + 127) << 23); }

} // namespace

bool build_bvh8(const float* verts, const uint32_t* inst, const uint32_t* prim, uint32_t n, Bvh8Host& out,
                std::string& err, float traversal_cost)
{
    auto t0 = std::chrono::steady_clock::now();
    for (size_t i = 0; i < 9 * (size_t)n; i++) {
        if (!std::isfinite(verts[i])) {
            err = "triangle " + std::to_string(i / 9) + " has a non-finite vertex";
            return false;
        }
    }
    Builder b;
    b.c_trav = traversal_cost;
    b.verts = verts;
    b.n = n;
    b.build();

    out.nodes.clear();
    out.tris.clear();
    out.binary_nodes = (uint32_t)b.nodes.size();

    // Breadth-first collapse. Each queue entry is a binary node that becomes the wide node at
    // `index`; the root wide node may hold a single leaf (scenes of at most three triangles).
    struct Item { uint32_t bnode, index, depth; };
    std::deque<Item> queue;
    uint32_t wide_count = 1;
    queue.push_back({0, 0, 1});
    out.nodes.assign(bvh8::NODE_WORDS, 0);
    uint32_t tri_count = 0;
    uint32_t wide_depth = 0;
    while (!queue.empty()) {
        Item it = queue.front();
        queue.pop_front();
        wide_depth = std::max(wide_depth, it.depth);
        std::vector<uint32_t> kids;
        const BNode& root = b.nodes[it.bnode];
        if (root.count > 0 || n == 0)
            kids.push_back(it.bnode);
        else {
            kids.push_back(root.a);
            kids.push_back(root.b);
        }
        while (kids.size() < 8) {
            int best = -1;
            float best_area = -1.0f;
            for (size_t k = 0; k < kids.size(); k++) {
                const BNode& c = b.nodes[kids[k]];
                if (c.count == 0 && c.box.area() > best_area) {
                    best_area = c.box.area();
                    best = (int)k;
                }
            }
            if (best < 0)
                break;
            uint32_t id = kids[best];
            kids[best] = b.nodes[id].a;
            kids.push_back(b.nodes[id].b);
        }
        // Node box and child centroids.
        Box nb;
        for (uint32_t k : kids)
            nb.grow(b.nodes[k].box);
        int m = (int)kids.size();
        if (n == 0)
            m = 0;
        // Slot assignment: slot s takes the child met first by rays of octant s.
        int slot_of[8];
        bool kid_done[8] = {};
        bool slot_done[8] = {};
        float cost[8][8];
        for (int k = 0; k < m; k++) {
            const Box& cb = b.nodes[kids[k]].box;
            float c[3];
            for (int a = 0; a < 3; a++)
                c[a] = 0.5f * (cb.lo[a] + cb.hi[a]) - 0.5f * (nb.lo[a] + nb.hi[a]);
            for (int s = 0; s < 8; s++)
                cost[k][s] = ((s & 1) ? -c[0] : c[0]) + ((s & 2) ? -c[1] : c[1]) + ((s & 4) ? -c[2] : c[2]);
        }
        for (int r = 0; r < m; r++) {
            int bk = -1, bs = -1;
            float bc = INFINITY;
            for (int k = 0; k < m; k++) {
                if (kid_done[k])
                    continue;
                for (int s = 0; s < 8; s++) {
                    if (!slot_done[s] && (bk < 0 || cost[k][s] < bc)) {
                        bc = cost[k][s];
                        bk = k;
                        bs = s;
                    }
                }
            }
            kid_done[bk] = true;
            slot_done[bs] = true;
            slot_of[bk] = bs;
        }
        int kid_in_slot[8];
        for (int s = 0; s < 8; s++)
            kid_in_slot[s] = -1;
        for (int k = 0; k < m; k++)
            kid_in_slot[slot_of[k]] = k;

        // Quantisation grid.
        float p[3];
        int ex[3];
        for (int a = 0; a < 3; a++) {
            p[a] = m > 0 ? nb.lo[a] : 0.0f;
            float extent = m > 0 ? nb.hi[a] - nb.lo[a] : 0.0f;
            int e = -126;
            if (extent > 0.0f) {
                int fe;
                std::frexp(extent / 255.0f, &fe); // extent/255 = f * 2^fe, f in [0.5, 1)
                e = std::max(fe, -126);
            }
            while (e < 127 && p[a] + 255.0f * pow2(e) < nb.hi[a])
                e++;
            if (e > 126) {
                err = "scene extent too large for the node grid";
                return false;
            }
            ex[a] = e;
        }
        uint32_t words[bvh8::NODE_WORDS] = {};
        uint8_t meta[8] = {};
        uint8_t qlo[3][8], qhi[3][8];
        for (int a = 0; a < 3; a++)
            for (int s = 0; s < 8; s++) {
                qlo[a][s] = 255;
                qhi[a][s] = 0;
            }
        uint32_t imask = 0;
        uint32_t child_base = wide_count;
        uint32_t tri_base = tri_count;
        uint32_t tri_off = 0;
        for (int s = 0; s < 8; s++) {
            int k = kid_in_slot[s];
            if (k < 0)
                continue;
            const BNode& c = b.nodes[kids[k]];
            for (int a = 0; a < 3; a++) {
                float sc = pow2(ex[a]);
                float lo = c.box.lo[a], hi = c.box.hi[a];
                int q0 = (int)std::floor((lo - p[a]) / sc);
                q0 = std::min(std::max(q0, 0), 255);
                while (q0 > 0 && p[a] + (float)q0 * sc > lo)
                    q0--;
                int q1 = (int)std::ceil((hi - p[a]) / sc);
                q1 = std::min(std::max(q1, 0), 255);
                while (q1 < 255 && p[a] + (float)q1 * sc < hi)
                    q1++;
                if (p[a] + (float)q0 * sc > lo || p[a] + (float)q1 * sc < hi) {
                    err = "quantised box does not contain its child";
                    return false;
                }
                qlo[a][s] = (uint8_t)q0;
                qhi[a][s] = (uint8_t)q1;
            }
            if (c.count == 0) {
                imask |= 1u << s;
            } else {
                meta[s] = (uint8_t)((c.count << 5) | tri_off);
                for (uint32_t i = 0; i < c.count; i++) {
                    uint32_t t = b.order[c.a + i];
                    const float* v = &verts[9 * (size_t)t];
                    float rec[bvh8::TRI_FLOATS] = {v[0], v[1], v[2], u2f(inst[t]),
                                                   v[3], v[4], v[5], u2f(prim[t]),
                                                   v[6], v[7], v[8], u2f(t)};
                    out.tris.insert(out.tris.end(), rec, rec + bvh8::TRI_FLOATS);
                }
                tri_off += c.count;
                tri_count += c.count;
            }
        }
        // Internal children get consecutive node indices in slot order.
        for (int s = 0; s < 8; s++) {
            int k = kid_in_slot[s];
            if (k >= 0 && (imask >> s & 1u)) {
                queue.push_back({kids[k], wide_count, it.depth + 1});
                wide_count++;
            }
        }
        words[0] = f2u(p[0]);
        words[1] = f2u(p[1]);
        words[2] = f2u(p[2]);
        words[3] = (uint32_t)(ex[0] + 127) | ((uint32_t)(ex[1] + 127) << 8) | ((uint32_t)(ex[2] + 127) << 16) |
                   (imask << 24);
        words[4] = child_base;
        words[5] = tri_base;
        memcpy(&words[6], meta, 8);
        memcpy(&words[8], qlo[0], 8);
        memcpy(&words[10], qlo[1], 8);
        memcpy(&words[12], qlo[2], 8);
        memcpy(&words[14], qhi[0], 8);
        memcpy(&words[16], qhi[1], 8);
        memcpy(&words[18], qhi[2], 8);
        out.nodes.resize((size_t)std::max(wide_count, it.index + 1) * bvh8::NODE_WORDS, 0);
        memcpy(&out.nodes[(size_t)it.index * bvh8::NODE_WORDS], words, sizeof(words));
    }
    out.nodes.resize((size_t)wide_count * bvh8::NODE_WORDS, 0);
    out.wide_nodes = wide_count;
    out.wide_depth = wide_depth;
    out.binary_depth = b.max_depth;
    out.triangles = n;
    out.build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (tri_count != n) {
        err = "collapse lost triangles";
        return false;
    }
    if (wide_depth > bvh8::MAX_WIDE_DEPTH) {
        err = "BVH deeper than the traversal stack allows";
        return false;
    }
    // Every index the traversal follows must stay inside the tables it reads.
    for (uint32_t i = 0; i < wide_count; i++) {
        const uint32_t* w = &out.nodes[(size_t)i * bvh8::NODE_WORDS];
        uint32_t imask = w[3] >> 24;
        uint8_t meta[8];
        memcpy(meta, &w[6], 8);
        uint32_t inner = (uint32_t)__builtin_popcount(imask);
        if (inner > 0 && (w[4] == 0 || (uint64_t)w[4] + inner > wide_count)) {
            err = "BVH child index out of range";
            return false;
        }
        for (int s = 0; s < 8; s++) {
            if ((imask >> s) & 1u) {
                if (meta[s] != 0) {
                    err = "BVH internal slot with leaf data";
                    return false;
                }
                continue;
            }
            uint32_t cnt = meta[s] >> 5, off = meta[s] & 31u;
            if (cnt > bvh8::MAX_LEAF_TRIS || (uint64_t)w[5] + off + cnt > tri_count) {
                err = "BVH triangle range out of range";
                return false;
            }
        }
    }
    return true;
}
