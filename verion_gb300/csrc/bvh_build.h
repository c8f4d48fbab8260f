// Host builder of the quantised 8-wide BVH; format in bvh8.h.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

struct Bvh8Host {
    std::vector<uint32_t> nodes; // bvh8::NODE_WORDS per node, node 0 is the root
    std::vector<float> tris;     // bvh8::TRI_FLOATS per triangle, in leaf order
    uint32_t wide_nodes = 0;
    uint32_t wide_depth = 0;
    uint32_t binary_nodes = 0;
    uint32_t binary_depth = 0;
    uint32_t triangles = 0;
    double build_seconds = 0.0;
};

// `verts`: 9 floats (three world-space vertices) per triangle; `inst`, `prim`: the instance and
// the primitive index within its mesh per triangle. The global index of a triangle (its position
// in `verts`) breaks ties between hits at equal distance. `traversal_cost`: the SAH cost of a node
// visit relative to a triangle test (smaller: deeper trees with smaller leaves).
bool build_bvh8(const float* verts, const uint32_t* inst, const uint32_t* prim, uint32_t n, Bvh8Host& out,
                std::string& err, float traversal_cost = 0.5f);
