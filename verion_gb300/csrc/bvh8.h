// Quantised 8-wide BVH: node and triangle record formats shared by the host builder and the
// CUDA traversal.
//
// Verion traces rays with the driver's hardware ray tracing (Metal intersector / Vulkan
// RayQuery, shaders/include/pt_core.slang:580-613,684-700); GB300 has no RT cores, so this
// backend builds its own acceleration structure on the host and walks it in software.
//
// Node (80 bytes = five 16-byte words, so a node is fetched with five 128-bit loads):
//   word 0: origin p (3 x f32) | exponents ex, ey, ez (biased, 8 bits each) and imask (8 bits)
//   word 1: child_base (first internal child) | tri_base (first triangle) | meta[8] (8 x u8)
//   word 2: qlo_x[8] | qlo_y[8]
//   word 3: qlo_z[8] | qhi_x[8]
//   word 4: qhi_y[8] | qhi_z[8]
// Child slot s has the box [p + qlo * 2^e, p + qhi * 2^e] per axis. Because qlo and qhi are
// 8-bit integers and 2^e a power of two, q * 2^e is exact and the decoded plane is one rounded
// add, which the builder reproduces to make every decoded box contain its child.
// imask bit s: slot s is an internal node, stored at child_base + popc(imask & ((1 << s) - 1)).
// meta[s] for a leaf slot: (count << 5) | offset, 1 <= count <= 3 triangles at tri_base + offset
// (offset < 24); 0 for internal and empty slots.
// Slots are assigned so that a ray whose direction has sign octant o (bit k set when component k
// is negative) meets the child in slot o first; traversal visits hit children in order of
// (slot XOR o), a front-to-back order without sorting (the ordering idea of Ylitie, Karras and
// Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs", HPG 2017).
//
// Triangle record (48 bytes = three 16-byte words): (v0.xyz, instance), (v1.xyz, primitive),
// (v2.xyz, global triangle index); world-space vertices, ids stored as integer bits.
#pragma once
#include <stdint.h>

namespace bvh8 {

constexpr uint32_t NODE_WORDS = 20;      // u32 words per node
constexpr uint32_t NODE_VEC4 = 5;        // 16-byte words per node
constexpr uint32_t TRI_FLOATS = 12;      // f32 words per triangle record
constexpr uint32_t TRI_VEC4 = 3;
constexpr uint32_t MAX_LEAF_TRIS = 3;
constexpr uint32_t STACK_SIZE = 32;      // traversal stack entries (node groups)
constexpr uint32_t MAX_WIDE_DEPTH = 30;  // the builder rejects trees deeper than this
constexpr uint32_t ERR_STACK = 1u;       // error-status bit: a traversal stack overflowed

// Direction components smaller than this are replaced by it (sign kept) for the slab test only.
constexpr float MIN_DIR = 1.0e-20f;

} // namespace bvh8
