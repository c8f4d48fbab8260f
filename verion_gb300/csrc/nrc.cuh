// Radiance cache: a multi-resolution hash-grid encoding of the position feeding a 64-wide MLP
// (4 hidden layers, ReLU, bf16 weights and activations, f32 accumulation) that predicts the
// radiance scattered at a path vertex toward the previous one. No reference counterpart: the
// learned termination of paths is an extension of the path tracer.
//
// Record (NRC_REC_WORDS floats): 0-2 world position, 3-5 outgoing direction (toward the previous
// vertex), 6-8 shading normal, 9 roughness, 10-12 base colour, 13 metallic, 14 transmission,
// 15 unused; 16-18 the training target (training records) or the path throughput (query records);
// 19 the pixel index bits (query records).
//
// Network input (64 columns): 0..2L-1 the L levels' two trilinear grid features, 32-34 direction
// and 35-37 normal mapped to [0,1], 38 roughness, 39-41 base colour, 42 metallic, 43 transmission,
// 44 the constant 1 (bias), 45-63 zero. Layers: z1 = W0 x, h1 = relu(z1), ... h4 = relu(W3 h3),
// out = W4 h4 with W4 16 x 64 of which rows 0-2 are used.
#pragma once
#include <stdint.h>

namespace vgn {

constexpr uint32_t REC_WORDS = 20;
constexpr uint32_t WIDTH = 64;
constexpr uint32_t OUT_ROWS = 16; // output layer rows in the MMA (3 used)
constexpr uint32_t HIDDEN_LAYERS = 4;
constexpr uint32_t MLP_PARAMS = HIDDEN_LAYERS * WIDTH * WIDTH + OUT_ROWS * WIDTH; // 17,408
constexpr uint32_t MAX_LEVELS = 16;
constexpr uint32_t TILE = 128; // records per MMA tile (M)

// Byte offsets of the bf16 weight image: the tiles exactly as the MMA reads them from shared
// memory (K-major, 128-byte swizzle). W0..W3 are 64 x 64 (forward B operands), W4 16 x 64; their
// transposes WT0..WT3 (64 x 64) and W4T (64 rows, 16 of 64 columns used) feed the backward pass.
constexpr uint32_t IMG_W = 0;
constexpr uint32_t IMG_W4 = 4 * 8192;
constexpr uint32_t IMG_WT = IMG_W4 + 2048;      // 34,816
constexpr uint32_t IMG_W4T = IMG_WT + 4 * 8192; // 67,584
constexpr uint32_t IMG_BYTES = IMG_W4T + 8192;  // 75,776
constexpr uint32_t IMG_FWD_BYTES = IMG_WT;      // what inference needs

// Offset of layer l's weights in the f32 parameter vector (row-major, out x in).
static __host__ __device__ constexpr uint32_t mlp_offset(uint32_t l) { return l * WIDTH * WIDTH; }

// Device view of one cache.
struct CacheDev {
    const uint32_t* grid;   // levels x 2^log2_t entries, two fp16 features each
    float* grid_grad;       // levels x 2^log2_t x 2 (f32), summed per training step
    const uint8_t* img;     // bf16 weight image (IMG_BYTES)
    float* mlp_grad;        // MLP_PARAMS (f32), summed per training step
    double* loss;           // loss sum of the last training step
    uint32_t* err;          // error flags (bit ERR_MMA_TIMEOUT)
    uint32_t levels;
    uint32_t log2_t;
    uint32_t dense_mask;    // bit l: level l is indexed densely ((res+1)^3 <= 2^log2_t)
    uint32_t res[MAX_LEVELS];
    float lo[3];            // scene box lower corner
    float inv_extent;       // 1 / largest side of the scene box
};

constexpr uint32_t ERR_MMA_TIMEOUT = 1u << 8; // an MMA completion wait gave up

// Hash of a grid vertex (the spatial hash of Teschner et al. 2003 with the primes of
// Mueller et al. 2022: 1, 2654435761, 805459861), reduced to the table size.
static __host__ __device__ __forceinline__ uint32_t grid_index(uint32_t x, uint32_t y, uint32_t z, uint32_t res,
                                                                bool dense, uint32_t mask)
{
    if (dense)
        return x + (res + 1u) * (y + (res + 1u) * z);
    return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & mask;
}

} // namespace vgn
