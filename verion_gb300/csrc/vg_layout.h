// Table layouts and parameter-block words shared by the host code and the kernels.
//
// The flat tables are the ones Verion's host packer produces (crates/verion-gpu/src/pack.rs:111-133)
// and its kernels read (shaders/include/pt_core.slang:12-63); a caller hands them over unchanged.
#pragma once
#include <stdint.h>

namespace vgl {

// Parameter block (pt_core.slang:23-28, pack.rs:828-874): 43 words.
constexpr int PARAM_WORDS = 43;
enum ParamWord : int {
    P_WIDTH = 0, P_HEIGHT = 1, P_TAN_HALF_FOV = 2, P_APERTURE = 3, P_FOCUS = 4,
    P_LIGHT_COUNT = 5, P_SAMPLE = 6, P_MAX_DEPTH = 7, P_CAMERA = 8, /* 8..19 camera-to-world 3x4 */
    P_SKY = 20, /* 20..22 */ P_EMITTER_COUNT = 23, P_ENV_W = 24, P_ENV_H = 25, P_ENV_PDF_SCALE = 26,
    P_PIXEL_CONE = 27, P_LIGHTING = 28, P_MULTISCATTER = 29, P_WF_DEPTH = 30, P_WF_PATHS = 31,
    P_ADAPTIVE = 32, P_ADAPTIVE_THRESHOLD = 33, P_ADAPTIVE_MIN_SPP = 34, P_SAMPLES_PER_DISPATCH = 35,
    P_RESTIR = 36, P_RESTIR_CANDIDATES = 37, P_RESTIR_HISTORY = 38, P_SHIFT_X = 39, P_SHIFT_Y = 40,
    P_VIRTUAL_LIGHT = 41, P_TRANSPARENT_BG = 42,
};

// Record sizes (pack.rs:13-34).
constexpr uint32_t DEFAULT_MAX_DEPTH = 8;
constexpr uint32_t MATERIAL_WORDS = 24;
constexpr uint32_t LIGHT_WORDS = 16;
constexpr uint32_t EMITTER_WORDS = 16;
constexpr uint32_t INSTANCE_WORDS = 16;

// Directional-albedo tables appended after the light table (pt_core.slang:188-195).
constexpr uint32_t GGX_ALBEDO_N = 32;
constexpr uint32_t SHEEN_ALBEDO_N = 16;
constexpr uint32_t DIEL_ALBEDO_N = 16;
constexpr uint32_t DIEL_ALBEDO_N_IOR = 9;
constexpr uint32_t ALBEDO_GGX = 0;
constexpr uint32_t ALBEDO_SHEEN = GGX_ALBEDO_N * GGX_ALBEDO_N;
constexpr uint32_t ALBEDO_DIEL = ALBEDO_SHEEN + SHEEN_ALBEDO_N * SHEEN_ALBEDO_N;
constexpr uint32_t ALBEDO_WORDS = ALBEDO_DIEL + DIEL_ALBEDO_N * DIEL_ALBEDO_N * DIEL_ALBEDO_N_IOR * 2;

// Lighting split (pt_core.slang:39-47, readback.rs:7-9): 17 words, then 4 light slots of 12.
constexpr uint32_t LIGHTING_STRIDE = 65;
constexpr uint32_t SLOT_WORDS = 12;
constexpr uint32_t LIGHT_SLOTS = 4;

// ReSTIR DI constants (pt_core.slang:704-713).
constexpr float RESTIR_MIN_ALPHA = 0.15f;
constexpr int RESTIR_RADIUS = 6;
constexpr uint32_t RESTIR_NEIGHBOURS = 2;

// Wavefront (wavefront.rs:7-12): path-state words of the reference layout, used for its size
// bookkeeping; this backend keeps the same words in 16-byte planes (see the state layout in
// pt_device.cuh).
constexpr uint32_t WF_BASE_WORDS = 16;
constexpr uint32_t WF_SPLIT_WORDS = 17;

} // namespace vgl
