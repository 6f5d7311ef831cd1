// Render levels, shared by the render kernel and the diffusion kernels'
// level planes (iterate_and_render).
#pragma once

#include <cuda_runtime.h>

namespace cg {

// ---------------------------------------------------------------------------
// Render (render.rs, render_main of compute_1024.wgsl:428-443): channels 0, 1
// and 2 become the R, G and B levels u32(sqrt(clamp(1.5 c, 0, 1)) * 255) of
// a packed 0x00RRGGBB word per pixel.  Channels a world lacks render as 0.
// In a rendering step, the diffusion kernel of channel c < 3 also writes its
// new values' levels to byte plane c (one byte per pixel, stored with the
// state), and k_pack_levels joins the planes into the words.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned render_level(float v) {
    return __float2uint_rz(__fsqrt_rn(fminf(fmaxf(v * 1.5f, 0.f), 1.f)) * 255.f);
}
__device__ __forceinline__ unsigned char render_level_byte(float v) {
    return static_cast<unsigned char>(render_level(v));
}

}  // namespace cg
