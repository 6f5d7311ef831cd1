// Render levels shared by the diffusion epilogue and the standalone render
// kernels.
#pragma once

#include <cuda_runtime.h>

namespace cg {

// ---------------------------------------------------------------------------
// Render (render.rs, render_main of compute_1024.wgsl:428-443): channels 0, 1
// and 2 become the R, G and B levels u32(sqrt(clamp(1.5 c, 0, 1)) * 255) of
// a packed 0x00RRGGBB word per pixel.  Channels a world lacks render as 0.
// As an epilogue of the per-channel diffusion kernel, channel c stores only
// its own bytes of the word (little-endian: B at byte 0, G at 1, R at 2),
// and the kernels of channels 0..2 together write all four.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned render_level(float v) {
    return __float2uint_rz(__fsqrt_rn(fminf(fmaxf(v * 1.5f, 0.f), 1.f)) * 255.f);
}

__device__ __forceinline__ void render_store(unsigned char* __restrict__ rb, int nch, int c,
                                             size_t p, float v) {
    const unsigned l = render_level(v);
    unsigned char* px = rb + 4 * p;
    if (c == 0) {
        if (nch == 1)
            *reinterpret_cast<unsigned*>(px) = l << 16;
        else
            *reinterpret_cast<unsigned short*>(px + 2) = static_cast<unsigned short>(l);
    } else if (c == 1) {
        if (nch == 2)
            *reinterpret_cast<unsigned short*>(px) = static_cast<unsigned short>(l << 8);
        else
            px[1] = static_cast<unsigned char>(l);
    } else if (c == 2) {
        px[0] = static_cast<unsigned char>(l);
    }
}

}  // namespace cg
