// Common definitions for the GB300 hologram kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "holovibes_gb300.h"
#include "hv_internal.h"

namespace hv {

// ---------------------------------------------------------------- complex helpers (float2)
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i: (x + iy)(-i) = y - ix
__host__ __device__ __forceinline__ float2 cmul_negi(float2 a) { return make_float2(a.y, -a.x); }
// multiply by +i
__host__ __device__ __forceinline__ float2 cmul_posi(float2 a) { return make_float2(-a.y, a.x); }

// Input pixel encodings accepted by the first spatial pass (camera PixelDepth, Camera/include/frame_desc.hh).
enum InKind : int
{
    IN_C64 = 0,     // complex64 (intermediate buffers)
    IN_U8 = 1,      // 8-bit camera pixels, scaled by 257
    IN_U16 = 2,     // 16-bit little-endian
    IN_F32 = 3,     // float pixels
    IN_U16_BE = 4,  // 16-bit big-endian (byte swapped on load)
};

__device__ __forceinline__ float2 load_pixel(const void* base, size_t idx, int kind)
{
    switch (kind)
    {
    case IN_U8:
        return make_float2(static_cast<float>(static_cast<const uint8_t*>(base)[idx]) * 257.0f, 0.f);
    case IN_U16:
        return make_float2(static_cast<float>(static_cast<const uint16_t*>(base)[idx]), 0.f);
    case IN_U16_BE:
    {
        uint16_t v = static_cast<const uint16_t*>(base)[idx];
        v = static_cast<uint16_t>((v << 8) | (v >> 8));
        return make_float2(static_cast<float>(v), 0.f);
    }
    case IN_F32:
        return make_float2(static_cast<const float*>(base)[idx], 0.f);
    default:
        return static_cast<const float2*>(base)[idx];
    }
}

inline int in_kind_bytes(int kind)
{
    switch (kind)
    {
    case IN_U8: return 1;
    case IN_U16:
    case IN_U16_BE: return 2;
    case IN_F32: return 4;
    default: return 8;
    }
}

// Maps batch frame b to its destination frame inside a circular buffer of `nslots` frames.
struct FrameMap
{
    size_t frame_stride;  // elements between consecutive slots
    int slot0;            // slot of frame 0
    int nslots;           // ring capacity (frame b -> (slot0 + b) % nslots)
    const int* slot0_dev = nullptr;  // device-side slot added to slot0 (a served cycle's ring_begin)
    __host__ __device__ __forceinline__ size_t offset(int b) const
    {
        int s0 = slot0;
#ifdef __CUDA_ARCH__
        if (slot0_dev)
            s0 += *slot0_dev;
#endif
        return static_cast<size_t>((s0 + b) % nslots) * frame_stride;
    }
};

}  // namespace hv
