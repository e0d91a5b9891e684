// Ingest: packed 10-bit and 12-bit camera data to 16-bit frames.
//
// Reference: unpack_12_to_16bit / unpack_10_to_16bit (Backend/cuda_sources/unpack.cu:4-60), called
// by the file reader for packed recordings (file_frame_read_worker.cc:220-240). The packing is
// MSB first: 12-bit pairs in 3 bytes (b0 b1 b2 -> (b0 << 8) | (b1 & 0xF0), ((b1 & 0x0F) << 12) |
// (b2 << 4)), 10-bit quadruples in 5 bytes; each value lands left-aligned in 16 bits.
//
// One thread per packed group (2 pixels / 3 bytes, or 4 pixels / 5 bytes) in a grid-stride loop
// (consecutive threads read consecutive groups); every output element is written only when it and
// the bytes it needs are inside the caller's buffers.
#include "hv_common.cuh"
#include "hv_internal.h"

namespace hv {

namespace {

__global__ void k_unpack12(const uint8_t* __restrict__ in, size_t in_bytes, uint16_t* __restrict__ out,
                           size_t out_count)
{
    const size_t groups = (out_count + 1) / 2;
    for (size_t g = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; g < groups;
         g += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        const size_t b = 3 * g, o = 2 * g;
        if (b + 1 < in_bytes)
            out[o] = static_cast<uint16_t>((in[b] << 8) | (in[b + 1] & 0xF0));
        if (o + 1 < out_count && b + 2 < in_bytes)
            out[o + 1] = static_cast<uint16_t>(((in[b + 1] & 0x0F) << 12) | (in[b + 2] << 4));
    }
}

__global__ void k_unpack10(const uint8_t* __restrict__ in, size_t in_bytes, uint16_t* __restrict__ out,
                           size_t out_count)
{
    const size_t groups = (out_count + 3) / 4;
    for (size_t g = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; g < groups;
         g += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        const size_t b = 5 * g, o = 4 * g;
        if (b + 1 < in_bytes)
            out[o] = static_cast<uint16_t>((in[b] << 8) | (in[b + 1] & 0xC0));
        if (o + 1 < out_count && b + 2 < in_bytes)
            out[o + 1] = static_cast<uint16_t>(((in[b + 1] & 0x3F) << 10) | ((in[b + 2] & 0xF0) << 2));
        if (o + 2 < out_count && b + 3 < in_bytes)
            out[o + 2] = static_cast<uint16_t>(((in[b + 2] & 0x0F) << 12) | ((in[b + 3] & 0xFC) << 4));
        if (o + 3 < out_count && b + 4 < in_bytes)
            out[o + 3] = static_cast<uint16_t>(((in[b + 3] & 0x03) << 14) | (in[b + 4] << 6));
    }
}

int unpack_grid(size_t groups)
{
    const size_t g = (groups + 255) / 256;
    return static_cast<int>(g < 152 * 16 ? (g < 1 ? 1 : g) : 152 * 16);
}

}  // namespace

hv_status unpack_packed(int bits, const void* in, size_t in_bytes, uint16_t* out, size_t out_count, cudaStream_t st)
{
    if (!in || !out)
        return HV_INVALID_VALUE;
    if (out_count == 0)
        return HV_OK;
    if (bits == 12)
        k_unpack12<<<unpack_grid((out_count + 1) / 2), 256, 0, st>>>(static_cast<const uint8_t*>(in), in_bytes, out,
                                                                      out_count);
    else if (bits == 10)
        k_unpack10<<<unpack_grid((out_count + 3) / 4), 256, 0, st>>>(static_cast<const uint8_t*>(in), in_bytes, out,
                                                                      out_count);
    else
        return HV_INVALID_VALUE;
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

}  // namespace hv
