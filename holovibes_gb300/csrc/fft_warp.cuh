// 1024-point FFT with 32 samples per thread: N = 32 x 32, two in-register 32-point DFTs and one
// shared-memory transpose between them.
//
// A thread owns one "group" n2 (0..31) of a transform and holds x[n2 + 32 j], j = 0..31. Stage A
// is a 32-point DFT over j, then the twiddle w1024^(n2 k1); after the transpose the thread owns
// group k1 and holds z[n2][k1] for every n2; stage B is a 32-point DFT over n2 and leaves
// X[k1 + 32 k2] in element k2 (natural order, stride 32: the same shape as stage A's input, so a
// forward transform can be followed by an inverse one without another exchange).
//
// Compared with the Stockham tile engine (16 x 8 x 8 at 16 samples per thread) this halves the
// shared-memory exchanges, replaces the per-element index arithmetic (lane / sample decoding,
// swizzles, twiddle indices) with compile-time register offsets and, for rows, keeps every
// exchange inside one warp (__syncwarp, no CTA barrier).
#pragma once

#include "fft_smem.cuh"

namespace hv {
namespace fftw {

constexpr int N = 1024;
constexpr int G = 32;                // groups (threads) per transform
constexpr int TW_COUNT = 31 * 32;    // table entry (k1 - 1) * 32 + n2 = exp(-2 pi i n2 k1 / 1024)

// cos / sin of 2 pi r / 32 for r = 0..7
__host__ __device__ constexpr float c32(int r)
{
    return r == 0   ? 1.0f
           : r == 1 ? 0.980785280403230449126182236134239037f
           : r == 2 ? 0.923879532511286756128183189396788933f
           : r == 3 ? 0.831469612302545237078788377617905756f
           : r == 4 ? 0.707106781186547524400844362104849039f
           : r == 5 ? 0.555570233019602224742830813948532874f
           : r == 6 ? 0.382683432365089771728459984030398866f
                    : 0.195090322016128267848284868477022240f;
}
__host__ __device__ constexpr float s32(int r) { return r == 0 ? 0.0f : c32(8 - r); }

// a * w32^m, w32 = exp(-2 pi i / 32); m is a constant after unrolling, so the branches fold
__device__ __forceinline__ float2 w32mul(int m, float2 a)
{
    const int r = m & 7, q = (m >> 3) & 3;
    float2 b;
    if (r == 0)
        b = a;
    else if (r == 4)
        b = fft::w8mul<1>(a);
    else
    {
        const float c = c32(r), s = s32(r);
        b = make_float2(fmaf(a.y, s, a.x * c), fmaf(-a.x, s, a.y * c));  // a * (c - i s)
    }
    if (q == 1)
        return cmul_negi(b);
    if (q == 2)
        return make_float2(-b.x, -b.y);
    if (q == 3)
        return cmul_posi(b);
    return b;
}

// Forward 32-point DFT in place (natural order): n = 4 n1 + n2, k = k1 + 8 k2; DFT8 over n1,
// twiddle w32^(n2 k1), DFT4 over n2.
__device__ __forceinline__ void dft32(float2 (&x)[32])
{
    float2 a[4][8];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2)
    {
#pragma unroll
        for (int n1 = 0; n1 < 8; ++n1)
            a[n2][n1] = x[4 * n1 + n2];
        fft::dft8(a[n2]);
    }
#pragma unroll
    for (int n2 = 1; n2 < 4; ++n2)
#pragma unroll
        for (int k1 = 1; k1 < 8; ++k1)
            a[n2][k1] = w32mul(n2 * k1, a[n2][k1]);
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1)
    {
        fft::dft4(a[0][k1], a[1][k1], a[2][k1], a[3][k1]);
        x[k1] = a[0][k1];
        x[k1 + 8] = a[1][k1];
        x[k1 + 16] = a[2][k1];
        x[k1 + 24] = a[3][k1];
    }
}

// Stage A of a transform: x[j] = input sample n2 + 32 j on entry, z[n2][k1] * w1024^(n2 k1) in
// element k1 on return. tw: shared-memory table, this thread's entries at tw[(k1 - 1) * 32 + n2].
__device__ __forceinline__ void stage_a(float2 (&x)[32], const float2* tw, int n2)
{
    dft32(x);
    const float2* t = tw + n2;
#pragma unroll
    for (int k1 = 1; k1 < 32; ++k1)
        x[k1] = cmul(x[k1], t[(k1 - 1) * 32]);
}

inline void twiddle_fill(float2* out)
{
    for (int k1 = 1; k1 < 32; ++k1)
        for (int n2 = 0; n2 < 32; ++n2)
        {
            const double a = -2.0 * 3.14159265358979323846 * static_cast<double>(n2) * k1 / static_cast<double>(N);
            *out++ = make_float2(static_cast<float>(cos(a)), static_cast<float>(sin(a)));
        }
}

}  // namespace fftw
}  // namespace hv
