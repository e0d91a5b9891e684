// 512- and 1024-point FFTs with 32 samples per thread: N = NG x 32 (NG = 16 or 32), stage-A
// DFTs of length NG, one shared-memory transpose, a 32-point stage-B DFT.
//
// A transform is owned by NG threads; thread g (0..NG-1) holds samples n = g + NG i, i = 0..31.
// Decomposition n = n2 + 32 n1 (n2 < 32, n1 < NG), k = k1 + NG k2 (k1 < NG, k2 < 32):
//   stage A  z[n2][k1] = w_N^(n2 k1) * sum_n1 x[n2 + 32 n1] w_NG^(n1 k1)   (thread g computes the
//            groups n2 = g, and n2 = g + 16 when NG = 16: its samples g + 16 i split by parity of i)
//   stage B  X[k1 + NG k2] = sum_n2 z[n2][k1] w_32^(n2 k2)                  (thread g owns k1 = g)
// so after stage B thread g holds X[g + NG k2] in element k2: the same shape as stage A's input,
// which lets a forward transform be followed by an inverse one without another exchange.
//
// Compared with the Stockham tile engine (16 x 8 x 8 at 16 samples per thread for N = 1024) this
// halves the shared-memory exchanges, replaces the per-element index arithmetic (lane / sample
// decoding, swizzles, twiddle indices) with compile-time register offsets and, for rows, keeps
// every exchange inside one warp (__syncwarp, no CTA barrier).
#pragma once

#include "fft_smem.cuh"

namespace hv {
namespace fftw {

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

template <int N>
struct Warp
{
    static_assert(N == 512 || N == 1024, "warp FFT lengths");
    static constexpr int NG = N / 32;               // threads per transform = stage-B outputs per thread
    static constexpr int TW_COUNT = (NG - 1) * 32;  // entry (k1 - 1) * 32 + n2 = exp(-2 pi i n2 k1 / N)

    // stage-A element e of thread g holds z[n2][k1] with n2 = g + 16 (e / 16) for NG = 16
    __device__ __forceinline__ static int n2_of(int e, int g) { return NG == 32 ? g : g + 16 * (e >> 4); }
    __device__ __host__ static constexpr int k1_of(int e) { return NG == 32 ? e : (e & 15); }

    // x[i] = sample g + NG i on entry; z[n2_of(e)][k1_of(e)] * w_N^(n2 k1) in element e on return.
    // tw: shared-memory table of this length.
    __device__ __forceinline__ static void stage_a(float2 (&x)[32], const float2* tw, int g)
    {
        if constexpr (NG == 32)
        {
            dft32(x);
            const float2* t = tw + g;
#pragma unroll
            for (int k1 = 1; k1 < 32; ++k1)
                x[k1] = cmul(x[k1], t[(k1 - 1) * 32]);
        }
        else
        {
            float2 a[16], b[16];
#pragma unroll
            for (int j = 0; j < 16; ++j)
            {
                a[j] = x[2 * j];      // group g:      samples g + 32 j
                b[j] = x[2 * j + 1];  // group g + 16: samples g + 16 + 32 j
            }
            fft::dft16(a);
            fft::dft16(b);
            const float2* ta = tw + g;
            const float2* tb = tw + g + 16;
            x[0] = a[0];
            x[16] = b[0];
#pragma unroll
            for (int k1 = 1; k1 < 16; ++k1)
            {
                x[k1] = cmul(a[k1], ta[(k1 - 1) * 32]);
                x[16 + k1] = cmul(b[k1], tb[(k1 - 1) * 32]);
            }
        }
    }

    static void twiddle_fill(float2* out)
    {
        for (int k1 = 1; k1 < NG; ++k1)
            for (int n2 = 0; n2 < 32; ++n2)
            {
                const double a = -2.0 * 3.14159265358979323846 * static_cast<double>(n2) * k1 / static_cast<double>(N);
                *out++ = make_float2(static_cast<float>(cos(a)), static_cast<float>(sin(a)));
            }
    }
};

// ------------------------------------------------------------------------- N = 768 = 24 x 32
// Two orders, each with 32 samples at most per thread:
//   V24 (DFT24 first): thread g < 32 holds samples g + 32 i (i < 24); stage A = DFT24 and the
//        twiddle w768^(g k1) (k1 < 24); after the transpose thread k1 < 24 holds z[n2][k1] for
//        n2 < 32, stage B = DFT32, leaving X[k1 + 24 k2] (k2 < 32) in element k2.
//   V32 (DFT32 first): thread g < 24 holds samples g + 24 i (i < 32); stage A = DFT32 and the
//        twiddle w768^(g k1) (k1 < 32); after the transpose thread k1 < 32 holds z[n2][k1] for
//        n2 < 24, stage B = DFT24, leaving X[k1 + 32 k2] (k2 < 24) in element k2.
// V24's output has V32's input shape and the other way round (the AS middle pass: V24 forward,
// * G, V32 inverse, no extra exchange).

// cos / sin of 2 pi r / 24 for r = 0..5
__host__ __device__ constexpr float c24(int r)
{
    return r == 0   ? 1.0f
           : r == 1 ? 0.965925826289068286749743199728897367f
           : r == 2 ? 0.866025403784438646763723170752936183f
           : r == 3 ? 0.707106781186547524400844362104849039f
           : r == 4 ? 0.5f
                    : 0.258819045102520762348898837624048328f;
}
__host__ __device__ constexpr float s24(int r) { return r == 0 ? 0.0f : c24(6 - r); }

// a * w24^m, w24 = exp(-2 pi i / 24) (w24^6 = -i); m is a constant after unrolling
__device__ __forceinline__ float2 w24mul(int m, float2 a)
{
    const int r = m % 6, q = (m / 6) & 3;
    float2 b;
    if (r == 0)
        b = a;
    else if (r == 3)
        b = fft::w8mul<1>(a);
    else
    {
        const float c = c24(r), s = s24(r);
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

// Forward 24-point DFT in place on x[0..23] (natural order): n = 3 n1 + n2, k = k1 + 8 k2; DFT8
// over n1, twiddle w24^(n2 k1), DFT3 over n2.
__device__ __forceinline__ void dft24(float2* x)
{
    float2 a[3][8];
#pragma unroll
    for (int n2 = 0; n2 < 3; ++n2)
    {
#pragma unroll
        for (int n1 = 0; n1 < 8; ++n1)
            a[n2][n1] = x[3 * n1 + n2];
        fft::dft8(a[n2]);
    }
#pragma unroll
    for (int n2 = 1; n2 < 3; ++n2)
#pragma unroll
        for (int k1 = 1; k1 < 8; ++k1)
            a[n2][k1] = w24mul(n2 * k1, a[n2][k1]);
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1)
    {
        fft::dft3(a[0][k1], a[1][k1], a[2][k1]);
        x[k1] = a[0][k1];
        x[k1 + 8] = a[1][k1];
        x[k1 + 16] = a[2][k1];
    }
}

struct W768
{
    static constexpr int N = 768;
    static constexpr int TW24 = 23 * 32;  // V24 entry (k1 - 1) * 32 + g = exp(-2 pi i g k1 / 768), g < 32
    static constexpr int TW32 = 31 * 24;  // V32 entry (k1 - 1) * 24 + g, g < 24 (stored after V24's)
    static constexpr int TW_COUNT = TW24 + TW32;

    // V24 stage A: x[i] = sample g + 32 i (i < 24) -> z[g][k1] * w^(g k1) in x[k1] (k1 < 24)
    __device__ __forceinline__ static void stage_a24(float2 (&x)[32], const float2* tw, int g)
    {
        dft24(x);
        const float2* t = tw + g;
#pragma unroll
        for (int k1 = 1; k1 < 24; ++k1)
            x[k1] = cmul(x[k1], t[(k1 - 1) * 32]);
    }
    // V32 stage A: x[i] = sample g + 24 i (i < 32, g < 24) -> z[g][k1] * w^(g k1) in x[k1]
    __device__ __forceinline__ static void stage_a32(float2 (&x)[32], const float2* tw, int g)
    {
        dft32(x);
        const float2* t = tw + TW24 + g;
#pragma unroll
        for (int k1 = 1; k1 < 32; ++k1)
            x[k1] = cmul(x[k1], t[(k1 - 1) * 24]);
    }

    static void twiddle_fill(float2* out)
    {
        for (int k1 = 1; k1 < 24; ++k1)
            for (int g = 0; g < 32; ++g)
            {
                const double a = -2.0 * 3.14159265358979323846 * static_cast<double>(g) * k1 / static_cast<double>(N);
                *out++ = make_float2(static_cast<float>(cos(a)), static_cast<float>(sin(a)));
            }
        for (int k1 = 1; k1 < 32; ++k1)
            for (int g = 0; g < 24; ++g)
            {
                const double a = -2.0 * 3.14159265358979323846 * static_cast<double>(g) * k1 / static_cast<double>(N);
                *out++ = make_float2(static_cast<float>(cos(a)), static_cast<float>(sin(a)));
            }
    }
};

}  // namespace fftw
}  // namespace hv
