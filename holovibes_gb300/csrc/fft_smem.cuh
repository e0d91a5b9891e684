// Shared-memory mixed-radix Stockham FFT for a tile of F independent transforms of length N.
//
// A CTA owns F "lanes" (rows or columns) of N complex samples. Every thread holds E samples in
// registers; a stage of radix r runs E/r butterflies per thread. Stage s with radix r and
// P = product of the previous radices reads x[i + j*N/r] (j < r), multiplies input j by
// w^(j*k) with k = i mod P and w = exp(-2*pi*i/(P*r)), applies an r-point DFT and writes output
// j to (i - k)*r + k + j*P (auto-sort: the last stage lands in natural order).
// The first stage gathers through a caller functor (global memory, fused convert / lens) and
// the last stage scatters through another (global memory, fused scale / conj / ring slot);
// the stages in between exchange through shared memory.
//
// Shared-memory layout: LANE_FAST tiles (columns) store lane f, sample n at n*F + f and map
// consecutive threads to consecutive lanes; IDX_FAST tiles (rows) store it at f*N + swz(n)
// with swz(n) = n ^ ((n >> 3) & 15), which keeps radix-8 exchanges free of bank conflicts.
#pragma once

#include "hv_common.cuh"

namespace hv {
namespace fft {

template <int... Rs>
struct RadixList
{
};

// Plan<N>: E = samples per thread, List = radices (product N, each divides E).
template <int N>
struct Plan;
#define HV_FFT_PLAN(N_, E_, ...)                                                                                       \
    template <>                                                                                                        \
    struct Plan<N_>                                                                                                    \
    {                                                                                                                  \
        static constexpr int E = E_;                                                                                   \
        using List = RadixList<__VA_ARGS__>;                                                                           \
    };
HV_FFT_PLAN(16, 8, 8, 2)
HV_FFT_PLAN(32, 8, 8, 4)
HV_FFT_PLAN(64, 8, 8, 8)
HV_FFT_PLAN(128, 8, 8, 4, 4)
HV_FFT_PLAN(256, 8, 8, 8, 4)
HV_FFT_PLAN(512, 8, 8, 8, 8)
HV_FFT_PLAN(1024, 16, 16, 8, 8)
HV_FFT_PLAN(2048, 16, 16, 16, 8)
HV_FFT_PLAN(4096, 16, 16, 16, 16)
HV_FFT_PLAN(48, 12, 4, 4, 3)
HV_FFT_PLAN(96, 24, 8, 4, 3)
HV_FFT_PLAN(192, 24, 8, 8, 3)
HV_FFT_PLAN(384, 24, 8, 4, 4, 3)
HV_FFT_PLAN(768, 24, 8, 8, 4, 3)
HV_FFT_PLAN(1536, 24, 8, 8, 8, 3)
#undef HV_FFT_PLAN

// ------------------------------------------------------------------------------ r-point DFTs
// Forward transforms (kernel exp(-2*pi*i*n*k/r)) on r consecutive registers.

__device__ __forceinline__ void dft2(float2& a, float2& b)
{
    const float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

__device__ __forceinline__ void dft4(float2& x0, float2& x1, float2& x2, float2& x3)
{
    const float2 s02 = cadd(x0, x2), d02 = csub(x0, x2);
    const float2 s13 = cadd(x1, x3), d13 = csub(x1, x3);
    x0 = cadd(s02, s13);
    x2 = csub(s02, s13);
    x1 = cadd(d02, cmul_negi(d13));
    x3 = csub(d02, cmul_negi(d13));
}

__device__ __forceinline__ void dft3(float2& x0, float2& x1, float2& x2)
{
    constexpr float s3 = 0.866025403784438646763723170752936183f;  // sin(2*pi/3)
    const float2 t = cadd(x1, x2);
    const float2 d = csub(x1, x2);
    const float2 m = make_float2(x0.x - 0.5f * t.x, x0.y - 0.5f * t.y);
    const float2 sd = make_float2(s3 * d.y, -s3 * d.x);  // -i * s3 * d
    x0 = cadd(x0, t);
    x1 = cadd(m, sd);
    x2 = csub(m, sd);
}

// multiply by w8^m, w8 = exp(-i*pi/4)
template <int m>
__device__ __forceinline__ float2 w8mul(float2 a)
{
    constexpr float c = 0.707106781186547524400844362104849039f;
    if constexpr (m == 0)
        return a;
    else if constexpr (m == 1)
        return make_float2(c * (a.x + a.y), c * (a.y - a.x));
    else if constexpr (m == 2)
        return cmul_negi(a);
    else
        return make_float2(c * (a.y - a.x), -c * (a.x + a.y));
}

__device__ __forceinline__ void dft8(float2* x)
{
    // split: even samples -> E, odd -> O; y_k = E_k + w8^k O_k, y_{k+4} = E_k - w8^k O_k
    float2 e0 = x[0], e1 = x[2], e2 = x[4], e3 = x[6];
    float2 o0 = x[1], o1 = x[3], o2 = x[5], o3 = x[7];
    dft4(e0, e1, e2, e3);
    dft4(o0, o1, o2, o3);
    o1 = w8mul<1>(o1);
    o2 = w8mul<2>(o2);
    o3 = w8mul<3>(o3);
    x[0] = cadd(e0, o0);
    x[4] = csub(e0, o0);
    x[1] = cadd(e1, o1);
    x[5] = csub(e1, o1);
    x[2] = cadd(e2, o2);
    x[6] = csub(e2, o2);
    x[3] = cadd(e3, o3);
    x[7] = csub(e3, o3);
}

// w16^m for m in [0, 9]
__device__ __forceinline__ float2 w16(int m)
{
    // cos / -sin of 2*pi*m/16
    constexpr float c1 = 0.923879532511286756128183189396788933f;
    constexpr float s1 = 0.382683432365089771728459984030398866f;
    constexpr float c2 = 0.707106781186547524400844362104849039f;
    switch (m)
    {
    case 0: return make_float2(1.f, 0.f);
    case 1: return make_float2(c1, -s1);
    case 2: return make_float2(c2, -c2);
    case 3: return make_float2(s1, -c1);
    case 4: return make_float2(0.f, -1.f);
    case 6: return make_float2(-c2, -c2);
    case 9: return make_float2(-c1, s1);
    default: return make_float2(0.f, 0.f);
    }
}

__device__ __forceinline__ void dft16(float2* x)
{
    // n = n2 + 4*n1, k = k1 + 4*k2: DFT4 over n1, twiddle w16^(n2*k1), DFT4 over n2.
    float2 a[4][4];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2)
    {
        a[n2][0] = x[n2];
        a[n2][1] = x[n2 + 4];
        a[n2][2] = x[n2 + 8];
        a[n2][3] = x[n2 + 12];
        dft4(a[n2][0], a[n2][1], a[n2][2], a[n2][3]);
    }
#pragma unroll
    for (int n2 = 1; n2 < 4; ++n2)
#pragma unroll
        for (int k1 = 1; k1 < 4; ++k1)
            a[n2][k1] = cmul(a[n2][k1], w16(n2 * k1));
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1)
    {
        float2 b0 = a[0][k1], b1 = a[1][k1], b2 = a[2][k1], b3 = a[3][k1];
        dft4(b0, b1, b2, b3);
        x[k1] = b0;
        x[k1 + 4] = b1;
        x[k1 + 8] = b2;
        x[k1 + 12] = b3;
    }
}

template <int r>
__device__ __forceinline__ void dft(float2* x)
{
    if constexpr (r == 2)
        dft2(x[0], x[1]);
    else if constexpr (r == 3)
        dft3(x[0], x[1], x[2]);
    else if constexpr (r == 4)
        dft4(x[0], x[1], x[2], x[3]);
    else if constexpr (r == 8)
        dft8(x);
    else if constexpr (r == 16)
        dft16(x);
    else
        static_assert(r == 2, "unsupported radix");
}

// ------------------------------------------------------------------------------ tile engine

template <int N, int F, bool LF>
struct Tile
{
    static constexpr int E = Plan<N>::E;
    static constexpr int NT = F * N / E;  // threads per CTA
    static_assert((F * N) % E == 0, "tile");

    __device__ __forceinline__ static int addr(int f, int n)
    {
        if constexpr (LF)
            return n * F + f;
        else
            return f * N + (n ^ ((n >> 3) & 15));
    }

    template <int r>
    __device__ __forceinline__ static void index(int b, int& f, int& i)
    {
        constexpr int M = N / r;
        if constexpr (LF)
        {
            f = b % F;
            i = b / F;
        }
        else
        {
            f = b / M;
            i = b % M;
        }
    }

    template <int r, class Src>
    __device__ __forceinline__ static void gather(float2 (&x)[E], Src& src)
    {
        constexpr int Q = E / r;
        constexpr int M = N / r;
#pragma unroll
        for (int q = 0; q < Q; ++q)
        {
            int f, i;
            index<r>(static_cast<int>(threadIdx.x) + q * NT, f, i);
#pragma unroll
            for (int j = 0; j < r; ++j)
                x[q * r + j] = src(f, i + j * M);
        }
    }

    // tw: this stage's table, entry (j-1)*P + k = exp(-2 pi i j k / (P r)), so consecutive k
    // (consecutive threads in row tiles) read consecutive entries
    template <int r, int P>
    __device__ __forceinline__ static void butterflies(float2 (&x)[E], const float2* tw)
    {
        constexpr int Q = E / r;
#pragma unroll
        for (int q = 0; q < Q; ++q)
        {
            if constexpr (P > 1)
            {
                int f, i;
                index<r>(static_cast<int>(threadIdx.x) + q * NT, f, i);
                const int k = i % P;
#pragma unroll
                for (int j = 1; j < r; ++j)
                    x[q * r + j] = cmul(x[q * r + j], tw[(j - 1) * P + k]);
            }
            dft<r>(&x[q * r]);
        }
    }

    template <int r, int P, class Dst>
    __device__ __forceinline__ static void scatter(float2 (&x)[E], Dst& dst)
    {
        constexpr int Q = E / r;
#pragma unroll
        for (int q = 0; q < Q; ++q)
        {
            int f, i;
            index<r>(static_cast<int>(threadIdx.x) + q * NT, f, i);
            const int k = i % P;
            const int base = (i - k) * r + k;
#pragma unroll
            for (int j = 0; j < r; ++j)
                dst(f, base + j * P, x[q * r + j]);
        }
    }

    template <int P, int r, int... Rest, class Dst>
    __device__ __forceinline__ static void chain(float2 (&x)[E], float2* sm, const float2* tw, Dst& dst)
    {
        butterflies<r, P>(x, tw);
        if constexpr (sizeof...(Rest) == 0)
        {
            scatter<r, P>(x, dst);
        }
        else
        {
            auto to_sm = [sm](int f, int n, float2 v) { sm[addr(f, n)] = v; };
            scatter<r, P>(x, to_sm);
            __syncthreads();
            auto from_sm = [sm](int f, int n) { return sm[addr(f, n)]; };
            gather<first<Rest...>()>(x, from_sm);
            __syncthreads();
            chain<P * r, Rest...>(x, sm, P > 1 ? tw + P * (r - 1) : tw, dst);
        }
    }

    template <int a, int... Rest>
    __device__ __host__ static constexpr int first()
    {
        return a;
    }

    template <int r0, int... Rest, class Src, class Dst>
    __device__ __forceinline__ static void run_list(RadixList<r0, Rest...>, float2* sm, const float2* tw, Src& src,
                                                    Dst& dst)
    {
        float2 x[E];
        gather<r0>(x, src);
        // the source may alias `sm` (second transform of a tile): finish all reads before the
        // first exchange writes
        __syncthreads();
        chain<1, r0, Rest...>(x, sm, tw, dst);
    }

    // Full forward transform of the tile: src(f, n) -> float2, dst(f, n, float2).
    template <class Src, class Dst>
    __device__ __forceinline__ static void run(float2* sm, const float2* tw, Src& src, Dst& dst)
    {
        run_list(typename Plan<N>::List{}, sm, tw, src, dst);
    }

    // Radix of the first stage and the (lane, sample) pairs a thread loads for it: element
    // q*r0 + j of x holds sample i + j*N/r0 of lane f, (f, i) = index<r0>(thread + q*NT).
    template <int r0, int... Rest>
    __device__ __host__ static constexpr int first_of(RadixList<r0, Rest...>)
    {
        return r0;
    }
    static constexpr int R0 = first_of(typename Plan<N>::List{});

    template <int r0, int... Rest, class Dst>
    __device__ __forceinline__ static void run_regs_list(RadixList<r0, Rest...>, float2 (&x)[E], float2* sm,
                                                         const float2* tw, Dst& dst)
    {
        chain<1, r0, Rest...>(x, sm, tw, dst);
    }

    // Transform of the tile whose first-stage inputs the caller already loaded into x.
    template <class Dst>
    __device__ __forceinline__ static void run_regs(float2 (&x)[E], float2* sm, const float2* tw, Dst& dst)
    {
        run_regs_list(typename Plan<N>::List{}, x, sm, tw, dst);
    }
};

// Host-side layout of the per-stage twiddle tables of Plan<N>: stages with P > 1 in order, each
// P * (r - 1) entries (j - 1) * P + k = exp(-2 pi i j k / (P r)).
template <int... Rs>
inline int twiddle_count(RadixList<Rs...>)
{
    int total = 0, P = 1;
    for (int r : {Rs...})
    {
        if (P > 1)
            total += P * (r - 1);
        P *= r;
    }
    return total;
}

template <int... Rs>
inline void twiddle_fill(RadixList<Rs...>, float2* out)
{
    int P = 1;
    for (int r : {Rs...})
    {
        if (P > 1)
        {
            for (int j = 1; j < r; ++j)
                for (int k = 0; k < P; ++k)
                {
                    const double a = -2.0 * 3.14159265358979323846 * static_cast<double>(j) * k / (static_cast<double>(P) * r);
                    *out++ = make_float2(static_cast<float>(cos(a)), static_cast<float>(sin(a)));
                }
        }
        P *= r;
    }
}

}  // namespace fft
}  // namespace hv
