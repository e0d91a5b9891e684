// Spatial stage: lenses, fused convert + 2-D FFT passes, Fresnel / angular-spectrum propagation.
//
// Reference behaviour (Holovibes):
//   convert        Backend/cuda_sources/tools_conversion.cu:107-171
//   Fresnel lens   Backend/cuda_sources/masks.cu:7-29, fresnel_transform.cu:14-63
//   AS lens        Backend/cuda_sources/masks.cu:31-59, angular_spectrum.cu:14-31, fourier_transform.cc:121-137
//   Fresnel        Backend/cuda_sources/fresnel_transform.cu:65-83   (x*L then forward FFT2, no 1/N)
//   angular spec.  Backend/cuda_sources/angular_spectrum.cu:33-63     (FFT2, *G, inverse FFT2, /(H*W))
//   ring enqueue   Backend/sources/data_struct/queue.cc:332-380
//   filter2D       Backend/cuda_sources/filter2D.cu:28-115, fourier_transform.cc:30-72,121-137
//                  (circular band-pass mask, shifted to FFT layout; x <- IFFT2(FFT2(x) M)
//                  unnormalised before Fresnel / no propagation, folded into G for AS)
//
// GB300 design: no cuFFT. A batch of B frames goes through two or three shared-memory passes:
//   row pass   : raw u8/u16/f32 -> complex (+ Fresnel lens) -> forward row FFT
//   column pass: forward column FFT (+ transfer function G, inverse column FFT for AS)
//   row pass   : inverse row FFT * 1/(H*W) (AS only)
// and the last pass writes straight into the time-ring slots, so the reference's separate
// mask, divide and ring-copy passes disappear. Passes of 512, 768 and 1024 points use the warp
// engine (fft_warp.cuh: 32 samples per thread, one transpose; the 1024-point passes persistent and
// fed by TMA where they apply), every other length the shared-memory Stockham tile engine
// (fft_smem.cuh).
#include <math.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "fft_smem.cuh"
#include "fft_warp.cuh"
#include "tc_common.cuh"
#include "hv_internal.h"

namespace hv {

// ====================================================================================== lenses

__global__ void k_fresnel_lens(float2* out, int W, int H, double lam, double z, double pixel_size_um, int mode)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= W || y >= H)
        return;
    const int S = W > H ? W : H;
    // centre crop of the S x S lens (fresnel_transform.cu:37-62)
    const int si = (H > W) ? x + (S - W) / 2 : x;
    const int sj = (W > H) ? y + (S - H) / 2 : y;
    float2 v;
    if (mode == HV_LENS_REF32)
    {
        const float lam32 = static_cast<float>(lam), z32 = static_cast<float>(z);
        const float c = static_cast<float>(M_PI / static_cast<double>(__fmul_rn(lam32, z32)));
        const float dx = __fmul_rn(static_cast<float>(pixel_size_um), 1.0e-6f);
        const float xf = __fmul_rn(__fsub_rn(static_cast<float>(si), static_cast<float>(S >> 1)), dx);
        const float yf = __fmul_rn(__fsub_rn(static_cast<float>(sj), static_cast<float>(S >> 1)), dx);
        // x * x + y * y contracted into one fused multiply-add, as the reference's build compiles it
        const float cs = __fmul_rn(c, __fmaf_rn(xf, xf, __fmul_rn(yf, yf)));
        v = make_float2(cosf(cs), sinf(cs));
    }
    else
    {
        const double dx = pixel_size_um * 1e-6;
        const double xd = (si - (S >> 1)) * dx;
        const double yd = (sj - (S >> 1)) * dx;
        double ph = M_PI / (lam * z) * (xd * xd + yd * yd);
        ph = fmod(ph, 2.0 * M_PI);
        double s, c;
        sincos(ph, &s, &c);
        v = make_float2(static_cast<float>(c), static_cast<float>(s));
    }
    out[static_cast<size_t>(y) * W + x] = v;
}

__global__ void k_spectral_lens(float2* out, int W, int H, double lam, double z, double pixel_size_um, int mode)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= W || y >= H)
        return;
    float2 v;
    if (mode == HV_LENS_REF32)
    {
        const float lam32 = static_cast<float>(lam), z32 = static_cast<float>(z);
        const float step = __fmul_rn(static_cast<float>(pixel_size_um), 1e-6f);
        const float u_step = __fdiv_rn(1.0f, __fmul_rn(static_cast<float>(W), step));
        const float v_step = __fdiv_rn(1.0f, __fmul_rn(static_cast<float>(H), step));
        const float u = __fmul_rn(static_cast<float>(x - (W >> 1)), u_step);
        const float vv = __fmul_rn(static_cast<float>(y - (H >> 1)), v_step);
        // the reference's build contracts u * u + v * v and 1 - (lam^2 * s) into fused multiply-adds
        // (matched bit for bit against its lens on the benchmark sizes)
        const float s2 = __fmaf_rn(u, u, __fmul_rn(vv, vv));
        float tmp = __fmaf_rn(-__fmul_rn(lam32, lam32), s2, 1.0f);
        if (tmp < 0.0f)
            tmp = 0.0f;
        const double ph_d = __dmul_rn(__ddiv_rn(__dmul_rn(2.0 * M_PI, static_cast<double>(z32)), static_cast<double>(lam32)),
                                      static_cast<double>(__fsqrt_rn(tmp)));
        const float ph = static_cast<float>(ph_d);
        v = make_float2(cosf(ph), sinf(ph));
    }
    else
    {
        const double step = pixel_size_um * 1e-6;
        const double u = (x - (W >> 1)) / (W * step);
        const double vv = (y - (H >> 1)) / (H * step);
        double tmp = 1.0 - lam * lam * (u * u + vv * vv);
        if (tmp < 0.0)
            tmp = 0.0;
        double ph = 2.0 * M_PI * z / lam * sqrt(tmp);
        ph = fmod(ph, 2.0 * M_PI);
        double s, c;
        sincos(ph, &s, &c);
        v = make_float2(static_cast<float>(c), static_cast<float>(s));
    }
    // quadrant swap into FFT layout (shift_corners on the lens, fourier_transform.cc:134)
    const int xs = (x + W / 2) % W;
    const int ys = (y + H / 2) % H;
    out[static_cast<size_t>(ys) * W + xs] = v;
}

// ====================================================================================== FFT passes

struct RowPass
{
    const void* in;        // batch of frames, row-major rows x N
    int in_kind;           // InKind
    size_t in_frame;       // elements between input frames
    float2* out;
    FrameMap out_map;      // output frame slots
    const float2* premul;  // rows x N multiplier applied before the transform (or null)
    int rows;              // rows per frame
    int inverse;           // 1: conj in / conj out (unnormalised inverse)
    float scale;
    const float2* tw;      // per-stage twiddle tables of the N-point plan (device)
    int tw_count;
    int stream_out;        // 1: output written with an evict-first hint (ring slots)
    const CycleCtl* ctl = nullptr;  // served cycle: gate (active) and, with raw_from_ctl, the input offset
    int raw_from_ctl = 0;           // 1: `in` is the input ring base, the batch is at ctl->raw_offset
    int reserve_sms = 0;            // persistent passes leave this many SMs to kernels of other streams
};

// Copies the plan's twiddle tables next to the tile in shared memory (read conflict-free:
// consecutive threads read consecutive entries in row tiles, one broadcast entry in column tiles).
__device__ __forceinline__ const float2* stage_twiddles(float2* dst, const float2* __restrict__ src, int count,
                                                        int nthreads)
{
    for (int e = threadIdx.x; e < count; e += nthreads)
        dst[e] = __ldg(src + e);
    __syncthreads();
    return dst;
}

template <int N, int F>
__global__ void __launch_bounds__(fft::Tile<N, F, false>::NT) k_fft_rows(RowPass p)
{
    using Tl = fft::Tile<N, F, false>;
    extern __shared__ float2 smem[];
    if (!ctl_active(p.ctl))
        return;
    const void* p_in = p.raw_from_ctl ? static_cast<const void*>(static_cast<const uint8_t*>(p.in) + p.ctl->raw_offset)
                                      : p.in;
    float2* sm = smem;
    const float2* tw = stage_twiddles(smem + F * N, p.tw, p.tw_count, Tl::NT);

    const int b = blockIdx.y;
    const int row0 = blockIdx.x * F;
    const size_t in_base = static_cast<size_t>(b) * p.in_frame;
    const int rows = p.rows;
    const bool inv = p.inverse != 0;
    constexpr int E = Tl::E, R0 = Tl::R0, Q0 = E / R0, M0 = N / R0;

    // First-stage inputs: every load of the thread is issued before any is used (the input kind
    // and the lens multiply are uniform branches outside the element loops).
    float2 x[E];
    size_t rb[Q0];  // element (q, j) sits at rb[q] + j * M0
    bool ok[Q0];
#pragma unroll
    for (int q = 0; q < Q0; ++q)
    {
        int f, i;
        Tl::template index<R0>(static_cast<int>(threadIdx.x) + q * Tl::NT, f, i);
        const int y = row0 + f;
        ok[q] = y < rows;
        rb[q] = static_cast<size_t>(ok[q] ? y : 0) * N + i;
    }
#define HV_EIDX(e) (rb[(e) / R0] + ((e) % R0) * M0)
    switch (p.in_kind)
    {
    case IN_U8:
    {
        const uint8_t* in = static_cast<const uint8_t*>(p_in) + in_base;
        uint8_t v[E];
#pragma unroll
        for (int e = 0; e < E; ++e)
            v[e] = __ldcs(in + HV_EIDX(e));
#pragma unroll
        for (int e = 0; e < E; ++e)
            x[e] = make_float2(static_cast<float>(v[e]) * 257.0f, 0.f);
        break;
    }
    case IN_U16:
    case IN_U16_BE:
    {
        const uint16_t* in = static_cast<const uint16_t*>(p_in) + in_base;
        uint16_t v[E];
#pragma unroll
        for (int e = 0; e < E; ++e)
            v[e] = __ldcs(in + HV_EIDX(e));
        const bool swap = p.in_kind == IN_U16_BE;
#pragma unroll
        for (int e = 0; e < E; ++e)
        {
            const uint16_t u = swap ? static_cast<uint16_t>((v[e] << 8) | (v[e] >> 8)) : v[e];
            x[e] = make_float2(static_cast<float>(u), 0.f);
        }
        break;
    }
    case IN_F32:
    {
        const float* in = static_cast<const float*>(p_in) + in_base;
#pragma unroll
        for (int e = 0; e < E; ++e)
            x[e] = make_float2(__ldcs(in + HV_EIDX(e)), 0.f);
        break;
    }
    default:
    {
        const float2* in = static_cast<const float2*>(p_in) + in_base;
#pragma unroll
        for (int e = 0; e < E; ++e)
            x[e] = __ldg(in + HV_EIDX(e));
        break;
    }
    }
    if (p.premul)
    {
        float2 L[E];
#pragma unroll
        for (int e = 0; e < E; ++e)
            L[e] = __ldg(p.premul + HV_EIDX(e));
#pragma unroll
        for (int e = 0; e < E; ++e)
            x[e] = cmul(x[e], L[e]);
    }
#undef HV_EIDX
#pragma unroll
    for (int q = 0; q < Q0; ++q)
#pragma unroll
        for (int j = 0; j < R0; ++j)
        {
            float2& v = x[q * R0 + j];
            if (!ok[q])
                v = make_float2(0.f, 0.f);
            else if (inv)
                v = cconj(v);
        }

    float2* out = p.out + p.out_map.offset(b);
    const float sc = p.scale;
    const bool stream_out = p.stream_out != 0;
    auto dst = [&](int f, int n, float2 v) {
        const int y = row0 + f;
        if (y >= rows)
            return;
        if (inv)
            v = cconj(v);
        float2* o = out + static_cast<size_t>(y) * N + n;
        if (stream_out)
            __stcs(o, cscale(v, sc));
        else
            *o = cscale(v, sc);
    };
    Tl::run_regs(x, sm, tw, dst);
}

struct ColPass
{
    const float2* in;
    size_t in_frame;
    float2* out;
    FrameMap out_map;
    const float2* postmul;  // rows x width multiplier applied between forward and inverse (AS), or null
    int width;              // row length (number of columns)
    int mode;               // 0 forward, 1 inverse, 2 forward * postmul then inverse
    float scale;
    const float2* tw;       // per-stage twiddle tables of the N-point plan (device)
    int tw_count;
    int stream_out;         // 1: output written with an evict-first hint (ring slots)
    const CycleCtl* ctl = nullptr;  // served cycle: gate (active)
    int reserve_sms = 0;            // persistent passes leave this many SMs to kernels of other streams
};

template <int N, int F>
__global__ void __launch_bounds__(fft::Tile<N, F, true>::NT) k_fft_cols(ColPass p)
{
    using Tl = fft::Tile<N, F, true>;
    extern __shared__ float2 smem[];
    if (!ctl_active(p.ctl))
        return;
    float2* sm = smem;
    const float2* tw = stage_twiddles(smem + F * N, p.tw, p.tw_count, Tl::NT);

    const int b = blockIdx.y;
    const int c0 = blockIdx.x * F;
    const int W = p.width;
    const float2* in = p.in + static_cast<size_t>(b) * p.in_frame;
    float2* out = p.out + p.out_map.offset(b);
    const float sc = p.scale;
    if (p.mode == 2)
    {
        auto src = [&](int f, int n) -> float2 {
            const int c = c0 + f;
            return (c < W) ? in[static_cast<size_t>(n) * W + c] : make_float2(0.f, 0.f);
        };
        const float2* G = p.postmul;
        // forward result * G, conjugated for the inverse transform, parked in shared memory
        auto mid = [&](int f, int n, float2 v) {
            const int c = c0 + f;
            const float2 g = (c < W) ? __ldg(G + static_cast<size_t>(n) * W + c) : make_float2(0.f, 0.f);
            sm[Tl::addr(f, n)] = cconj(cmul(v, g));
        };
        Tl::run(sm, tw, src, mid);
        __syncthreads();
        auto src2 = [&](int f, int n) -> float2 { return sm[Tl::addr(f, n)]; };
        auto dst2 = [&](int f, int n, float2 v) {
            const int c = c0 + f;
            if (c < W)
                out[static_cast<size_t>(n) * W + c] = cscale(cconj(v), sc);
        };
        Tl::run(sm, tw, src2, dst2);
    }
    else
    {
        const bool inv = p.mode == 1;
        auto src = [&](int f, int n) -> float2 {
            const int c = c0 + f;
            if (c >= W)
                return make_float2(0.f, 0.f);
            const float2 v = in[static_cast<size_t>(n) * W + c];
            return inv ? cconj(v) : v;
        };
        const bool stream_out = p.stream_out != 0;
        auto dst = [&](int f, int n, float2 v) {
            const int c = c0 + f;
            if (c >= W)
                return;
            if (inv)
                v = cconj(v);
            float2* o = out + static_cast<size_t>(n) * W + c;
            if (stream_out)
                __stcs(o, cscale(v, sc));
            else
                *o = cscale(v, sc);
        };
        Tl::run(sm, tw, src, dst);
    }
}

// ------------------------------------------------------------------ warp engine (N = 512, 1024)
// Rows: 32 / NG rows per warp (1 or 2), 8 warps per CTA; lane (r, g) = (lane / NG, lane % NG);
// the transpose in the warp's own [row][n2][k1] block, k1 rows padded to NG + 1 entries
// (conflict-free both ways). Columns: 256 / NG adjacent columns per CTA (8 or 16), thread
// (c, g) = (t % C, t / C) holds samples g + NG i of column c (a warp load covers 32 / C rows of
// C * 8 bytes); the transpose goes through a [k1][n2][c] block (conflict-free: k1 rows padded
// to 264 entries when C = 8).
constexpr int W32_WARPS = 8;
constexpr int W32_THREADS = 256;

template <int N>
struct W32Geom
{
    static constexpr int NG = fftw::Warp<N>::NG;
    static constexpr int RPW = 32 / NG;                 // rows per warp
    static constexpr int ROWS = W32_WARPS * RPW;        // rows per CTA
    static constexpr int ROW_PAD = NG + 1;
    static constexpr int ROW_BUF = RPW * 32 * ROW_PAD;  // per warp
    static constexpr int COLS = W32_THREADS / NG;       // columns per CTA
    static constexpr int COL_PAD = 32 * COLS + (COLS == 8 ? 8 : 0);
    static constexpr int TW = fftw::Warp<N>::TW_COUNT;
    static constexpr size_t ROW_SMEM = (TW + static_cast<size_t>(W32_WARPS) * ROW_BUF) * sizeof(float2);
    static constexpr size_t COL_SMEM = (TW + static_cast<size_t>(NG) * COL_PAD) * sizeof(float2);
};

// First-stage samples of one row: x[j] = converted sample at e0 + STRIDE j (j < NS) of the input,
// times premul[l0 + STRIDE j] when the pass has one, conjugated for an inverse pass. Every load of
// the thread is issued before any is used (the input kind is a uniform branch).
template <int NS, int STRIDE>
__device__ __forceinline__ void load_row_samples(const RowPass& p, const void* p_in, size_t e0, size_t l0,
                                                 float2 (&x)[32])
{
    const bool inv = p.inverse != 0;
    if (p.in_kind == IN_C64)
    {
        const float2* in = static_cast<const float2*>(p_in) + e0;
#pragma unroll
        for (int j = 0; j < NS; ++j)
            x[j] = __ldg(in + STRIDE * j);
        if (p.premul)
        {
            const float2* L = p.premul + l0;
#pragma unroll
            for (int j = 0; j < NS; ++j)
                x[j] = cmul(x[j], __ldg(L + STRIDE * j));
        }
    }
    else
    {
        float v[NS];
        bool pre_done = false;  // x already holds the converted, premultiplied samples
        switch (p.in_kind)
        {
        case IN_U8:
        {
            const uint8_t* in = static_cast<const uint8_t*>(p_in) + e0;
            uint8_t u[NS];
#pragma unroll
            for (int j = 0; j < NS; ++j)
                u[j] = __ldcs(in + STRIDE * j);
            if (p.premul)
            {
                // the lens loads go out before the pixels are used: one memory round trip, not two
                const float2* L = p.premul + l0;
#pragma unroll
                for (int j = 0; j < NS; ++j)
                    x[j] = __ldg(L + STRIDE * j);
#pragma unroll
                for (int j = 0; j < NS; ++j)
                {
                    const float f = static_cast<float>(u[j]) * 257.0f;
                    x[j] = make_float2(f * x[j].x, f * x[j].y);
                }
                pre_done = true;
                break;
            }
#pragma unroll
            for (int j = 0; j < NS; ++j)
                v[j] = static_cast<float>(u[j]) * 257.0f;
            break;
        }
        case IN_U16:
        case IN_U16_BE:
        {
            const uint16_t* in = static_cast<const uint16_t*>(p_in) + e0;
            uint16_t u[NS];
#pragma unroll
            for (int j = 0; j < NS; ++j)
                u[j] = __ldcs(in + STRIDE * j);
            const bool swap = p.in_kind == IN_U16_BE;
#pragma unroll
            for (int j = 0; j < NS; ++j)
                v[j] = static_cast<float>(swap ? static_cast<uint16_t>((u[j] << 8) | (u[j] >> 8)) : u[j]);
            break;
        }
        default:
        {
            const float* in = static_cast<const float*>(p_in) + e0;
#pragma unroll
            for (int j = 0; j < NS; ++j)
                v[j] = __ldcs(in + STRIDE * j);
            break;
        }
        }
        if (pre_done)
        {
        }
        else if (p.premul)
        {
            const float2* L = p.premul + l0;
#pragma unroll
            for (int j = 0; j < NS; ++j)
            {
                const float2 l = __ldg(L + STRIDE * j);
                x[j] = make_float2(v[j] * l.x, v[j] * l.y);
            }
        }
        else
        {
#pragma unroll
            for (int j = 0; j < NS; ++j)
                x[j] = make_float2(v[j], 0.f);
        }
    }
    if (inv)
    {
#pragma unroll
        for (int j = 0; j < NS; ++j)
            x[j] = cconj(x[j]);
    }
}

template <int N>
__global__ void __launch_bounds__(W32_THREADS, 2) k_fft_rows_w32(RowPass p)
{
    using Gm = W32Geom<N>;
    using Wp = fftw::Warp<N>;
    constexpr int NG = Gm::NG;
    extern __shared__ float2 smem[];
    if (!ctl_active(p.ctl))
        return;
    const float2* tw = stage_twiddles(smem, p.tw, Gm::TW, W32_THREADS);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = lane / NG, g = lane % NG;
    const int y = blockIdx.x * Gm::ROWS + warp * Gm::RPW + r;
    // lanes of a row past the frame's last row compute on zeros and store nothing (they take part
    // in the warp's transpose)
    const bool row_ok = y < p.rows;
    const int yc = row_ok ? y : 0;
    float2* buf = smem + Gm::TW + warp * Gm::ROW_BUF + r * 32 * Gm::ROW_PAD;
    const int b = blockIdx.y;
    const void* p_in = p.raw_from_ctl ? static_cast<const void*>(static_cast<const uint8_t*>(p.in) + p.ctl->raw_offset)
                                      : p.in;
    const size_t e0 = static_cast<size_t>(b) * p.in_frame + static_cast<size_t>(yc) * N + g;
    const bool inv = p.inverse != 0;

    float2 x[32];
    load_row_samples<32, NG>(p, p_in, e0, static_cast<size_t>(yc) * N + g, x);
    Wp::stage_a(x, tw, g);
    // transpose: z[n2][k1] at buf[n2 * ROW_PAD + k1]; thread g then reads z[n2][g] for every n2
#pragma unroll
    for (int e = 0; e < 32; ++e)
        buf[Wp::n2_of(e, g) * Gm::ROW_PAD + Wp::k1_of(e)] = x[e];
    __syncwarp();
#pragma unroll
    for (int n2 = 0; n2 < 32; ++n2)
        x[n2] = buf[n2 * Gm::ROW_PAD + g];
    fftw::dft32(x);

    if (!row_ok)
        return;
    float2* o = p.out + p.out_map.offset(b) + static_cast<size_t>(y) * N + g;
    const float sc = p.scale;
#pragma unroll
    for (int k2 = 0; k2 < 32; ++k2)
    {
        float2 v = x[k2];
        if (inv)
            v = cconj(v);
        v = cscale(v, sc);
        if (p.stream_out)
            __stcs(o + NG * k2, v);
        else
            o[NG * k2] = v;
    }
}

// Column transpose through shared memory: thread (c, g) writes its z[n2][k1], then reads z[n2][g]
// for every n2 (g now the k1 it owns). Ends with a barrier so the block can be reused.
template <int N>
__device__ __forceinline__ void w32_col_exchange(float2 (&x)[32], float2* S, int c, int g)
{
    using Gm = W32Geom<N>;
    using Wp = fftw::Warp<N>;
#pragma unroll
    for (int e = 0; e < 32; ++e)
        S[Wp::k1_of(e) * Gm::COL_PAD + Wp::n2_of(e, g) * Gm::COLS + c] = x[e];
    __syncthreads();
    const float2* rd = S + g * Gm::COL_PAD + c;
#pragma unroll
    for (int n2 = 0; n2 < 32; ++n2)
        x[n2] = rd[n2 * Gm::COLS];
    __syncthreads();
}

template <int N>
__global__ void __launch_bounds__(W32_THREADS, 2) k_fft_cols_w32(ColPass p)
{
    using Gm = W32Geom<N>;
    using Wp = fftw::Warp<N>;
    constexpr int NG = Gm::NG;
    extern __shared__ float2 smem[];
    if (!ctl_active(p.ctl))
        return;
    const float2* tw = stage_twiddles(smem, p.tw, Gm::TW, W32_THREADS);
    float2* S = smem + Gm::TW;
    const int c = threadIdx.x % Gm::COLS, g = threadIdx.x / Gm::COLS;
    const int W = p.width;
    const int col = blockIdx.x * Gm::COLS + c;
    const bool in_range = col < W;
    const int b = blockIdx.y;
    // sample g + NG j of column `col` sits at g W + col + j (NG W)
    const size_t e0 = static_cast<size_t>(g) * W + col;
    const size_t step = static_cast<size_t>(NG) * W;
    const float2* in = p.in + static_cast<size_t>(b) * p.in_frame + e0;
    const bool inv_in = p.mode == 1;

    float2 x[32];
#pragma unroll
    for (int j = 0; j < 32; ++j)
        x[j] = in_range ? in[j * step] : make_float2(0.f, 0.f);
    if (inv_in)
    {
#pragma unroll
        for (int j = 0; j < 32; ++j)
            x[j] = cconj(x[j]);
    }
    Wp::stage_a(x, tw, g);
    w32_col_exchange<N>(x, S, c, g);
    fftw::dft32(x);

    float2* o = p.out + p.out_map.offset(b) + e0;
    const float sc = p.scale;
    if (p.mode == 2)
    {
        // * G, conjugate, inverse transform (stage B left X[g + NG k2], stage A's input shape)
        const float2* Gp = p.postmul + e0;
#pragma unroll
        for (int k2 = 0; k2 < 32; ++k2)
        {
            const float2 gv = in_range ? __ldg(Gp + k2 * step) : make_float2(0.f, 0.f);
            x[k2] = cconj(cmul(x[k2], gv));
        }
        Wp::stage_a(x, tw, g);
        w32_col_exchange<N>(x, S, c, g);
        fftw::dft32(x);
        if (in_range)
        {
#pragma unroll
            for (int k2 = 0; k2 < 32; ++k2)
                o[k2 * step] = cscale(cconj(x[k2]), sc);
        }
        return;
    }
    if (!in_range)
        return;
#pragma unroll
    for (int k2 = 0; k2 < 32; ++k2)
    {
        float2 v = x[k2];
        if (inv_in)
            v = cconj(v);
        v = cscale(v, sc);
        if (p.stream_out)
            __stcs(o + k2 * step, v);
        else
            o[k2 * step] = v;
    }
}

// ------------------------------------------------------------------ warp engine, TMA-fed columns
// Persistent column pass (N = 1024): one CTA per SM walks the tiles blockIdx.x, + gridDim.x, ...
// (a tile = 8 columns x 1024 rows of one frame, 64 KB). The tile two steps ahead is loaded by TMA
// (four 256-row boxes) into one of two staging buffers while the current tile is transformed
// from registers, so the column reads stream without the per-tile load latency of the
// register-loading kernel. The waits are bounded; a wait that gives up sets g_fft_wait_error,
// lets the copies already issued land and ends the CTA.
__device__ int g_fft_wait_error = 0;

constexpr int WT_N = 1024;
constexpr int WT_COLS = W32Geom<WT_N>::COLS;
constexpr int WT_TILE = WT_N * WT_COLS;  // float2 per tile
constexpr size_t WT_SMEM = 1024 + (2 * static_cast<size_t>(WT_TILE) + fftw::Warp<WT_N>::NG * W32Geom<WT_N>::COL_PAD +
                                   fftw::Warp<WT_N>::TW_COUNT) * sizeof(float2) + 64;

__global__ void __launch_bounds__(W32_THREADS, 1) k_fft_cols_w32_tma(const __grid_constant__ CUtensorMap tmap,
                                                                       ColPass p, int tiles_x, int ntiles)
{
    using Gm = W32Geom<WT_N>;
    using Wp = fftw::Warp<WT_N>;
    constexpr int NG = Gm::NG;
    constexpr int COLS = Gm::COLS;
    extern __shared__ unsigned char smem_raw[];
    if (!ctl_active(p.ctl))
        return;
    float2* stage = reinterpret_cast<float2*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    float2* S = stage + 2 * WT_TILE;
    float2* tws = S + NG * Gm::COL_PAD;
    uint64_t* bar = reinterpret_cast<uint64_t*>(tws + Gm::TW);
    __shared__ int s_abort;
    volatile int* abort = &s_abort;
    const int tid = threadIdx.x;
    if (tid == 0)
    {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int e = tid; e < Gm::TW; e += W32_THREADS)
        tws[e] = __ldg(p.tw + e);
    tc::fence_async_smem();
    __syncthreads();

    auto issue = [&](int t, int sb) {
        const int fb = t / tiles_x, tx = t - fb * tiles_x;
        tc::mbar_arrive_expect_tx(&bar[sb], WT_TILE * sizeof(float2));
#pragma unroll
        for (int q = 0; q < WT_N / 256; ++q)
            tc::tma_load_2d(stage + sb * WT_TILE + q * 256 * COLS, &tmap, tx * COLS * 2, fb * WT_N + q * 256, &bar[sb]);
    };
    if (tid == 0)
    {
        if (static_cast<int>(blockIdx.x) < ntiles)
            issue(blockIdx.x, 0);
        if (static_cast<int>(blockIdx.x + gridDim.x) < ntiles)
            issue(blockIdx.x + gridDim.x, 1);
    }
    const int c = tid % COLS, g = tid / COLS;
    const int W = p.width;
    const size_t step = static_cast<size_t>(NG) * W;
    const bool inv_in = p.mode == 1;
    const float sc = p.scale;
    int k = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++k)
    {
        const int sb = k & 1;
        // every thread waits; the CTA agrees on the outcome so that all of it leaves together
        const bool landed = tc::mbar_wait(&bar[sb], static_cast<uint32_t>((k >> 1) & 1), abort);
        if (!__syncthreads_and(landed))
        {
            if (tid == 0)
                s_abort = 1;
            break;
        }
        float2 x[32];
        {
            const float2* src = stage + sb * WT_TILE + g * COLS + c;  // row g + NG j at (g + NG j) * COLS
#pragma unroll
            for (int j = 0; j < 32; ++j)
                x[j] = src[j * NG * COLS];
        }
        __syncthreads();  // stage sb fully read: refill it with the tile two steps ahead
        if (tid == 0 && t + 2 * static_cast<int>(gridDim.x) < ntiles)
            issue(t + 2 * gridDim.x, sb);
        if (inv_in)
        {
#pragma unroll
            for (int j = 0; j < 32; ++j)
                x[j] = cconj(x[j]);
        }
        const int fb = t / tiles_x, tx = t - fb * tiles_x;
        const int col = tx * COLS + c;
        const bool in_range = col < W;
        const size_t e0 = static_cast<size_t>(g) * W + col;
        Wp::stage_a(x, tws, g);
        w32_col_exchange<WT_N>(x, S, c, g);
        fftw::dft32(x);
        float2* o = p.out + p.out_map.offset(fb) + e0;
        if (p.mode == 2)
        {
            const float2* Gp = p.postmul + e0;
#pragma unroll
            for (int k2 = 0; k2 < 32; ++k2)
            {
                const float2 gv = in_range ? __ldg(Gp + k2 * step) : make_float2(0.f, 0.f);
                x[k2] = cconj(cmul(x[k2], gv));
            }
            Wp::stage_a(x, tws, g);
            w32_col_exchange<WT_N>(x, S, c, g);
            fftw::dft32(x);
            if (in_range)
            {
#pragma unroll
                for (int k2 = 0; k2 < 32; ++k2)
                    o[k2 * step] = cscale(cconj(x[k2]), sc);
            }
            continue;
        }
        if (!in_range)
            continue;
#pragma unroll
        for (int k2 = 0; k2 < 32; ++k2)
        {
            float2 v = x[k2];
            if (inv_in)
                v = cconj(v);
            v = cscale(v, sc);
            if (p.stream_out)
                __stcs(o + k2 * step, v);
            else
                o[k2 * step] = v;
        }
    }
    __syncthreads();
    if (s_abort && tid == 0)
    {
        // a wait gave up at step k: let the (at most two) copies still in flight land before the
        // CTA's shared memory is released (bounded waits without the abort shortcut)
        const int t = blockIdx.x + k * gridDim.x;
        if (t < ntiles)
            tc::mbar_wait(&bar[k & 1], static_cast<uint32_t>((k >> 1) & 1));
        if (t + static_cast<int>(gridDim.x) < ntiles)
            tc::mbar_wait(&bar[(k + 1) & 1], static_cast<uint32_t>(((k + 1) >> 1) & 1));
        atomicExch(&g_fft_wait_error, 1);
    }
}

// Persistent row pass (N = 1024, 8-/16-bit camera input, optional premultiply): tile = 8 rows of
// one frame (one row per warp), two CTAs per SM, CTA i takes the contiguous tile range
// [i per, (i + 1) per) (row block major, frame minor). The raw rows of the tile two steps ahead
// (8 or 16 KB) are loaded by TMA during the current tile; the lens rows come from L2 with their
// loads issued before the staged pixels are used. Bounded waits as in k_fft_cols_w32_tma.
// (Staging the lens rows in shared memory as well, one CTA per SM, measured slower.)
constexpr int RT_ROWS = 8;
constexpr size_t RT_RAW_MAX = static_cast<size_t>(RT_ROWS) * WT_N * 2;  // 16-bit input
constexpr int RT_XBUF = W32Geom<WT_N>::ROW_BUF;                          // per warp (32 x 33)
constexpr size_t RT_SMEM =
    1024 + 2 * RT_RAW_MAX + (static_cast<size_t>(W32_WARPS) * RT_XBUF + fftw::Warp<WT_N>::TW_COUNT) * sizeof(float2) + 64;

template <int ESIZE>
__global__ void __launch_bounds__(W32_THREADS, 2) k_fft_rows_w32_tma(const __grid_constant__ CUtensorMap raw_map,
                                                                       RowPass p, int nframes, int ntiles, int per)
{
    using Wp = fftw::Warp<WT_N>;
    extern __shared__ unsigned char smem_raw[];
    if (!ctl_active(p.ctl))
        return;
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    unsigned char* raw_st = base;  // 2 x RT_RAW_MAX
    float2* xbuf = reinterpret_cast<float2*>(base + 2 * RT_RAW_MAX);
    float2* tws = xbuf + W32_WARPS * RT_XBUF;
    uint64_t* bar = reinterpret_cast<uint64_t*>(tws + Wp::TW_COUNT);
    __shared__ int s_abort;
    volatile int* abort = &s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0)
    {
        tc::mbar_init(&bar[0], 1);
        tc::mbar_init(&bar[1], 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int e = tid; e < Wp::TW_COUNT; e += W32_THREADS)
        tws[e] = __ldg(p.tw + e);
    tc::fence_async_smem();
    __syncthreads();

    const int t0 = blockIdx.x * per;
    const int t1 = min(t0 + per, ntiles);
    constexpr uint32_t RAW_TILE = RT_ROWS * WT_N * ESIZE;
    auto issue_raw = [&](int t, int sb) {
        const int rb = t / nframes, f = t - rb * nframes;
        tc::mbar_arrive_expect_tx(&bar[sb], RAW_TILE);
#pragma unroll
        for (int q = 0; q < WT_N / 256; ++q)
            tc::tma_load_2d(raw_st + sb * RT_RAW_MAX + q * RT_ROWS * 256 * ESIZE, &raw_map, q * 256,
                            f * p.rows + rb * RT_ROWS, &bar[sb]);
    };
    if (tid == 0 && t0 < t1)
    {
        issue_raw(t0, 0);
        if (t0 + 1 < t1)
            issue_raw(t0 + 1, 1);
    }
    const bool inv = p.inverse != 0;
    const bool swap = ESIZE == 2 && p.in_kind == IN_U16_BE;
    const float sc = p.scale;
    int k = 0;
    for (int t = t0; t < t1; ++t, ++k)
    {
        const int sb = k & 1;
        const int rb = t / nframes, f = t - rb * nframes;
        const size_t row = static_cast<size_t>(rb * RT_ROWS + warp) * WT_N + lane;
        float2 x[32];
        if (p.premul)
        {
#pragma unroll
            for (int j = 0; j < 32; ++j)
                x[j] = __ldg(p.premul + row + 32 * j);
        }
        const bool landed = tc::mbar_wait(&bar[sb], static_cast<uint32_t>((k >> 1) & 1), abort);
        if (!__syncthreads_and(landed))
        {
            if (tid == 0)
                s_abort = 1;
            break;
        }
        // sample n = lane + 32 j of row `warp`: box j / 8 at (warp * 256 + lane + 32 (j % 8))
        {
            const unsigned char* rs = raw_st + sb * RT_RAW_MAX;
#pragma unroll
            for (int j = 0; j < 32; ++j)
            {
                const int off = (j >> 3) * RT_ROWS * 256 + warp * 256 + lane + 32 * (j & 7);
                float v;
                if constexpr (ESIZE == 1)
                    v = static_cast<float>(rs[off]) * 257.0f;
                else
                {
                    uint16_t u = reinterpret_cast<const uint16_t*>(rs)[off];
                    if (swap)
                        u = static_cast<uint16_t>((u << 8) | (u >> 8));
                    v = static_cast<float>(u);
                }
                x[j] = p.premul ? make_float2(v * x[j].x, v * x[j].y) : make_float2(v, 0.f);
                if (inv)
                    x[j] = cconj(x[j]);
            }
        }
        __syncthreads();  // raw stage sb fully read: refill it with the tile two steps ahead
        if (tid == 0 && t + 2 < t1)
            issue_raw(t + 2, sb);

        Wp::stage_a(x, tws, lane);
        float2* buf = xbuf + warp * RT_XBUF;
#pragma unroll
        for (int e = 0; e < 32; ++e)
            buf[lane * W32Geom<WT_N>::ROW_PAD + e] = x[e];
        __syncwarp();
#pragma unroll
        for (int n2 = 0; n2 < 32; ++n2)
            x[n2] = buf[n2 * W32Geom<WT_N>::ROW_PAD + lane];
        __syncwarp();  // the block is rewritten by the next tile
        fftw::dft32(x);

        float2* o = p.out + p.out_map.offset(f) + row;
#pragma unroll
        for (int k2 = 0; k2 < 32; ++k2)
        {
            float2 v = x[k2];
            if (inv)
                v = cconj(v);
            v = cscale(v, sc);
            if (p.stream_out)
                __stcs(o + 32 * k2, v);
            else
                o[32 * k2] = v;
        }
    }
    __syncthreads();
    if (s_abort && tid == 0)
    {
        // copies still in flight at the failed step k land before the shared memory is released
        const int t = t0 + k;
        if (t < t1)
            tc::mbar_wait(&bar[k & 1], static_cast<uint32_t>((k >> 1) & 1));
        if (t + 1 < t1)
            tc::mbar_wait(&bar[(k + 1) & 1], static_cast<uint32_t>(((k + 1) >> 1) & 1));
        atomicExch(&g_fft_wait_error, 1);
    }
}

// ------------------------------------------------------------------ warp engine, N = 768
// Rows: one warp per row (V24: 32 lanes load and run DFT24, lanes 0..23 run the DFT32 and store).
// Columns: 8 columns per CTA, thread (c, g) = (t & 7, t >> 3); forward = V24 (warps 6-7 idle in
// stage B), the AS middle pass continues with V32 (warps 6-7 idle in its stage A).
constexpr int W768_ROWS = 8;
constexpr int W768_ROW_PAD = 25;
constexpr int W768_COLS = 8;
constexpr int W768_COL_PAD = 32 * W768_COLS + 8;
constexpr size_t W768_ROW_SMEM =
    (fftw::W768::TW_COUNT + static_cast<size_t>(W768_ROWS) * 32 * W768_ROW_PAD) * sizeof(float2);
constexpr size_t W768_COL_SMEM = (fftw::W768::TW_COUNT + static_cast<size_t>(32) * W768_COL_PAD) * sizeof(float2);

__global__ void __launch_bounds__(W32_THREADS, 2) k_fft_rows_w768(RowPass p)
{
    using W = fftw::W768;
    extern __shared__ float2 smem[];
    if (!ctl_active(p.ctl))
        return;
    const float2* tw = stage_twiddles(smem, p.tw, W::TW_COUNT, W32_THREADS);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int y = blockIdx.x * W768_ROWS + warp;
    if (y >= p.rows)
        return;
    float2* buf = smem + W::TW_COUNT + warp * 32 * W768_ROW_PAD;
    const int b = blockIdx.y;
    const void* p_in = p.raw_from_ctl ? static_cast<const void*>(static_cast<const uint8_t*>(p.in) + p.ctl->raw_offset)
                                      : p.in;
    const size_t l0 = static_cast<size_t>(y) * W::N + lane;
    float2 x[32];
    load_row_samples<24, 32>(p, p_in, static_cast<size_t>(b) * p.in_frame + l0, l0, x);
    W::stage_a24(x, tw, lane);
#pragma unroll
    for (int k1 = 0; k1 < 24; ++k1)
        buf[lane * W768_ROW_PAD + k1] = x[k1];
    __syncwarp();
    if (lane >= 24)
        return;
#pragma unroll
    for (int n2 = 0; n2 < 32; ++n2)
        x[n2] = buf[n2 * W768_ROW_PAD + lane];
    fftw::dft32(x);
    const bool inv = p.inverse != 0;
    float2* o = p.out + p.out_map.offset(b) + l0;
    const float sc = p.scale;
#pragma unroll
    for (int k2 = 0; k2 < 32; ++k2)
    {
        float2 v = x[k2];
        if (inv)
            v = cconj(v);
        v = cscale(v, sc);
        if (p.stream_out)
            __stcs(o + 24 * k2, v);
        else
            o[24 * k2] = v;
    }
}

__global__ void __launch_bounds__(W32_THREADS, 2) k_fft_cols_w768(ColPass p)
{
    using W7 = fftw::W768;
    extern __shared__ float2 smem[];
    if (!ctl_active(p.ctl))
        return;
    const float2* tw = stage_twiddles(smem, p.tw, W7::TW_COUNT, W32_THREADS);
    float2* S = smem + W7::TW_COUNT;
    const int c = threadIdx.x & (W768_COLS - 1), g = threadIdx.x / W768_COLS;
    const int W = p.width;
    const int col = blockIdx.x * W768_COLS + c;
    const bool in_range = col < W;
    const int b = blockIdx.y;
    const size_t Ws = static_cast<size_t>(W);
    const float2* in = p.in + static_cast<size_t>(b) * p.in_frame + col;
    float2* o = p.out + p.out_map.offset(b) + col;
    const bool inv_in = p.mode == 1;
    const bool active_b = g < 24;  // stage B of V24 / stage A of V32

    // V24 forward: samples g + 32 i (i < 24)
    float2 x[32];
#pragma unroll
    for (int i = 0; i < 24; ++i)
        x[i] = in_range ? in[(static_cast<size_t>(g) + 32 * i) * Ws] : make_float2(0.f, 0.f);
    if (inv_in)
    {
#pragma unroll
        for (int i = 0; i < 24; ++i)
            x[i] = cconj(x[i]);
    }
    W7::stage_a24(x, tw, g);
#pragma unroll
    for (int k1 = 0; k1 < 24; ++k1)
        S[k1 * W768_COL_PAD + g * W768_COLS + c] = x[k1];
    __syncthreads();
    if (active_b)
    {
#pragma unroll
        for (int n2 = 0; n2 < 32; ++n2)
            x[n2] = S[g * W768_COL_PAD + n2 * W768_COLS + c];
        fftw::dft32(x);  // X[g + 24 k2], k2 < 32
    }
    __syncthreads();
    const float sc = p.scale;
    if (p.mode != 2)
    {
        if (!active_b || !in_range)
            return;
#pragma unroll
        for (int k2 = 0; k2 < 32; ++k2)
        {
            float2 v = x[k2];
            if (inv_in)
                v = cconj(v);
            v = cscale(v, sc);
            float2* d = o + (static_cast<size_t>(g) + 24 * k2) * Ws;
            if (p.stream_out)
                __stcs(d, v);
            else
                *d = v;
        }
        return;
    }
    // * G, conjugate, V32 inverse (samples g + 24 i, i < 32, g < 24)
    if (active_b)
    {
        const float2* Gp = p.postmul + col;
#pragma unroll
        for (int k2 = 0; k2 < 32; ++k2)
        {
            const float2 gv = in_range ? __ldg(Gp + (static_cast<size_t>(g) + 24 * k2) * Ws) : make_float2(0.f, 0.f);
            x[k2] = cconj(cmul(x[k2], gv));
        }
        W7::stage_a32(x, tw, g);
#pragma unroll
        for (int k1 = 0; k1 < 32; ++k1)
            S[k1 * W768_COL_PAD + g * W768_COLS + c] = x[k1];
    }
    __syncthreads();
#pragma unroll
    for (int n2 = 0; n2 < 24; ++n2)
        x[n2] = S[g * W768_COL_PAD + n2 * W768_COLS + c];
    fftw::dft24(x);  // X[g + 32 k2], k2 < 24
    if (!in_range)
        return;
#pragma unroll
    for (int k2 = 0; k2 < 24; ++k2)
        o[(static_cast<size_t>(g) + 32 * k2) * Ws] = cscale(cconj(x[k2]), sc);
}

// Raw -> complex into ring slots (space transformation NONE), 8 pixels of one frame per thread
// (frames of a multiple of 8 pixels, 16-byte aligned rows of the raw batch); with `planes`, the
// real rows of the ring's split-BF16 planes of those slots as well (planes[p][slot][px]: the
// covariance operands of a ring with zero imaginary parts), so the frame is read once.
__global__ void k_convert8(const void* in, int kind, size_t frame_px, int batch, float2* ring, FrameMap map,
                           const CycleCtl* ctl, uint16_t* planes)
{
    if (!ctl_active(ctl))
        return;
    if (ctl)
        in = static_cast<const uint8_t*>(in) + ctl->raw_offset;
    const size_t groups = frame_px / 8;
    const size_t total = groups * batch;
    const size_t plane = static_cast<size_t>(map.nslots) * frame_px;
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        const int b = static_cast<int>(e / groups);
        const size_t px = (e - static_cast<size_t>(b) * groups) * 8;
        const size_t src = static_cast<size_t>(b) * frame_px + px;
        float v[8];
        if (kind == IN_U8)
        {
            const uint2 w = *reinterpret_cast<const uint2*>(static_cast<const uint8_t*>(in) + src);
#pragma unroll
            for (int i = 0; i < 4; ++i)
            {
                v[i] = static_cast<float>((w.x >> (8 * i)) & 0xffu) * 257.0f;
                v[4 + i] = static_cast<float>((w.y >> (8 * i)) & 0xffu) * 257.0f;
            }
        }
        else if (kind == IN_U16 || kind == IN_U16_BE)
        {
            const uint4 w = *reinterpret_cast<const uint4*>(static_cast<const uint16_t*>(in) + src);
            const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
            {
                uint32_t x = ww[i];
                if (kind == IN_U16_BE)
                    x = ((x & 0x00ff00ffu) << 8) | ((x >> 8) & 0x00ff00ffu);
                v[2 * i] = static_cast<float>(x & 0xffffu);
                v[2 * i + 1] = static_cast<float>(x >> 16);
            }
        }
        else
        {
            const float4* f = reinterpret_cast<const float4*>(static_cast<const float*>(in) + src);
            const float4 a = f[0], c = f[1];
            v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = c.x, v[5] = c.y, v[6] = c.z, v[7] = c.w;
        }
        const size_t off = map.offset(b);
        if (ring)
        {
            float4* o = reinterpret_cast<float4*>(ring + off + px);
#pragma unroll
            for (int i = 0; i < 4; ++i)
                __stcs(o + i, make_float4(v[2 * i], 0.f, v[2 * i + 1], 0.f));
        }
        if (planes)
        {
            uint4 hi, lo;
            tc::split2(v[0], v[1], hi.x, lo.x);
            tc::split2(v[2], v[3], hi.y, lo.y);
            tc::split2(v[4], v[5], hi.z, lo.z);
            tc::split2(v[6], v[7], hi.w, lo.w);
            const size_t slot_px = off / map.frame_stride * frame_px + px;
            *reinterpret_cast<uint4*>(planes + slot_px) = hi;
            *reinterpret_cast<uint4*>(planes + plane + slot_px) = lo;
        }
    }
}

// Ring slots slot0 .. slot0 + n - 1 (mod T) from their real split planes: x = hi + lo, exact for
// integer pixels below 2^16 (hi keeps the top 8 significant bits, lo the rest), imaginary part 0.
__global__ void k_ring_from_planes(const uint16_t* __restrict__ planes, int T, size_t frame_px, int slot0, int n,
                                   float2* __restrict__ ring)
{
    const size_t groups = frame_px / 8;
    const size_t total = groups * n;
    const size_t plane = static_cast<size_t>(T) * frame_px;
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        const int f = static_cast<int>(e / groups);
        const size_t px = (e - static_cast<size_t>(f) * groups) * 8;
        const size_t at = static_cast<size_t>((slot0 + f) % T) * frame_px + px;
        const uint4 hi = *reinterpret_cast<const uint4*>(planes + at);
        const uint4 lo = *reinterpret_cast<const uint4*>(planes + plane + at);
        const uint32_t h[4] = {hi.x, hi.y, hi.z, hi.w}, l[4] = {lo.x, lo.y, lo.z, lo.w};
        float4* o = reinterpret_cast<float4*>(ring + at);
#pragma unroll
        for (int i = 0; i < 4; ++i)
        {
            // bf16 = the top half of an FP32 word
            const float a = __uint_as_float(h[i] << 16) + __uint_as_float(l[i] << 16);
            const float b = __uint_as_float(h[i] & 0xffff0000u) + __uint_as_float(l[i] & 0xffff0000u);
            __stcs(o + i, make_float4(a, 0.f, b, 0.f));
        }
    }
}

// Raw -> complex into ring slots (space transformation NONE).
__global__ void k_convert(const void* in, int kind, size_t frame_px, int batch, float2* ring, FrameMap map,
                          const CycleCtl* ctl)
{
    if (!ctl_active(ctl))
        return;
    if (ctl)
        in = static_cast<const uint8_t*>(in) + ctl->raw_offset;
    const size_t total = frame_px * batch;
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < total;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        const int b = static_cast<int>(e / frame_px);
        const size_t px = e - static_cast<size_t>(b) * frame_px;
        ring[map.offset(b) + px] = load_pixel(in, e, kind);
    }
}

// ====================================================================================== twiddles
// All plans' per-stage twiddle tables live in one static device array, filled from the host (FP64
// cos/sin rounded to FP32) by a synchronous copy the first time a size is used on a device: no
// device allocation, so the allocation-free entry points can use the FFT too. That first use on a
// device must not happen inside a stream capture.

#define HV_FFT_SIZES(X)                                                                                                \
    X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096) X(48) X(96) X(192) X(384) X(768) X(1536)

constexpr int kTwiddleCapacity = 32768;
static __device__ float2 g_fft_twiddles[kTwiddleCapacity];

namespace {

constexpr int kMaxTwDevices = 64;
std::mutex g_tw_mu;
const float2* g_tw_base[kMaxTwDevices] = {};
int g_tw_offset[8192];  // offset of size N's tables in g_fft_twiddles
int g_tw_w32_offset[2] = {};  // offsets of the warp engine's tables (N = 512, 1024)
int g_tw_w768_offset = 0;    // offset of the warp engine's N = 768 tables
bool g_tw_layout_ready = false;
std::vector<float2> g_tw_host;

void tw_layout()
{
    if (g_tw_layout_ready)
        return;
    int off = 0;
#define HV_TW(N)                                                                                                       \
    {                                                                                                                  \
        g_tw_offset[N] = off;                                                                                          \
        const int cnt = fft::twiddle_count(typename fft::Plan<N>::List{});                                             \
        g_tw_host.resize(off + cnt + 1);                                                                               \
        fft::twiddle_fill(typename fft::Plan<N>::List{}, g_tw_host.data() + off);                                      \
        off += cnt;                                                                                                    \
    }
    HV_FFT_SIZES(HV_TW)
#undef HV_TW
    g_tw_w32_offset[1] = off;
    g_tw_host.resize(off + fftw::Warp<1024>::TW_COUNT + 1);
    fftw::Warp<1024>::twiddle_fill(g_tw_host.data() + off);
    off += fftw::Warp<1024>::TW_COUNT;
    g_tw_w32_offset[0] = off;
    g_tw_host.resize(off + fftw::Warp<512>::TW_COUNT + 1);
    fftw::Warp<512>::twiddle_fill(g_tw_host.data() + off);
    off += fftw::Warp<512>::TW_COUNT;
    g_tw_w768_offset = off;
    g_tw_host.resize(off + fftw::W768::TW_COUNT + 1);
    fftw::W768::twiddle_fill(g_tw_host.data() + off);
    off += fftw::W768::TW_COUNT;
    g_tw_layout_ready = true;
}

// Base of the twiddle array on the current device (uploaded on first use), or null.
const float2* twiddle_base()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxTwDevices)
        return nullptr;
    std::lock_guard<std::mutex> g(g_tw_mu);
    if (!g_tw_base[dev])
    {
        tw_layout();
        if (g_tw_host.size() > static_cast<size_t>(kTwiddleCapacity))
            return nullptr;
        if (cudaMemcpyToSymbol(g_fft_twiddles, g_tw_host.data(), g_tw_host.size() * sizeof(float2)) != cudaSuccess)
            return nullptr;
        void* base = nullptr;
        if (cudaGetSymbolAddress(&base, g_fft_twiddles) != cudaSuccess)
            return nullptr;
        g_tw_base[dev] = static_cast<const float2*>(base);
    }
    return g_tw_base[dev];
}

template <int N>
const float2* twiddles()
{
    const float2* base = twiddle_base();
    return base ? base + g_tw_offset[N] : nullptr;
}

const float2* twiddles_w768()
{
    const float2* base = twiddle_base();
    return base ? base + g_tw_w768_offset : nullptr;
}

template <int N>
const float2* twiddles_w32()
{
    const float2* base = twiddle_base();
    return base ? base + g_tw_w32_offset[N == 1024 ? 1 : 0] : nullptr;
}

}  // namespace

// ====================================================================================== dispatch

namespace {

// Rows per CTA for the row pass (about 256 threads) and columns per CTA for the column pass.
template <int N>
constexpr int row_lanes()
{
    constexpr int per_row = N / fft::Plan<N>::E;
    return per_row >= 256 ? 1 : 256 / per_row;
}
template <int N>
constexpr int col_lanes()
{
    constexpr int E = fft::Plan<N>::E;
    // at most 512 threads and 128 KB of tile per CTA
    int f = 16;
    while (f > 1 && (f * N / E > 512 || f * N * 8 > 128 * 1024))
        f /= 2;
    return f;
}

std::atomic<int> g_fft_engine{0};  // 0 automatic (warp engine for 512-, 768- and 1024-point transforms), 1 tile engine only

std::atomic<int> g_fft_tma{1};  // 1: TMA-fed persistent row / column passes where they apply

int device_sms()
{
    static const int sms = [] {
        int dev = 0, n = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return 0;
        return n;
    }();
    return sms;
}

// Persistent TMA-fed row pass for N = 1024 (8-/16-bit input outside served cycles); false when it
// does not apply (the caller then launches the register-loading kernel).
bool launch_rows_w32_tma(const RowPass& p, int nframes, cudaStream_t st, hv_status* status)
{
    const int esize = p.in_kind == IN_U8 ? 1 : (p.in_kind == IN_U16 || p.in_kind == IN_U16_BE) ? 2 : 0;
    if (!g_fft_tma.load() || esize == 0 || p.raw_from_ctl || (p.rows % RT_ROWS) != 0 ||
        p.in_frame != static_cast<size_t>(p.rows) * WT_N)
        return false;
    const int sms = device_sms();
    if (sms <= 0)
        return false;
    CUtensorMap raw_map;
    if (!tc::encode_tmap_2d(&raw_map, esize == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16,
                            p.in, WT_N, static_cast<uint64_t>(nframes) * p.rows, static_cast<uint64_t>(WT_N) * esize,
                            256, RT_ROWS))
        return false;
    *status = HV_OK;
    const int ntiles = (p.rows / RT_ROWS) * nframes;
    const int use = sms - p.reserve_sms > 0 ? sms - p.reserve_sms : 1;
    const int per = (ntiles + 2 * use - 1) / (2 * use);  // two CTAs per SM
    const int grid = (ntiles + per - 1) / per;
    RowPass q = p;
    if ((q.tw = twiddles_w32<WT_N>()) == nullptr)
    {
        *status = HV_ERR_CUDA;
        return true;
    }
    q.tw_count = fftw::Warp<WT_N>::TW_COUNT;
    cudaError_t e;
    if (esize == 1)
    {
        e = cudaFuncSetAttribute(k_fft_rows_w32_tma<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(RT_SMEM));
        if (e == cudaSuccess)
            k_fft_rows_w32_tma<1><<<grid, W32_THREADS, RT_SMEM, st>>>(raw_map, q, nframes, ntiles, per);
    }
    else
    {
        e = cudaFuncSetAttribute(k_fft_rows_w32_tma<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(RT_SMEM));
        if (e == cudaSuccess)
            k_fft_rows_w32_tma<2><<<grid, W32_THREADS, RT_SMEM, st>>>(raw_map, q, nframes, ntiles, per);
    }
    if (e == cudaSuccess)
        e = cudaGetLastError();
    if (e != cudaSuccess)
    {
        set_last_error_msg(cudaGetErrorString(e));
        *status = HV_ERR_CUDA;
        return true;
    }
    count_launch();
    return true;
}

template <int N>
hv_status launch_rows_w32(const RowPass& p, int nframes, cudaStream_t st)
{
    if constexpr (N == WT_N)
    {
        hv_status r;
        if (launch_rows_w32_tma(p, nframes, st, &r))
            return r;
    }
    using Gm = W32Geom<N>;
    HV_CUDA_TRY(cudaFuncSetAttribute(k_fft_rows_w32<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(Gm::ROW_SMEM)));
    RowPass q = p;
    if ((q.tw = twiddles_w32<N>()) == nullptr)
        return HV_ERR_CUDA;
    q.tw_count = Gm::TW;
    dim3 grid((p.rows + Gm::ROWS - 1) / Gm::ROWS, nframes);
    k_fft_rows_w32<N><<<grid, W32_THREADS, Gm::ROW_SMEM, st>>>(q);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

// Persistent TMA-fed column pass for N = 1024; false when it does not apply (the caller then
// launches the register-loading kernel).
bool launch_cols_w32_tma(const ColPass& p, int nframes, cudaStream_t st, hv_status* status)
{
    // forward / inverse passes only: the AS middle pass (two transforms per tile) is compute-bound
    // at one CTA of 8 warps per SM and stays on the register-loading kernel (2 CTAs per SM)
    if (!g_fft_tma.load() || p.mode == 2 || p.in_frame != static_cast<size_t>(p.width) * WT_N ||
        (p.width % WT_COLS) != 0)
        return false;
    CUtensorMap map;
    if (!tc::encode_tmap_2d_f32(&map, p.in, static_cast<uint64_t>(p.width) * 2, static_cast<uint64_t>(nframes) * WT_N,
                                static_cast<uint64_t>(p.width) * sizeof(float2), WT_COLS * 2, 256))
        return false;
    const int sms = device_sms();
    if (sms <= 0)
        return false;
    *status = HV_OK;
    const cudaError_t e = cudaFuncSetAttribute(k_fft_cols_w32_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(WT_SMEM));
    if (e != cudaSuccess)
    {
        *status = HV_ERR_CUDA;
        return true;
    }
    ColPass q = p;
    if ((q.tw = twiddles_w32<WT_N>()) == nullptr)
    {
        *status = HV_ERR_CUDA;
        return true;
    }
    q.tw_count = fftw::Warp<WT_N>::TW_COUNT;
    const int tiles_x = p.width / WT_COLS;
    const int ntiles = tiles_x * nframes;
    const int use = sms - p.reserve_sms > 0 ? sms - p.reserve_sms : 1;
    const int grid = ntiles < use ? ntiles : use;
    k_fft_cols_w32_tma<<<grid, W32_THREADS, WT_SMEM, st>>>(map, q, tiles_x, ntiles);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess)
    {
        set_last_error_msg(cudaGetErrorString(le));
        *status = HV_ERR_CUDA;
        return true;
    }
    count_launch();
    return true;
}

template <int N>
hv_status launch_cols_w32(const ColPass& p, int nframes, cudaStream_t st)
{
    if constexpr (N == WT_N)
    {
        hv_status r;
        if (launch_cols_w32_tma(p, nframes, st, &r))
            return r;
    }
    using Gm = W32Geom<N>;
    HV_CUDA_TRY(cudaFuncSetAttribute(k_fft_cols_w32<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(Gm::COL_SMEM)));
    ColPass q = p;
    if ((q.tw = twiddles_w32<N>()) == nullptr)
        return HV_ERR_CUDA;
    q.tw_count = Gm::TW;
    dim3 grid((p.width + Gm::COLS - 1) / Gm::COLS, nframes);
    k_fft_cols_w32<N><<<grid, W32_THREADS, Gm::COL_SMEM, st>>>(q);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status launch_rows_w768(const RowPass& p, int nframes, cudaStream_t st)
{
    HV_CUDA_TRY(cudaFuncSetAttribute(k_fft_rows_w768, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(W768_ROW_SMEM)));
    RowPass q = p;
    if ((q.tw = twiddles_w768()) == nullptr)
        return HV_ERR_CUDA;
    q.tw_count = fftw::W768::TW_COUNT;
    dim3 grid((p.rows + W768_ROWS - 1) / W768_ROWS, nframes);
    k_fft_rows_w768<<<grid, W32_THREADS, W768_ROW_SMEM, st>>>(q);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status launch_cols_w768(const ColPass& p, int nframes, cudaStream_t st)
{
    HV_CUDA_TRY(cudaFuncSetAttribute(k_fft_cols_w768, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(W768_COL_SMEM)));
    ColPass q = p;
    if ((q.tw = twiddles_w768()) == nullptr)
        return HV_ERR_CUDA;
    q.tw_count = fftw::W768::TW_COUNT;
    dim3 grid((p.width + W768_COLS - 1) / W768_COLS, nframes);
    k_fft_cols_w768<<<grid, W32_THREADS, W768_COL_SMEM, st>>>(q);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

template <int N>
hv_status launch_rows(const RowPass& p, int nframes, cudaStream_t st)
{
    if constexpr (N == 768)
        if (g_fft_engine.load() == 0)
            return launch_rows_w768(p, nframes, st);
    if constexpr (N == 512 || N == 1024)
        if (g_fft_engine.load() == 0)
            return launch_rows_w32<N>(p, nframes, st);
    constexpr int F = row_lanes<N>();
    using Tl = fft::Tile<N, F, false>;
    const int tw_count = fft::twiddle_count(typename fft::Plan<N>::List{});
    const size_t smem = (static_cast<size_t>(F) * N + tw_count) * sizeof(float2);
    if (smem > 48 * 1024)
        HV_CUDA_TRY(cudaFuncSetAttribute(k_fft_rows<N, F>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem)));
    RowPass q = p;
    if ((q.tw = twiddles<N>()) == nullptr)
        return HV_ERR_CUDA;
    q.tw_count = tw_count;
    dim3 grid((p.rows + F - 1) / F, nframes);
    k_fft_rows<N, F><<<grid, Tl::NT, smem, st>>>(q);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

template <int N>
hv_status launch_cols(const ColPass& p, int nframes, cudaStream_t st)
{
    if constexpr (N == 768)
        if (g_fft_engine.load() == 0)
            return launch_cols_w768(p, nframes, st);
    if constexpr (N == 512 || N == 1024)
        if (g_fft_engine.load() == 0)
            return launch_cols_w32<N>(p, nframes, st);
    constexpr int F = col_lanes<N>();
    using Tl = fft::Tile<N, F, true>;
    const int tw_count = fft::twiddle_count(typename fft::Plan<N>::List{});
    const size_t smem = (static_cast<size_t>(F) * N + tw_count) * sizeof(float2);
    if (smem > 48 * 1024)
        HV_CUDA_TRY(cudaFuncSetAttribute(k_fft_cols<N, F>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem)));
    ColPass q = p;
    if ((q.tw = twiddles<N>()) == nullptr)
        return HV_ERR_CUDA;
    q.tw_count = tw_count;
    dim3 grid((p.width + F - 1) / F, nframes);
    k_fft_cols<N, F><<<grid, Tl::NT, smem, st>>>(q);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

}  // namespace

void set_fft_engine(int mode)
{
    g_fft_engine = mode == 2 ? 0 : mode;
    g_fft_tma = mode == 2 ? 0 : 1;
}

hv_status fft_status()
{
    int err = 0;
    HV_CUDA_TRY(cudaMemcpyFromSymbol(&err, g_fft_wait_error, sizeof(int)));
    return err ? HV_ERR_TIMEOUT : HV_OK;
}

bool fft_size_supported(int n)
{
    switch (n)
    {
#define HV_CASE(N)                                                                                                     \
    case N: return true;
        HV_FFT_SIZES(HV_CASE)
#undef HV_CASE
    default: return false;
    }
}

hv_status fft_rows(const RowPass& p, int N, int nframes, cudaStream_t st)
{
    switch (N)
    {
#define HV_CASE(NN)                                                                                                    \
    case NN: return launch_rows<NN>(p, nframes, st);
        HV_FFT_SIZES(HV_CASE)
#undef HV_CASE
    default: set_last_error_msg("unsupported FFT length"); return HV_ERR_UNSUPPORTED;
    }
}

hv_status fft_cols(const ColPass& p, int N, int nframes, cudaStream_t st)
{
    switch (N)
    {
#define HV_CASE(NN)                                                                                                    \
    case NN: return launch_cols<NN>(p, nframes, st);
        HV_FFT_SIZES(HV_CASE)
#undef HV_CASE
    default: set_last_error_msg("unsupported FFT length"); return HV_ERR_UNSUPPORTED;
    }
}

hv_status make_fresnel_lens(float2* lens, int W, int H, float lam, float z, float ps, int mode, cudaStream_t st)
{
    dim3 block(128), grid((W + 127) / 128, H);
    k_fresnel_lens<<<grid, block, 0, st>>>(lens, W, H, lam, z, ps, mode);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status make_spectral_lens(float2* lens, int W, int H, float lam, float z, float ps, int mode, cudaStream_t st)
{
    dim3 block(128), grid((W + 127) / 128, H);
    k_spectral_lens<<<grid, block, 0, st>>>(lens, W, H, lam, z, ps, mode);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

// ====================================================================================== filter2D

// Band-pass mask of kernel_update_filter2d_circles_mask (filter2D.cu:52-88) in the reference's
// float arithmetic: r = hypotf(x - W/2, y - H/2), A = 1 inside radius n2 with a cosine roll-off of
// width sh, B the same for n1 / sl, mask = A (1 - B); written quadrant-swapped (FFT layout, the
// shift_corners of update_filter2d_circles_mask) as complex (multiply = 0) or multiplied into an
// FFT-layout complex array in place (multiply = 1: the AS transfer function, fourier_transform.cc:134-137).
__global__ void k_filter2d_mask(float2* dst, int W, int H, int n1, int n2, int sl, int sh, int multiply)
{
    const int X = blockIdx.x * blockDim.x + threadIdx.x, Y = blockIdx.y;
    if (X >= W || Y >= H)
        return;
    const int x = (X + W / 2) % W, y = (Y + H / 2) % H;  // source of the quadrant swap (even W, H)
    const float rx = static_cast<float>(x) - static_cast<float>(W / 2);
    const float ry = static_cast<float>(y) - static_cast<float>(H / 2);
    const float len = hypotf(rx, ry);
    float a = 0.0f, b = 0.0f;
    if (len < static_cast<float>(n2))
        a = 1.0f;
    else if (len < static_cast<float>(n2 + sh))
        a = cosf(static_cast<float>(static_cast<double>(__fdiv_rn(len - static_cast<float>(n2), static_cast<float>(sh))) *
                                    1.57079632679489661923));
    if (len < static_cast<float>(n1))
        b = 1.0f;
    else if (len < static_cast<float>(n1 + sl))
        b = cosf(static_cast<float>(static_cast<double>(__fdiv_rn(len - static_cast<float>(n1), static_cast<float>(sl))) *
                                    1.57079632679489661923));
    const float m = a * (1.0f - b);
    float2* o = dst + static_cast<size_t>(Y) * W + X;
    if (multiply)
    {
        const float2 v = *o;
        *o = make_float2(v.x * m, v.y * m);
    }
    else
        *o = make_float2(m, 0.0f);
}

hv_status filter2d_mask(float2* dst, int W, int H, int n1, int n2, int smooth_low, int smooth_high, int multiply,
                        cudaStream_t st)
{
    if (!dst || W <= 0 || H <= 0 || (W & 1) || (H & 1) || n1 < 0 || n2 <= n1 || smooth_low < 0 || smooth_high < 0)
        return HV_INVALID_VALUE;
    dim3 block(128), grid((W + 127) / 128, H);
    k_filter2d_mask<<<grid, block, 0, st>>>(dst, W, H, n1, n2, smooth_low, smooth_high, multiply);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

int raw_kind(int raw_bytes, int big_endian)
{
    switch (raw_bytes)
    {
    case 1: return IN_U8;
    case 2: return big_endian ? IN_U16_BE : IN_U16;
    case 4: return IN_F32;
    case 8: return IN_C64;
    default: return -1;
    }
}

static std::atomic<int> g_spatial_sub_mb{0};
void set_spatial_sub_batch_mb(int mb) { g_spatial_sub_mb = mb < 0 ? 0 : mb; }

hv_status spatial_transform(const void* raw, int kind, int W, int H, int batch, int space, const float2* lens,
                            float2* work, float2* ring, int slot0, int nslots, cudaStream_t st, const CycleCtl* ctl,
                            const float2* f2d_mask, float2* work2, uint16_t* real_planes, int reserve_sms)
{
    // With a cycle control block, `raw` is the input ring base (the batch sits at ctl->raw_offset)
    // and the ring slot of frame 0 is slot0 + ctl->ring_begin; every pass is gated by ctl->active.
    const int* begin_dev = ctl ? &ctl->ring_begin : nullptr;
    const size_t HW = static_cast<size_t>(W) * H;
    const FrameMap ring_map{HW, slot0, nslots, begin_dev};
    const FrameMap work_map{HW, 0, batch > 0 ? batch : 1};
    if (batch <= 0)
        return HV_OK;
    // filter2D before Fresnel or without propagation (fourier_transform.cc:55-58, filter2D.cu:28-46);
    // for AS the mask is part of the transfer function and nothing changes here
    const bool f2d = f2d_mask && space != HV_SPACE_ANGULARSP;
    if (f2d && (!work || (space == HV_SPACE_FRESNELTR && !work2)))
        return HV_INVALID_VALUE;
    if (space == HV_SPACE_NONE && !f2d)
    {
        const int block = 256;
        // 8-pixel groups: 8-byte (8-bit), 16-byte (16-bit) and 32-byte (float) aligned loads when the
        // batch starts on 16 bytes and frames hold a multiple of 8 pixels
        if (HW % 8 == 0 && kind != IN_C64 && (reinterpret_cast<uintptr_t>(raw) & 15) == 0 &&
            (reinterpret_cast<uintptr_t>(ring) & 15) == 0)
        {
            const size_t total = HW / 8 * batch;
            const int grid = static_cast<int>((total + block - 1) / block < 152 * 8 ? (total + block - 1) / block : 152 * 8);
            k_convert8<<<grid, block, 0, st>>>(raw, kind, HW, batch, ring, ring_map, ctl, real_planes);
            HV_LAUNCH_CHECK();
            count_launch();
            return HV_OK;
        }
        if (real_planes)
        {
            set_last_error_msg("converting into the split planes needs frames of a multiple of 8 pixels");
            return HV_ERR_UNSUPPORTED;
        }
        const size_t total = HW * batch;
        const int grid = static_cast<int>((total + block - 1) / block < 152 * 16 ? (total + block - 1) / block : 152 * 16);
        k_convert<<<grid, block, 0, st>>>(raw, kind, HW, batch, ring, ring_map, ctl);
        HV_LAUNCH_CHECK();
        count_launch();
        return HV_OK;
    }
    if (!fft_size_supported(W) || !fft_size_supported(H))
    {
        set_last_error_msg("frame width/height not supported by the shared-memory FFT");
        return HV_ERR_UNSUPPORTED;
    }
    // One launch per pass over the whole batch when g_spatial_sub_mb is 0; otherwise sub-batches
    // whose complex intermediate (sb frames) fits in that many MB of L2 between the passes. Raw
    // input is read and ring slots are written with streaming hints.
    const size_t frame_c64 = HW * sizeof(float2);
    const int sub_mb = g_spatial_sub_mb.load();
    int sb = sub_mb > 0 ? static_cast<int>((static_cast<size_t>(sub_mb) << 20) / frame_c64) : batch;
    if (sb < 1)
        sb = 1;
    if (sb > batch)
        sb = batch;
    const size_t raw_frame_bytes = HW * static_cast<size_t>(in_kind_bytes(kind));
    for (int b0 = 0; b0 < batch; b0 += sb)
    {
        const int nb = (batch - b0) < sb ? (batch - b0) : sb;
        const void* raw_b = static_cast<const uint8_t*>(raw) + static_cast<size_t>(b0) * raw_frame_bytes;
        const FrameMap ring_b{HW, (slot0 + b0) % nslots, nslots, begin_dev};
        const FrameMap work_b{HW, 0, nb};
        hv_status s;
        if (f2d)
        {
            // forward rows -> work; columns: forward, *M, inverse (in place); then the unnormalised
            // inverse rows: -> ring slots (no propagation) or -> work2, *L and forward rows -> work,
            // forward columns -> ring slots (Fresnel)
            RowPass r{raw_b, kind, HW, work, work_b, nullptr, H, 0, 1.0f};
            r.ctl = ctl;
            r.raw_from_ctl = ctl ? 1 : 0;
            if ((s = fft_rows(r, W, nb, st)) != HV_OK)
                return s;
            ColPass c{work, HW, work, work_b, f2d_mask, W, 2, 1.0f};
            c.ctl = ctl;
            if ((s = fft_cols(c, H, nb, st)) != HV_OK)
                return s;
            if (space == HV_SPACE_NONE)
            {
                RowPass r2{work, IN_C64, HW, ring, ring_b, nullptr, H, 1, 1.0f};
                r2.stream_out = 1;
                r2.ctl = ctl;
                if ((s = fft_rows(r2, W, nb, st)) != HV_OK)
                    return s;
                continue;
            }
            RowPass r2{work, IN_C64, HW, work2, work_b, nullptr, H, 1, 1.0f};
            r2.ctl = ctl;
            if ((s = fft_rows(r2, W, nb, st)) != HV_OK)
                return s;
            RowPass r3{work2, IN_C64, HW, work, work_b, lens, H, 0, 1.0f};
            r3.ctl = ctl;
            if ((s = fft_rows(r3, W, nb, st)) != HV_OK)
                return s;
            ColPass c2{work, HW, ring, ring_b, nullptr, W, 0, 1.0f};
            c2.stream_out = 1;
            c2.ctl = ctl;
            if ((s = fft_cols(c2, H, nb, st)) != HV_OK)
                return s;
            continue;
        }
        if (space == HV_SPACE_FRESNELTR)
        {
            // x*L, forward rows -> work; forward columns -> ring slots
            RowPass r{raw_b, kind, HW, work, work_b, lens, H, 0, 1.0f};
            r.ctl = ctl;
            r.raw_from_ctl = ctl ? 1 : 0;
            r.reserve_sms = reserve_sms;
            if ((s = fft_rows(r, W, nb, st)) != HV_OK)
                return s;
            ColPass c{work, HW, ring, ring_b, nullptr, W, 0, 1.0f};
            c.stream_out = 1;
            c.ctl = ctl;
            c.reserve_sms = reserve_sms;
            if ((s = fft_cols(c, H, nb, st)) != HV_OK)
                return s;
        }
        else if (space == HV_SPACE_ANGULARSP)
        {
            // forward rows -> work; columns: forward, *G, inverse (in place); inverse rows /(H*W) -> ring
            RowPass r{raw_b, kind, HW, work, work_b, nullptr, H, 0, 1.0f};
            r.ctl = ctl;
            r.raw_from_ctl = ctl ? 1 : 0;
            r.reserve_sms = reserve_sms;
            if ((s = fft_rows(r, W, nb, st)) != HV_OK)
                return s;
            ColPass c{work, HW, work, work_b, lens, W, 2, 1.0f};
            c.ctl = ctl;
            if ((s = fft_cols(c, H, nb, st)) != HV_OK)
                return s;
            RowPass r2{work, IN_C64, HW, ring, ring_b, nullptr, H, 1, 1.0f / static_cast<float>(HW)};
            r2.stream_out = 1;
            r2.ctl = ctl;
            if ((s = fft_rows(r2, W, nb, st)) != HV_OK)
                return s;
        }
        else
        {
            set_last_error_msg("unknown space transformation");
            return HV_INVALID_VALUE;
        }
    }
    return HV_OK;
    set_last_error_msg("unknown space transformation");
    return HV_INVALID_VALUE;
}

hv_status convert_to_planes(const void* raw, int kind, size_t HW, int batch, int slot0, int T, uint16_t* planes,
                            cudaStream_t st)
{
    if (HW % 8 != 0 || kind == IN_C64 || (reinterpret_cast<uintptr_t>(raw) & 15) != 0 || batch <= 0)
        return HV_ERR_UNSUPPORTED;
    const FrameMap map{HW, slot0, T};
    const size_t total = HW / 8 * batch;
    const int block = 256;
    // three quarters of the SMs' thread slots: the pipelined windows' eigensolve kernels (another
    // stream) find room beside this pass
    const int cap = device_sms() * 6;
    const int grid = static_cast<int>((total + block - 1) / block < static_cast<size_t>(cap) ? (total + block - 1) / block : cap);
    k_convert8<<<grid, block, 0, st>>>(raw, kind, HW, batch, nullptr, map, nullptr, planes);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status ring_from_planes(const uint16_t* planes, int T, size_t HW, int slot0, int n, float2* ring, cudaStream_t st)
{
    if (HW % 8 != 0 || n <= 0)
        return n <= 0 ? HV_OK : HV_ERR_UNSUPPORTED;
    const size_t total = HW / 8 * n;
    const int block = 256;
    const int cap = device_sms() * 6;  // as convert_to_planes: room for the eigensolve stream's kernels
    const int grid = static_cast<int>((total + block - 1) / block < static_cast<size_t>(cap) ? (total + block - 1) / block : cap);
    k_ring_from_planes<<<grid, block, 0, st>>>(planes, T, HW, slot0, n, ring);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status fft_rows_pass(const void* in, int kind, float2* out, int W, int H, int batch, const float2* premul,
                        int inverse, float scale, int slot0, int nslots, cudaStream_t st)
{
    const size_t HW = static_cast<size_t>(W) * H;
    RowPass r{in, kind, HW, out, FrameMap{HW, slot0, nslots}, premul, H, inverse, scale};
    return fft_rows(r, W, batch, st);
}

hv_status fft_cols_pass(const float2* in, float2* out, int W, int H, int batch, const float2* postmul, int mode,
                        float scale, int slot0, int nslots, cudaStream_t st)
{
    const size_t HW = static_cast<size_t>(W) * H;
    ColPass c{in, HW, out, FrameMap{HW, slot0, nslots}, postmul, W, mode, scale};
    return fft_cols(c, H, batch, st);
}

hv_status fft2d(const float2* in, float2* out, int n0, int n1, int batch, int inverse, float scale, cudaStream_t st)
{
    if (!fft_size_supported(n0) || !fft_size_supported(n1))
    {
        set_last_error_msg("FFT length not supported");
        return HV_ERR_UNSUPPORTED;
    }
    const size_t HW = static_cast<size_t>(n0) * n1;
    const FrameMap map{HW, 0, batch};
    RowPass r{in, IN_C64, HW, out, map, nullptr, n0, inverse, 1.0f};
    hv_status s = fft_rows(r, n1, batch, st);
    if (s != HV_OK)
        return s;
    ColPass c{out, HW, out, map, nullptr, n1, inverse ? 1 : 0, scale};
    return fft_cols(c, n0, batch, st);
}

}  // namespace hv
