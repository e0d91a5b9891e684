// Time transforms over the ring of T complex frames, fused with the view.
//
// Reference behaviour (Holovibes):
//   STFT           Backend/cuda_sources/stft.cu:9-15 with the plan of Backend/sources/core/icompute.cc:109-115:
//                  a forward T-point DFT along time over the ring STORAGE order, all T bins.
//   PCA            Backend/sources/compute/matrix_operations.cc:9-103, fourier_transform.cc:340-377:
//                  cov = H^H H (Cgemm3m), cusolverDnCheevd (ascending), p_acc = H V (Cgemm3m).
//   p range        Backend/sources/compute/converts.cc:76-92
//   views          Backend/cuda_sources/tools_conversion.cu:11-103,199-232 (mean over [pmin, pmax]
//                  of hypotf, hypotf^2 or atan2)
//   PCA x131071    Backend/sources/compute/converts.cc:50-62
//   SSA_STFT       Backend/sources/compute/fourier_transform.cc:379-444: eigenvectors q..q+q_acc of
//                  H^H H kept, tmp = V V^H, p_acc = FFT_t(H tmp)
//   phase increase Backend/cuda_sources/tools_unwrap.cu:210-267, converts.cc:251-300,
//                  rescale_float tools_conversion.cu:245-313
//
// GB300 design: only the K = pmax - pmin + 1 bins the view reads are computed, as a dense
// contraction X[k][pix] = sum_t W[k][t] ring[t][pix] with W = DFT twiddles (STFT) or the selected
// eigenvector columns (PCA); the view, the bin average, the PCA scale, the fftshift permutation
// and the renormalisation partial sums are fused into the same kernel, so the T x HW p_acc
// buffer of the reference never exists.
#include <math.h>

#include <atomic>
#include <vector>

#include "hv_common.cuh"
#include "hv_internal.h"

namespace hv {

constexpr int TV_THREADS = 128;  // one renormalisation partial per 128 pixels (same as the tensor-core view)
constexpr int TV_KMAX = 16;  // bins per register chunk at most

__device__ __forceinline__ float view_value(float2 X, int img_type)
{
    if (img_type == HV_IMG_MODULUS)
        return hypotf(X.x, X.y);
    if (img_type == HV_IMG_SQUARED_MODULUS)
    {
        const float t = hypotf(X.x, X.y);
        return t * t;
    }
    return atan2f(X.y, X.x);
}

// ring: [T][HW] complex; weights: [K][T] complex. One pixel per thread; the K bins are done in
// chunks of KC (registers), the chunk's weights staged in shared memory as [T][KC].
template <int KC>
__global__ void __launch_bounds__(TV_THREADS) k_time_view(const float2* __restrict__ ring, int T, int W, int H,
                                                           const float2* __restrict__ weights, int K, int img_type,
                                                           float scale, int shift, float* __restrict__ out,
                                                           double* __restrict__ partials, const CycleCtl* ctl,
                                                           const float* __restrict__ bin_w)
{
    // bin_w (moments): out = sum_k |X_k|^2 bin_w[k] instead of the mean of the view over the bins
    if (!ctl_render(ctl))
        return;
    extern __shared__ __align__(16) float2 wsm[];  // [T][KC]
    __shared__ double red[TV_THREADS / 32];
    const size_t HW = static_cast<size_t>(W) * H;
    const size_t pix = blockIdx.x * static_cast<size_t>(TV_THREADS) + threadIdx.x;
    const bool valid = pix < HW;
    float acc_view = 0.f;
    for (int k0 = 0; k0 < K; k0 += KC)
    {
        __syncthreads();
        for (int e = threadIdx.x; e < T * KC; e += TV_THREADS)
        {
            const int t = e / KC, kk = e - t * KC;
            const int k = k0 + kk;
            wsm[e] = (k < K) ? weights[static_cast<size_t>(k) * T + t] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        float2 acc[KC];
#pragma unroll
        for (int kk = 0; kk < KC; ++kk)
            acc[kk] = make_float2(0.f, 0.f);
        if (valid)
        {
            const float2* src = ring + pix;
#pragma unroll 8
            for (int t = 0; t < T; ++t)
            {
                const float2 x = __ldg(src + static_cast<size_t>(t) * HW);
                const float2* wt = wsm + t * KC;
#pragma unroll
                for (int kk = 0; kk < KC; ++kk)
                {
                    const float2 w = wt[kk];
                    acc[kk].x = fmaf(x.x, w.x, fmaf(-x.y, w.y, acc[kk].x));
                    acc[kk].y = fmaf(x.x, w.y, fmaf(x.y, w.x, acc[kk].y));
                }
            }
            const int kn = (K - k0) < KC ? (K - k0) : KC;
            if (bin_w)
            {
#pragma unroll
                for (int kk = 0; kk < KC; ++kk)
                    if (kk < kn)
                        acc_view += (acc[kk].x * acc[kk].x + acc[kk].y * acc[kk].y) * __ldg(bin_w + k0 + kk);
            }
            else
            {
#pragma unroll
                for (int kk = 0; kk < KC; ++kk)
                    if (kk < kn)
                        acc_view += view_value(acc[kk], img_type);
            }
        }
    }
    float v = 0.f;
    if (valid)
    {
        v = bin_w ? acc_view : acc_view / static_cast<float>(K);
        if (scale != 1.0f)
            v = v * scale;
        const int x = static_cast<int>(pix % W);
        const int y = static_cast<int>(pix / W);
        size_t dst = pix;
        if (shift)
            dst = static_cast<size_t>((y + H / 2) % H) * W + (x + W / 2) % W;
        out[dst] = v;
    }
    if (partials)
    {
        double d = valid ? static_cast<double>(v) : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            d += __shfl_down_sync(0xffffffffu, d, o);
        if ((threadIdx.x & 31) == 0)
            red[threadIdx.x >> 5] = d;
        __syncthreads();
        if (threadIdx.x == 0)
        {
            double s = 0.0;
            for (int i = 0; i < TV_THREADS / 32; ++i)
                s += red[i];
            partials[blockIdx.x] = s;
        }
    }
}

// Two adjacent pixels per thread (16-byte ring loads: 512 contiguous bytes per warp and frame;
// HW even). 128 threads cover 256 pixels and write the two 128-pixel renormalisation partials of
// their CTA, the same partials as k_time_view.
template <int KC>
__global__ void __launch_bounds__(TV_THREADS) k_time_view2(const float2* __restrict__ ring, int T, int W, int H,
                                                            const float2* __restrict__ weights, int K, int img_type,
                                                            float scale, int shift, float* __restrict__ out,
                                                            double* __restrict__ partials, int npartials,
                                                            const CycleCtl* ctl, const float* __restrict__ bin_w)
{
    if (!ctl_render(ctl))
        return;
    extern __shared__ __align__(16) float2 wsm[];  // [T][KC]
    __shared__ double red[TV_THREADS / 32];
    const size_t HW = static_cast<size_t>(W) * H;
    const size_t pix0 = 2 * (blockIdx.x * static_cast<size_t>(TV_THREADS) + threadIdx.x);
    const bool valid = pix0 < HW;
    float view0 = 0.f, view1 = 0.f;
    for (int k0 = 0; k0 < K; k0 += KC)
    {
        __syncthreads();
        for (int e = threadIdx.x; e < T * KC; e += TV_THREADS)
        {
            const int t = e / KC, kk = e - t * KC;
            const int k = k0 + kk;
            wsm[e] = (k < K) ? weights[static_cast<size_t>(k) * T + t] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        float2 a0[KC], a1[KC];
#pragma unroll
        for (int kk = 0; kk < KC; ++kk)
            a0[kk] = a1[kk] = make_float2(0.f, 0.f);
        if (valid)
        {
            const float4* src = reinterpret_cast<const float4*>(ring + pix0);
            const size_t step = HW / 2;
#pragma unroll 8
            for (int t = 0; t < T; ++t)
            {
                const float4 x = __ldg(src + static_cast<size_t>(t) * step);
                const float2* wt = wsm + t * KC;
#pragma unroll
                for (int kk = 0; kk < KC; ++kk)
                {
                    const float2 w = wt[kk];
                    a0[kk].x = fmaf(x.x, w.x, fmaf(-x.y, w.y, a0[kk].x));
                    a0[kk].y = fmaf(x.x, w.y, fmaf(x.y, w.x, a0[kk].y));
                    a1[kk].x = fmaf(x.z, w.x, fmaf(-x.w, w.y, a1[kk].x));
                    a1[kk].y = fmaf(x.z, w.y, fmaf(x.w, w.x, a1[kk].y));
                }
            }
            const int kn = (K - k0) < KC ? (K - k0) : KC;
#pragma unroll
            for (int kk = 0; kk < KC; ++kk)
                if (kk < kn)
                {
                    if (bin_w)
                    {
                        const float bw = __ldg(bin_w + k0 + kk);
                        view0 += (a0[kk].x * a0[kk].x + a0[kk].y * a0[kk].y) * bw;
                        view1 += (a1[kk].x * a1[kk].x + a1[kk].y * a1[kk].y) * bw;
                    }
                    else
                    {
                        view0 += view_value(a0[kk], img_type);
                        view1 += view_value(a1[kk], img_type);
                    }
                }
        }
    }
    float v0 = 0.f, v1 = 0.f;
    if (valid)
    {
        v0 = bin_w ? view0 : view0 / static_cast<float>(K);
        v1 = bin_w ? view1 : view1 / static_cast<float>(K);
        if (scale != 1.0f)
        {
            v0 = v0 * scale;
            v1 = v1 * scale;
        }
#pragma unroll
        for (int q = 0; q < 2; ++q)
        {
            const size_t pix = pix0 + q;
            const int x = static_cast<int>(pix % W);
            const int y = static_cast<int>(pix / W);
            size_t dst = pix;
            if (shift)
                dst = static_cast<size_t>((y + H / 2) % H) * W + (x + W / 2) % W;
            out[dst] = q ? v1 : v0;
        }
    }
    if (partials)
    {
        double d = valid ? static_cast<double>(v0) + static_cast<double>(v1) : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            d += __shfl_down_sync(0xffffffffu, d, o);
        if ((threadIdx.x & 31) == 0)
            red[threadIdx.x >> 5] = d;
        __syncthreads();
        // warps 0-1: pixels 0..127 of the CTA, warps 2-3: 128..255
        if (threadIdx.x < 2)
        {
            const int pi = 2 * blockIdx.x + threadIdx.x;
            if (pi < npartials)
                partials[pi] = red[2 * threadIdx.x] + red[2 * threadIdx.x + 1];
        }
    }
}

// sum_t x_t W[k][t] over slots [t0, t1) of a real ring, two adjacent pixels, from the split-BF16
// planes (hi = bf16(x), lo = bf16(x - hi): a 4-byte load from each plane) or from the complex ring
// (real parts of one 16-byte load). Either source takes the same FMAs in the same order as
// k_time_view / k_time_view2 on the ring (the zero imaginary parts leave those sums unchanged).
// The planes hold half the bytes per sample: twice the frames per unrolled step keep as many bytes
// in flight as the ring view.
template <int KC>
__device__ __forceinline__ void tvp_accumulate(float2 (&a)[2][KC], uint32_t h, uint32_t l, const float2* wt)
{
    // bf16 = the top half of an FP32 word; hi + lo is exact for integer pixels below 2^16
    const float x0 = __uint_as_float(h << 16) + __uint_as_float(l << 16);
    const float x1 = __uint_as_float(h & 0xffff0000u) + __uint_as_float(l & 0xffff0000u);
#pragma unroll
    for (int kk = 0; kk < KC; ++kk)
    {
        const float2 w = wt[kk];
        a[0][kk].x = fmaf(x0, w.x, a[0][kk].x);
        a[0][kk].y = fmaf(x0, w.y, a[0][kk].y);
        a[1][kk].x = fmaf(x1, w.x, a[1][kk].x);
        a[1][kk].y = fmaf(x1, w.y, a[1][kk].y);
    }
}

template <int KC>
__device__ __forceinline__ void tvp_planes(float2 (&a)[2][KC], const uint32_t* __restrict__ hi,
                                           const uint32_t* __restrict__ lo, size_t step, int t0, int t1,
                                           const float2* wsm)
{
    constexpr int D = 12;  // frames whose loads are issued before the first is used
    int t = t0;
    for (; t + D <= t1; t += D)
    {
        uint32_t h[D], l[D];
#pragma unroll
        for (int i = 0; i < D; ++i)
        {
            h[i] = __ldcs(hi + static_cast<size_t>(t + i) * step);
            l[i] = __ldcs(lo + static_cast<size_t>(t + i) * step);
        }
#pragma unroll
        for (int i = 0; i < D; ++i)
            tvp_accumulate<KC>(a, h[i], l[i], wsm + (t + i) * KC);
    }
    for (; t < t1; ++t)
        tvp_accumulate<KC>(a, __ldcs(hi + static_cast<size_t>(t) * step), __ldcs(lo + static_cast<size_t>(t) * step),
                           wsm + t * KC);
}

template <int KC>
__device__ __forceinline__ void tvp_ring(float2 (&a)[2][KC], const float4* __restrict__ ring, size_t step, int t0,
                                         int t1, const float2* wsm)
{
#pragma unroll 8
    for (int t = t0; t < t1; ++t)
    {
        const float4 r = __ldg(ring + static_cast<size_t>(t) * step);
        const float2* wt = wsm + t * KC;
#pragma unroll
        for (int kk = 0; kk < KC; ++kk)
        {
            const float2 w = wt[kk];
            a[0][kk].x = fmaf(r.x, w.x, a[0][kk].x);
            a[0][kk].y = fmaf(r.x, w.y, a[0][kk].y);
            a[1][kk].x = fmaf(r.z, w.x, a[1][kk].x);
            a[1][kk].y = fmaf(r.z, w.y, a[1][kk].y);
        }
    }
}

// The view of a real ring (zero imaginary parts) read from its split-BF16 planes ([2][T][HW] bf16,
// hi then lo): 4 bytes per sample instead of the 8 of the complex ring. The ring slots
// [r0, r0 + rn) mod T are read from the complex ring instead (the slots that the next batch's
// planes overwrite while this view may still run). Two adjacent pixels per thread, 128 threads
// cover 256 pixels and write their two 128-pixel renormalisation partials (those of k_time_view).
// The view values equal k_time_view's on the same ring. 64 registers: the grid leaves a CTA slot
// free on most SMs for the pipelined windows' eigensolve kernels (another stream).
template <int KC>
__global__ void __launch_bounds__(TV_THREADS, 8) k_time_view_planes(const uint16_t* __restrict__ planes,
                                                                 const float2* __restrict__ ring, int r0, int rn, int T,
                                                                 int W, int H, const float2* __restrict__ weights,
                                                                 int K, int img_type, float scale, int shift,
                                                                 float* __restrict__ out, double* __restrict__ partials,
                                                                 int npartials, const CycleCtl* ctl,
                                                                 const float* __restrict__ bin_w)
{
    if (!ctl_render(ctl))
        return;
    extern __shared__ __align__(16) float2 wsm[];  // [T][KC]
    __shared__ double red[TV_THREADS / 32];
    const size_t HW = static_cast<size_t>(W) * H;
    const size_t pix0 = 2 * (blockIdx.x * static_cast<size_t>(TV_THREADS) + threadIdx.x);
    const bool valid = pix0 < HW;  // HW even: both pixels or none
    // slot order [0, T) cut into at most three runs, each from one source
    int cut[4], src[3], nrun;
    if (rn <= 0)
    {
        cut[0] = 0, cut[1] = T, src[0] = 0, nrun = 1;
    }
    else if (r0 + rn <= T)
    {
        cut[0] = 0, cut[1] = r0, cut[2] = r0 + rn, cut[3] = T;
        src[0] = 0, src[1] = 1, src[2] = 0, nrun = 3;
    }
    else
    {
        cut[0] = 0, cut[1] = r0 + rn - T, cut[2] = r0, cut[3] = T;
        src[0] = 1, src[1] = 0, src[2] = 1, nrun = 3;
    }
    float view0 = 0.f, view1 = 0.f;
    for (int k0 = 0; k0 < K; k0 += KC)
    {
        __syncthreads();
        for (int e = threadIdx.x; e < T * KC; e += TV_THREADS)
        {
            const int t = e / KC, kk = e - t * KC;
            const int k = k0 + kk;
            wsm[e] = (k < K) ? weights[static_cast<size_t>(k) * T + t] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        float2 a[2][KC];
#pragma unroll
        for (int kk = 0; kk < KC; ++kk)
            a[0][kk] = a[1][kk] = make_float2(0.f, 0.f);
        if (valid)
        {
            for (int r = 0; r < nrun; ++r)
            {
                if (src[r])
                    tvp_ring<KC>(a, reinterpret_cast<const float4*>(ring + pix0), HW / 2, cut[r], cut[r + 1], wsm);
                else
                    tvp_planes<KC>(a, reinterpret_cast<const uint32_t*>(planes + pix0),
                                   reinterpret_cast<const uint32_t*>(planes + static_cast<size_t>(T) * HW + pix0),
                                   HW / 2, cut[r], cut[r + 1], wsm);
            }
            const int kn = (K - k0) < KC ? (K - k0) : KC;
#pragma unroll
            for (int kk = 0; kk < KC; ++kk)
                if (kk < kn)
                {
                    if (bin_w)
                    {
                        const float bw = __ldg(bin_w + k0 + kk);
                        view0 += (a[0][kk].x * a[0][kk].x + a[0][kk].y * a[0][kk].y) * bw;
                        view1 += (a[1][kk].x * a[1][kk].x + a[1][kk].y * a[1][kk].y) * bw;
                    }
                    else
                    {
                        view0 += view_value(a[0][kk], img_type);
                        view1 += view_value(a[1][kk], img_type);
                    }
                }
        }
    }
    float v0 = 0.f, v1 = 0.f;
    if (valid)
    {
        v0 = bin_w ? view0 : view0 / static_cast<float>(K);
        v1 = bin_w ? view1 : view1 / static_cast<float>(K);
        if (scale != 1.0f)
        {
            v0 = v0 * scale;
            v1 = v1 * scale;
        }
#pragma unroll
        for (int q = 0; q < 2; ++q)
        {
            const size_t pix = pix0 + q;
            const int x = static_cast<int>(pix % W);
            const int y = static_cast<int>(pix / W);
            size_t dst = pix;
            if (shift)
                dst = static_cast<size_t>((y + H / 2) % H) * W + (x + W / 2) % W;
            out[dst] = q ? v1 : v0;
        }
    }
    if (partials)
    {
        double d = valid ? static_cast<double>(v0) + static_cast<double>(v1) : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            d += __shfl_down_sync(0xffffffffu, d, o);
        if ((threadIdx.x & 31) == 0)
            red[threadIdx.x >> 5] = d;
        __syncthreads();
        // warps 0-1: pixels 0..127 of the CTA, warps 2-3: 128..255
        if (threadIdx.x < 2)
        {
            const int pi = 2 * blockIdx.x + threadIdx.x;
            if (pi < npartials)
                partials[pi] = red[2 * threadIdx.x] + red[2 * threadIdx.x + 1];
        }
    }
}

int time_view_partials(int W, int H)
{
    const size_t HW = static_cast<size_t>(W) * H;
    return static_cast<int>((HW + TV_THREADS - 1) / TV_THREADS);
}

template <int KC>
static hv_status launch_time_view(const float2* ring, int T, int W, int H, const float2* weights, int K, int img_type,
                                  float scale, int shift, float* out, double* partials, cudaStream_t st,
                                  const CycleCtl* ctl, const float* bin_w)
{
    const size_t smem = static_cast<size_t>(T) * KC * sizeof(float2);
    if (smem > 200 * 1024)
    {
        set_last_error_msg("time window too large for the time-view kernel");
        return HV_ERR_UNSUPPORTED;
    }
    if (smem > 48 * 1024)
        HV_CUDA_TRY(cudaFuncSetAttribute(k_time_view<KC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem)));
    const int np = time_view_partials(W, H);
    const size_t HW = static_cast<size_t>(W) * H;
    if (KC <= 4 && HW % 2 == 0)
    {
        if (smem > 48 * 1024)
            HV_CUDA_TRY(cudaFuncSetAttribute(k_time_view2<KC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem)));
        const int grid2 = static_cast<int>((HW + 2 * TV_THREADS - 1) / (2 * TV_THREADS));
        k_time_view2<KC><<<grid2, TV_THREADS, smem, st>>>(ring, T, W, H, weights, K, img_type, scale, shift, out,
                                                          partials, np, ctl, bin_w);
        HV_LAUNCH_CHECK();
        count_launch();
        return HV_OK;
    }
    const int grid = np;
    k_time_view<KC><<<grid, TV_THREADS, smem, st>>>(ring, T, W, H, weights, K, img_type, scale, shift, out, partials,
                                                    ctl, bin_w);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status time_view(const float2* ring, int T, int W, int H, const float2* weights, int K, int img_type, float scale,
                    int shift, float* out, double* partials, cudaStream_t st, const CycleCtl* ctl, const float* bin_w)
{
    if (T <= 0 || K <= 0 || W <= 0 || H <= 0)
    {
        set_last_error_msg("time_view: bad sizes");
        return HV_INVALID_VALUE;
    }
    if (shift && ((W & 1) || (H & 1)))
    {
        set_last_error_msg("fftshift needs even width and height");
        return HV_INVALID_VALUE;
    }
    // fewest register chunks, then the smallest instantiated chunk that covers K / chunks
    const int chunks = (K + TV_KMAX - 1) / TV_KMAX;
    const int need = (K + chunks - 1) / chunks;
    if (need <= 1)
        return launch_time_view<1>(ring, T, W, H, weights, K, img_type, scale, shift, out, partials, st, ctl, bin_w);
    if (need <= 2)
        return launch_time_view<2>(ring, T, W, H, weights, K, img_type, scale, shift, out, partials, st, ctl, bin_w);
    if (need <= 4)
        return launch_time_view<4>(ring, T, W, H, weights, K, img_type, scale, shift, out, partials, st, ctl, bin_w);
    if (need <= 6)
        return launch_time_view<6>(ring, T, W, H, weights, K, img_type, scale, shift, out, partials, st, ctl, bin_w);
    if (need <= 8)
        return launch_time_view<8>(ring, T, W, H, weights, K, img_type, scale, shift, out, partials, st, ctl, bin_w);
    if (need <= 11)
        return launch_time_view<11>(ring, T, W, H, weights, K, img_type, scale, shift, out, partials, st, ctl, bin_w);
    return launch_time_view<16>(ring, T, W, H, weights, K, img_type, scale, shift, out, partials, st, ctl, bin_w);
}

template <int KC>
static hv_status launch_time_view_planes(const uint16_t* planes, const float2* ring, int r0, int rn, int T, int W,
                                         int H, const float2* weights, int K, int img_type, float scale, int shift,
                                         float* out, double* partials, cudaStream_t st, const CycleCtl* ctl,
                                         const float* bin_w)
{
    const size_t smem = static_cast<size_t>(T) * KC * sizeof(float2);
    if (smem > 200 * 1024)
    {
        set_last_error_msg("time window too large for the time-view kernel");
        return HV_ERR_UNSUPPORTED;
    }
    if (smem > 48 * 1024)
        HV_CUDA_TRY(cudaFuncSetAttribute(k_time_view_planes<KC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem)));
    const size_t HW = static_cast<size_t>(W) * H;
    const int grid = static_cast<int>((HW + 2 * TV_THREADS - 1) / (2 * TV_THREADS));
    k_time_view_planes<KC><<<grid, TV_THREADS, smem, st>>>(planes, ring, r0, rn, T, W, H, weights, K, img_type, scale,
                                                           shift, out, partials, time_view_partials(W, H), ctl,
                                                           bin_w);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status time_view_planes(const uint16_t* planes, const float2* ring, int ring_slot0, int ring_n, int T, int W, int H,
                           const float2* weights, int K, int img_type, float scale, int shift, float* out,
                           double* partials, cudaStream_t st, const CycleCtl* ctl, const float* bin_w)
{
    if (T <= 0 || K <= 0 || W <= 0 || H <= 0 || ring_n < 0 || ring_n > T || ring_slot0 < 0 || ring_slot0 >= T)
    {
        set_last_error_msg("time_view_planes: bad sizes");
        return HV_INVALID_VALUE;
    }
    if (shift && ((W & 1) || (H & 1)))
    {
        set_last_error_msg("fftshift needs even width and height");
        return HV_INVALID_VALUE;
    }
    const size_t HW = static_cast<size_t>(W) * H;
    if (HW % 8 != 0 || (reinterpret_cast<uintptr_t>(planes) & 15) != 0 ||
        (ring_n > 0 && (reinterpret_cast<uintptr_t>(ring) & 15) != 0))
    {
        set_last_error_msg("time_view_planes: W x H must be a multiple of 8 and the planes and ring 16-byte aligned");
        return HV_ERR_UNSUPPORTED;
    }
    // chunks of up to 4 bins (2 KC complex accumulators per thread)
    if (K == 1)
        return launch_time_view_planes<1>(planes, ring, ring_slot0, ring_n, T, W, H, weights, K, img_type, scale, shift,
                                          out, partials, st, ctl, bin_w);
    if (K == 2)
        return launch_time_view_planes<2>(planes, ring, ring_slot0, ring_n, T, W, H, weights, K, img_type, scale, shift,
                                          out, partials, st, ctl, bin_w);
    return launch_time_view_planes<4>(planes, ring, ring_slot0, ring_n, T, W, H, weights, K, img_type, scale, shift,
                                      out, partials, st, ctl, bin_w);
}

// ------------------------------------------------------------------------------ weights

__global__ void k_stft_weights(float2* w, int T, int pmin, int K)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= K * T)
        return;
    const int k = e / T, t = e - k * T;
    const long long m = (static_cast<long long>(pmin + k) * t) % T;
    double s, c;
    sincospi(-2.0 * static_cast<double>(m) / static_cast<double>(T), &s, &c);
    w[e] = make_float2(static_cast<float>(c), static_cast<float>(s));
}

__global__ void k_delta_weights(float2* w, int T, int pmin, int K)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= K * T)
        return;
    const int k = e / T, t = e - k * T;
    w[e] = make_float2(t == pmin + k ? 1.f : 0.f, 0.f);
}

// f_k^n of the bins pmin..pmax with the Nyquist compensation, in the reference's float arithmetic:
// d = (float)camera_fps / T, f1 = i d for the first half and -(T - i) d (even T) or (i - T) d
// (odd T) for the second (icompute.cc:26-69); the Nyquist bin of an even window counts twice for
// orders 0 and 2 and not at all for order 1 (tools_compute.cu:60-69).
hv_status moment_bin_weights(float* bin_w, int T, int pmin, int pmax, int order, float camera_fps, cudaStream_t st)
{
    if (T <= 0 || pmin < 0 || pmax < pmin || pmax >= T || order < 0 || order > 2 || !bin_w)
        return HV_INVALID_VALUE;
    const float d = camera_fps / static_cast<float>(T);
    std::vector<float> w(static_cast<size_t>(pmax - pmin + 1));
    const bool even = T % 2 == 0;
    for (int i = pmin; i <= pmax; ++i)
    {
        float f1;
        if (even)
            f1 = i < T / 2 ? static_cast<float>(i) * d : -(static_cast<float>(T) - static_cast<float>(i)) * d;
        else
            f1 = i < (T + 1) / 2 ? static_cast<float>(i) * d : (static_cast<float>(i) - static_cast<float>(T)) * d;
        float f = order == 0 ? 1.0f : (order == 1 ? f1 : f1 * f1);
        if (even && i == T / 2)
            f = order == 1 ? 0.0f : 2.0f * f;
        w[static_cast<size_t>(i - pmin)] = f;
    }
    HV_CUDA_TRY(cudaMemcpyAsync(bin_w, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    HV_CUDA_TRY(cudaStreamSynchronize(st));  // the host table goes out of scope
    return HV_OK;
}

hv_status stft_weights(float2* weights, int T, int pmin, int pmax, cudaStream_t st)
{
    const int K = pmax - pmin + 1;
    if (K <= 0 || T <= 0)
        return HV_INVALID_VALUE;
    k_stft_weights<<<(K * T + 255) / 256, 256, 0, st>>>(weights, T, pmin, K);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status delta_weights(float2* weights, int T, int pmin, int pmax, cudaStream_t st)
{
    const int K = pmax - pmin + 1;
    if (K <= 0 || T <= 0)
        return HV_INVALID_VALUE;
    k_delta_weights<<<(K * T + 255) / 256, 256, 0, st>>>(weights, T, pmin, K);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

// ------------------------------------------------------------------------------ PCA covariance
// C[i][j] = sum_pix conj(H[pix][i]) H[pix][j], H[pix][t] = ring[t][pix]. Split-K over pixel
// chunks: CTA (tile, chunk) accumulates a 32 x 32 complex tile in FP32 registers, partial tiles
// are summed in FP64 by k_cov_reduce, which also mirrors the Hermitian triangle.

constexpr int COV_TILE = 32;
constexpr int COV_THREADS = 256;
constexpr int COV_PX = 32;  // pixels per shared-memory stage

struct CovPlan
{
    int tiles1d, ntiles, chunks;
    size_t chunk_px;
};

static CovPlan cov_plan(int T, size_t npix)
{
    CovPlan p;
    p.tiles1d = (T + COV_TILE - 1) / COV_TILE;
    p.ntiles = p.tiles1d * (p.tiles1d + 1) / 2;
    int chunks = (152 * 8 + p.ntiles - 1) / p.ntiles;
    const size_t max_chunks = (npix + COV_PX - 1) / COV_PX;
    if (static_cast<size_t>(chunks) > max_chunks)
        chunks = static_cast<int>(max_chunks);
    if (chunks < 1)
        chunks = 1;
    p.chunks = chunks;
    p.chunk_px = ((npix + chunks - 1) / chunks + COV_PX - 1) / COV_PX * COV_PX;
    return p;
}

__global__ void __launch_bounds__(COV_THREADS) k_cov_partial(const float2* __restrict__ ring, int T, size_t npix,
                                                              int tiles1d, size_t chunk_px, float2* __restrict__ part)
{
    __shared__ float2 A[COV_PX][COV_TILE + 1];
    __shared__ float2 B[COV_PX][COV_TILE + 1];
    // tile index -> (ti, tj) with ti <= tj
    int t = blockIdx.x, ti = 0;
    while (t >= tiles1d - ti)
    {
        t -= tiles1d - ti;
        ++ti;
    }
    const int tj = ti + t;
    const int chunk = blockIdx.y;
    const size_t p0 = chunk * chunk_px;
    const size_t p1 = (p0 + chunk_px < npix) ? p0 + chunk_px : npix;
    // thread -> 2 x 2 outputs: rows ri*2 + {0,1}, cols cj*2 + {0,1}
    const int ri = threadIdx.x / 16, cj = threadIdx.x % 16;
    float2 acc[2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
            acc[a][b] = make_float2(0.f, 0.f);
    for (size_t px0 = p0; px0 < p1; px0 += COV_PX)
    {
        __syncthreads();
        for (int e = threadIdx.x; e < COV_PX * COV_TILE; e += COV_THREADS)
        {
            const int c = e / COV_PX, pp = e % COV_PX;  // pixel fastest: coalesced ring reads
            const size_t px = px0 + pp;
            const int ia = ti * COV_TILE + c, ib = tj * COV_TILE + c;
            A[pp][c] = (px < p1 && ia < T) ? __ldg(ring + static_cast<size_t>(ia) * npix + px) : make_float2(0.f, 0.f);
            B[pp][c] = (px < p1 && ib < T) ? __ldg(ring + static_cast<size_t>(ib) * npix + px) : make_float2(0.f, 0.f);
        }
        __syncthreads();
#pragma unroll 4
        for (int pp = 0; pp < COV_PX; ++pp)
        {
            const float2 a0 = A[pp][ri * 2], a1 = A[pp][ri * 2 + 1];
            const float2 b0 = B[pp][cj * 2], b1 = B[pp][cj * 2 + 1];
            // conj(a) * b
            acc[0][0].x = fmaf(a0.x, b0.x, fmaf(a0.y, b0.y, acc[0][0].x));
            acc[0][0].y = fmaf(a0.x, b0.y, fmaf(-a0.y, b0.x, acc[0][0].y));
            acc[0][1].x = fmaf(a0.x, b1.x, fmaf(a0.y, b1.y, acc[0][1].x));
            acc[0][1].y = fmaf(a0.x, b1.y, fmaf(-a0.y, b1.x, acc[0][1].y));
            acc[1][0].x = fmaf(a1.x, b0.x, fmaf(a1.y, b0.y, acc[1][0].x));
            acc[1][0].y = fmaf(a1.x, b0.y, fmaf(-a1.y, b0.x, acc[1][0].y));
            acc[1][1].x = fmaf(a1.x, b1.x, fmaf(a1.y, b1.y, acc[1][1].x));
            acc[1][1].y = fmaf(a1.x, b1.y, fmaf(-a1.y, b1.x, acc[1][1].y));
        }
    }
    // part layout: [chunk][tile][32][32]
    float2* dst = part + (static_cast<size_t>(chunk) * gridDim.x + blockIdx.x) * COV_TILE * COV_TILE;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
            dst[(ri * 2 + a) * COV_TILE + cj * 2 + b] = acc[a][b];
}

// Sums the partial tiles of a slice of chunks in FP64 and adds them atomically into cov
// (zeroed before); grid.y splits the chunks so the reduction is not latency bound.
__global__ void k_cov_reduce(const float2* __restrict__ part, int T, int tiles1d, int ntiles, int chunks,
                             int chunks_per_slice, double2* __restrict__ cov)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;  // over T*T
    if (e >= T * T)
        return;
    int i = e / T, j = e % T;
    const bool mirror = i > j;  // lower triangle: conj of (j, i)
    if (mirror)
    {
        const int s = i;
        i = j;
        j = s;
    }
    const int ti = i / COV_TILE, tj = j / COV_TILE;
    const int tile = ti * tiles1d - ti * (ti - 1) / 2 + (tj - ti);
    const int li = i % COV_TILE, lj = j % COV_TILE;
    const int c0 = blockIdx.y * chunks_per_slice;
    const int c1 = min(chunks, c0 + chunks_per_slice);
    double re = 0.0, im = 0.0;
#pragma unroll 4
    for (int c = c0; c < c1; ++c)
    {
        const float2 v = part[(static_cast<size_t>(c) * ntiles + tile) * COV_TILE * COV_TILE + li * COV_TILE + lj];
        re += v.x;
        im += v.y;
    }
    atomicAdd(&cov[e].x, re);
    if (i != j)  // Hermitian: the diagonal is real
        atomicAdd(&cov[e].y, mirror ? -im : im);
}

static std::atomic<int> g_cov_mode{0};  // 0 auto (tensor cores when supported), 1 SIMT, 2 tensor cores

constexpr size_t COV_FLAGS = 256;

size_t pca_cov_workspace(int T, size_t npix)
{
    const CovPlan p = cov_plan(T, npix);
    size_t simt = static_cast<size_t>(p.chunks) * p.ntiles * COV_TILE * COV_TILE * sizeof(float2);
    size_t tc = cov_tc_supported(T) ? cov_tc_workspace(T, npix) : 0;
    return COV_FLAGS + (simt > tc ? simt : tc);
}

size_t pca_cov_workspace_planes(int T, size_t npix)
{
    const CovPlan p = cov_plan(T, npix);
    size_t simt = static_cast<size_t>(p.chunks) * p.ntiles * COV_TILE * COV_TILE * sizeof(float2);
    size_t tc = cov_tc_supported(T) ? (2 * T > 128 ? cov_tc_partial_bytes(T, npix) : cov_tc_workspace(T, npix)) : 0;
    return COV_FLAGS + (simt > tc ? simt : tc);
}

void set_cov_mode(int mode) { g_cov_mode = mode; }
int cov_mode() { return g_cov_mode.load(); }

static std::atomic<bool> g_cov_incremental{true};
void set_cov_incremental(bool on) { g_cov_incremental = on; }
bool cov_incremental() { return g_cov_incremental.load(); }

hv_status pca_covariance(const float2* ring, int T, size_t npix, double2* cov, void* work, cudaStream_t st)
{
    if (T <= 0 || npix == 0)
        return HV_INVALID_VALUE;
    int* err = static_cast<int*>(work);
    char* ws = static_cast<char*>(work) + COV_FLAGS;
    HV_CUDA_TRY(cudaMemsetAsync(cov, 0, static_cast<size_t>(T) * T * sizeof(double2), st));
    HV_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
    const bool tc_ok = cov_tc_supported(T) && npix % 8 == 0 && (reinterpret_cast<uintptr_t>(ring) & 15) == 0;
    const int mode = g_cov_mode.load();
    if ((mode == 0 && tc_ok) || mode == 2)
    {
        if (!tc_ok)
        {
            set_last_error_msg("tensor-core covariance unsupported for this shape");
            return HV_ERR_UNSUPPORTED;
        }
        return cov_tc(ring, T, npix, cov, ws, err, st);
    }
    const CovPlan p = cov_plan(T, npix);
    float2* part = reinterpret_cast<float2*>(ws);
    dim3 grid(p.ntiles, p.chunks);
    k_cov_partial<<<grid, COV_THREADS, 0, st>>>(ring, T, npix, p.tiles1d, p.chunk_px, part);
    HV_LAUNCH_CHECK();
    const int slices = p.chunks < 32 ? p.chunks : 32;
    const int per = (p.chunks + slices - 1) / slices;
    dim3 rgrid((T * T + 255) / 256, (p.chunks + per - 1) / per);
    k_cov_reduce<<<rgrid, 256, 0, st>>>(part, T, p.tiles1d, p.ntiles, p.chunks, per, cov);
    HV_LAUNCH_CHECK();
    count_launch(2);
    return HV_OK;
}

hv_status pca_covariance_planes(const uint16_t* planes, int T, size_t npix, double2* cov, void* work, uint32_t blocks,
                                int real, cudaStream_t st)
{
    if (T <= 0 || npix == 0 || !planes || !cov || !work)
        return HV_INVALID_VALUE;
    if (g_cov_mode.load() == 1)
        return HV_ERR_UNSUPPORTED;
    int* err = static_cast<int*>(work);
    char* ws = static_cast<char*>(work) + COV_FLAGS;
    HV_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
    return cov_tc_planes(planes, T, npix, cov, ws, err, blocks, real, st);
}

hv_status pca_cov_status(const void* work)
{
    int flag = 0;
    HV_CUDA_TRY(cudaMemcpy(&flag, work, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag)
    {
        set_last_error_msg("tensor-core covariance: a bounded wait gave up");
        return HV_ERR_TIMEOUT;
    }
    return HV_OK;
}

// ------------------------------------------------------------------------------ FP64 Jacobi
// Cyclic two-sided Jacobi with the round-robin (tournament) ordering: each step rotates T/2
// disjoint (p, q) pairs in parallel. A rotation first turns A[p][q] real with a phase on index q
// and then applies the real symmetric Schur rotation (Golub & Van Loan, Alg. 8.4.1), i.e.
// J = diag(1, e^{-i phi}) R(c, s). Matrix in global memory (row-major, complex128), one CTA.
// The sweep count is bounded; the global variant stops when the off-diagonal norm is below 1e-13 of the
// total, the shared-memory variant after a sweep without rotation (threshold 1e-15 relative).

constexpr int JAC_THREADS = 512;
constexpr int JAC_MAX_SWEEPS = 40;

__device__ __forceinline__ double2 zmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__global__ void __launch_bounds__(JAC_THREADS) k_jacobi(double2* A, double2* V, int T, int Tp, double* evals,
                                                         int* pair_buf, double* rot_buf)
{
    // pair_buf: 2*(Tp/2) ints; rot_buf: 4*(Tp/2) doubles (c, s, cos phi, sin phi)
    __shared__ double red[JAC_THREADS / 32];
    __shared__ double s_off, s_norm;
    const int tid = threadIdx.x;
    // V = I
    for (int e = tid; e < T * T; e += JAC_THREADS)
        V[e] = make_double2((e / T) == (e % T) ? 1.0 : 0.0, 0.0);
    __syncthreads();
    const int npairs = Tp / 2;
    for (int sweep = 0; sweep < JAC_MAX_SWEEPS; ++sweep)
    {
        // off-diagonal norm and total norm
        double off = 0.0, nrm = 0.0;
        for (int e = tid; e < T * T; e += JAC_THREADS)
        {
            const double2 a = A[e];
            const double m = a.x * a.x + a.y * a.y;
            nrm += m;
            if ((e / T) != (e % T))
                off += m;
        }
        for (int o = 16; o > 0; o >>= 1)
        {
            off += __shfl_down_sync(0xffffffffu, off, o);
            nrm += __shfl_down_sync(0xffffffffu, nrm, o);
        }
        if ((tid & 31) == 0)
            red[tid >> 5] = off;
        __syncthreads();
        if (tid == 0)
        {
            double s = 0.0;
            for (int i = 0; i < JAC_THREADS / 32; ++i)
                s += red[i];
            s_off = s;
        }
        __syncthreads();
        if ((tid & 31) == 0)
            red[tid >> 5] = nrm;
        __syncthreads();
        if (tid == 0)
        {
            double s = 0.0;
            for (int i = 0; i < JAC_THREADS / 32; ++i)
                s += red[i];
            s_norm = s;
        }
        __syncthreads();
        if (s_off <= 1e-26 * s_norm || s_norm == 0.0)
            break;
        for (int step = 0; step < Tp - 1; ++step)
        {
            // round-robin pairing: player Tp-1 fixed, others rotate
            for (int k = tid; k < npairs; k += JAC_THREADS)
            {
                int a, b;
                if (k == 0)
                {
                    a = Tp - 1;
                    b = step % (Tp - 1);
                }
                else
                {
                    a = (step + k) % (Tp - 1);
                    b = (step - k + (Tp - 1)) % (Tp - 1);
                }
                const int p = a < b ? a : b, q = a < b ? b : a;
                pair_buf[2 * k] = p;
                pair_buf[2 * k + 1] = q;
                double c = 1.0, s = 0.0, cph = 1.0, sph = 0.0;
                if (q < T)
                {
                    const double2 apq = A[p * T + q];
                    const double mag = hypot(apq.x, apq.y);
                    const double app = A[p * T + p].x, aqq = A[q * T + q].x;
                    if (mag > 1e-300 && mag > 1e-15 * sqrt(fabs(app * aqq)))
                    {
                        cph = apq.x / mag;
                        sph = apq.y / mag;
                        const double tau = (aqq - app) / (2.0 * mag);
                        const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                        c = 1.0 / sqrt(1.0 + t * t);
                        s = t * c;
                    }
                }
                rot_buf[4 * k] = c;
                rot_buf[4 * k + 1] = s;
                rot_buf[4 * k + 2] = cph;
                rot_buf[4 * k + 3] = sph;
            }
            __syncthreads();
            // column update A <- A J and V <- V J; J = [[c, s], [-s e^{-i phi}, c e^{-i phi}]]
            for (int e = tid; e < npairs * T; e += JAC_THREADS)
            {
                const int k = e / T, r = e % T;
                const int p = pair_buf[2 * k], q = pair_buf[2 * k + 1];
                if (q >= T)
                    continue;
                const double c = rot_buf[4 * k], s = rot_buf[4 * k + 1];
                const double2 em = make_double2(rot_buf[4 * k + 2], -rot_buf[4 * k + 3]);  // e^{-i phi}
                {
                    const double2 ap = A[r * T + p], aq = A[r * T + q];
                    const double2 aqe = zmul(aq, em);
                    A[r * T + p] = make_double2(c * ap.x - s * aqe.x, c * ap.y - s * aqe.y);
                    A[r * T + q] = make_double2(s * ap.x + c * aqe.x, s * ap.y + c * aqe.y);
                }
                {
                    const double2 vp = V[r * T + p], vq = V[r * T + q];
                    const double2 vqe = zmul(vq, em);
                    V[r * T + p] = make_double2(c * vp.x - s * vqe.x, c * vp.y - s * vqe.y);
                    V[r * T + q] = make_double2(s * vp.x + c * vqe.x, s * vp.y + c * vqe.y);
                }
            }
            __syncthreads();
            // row update A <- J^H A: row p <- c A_p - s e^{i phi} A_q, row q <- s A_p + c e^{i phi} A_q
            for (int e = tid; e < npairs * T; e += JAC_THREADS)
            {
                const int k = e / T, col = e % T;
                const int p = pair_buf[2 * k], q = pair_buf[2 * k + 1];
                if (q >= T)
                    continue;
                const double c = rot_buf[4 * k], s = rot_buf[4 * k + 1];
                const double2 ep = make_double2(rot_buf[4 * k + 2], rot_buf[4 * k + 3]);  // e^{i phi}
                const double2 ap = A[p * T + col], aq = A[q * T + col];
                const double2 aqe = zmul(aq, ep);
                A[p * T + col] = make_double2(c * ap.x - s * aqe.x, c * ap.y - s * aqe.y);
                A[q * T + col] = make_double2(s * ap.x + c * aqe.x, s * ap.y + c * aqe.y);
            }
            __syncthreads();
            // exact zeros / real diagonal for the rotated pairs
            for (int k = tid; k < npairs; k += JAC_THREADS)
            {
                const int p = pair_buf[2 * k], q = pair_buf[2 * k + 1];
                if (q >= T || rot_buf[4 * k + 1] == 0.0)
                    continue;
                A[p * T + q] = make_double2(0.0, 0.0);
                A[q * T + p] = make_double2(0.0, 0.0);
                A[p * T + p].y = 0.0;
                A[q * T + q].y = 0.0;
            }
            __syncthreads();
        }
    }
    for (int i = tid; i < T; i += JAC_THREADS)
        evals[i] = A[i * T + i].x;
}

// Shared-memory variant for T <= 64 (A and V resident in shared memory, one CTA), templated on
// the sweep precision. The step update works on 2 x 2 blocks: for row pair k1 and column pair k2
// the block of A becomes J1^H B J2 and the mirrored block its conjugate transpose (A stays
// Hermitian), so each step is one barrier-separated phase; steps whose rotations are all
// identities are skipped and the sweeps stop after a sweep without rotation. The skip threshold is
// a few units of the working precision relative to sqrt(|a_pp a_qq|).
constexpr int JS_THREADS = 256;
constexpr int JS_MAX_T = 64;

template <class R>
struct Cx
{
    R x, y;
};
template <class R>
__device__ __forceinline__ Cx<R> cxmul(Cx<R> a, Cx<R> b)
{
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}

template <class R>
__device__ __forceinline__ R jac_threshold();
template <>
__device__ __forceinline__ double jac_threshold<double>() { return 1e-15; }
template <>
__device__ __forceinline__ float jac_threshold<float>() { return 2.5e-7f; }

template <class R>
struct JacRot
{
    R c, s, cph, sph;  // J = [[c, s], [-s e^{-i phi}, c e^{-i phi}]], e^{i phi} = cph + i sph
};

template <class R>
struct JacScratch
{
    int2 pq[JS_MAX_T / 2];  // the step's pairs (p < q)
    int act[JS_MAX_T / 2];
    JacRot<R> rot[JS_MAX_T / 2];
    short2 blk[(JS_MAX_T / 2) * (JS_MAX_T / 2 + 1) / 2];
};

// Power of two that brings the largest diagonal entry of a Hermitian positive semi-definite matrix
// (its largest entry in magnitude) near 1: the FP32 sweeps square entries (|a_pq|^2, a_pp a_qq),
// which overflow for covariances of large frames (1024 x 1024 pixels of 8-bit data scaled by 257
// give entries near 1e22). Scaling by a power of two changes no eigenvector and no relative
// rounding. 1 for a zero or non-finite maximum.
__device__ __forceinline__ double jac_scale(double max_diag)
{
    if (!(max_diag > 0.0) || !isfinite(max_diag))
        return 1.0;
    return ldexp(1.0, -ilogb(max_diag));
}

// Rotation annihilating a_pq of the 2 x 2 Hermitian block [[app, apq], [conj(apq), aqq]] when |apq|
// exceeds the relative threshold thr * sqrt(|app aqq|) and `floor` (and is not 0); returns false (identity)
// otherwise. The FP32 form uses reciprocal square roots and one division (the sweeps only need an
// orthogonal rotation to FP32 accuracy; the eigenpairs are finished in FP64).
__device__ __forceinline__ bool jac_rotation(Cx<float> apq, float app, float aqq, float thr, float floor,
                                             JacRot<float>& r)
{
    const float m2 = apq.x * apq.x + apq.y * apq.y;
    if (!(m2 > 0.0f) || !(m2 > floor * floor) || !(m2 > thr * thr * fabsf(app * aqq)))
        return false;
    const float inv = rsqrtf(m2);
    r.cph = apq.x * inv;
    r.sph = apq.y * inv;
    const float tau = 0.5f * (aqq - app) * inv;
    const float t = copysignf(1.0f, tau) / (fabsf(tau) + sqrtf(fmaf(tau, tau, 1.0f)));
    r.c = rsqrtf(fmaf(t, t, 1.0f));
    r.s = t * r.c;
    return true;
}

__device__ __forceinline__ bool jac_rotation(Cx<double> apq, double app, double aqq, double thr, double floor,
                                             JacRot<double>& r)
{
    const double mag = hypot(apq.x, apq.y);
    if (!(mag > 1e-30) || !(mag > floor) || !(mag > thr * sqrt(fabs(app * aqq))))
        return false;
    r.cph = apq.x / mag;
    r.sph = apq.y / mag;
    const double tau = (aqq - app) / (2.0 * mag);
    const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
    r.c = 1.0 / sqrt(1.0 + t * t);
    r.s = t * r.c;
    return true;
}

// Cyclic sweeps over the T x T Hermitian A (T <= 64, shared memory, leading dimension LD) with the
// round-robin pairing, accumulating V <- V J; at most max_sweeps sweeps, ending after a sweep
// without rotation. A rotation is applied when |a_pq| exceeds both the relative threshold and
// `floor`. Every thread of the block (NT of them) calls it; returns whether any rotation was applied.
// Pair k of step `step` of a sweep over Tp indices. Round-robin order; with `split` (Tp = 2h, the
// two halves already nearly diagonal) the h cross steps (i, h + (i + step) mod h) come first, then
// the h - 1 round-robin steps inside both halves at once.
__device__ __forceinline__ void sweep_pair(int step, int k, int Tp, bool split, int& p, int& q)
{
    int n = Tp, s = step, kk = k, base = 0;
    if (split)
    {
        const int h = Tp / 2;
        if (step < h)
        {
            p = k;
            q = h + (k + step) % h;
            return;
        }
        n = h;
        s = step - h;
        kk = k % (h / 2);
        base = (k / (h / 2)) * h;
    }
    int a, b;
    if (kk == 0)
    {
        a = n - 1;
        b = s % (n - 1);
    }
    else
    {
        a = (s + kk) % (n - 1);
        b = (s - kk + (n - 1)) % (n - 1);
    }
    p = base + (a < b ? a : b);
    q = base + (a < b ? b : a);
}

// N > 0 fixes T = Tp = N and LD = N + 1 at compile time (index arithmetic by shifts). A sweep runs
// the steps [step_begin, step_end) of its ordering (step_end < 0: all Tp - 1 steps).
template <class R, int NT, int N = 0>
__device__ bool smem_sweeps(Cx<R>* A, Cx<R>* V, int T_, int Tp_, int LD_, JacScratch<R>& sc, R floor, int max_sweeps,
                            bool split = false, int step_begin = 0, int step_end = -1)
{
    const int T = N > 0 ? N : T_, Tp = N > 0 ? N : Tp_, LD = N > 0 ? N + 1 : LD_;
    const int tid = threadIdx.x;
    const int npairs = Tp / 2;
    const int nblocks = npairs * (npairs + 1) / 2;
    for (int e = tid; e < nblocks; e += NT)
    {
        int k1 = 0;
        while ((k1 + 1) * (k1 + 2) / 2 <= e)
            ++k1;
        sc.blk[e] = make_short2(static_cast<short>(k1), static_cast<short>(e - k1 * (k1 + 1) / 2));
    }
    __syncthreads();
    const R thr = jac_threshold<R>();
    bool any = false;
    for (int sweep = 0; sweep < max_sweeps; ++sweep)
    {
        int sweep_active = 0;
        const int s_end = step_end < 0 ? Tp - 1 : step_end;
        for (int step = step_begin; step < s_end; ++step)
        {
            int active = 0;
            if (tid < npairs)
            {
                const int k = tid;
                int p, q;
                sweep_pair(step, k, Tp, split, p, q);
                sc.pq[k] = make_int2(p, q);
                JacRot<R> r = {1, 0, 1, 0};
                if (q < T && jac_rotation(A[p * LD + q], A[p * LD + p].x, A[q * LD + q].x, thr, floor, r))
                    active = 1;
                sc.rot[k] = r;
                sc.act[k] = active;
            }
            if (!__syncthreads_or(active))
                continue;
            sweep_active = 1;
            // A <- J^H A J, block by block (k1 >= k2) with the mirror block
            for (int e = tid; e < nblocks; e += NT)
            {
                const int k1 = sc.blk[e].x, k2 = sc.blk[e].y;
                if (!sc.act[k1] && !sc.act[k2])
                    continue;
                const int2 P1 = sc.pq[k1], P2 = sc.pq[k2];
                const int r0 = P1.x, r1 = P1.y, c0 = P2.x, c1 = P2.y;
                const bool hr1 = r1 < T, hc1 = c1 < T;
                const Cx<R> z = {0, 0};
                Cx<R> B[2][2];
                B[0][0] = A[r0 * LD + c0];
                B[0][1] = hc1 ? A[r0 * LD + c1] : z;
                B[1][0] = hr1 ? A[r1 * LD + c0] : z;
                B[1][1] = (hr1 && hc1) ? A[r1 * LD + c1] : z;
                // X = B J2, J2 = [[c, s], [-s e^{-i phi}, c e^{-i phi}]]
                const JacRot<R> J1 = sc.rot[k1], J2 = sc.rot[k2];
                const R c2 = J2.c, s2 = J2.s;
                const Cx<R> em2 = {J2.cph, -J2.sph};
                Cx<R> X[2][2];
#pragma unroll
                for (int r = 0; r < 2; ++r)
                {
                    const Cx<R> b1 = cxmul(B[r][1], em2);
                    X[r][0] = {c2 * B[r][0].x - s2 * b1.x, c2 * B[r][0].y - s2 * b1.y};
                    X[r][1] = {s2 * B[r][0].x + c2 * b1.x, s2 * B[r][0].y + c2 * b1.y};
                }
                // Y = J1^H X: row0 = c X0 - s e^{i phi} X1, row1 = s X0 + c e^{i phi} X1
                const R c1r = J1.c, s1r = J1.s;
                const Cx<R> ep1 = {J1.cph, J1.sph};
                Cx<R> Y[2][2];
#pragma unroll
                for (int cc = 0; cc < 2; ++cc)
                {
                    const Cx<R> x1 = cxmul(X[1][cc], ep1);
                    Y[0][cc] = {c1r * X[0][cc].x - s1r * x1.x, c1r * X[0][cc].y - s1r * x1.y};
                    Y[1][cc] = {s1r * X[0][cc].x + c1r * x1.x, s1r * X[0][cc].y + c1r * x1.y};
                }
                if (k1 == k2 && sc.act[k1])
                {
                    Y[0][1] = z;
                    Y[1][0] = z;
                    Y[0][0].y = 0;
                    Y[1][1].y = 0;
                }
                A[r0 * LD + c0] = Y[0][0];
                if (hc1)
                    A[r0 * LD + c1] = Y[0][1];
                if (hr1)
                    A[r1 * LD + c0] = Y[1][0];
                if (hr1 && hc1)
                    A[r1 * LD + c1] = Y[1][1];
                if (k1 != k2)
                {
                    A[c0 * LD + r0] = {Y[0][0].x, -Y[0][0].y};
                    if (hc1)
                        A[c1 * LD + r0] = {Y[0][1].x, -Y[0][1].y};
                    if (hr1)
                        A[c0 * LD + r1] = {Y[1][0].x, -Y[1][0].y};
                    if (hr1 && hc1)
                        A[c1 * LD + r1] = {Y[1][1].x, -Y[1][1].y};
                }
            }
            // V <- V J for the active pairs
            for (int e = tid; e < npairs * T; e += NT)
            {
                const int k = e / T, r = e % T;
                if (!sc.act[k])
                    continue;
                const int p = sc.pq[k].x, q = sc.pq[k].y;
                const JacRot<R> J = sc.rot[k];
                const R c = J.c, s = J.s;
                const Cx<R> em = {J.cph, -J.sph};
                const Cx<R> vp = V[r * LD + p], vq = cxmul(V[r * LD + q], em);
                V[r * LD + p] = {c * vp.x - s * vq.x, c * vp.y - s * vq.y};
                V[r * LD + q] = {s * vp.x + c * vq.x, s * vp.y + c * vq.y};
            }
            __syncthreads();
        }
        if (!sweep_active)
            break;
        any = true;
    }
    return any;
}

// C = op(X) Y for T x T shared-memory matrices (leading dimension LD), op(X) = X or X^H; every
// thread of the block takes output elements in turn.
template <class R, int NT>
__device__ void smem_cgemm(const Cx<R>* X, const Cx<R>* Y, Cx<R>* C, int T, int LD, bool conj_x)
{
    for (int e = threadIdx.x; e < T * T; e += NT)
    {
        const int i = e / T, j = e % T;
        R re = 0, im = 0;
        for (int k = 0; k < T; ++k)
        {
            Cx<R> x = conj_x ? X[k * LD + i] : X[i * LD + k];
            if (conj_x)
                x.y = -x.y;
            const Cx<R> y = Y[k * LD + j];
            re += x.x * y.x - x.y * y.y;
            im += x.x * y.y + x.y * y.x;
        }
        C[i * LD + j] = {re, im};
    }
}

// Shared-memory bytes of k_jacobi_smem: A and V, plus two work matrices for a warm start.
template <class R>
size_t jacobi_smem_bytes(int T, bool warm)
{
    return (warm ? 4 : 2) * static_cast<size_t>(T) * (T + 1) * sizeof(Cx<R>);
}

// `warm` (FP32 only): Vout holds the orthonormal eigenvector basis of the previous call on this
// workspace (a window of the same stream): the sweeps start from A' = V0^H A V0 with V = V0, which
// is nearly diagonal when consecutive windows share their temporal modes, so one or two sweeps
// finish it. V0 is first re-orthonormalised by one Newton-Schulz step V0 (3 I - V0^H V0) / 2, so
// rounding does not accumulate from window to window.
template <class R>
__global__ void __launch_bounds__(JS_THREADS) k_jacobi_smem(const double2* __restrict__ Ain, double2* __restrict__ Vout,
                                                            int T, int Tp, double* __restrict__ evals, int warm,
                                                            float floor_rel)
{
    extern __shared__ __align__(16) unsigned char js_raw[];
    Cx<R>* js = reinterpret_cast<Cx<R>*>(js_raw);
    const int LD = T + 1;
    Cx<R>* A = js;
    Cx<R>* V = js + T * LD;
    Cx<R>* X = V + T * LD;  // warm start only
    Cx<R>* N = X + T * LD;
    __shared__ JacScratch<R> sc;
    __shared__ double s_scale;
    const int tid = threadIdx.x;
    if (tid < 32)
    {
        double m = 0.0;
        for (int i = tid; i < T; i += 32)
            m = fmax(m, fabs(Ain[static_cast<size_t>(i) * T + i].x));
        for (int o = 16; o > 0; o >>= 1)
            m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (tid == 0)
            s_scale = jac_scale(m);
    }
    __syncthreads();
    // the sweeps run on 2^-e A (exact scaling): the squares of the entries stay finite in FP32
    const double scale = s_scale;
    for (int e = tid; e < T * T; e += JS_THREADS)
    {
        const int i = e / T, j = e % T;
        const double2 a = Ain[e];
        A[i * LD + j] = {static_cast<R>(a.x * scale), static_cast<R>(i == j ? 0.0 : a.y * scale)};
        if (warm)
        {
            const double2 v = Vout[e];
            N[i * LD + j] = {static_cast<R>(v.x), static_cast<R>(v.y)};
        }
        else
            V[i * LD + j] = {static_cast<R>(i == j ? 1 : 0), static_cast<R>(0)};
    }
    __syncthreads();
    if (warm)
    {
        // V = V0 (3 I - V0^H V0) / 2 (V0 in N), then A <- V^H A V
        smem_cgemm<R, JS_THREADS>(N, N, X, T, LD, true);
        __syncthreads();
        for (int e = tid; e < T * T; e += JS_THREADS)
        {
            const int i = e / T, j = e % T;
            const Cx<R> x = X[i * LD + j];
            X[i * LD + j] = {R(-0.5) * x.x + (i == j ? R(1.5) : R(0)), R(-0.5) * x.y};
        }
        __syncthreads();
        smem_cgemm<R, JS_THREADS>(N, X, V, T, LD, false);
        __syncthreads();
        smem_cgemm<R, JS_THREADS>(A, V, X, T, LD, false);
        __syncthreads();
        smem_cgemm<R, JS_THREADS>(V, X, N, T, LD, true);
        __syncthreads();
        for (int e = tid; e < T * T; e += JS_THREADS)
        {
            const int i = e / T, j = e % T;
            const Cx<R> a = N[i * LD + j], b = N[j * LD + i];
            A[i * LD + j] = {R(0.5) * (a.x + b.x), i == j ? R(0) : R(0.5) * (a.y - b.y)};
        }
        __syncthreads();
    }
    // FP32 sweeps: rotations below floor_rel of the matrix's Frobenius norm are not applied (5e-7:
    // the round-off level of the FP32 updates, below which they keep regenerating off-diagonal
    // entries of the small eigenvalues and the sweeps would run to their limit; 2e-5 when only the
    // kept eigenvectors are used, which are refined in FP64 afterwards).
    __shared__ double s_fro[JS_THREADS / 32];
    R floor = R(0);
    if constexpr (sizeof(R) == sizeof(float))
    {
        double f2 = 0.0;
        for (int e = tid; e < T * T; e += JS_THREADS)
        {
            const Cx<R> a = A[(e / T) * LD + e % T];
            f2 += static_cast<double>(a.x) * a.x + static_cast<double>(a.y) * a.y;
        }
        for (int o = 16; o > 0; o >>= 1)
            f2 += __shfl_xor_sync(0xffffffffu, f2, o);
        if ((tid & 31) == 0)
            s_fro[tid >> 5] = f2;
        __syncthreads();
        double t2 = 0.0;
        for (int w = 0; w < JS_THREADS / 32; ++w)
            t2 += s_fro[w];
        floor = static_cast<R>(static_cast<double>(floor_rel) * sqrt(t2));
    }
    smem_sweeps<R, JS_THREADS>(A, V, T, Tp, LD, sc, floor, JAC_MAX_SWEEPS);
    __syncthreads();
    for (int e = tid; e < T * T; e += JS_THREADS)
    {
        const int i = e / T, j = e % T;
        Vout[e] = make_double2(static_cast<double>(V[i * LD + j].x), static_cast<double>(V[i * LD + j].y));
    }
    for (int i = tid; i < T; i += JS_THREADS)
        evals[i] = static_cast<double>(A[i * LD + i].x) / scale;
}

// Grid-wide kernels (64 < T <= JC_MAX_T) synchronise through a bounded sense-reversal barrier: a
// wait that exceeds about 2 s sets the error flag and every later barrier returns at once, so the
// kernel ends.
constexpr int JC_MAX_T = 512;

// Loads of A and V in the grid kernel bypass L1 (other SMs wrote them before the last barrier).
__device__ __forceinline__ Cx<float> ldcg(const Cx<float>* p)
{
    const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
    return {v.x, v.y};
}

struct GridBarrier
{
    unsigned int count;
    unsigned int gen;
    int err;
};

__device__ __forceinline__ void grid_barrier(GridBarrier* b)
{
    __syncthreads();
    if (threadIdx.x == 0)
    {
        volatile unsigned int* vgen = &b->gen;
        volatile int* verr = &b->err;
        const unsigned int g = *vgen;
        __threadfence();
        if (atomicAdd(&b->count, 1u) == gridDim.x - 1)
        {
            b->count = 0;
            __threadfence();
            atomicAdd(&b->gen, 1u);
        }
        else
        {
            uint64_t t0 = 0;
            for (unsigned int i = 0; *vgen == g && !*verr; ++i)
            {
                if ((i & 1023u) == 1023u)
                {
                    uint64_t now;
                    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
                    if (t0 == 0)
                        t0 = now;
                    else if (now - t0 > 2000000000ull)
                        *verr = 1;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// Block-cyclic variant for 64 < T <= JC_MAX_T: the indices form blocks of 32 (T rounded up to 64
// with zero rows and columns, which no rotation ever touches), and a sweep pairs the blocks in the
// round-robin order. A step (one of nblk - 1 per sweep) has two grid phases:
//   1. each of the nblk / 2 block pairs (I, J) loads its 64 x 64 subproblem A[I u J][I u J] into
//      shared memory and applies one pass of 2 x 2 rotations to it (smem_sweeps over part of the
//      split ordering, see below), giving the pair's unitary U (64 x 64);
//   2. every CTA applies the step's unitaries to 64 x 64 blocks: A[P][Q] <- U_P^H A[P][Q] U_Q for
//      pair groups P <= Q (and the mirror), V[rows][P] <- V[rows][P] U_P, from one copy of A and V
//      into the other.
// The nblk - 1 round-robin steps rotate only the I x J pairs (32 inner steps each) and one more
// step pairs blocks (2k, 2k + 1) to rotate the pairs inside every block (31 inner steps), so a
// sweep visits every index pair once, like a scalar sweep, with nblk grid steps instead of T - 1. FP32, the same absolute floor as the scalar kernels; the sweeps end after one without a
// rotation. Bounded grid barriers as above.
constexpr int BJ_B = 32;                 // indices per block
constexpr int BJ_S = 2 * BJ_B;           // subproblem size
constexpr int BJ_LD = BJ_S + 1;          // shared-memory leading dimension
constexpr int BJ_THREADS = 512;
constexpr int BJ_MAX_SWEEPS = 40;
constexpr size_t BJ_SMEM = 3 * static_cast<size_t>(BJ_S) * BJ_LD * sizeof(float2);

__device__ __forceinline__ void bj_pair(int step, int k, int nblk, int& I, int& J)
{
    int a, b;
    if (k == 0)
    {
        a = nblk - 1;
        b = step % (nblk - 1);
    }
    else
    {
        a = (step + k) % (nblk - 1);
        b = (step - k + (nblk - 1)) % (nblk - 1);
    }
    I = a < b ? a : b;
    J = a < b ? b : a;
}

// Blocks of pair k in step `step` of a sweep: the round-robin pairs for the nblk - 1 cross steps,
// then one step pairing blocks (2k, 2k + 1) for the pairs inside each block.
__device__ __forceinline__ void bj_step_pair(int step, int k, int nblk, int& I, int& J)
{
    if (step < nblk - 1)
        bj_pair(step, k, nblk, I, J);
    else
    {
        I = 2 * k;
        J = 2 * k + 1;
    }
}

// index i < 64 of pair group (I, J): block I then block J
__device__ __forceinline__ int bj_index(int I, int J, int i) { return i < BJ_B ? I * BJ_B + i : J * BJ_B + i - BJ_B; }

// C = op(A) B for 64 x 64 shared-memory matrices (leading dimension BJ_LD), op(A) = A or A^H.
// Thread t computes rows BJ_RPT (t / 16) .. + BJ_RPT - 1 and columns t % 16 + 16 j (conflict-free B rows).
constexpr int BJ_RPT = BJ_S * BJ_S / (BJ_THREADS * 4);  // rows per thread
static_assert(BJ_RPT * 16 * (BJ_THREADS / 16) == BJ_S * BJ_S / 4 && BJ_RPT * (BJ_THREADS / 16) == BJ_S, "gemm map");
template <bool AH>
__device__ __forceinline__ void bj_gemm(const Cx<float>* A, const Cx<float>* B, Cx<float>* C)
{
    const int r0 = (threadIdx.x >> 4) * BJ_RPT, cb = threadIdx.x & 15;
    float2 acc[BJ_RPT][4];
#pragma unroll
    for (int i = 0; i < BJ_RPT; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
            acc[i][j] = make_float2(0.f, 0.f);
    for (int k = 0; k < BJ_S; ++k)
    {
        Cx<float> a[BJ_RPT], b[4];
#pragma unroll
        for (int i = 0; i < BJ_RPT; ++i)
        {
            if (AH)
            {
                const Cx<float> v = A[k * BJ_LD + r0 + i];
                a[i] = {v.x, -v.y};
            }
            else
                a[i] = A[(r0 + i) * BJ_LD + k];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            b[j] = B[k * BJ_LD + cb + 16 * j];
#pragma unroll
        for (int i = 0; i < BJ_RPT; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j)
            {
                acc[i][j].x = fmaf(a[i].x, b[j].x, fmaf(-a[i].y, b[j].y, acc[i][j].x));
                acc[i][j].y = fmaf(a[i].x, b[j].y, fmaf(a[i].y, b[j].x, acc[i][j].y));
            }
    }
#pragma unroll
    for (int i = 0; i < BJ_RPT; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
            C[(r0 + i) * BJ_LD + cb + 16 * j] = {acc[i][j].x, acc[i][j].y};
}

__global__ void __launch_bounds__(BJ_THREADS) k_jacobi_block(const double2* __restrict__ Ain, int T, int Tp,
                                                             Cx<float>* A0, Cx<float>* A1, Cx<float>* V0,
                                                             Cx<float>* V1, Cx<float>* U, int* flags,
                                                             double* fro2, GridBarrier* bar,
                                                             double2* __restrict__ Vout,
                                                             double* __restrict__ evals, double floor_rel)
{
    using R = float;
    extern __shared__ __align__(16) unsigned char bj_raw[];
    Cx<R>* sm0 = reinterpret_cast<Cx<R>*>(bj_raw);
    Cx<R>* sm1 = sm0 + BJ_S * BJ_LD;
    Cx<R>* sm2 = sm1 + BJ_S * BJ_LD;
    __shared__ JacScratch<R> sc;
    __shared__ R s_floor;
    __shared__ int s_rot;
    const int tid = threadIdx.x;
    const size_t gtid = static_cast<size_t>(blockIdx.x) * BJ_THREADS + tid;
    const size_t gsz = static_cast<size_t>(gridDim.x) * BJ_THREADS;
    const size_t TT = static_cast<size_t>(Tp) * Tp;
    const int nblk = Tp / BJ_B, npb = nblk / 2;
    // the sweeps run on 2^-e A (exact scaling, every CTA derives the same factor): FP32 squares of
    // the entries stay finite
    __shared__ double s_scale;
    if (tid < 32)
    {
        double m = 0.0;
        for (int i = tid; i < T; i += 32)
            m = fmax(m, fabs(Ain[static_cast<size_t>(i) * T + i].x));
        for (int o = 16; o > 0; o >>= 1)
            m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (tid == 0)
            s_scale = jac_scale(m);
    }
    __syncthreads();
    const double scale = s_scale;
    // the squared Frobenius norm is summed on the way (FP64, one atomic per CTA into fro2)
    __shared__ double s_fro[BJ_THREADS / 32];
    double fro = 0.0;
    for (size_t e = gtid; e < TT; e += gsz)
    {
        const int i = static_cast<int>(e / Tp), j = static_cast<int>(e % Tp);
        double2 a = (i < T && j < T) ? Ain[static_cast<size_t>(i) * T + j] : make_double2(0.0, 0.0);
        a.x *= scale;
        a.y *= scale;
        fro += a.x * a.x + (i == j ? 0.0 : a.y * a.y);
        A0[e] = {static_cast<R>(a.x), static_cast<R>(i == j ? 0.0 : a.y)};
        V0[e] = {static_cast<R>(i == j ? 1 : 0), static_cast<R>(0)};
    }
    for (int o = 16; o > 0; o >>= 1)
        fro += __shfl_down_sync(0xffffffffu, fro, o);
    if ((tid & 31) == 0)
        s_fro[tid >> 5] = fro;
    __syncthreads();
    if (tid == 0)
    {
        double t = 0.0;
        for (int w = 0; w < BJ_THREADS / 32; ++w)
            t += s_fro[w];
        atomicAdd(fro2, t);
    }
    grid_barrier(bar);
    // rotations below the FP32 round-off level of the matrix are not applied: 5e-7 of its Frobenius
    // norm. The FP32 block updates leave off-diagonal entries near that size, which would keep the
    // sweeps going; at this floor the eigenvectors of separated eigenvalues keep FP32 accuracy
    // (residual ~3e-6 of the largest eigenvalue at T = 512, the level of the sweeps' own round-off)
    if (tid == 0)
        s_floor = static_cast<R>(sqrt(*reinterpret_cast<volatile double*>(fro2)) * floor_rel);
    __syncthreads();
    Cx<R>*A = A0, *An = A1, *V = V0, *Vn = V1;
    const int na = npb * (npb + 1) / 2, nrow = Tp / BJ_S;
    for (int sweep = 0; sweep < BJ_MAX_SWEEPS; ++sweep)
    {
        // three rotating flags: sweep s sets flags[s % 3] and every CTA reads it after the sweep's last
        // barrier; the one zeroed here was last read before the previous sweep's barriers
        if (gtid == 0)
            flags[(sweep + 1) % 3] = 0;
        for (int step = 0; step < nblk; ++step)
        {
            // cross steps rotate the I x J pairs (first half of the split ordering), the last step
            // the pairs inside each block (second half): every pair once per sweep
            const bool diag_step = step == nblk - 1;
            // phase 1: one sweep on each pair's subproblem
            for (int k = blockIdx.x; k < npb; k += gridDim.x)
            {
                int I, J;
                bj_step_pair(step, k, nblk, I, J);
                for (int e = tid; e < BJ_S * BJ_S; e += BJ_THREADS)
                {
                    const int i = e / BJ_S, j = e % BJ_S;
                    sm0[i * BJ_LD + j] =
                        ldcg(A + static_cast<size_t>(bj_index(I, J, i)) * Tp + static_cast<size_t>(bj_index(I, J, j)));
                    sm1[i * BJ_LD + j] = {static_cast<R>(i == j ? 1 : 0), static_cast<R>(0)};
                }
                __syncthreads();
                const bool rot = smem_sweeps<R, BJ_THREADS, BJ_S>(sm0, sm1, BJ_S, BJ_S, BJ_LD, sc, s_floor, 1, true,
                                                                  diag_step ? BJ_B : 0, diag_step ? -1 : BJ_B);
                for (int e = tid; e < BJ_S * BJ_S; e += BJ_THREADS)
                {
                    const int i = e / BJ_S, j = e % BJ_S;
                    const Cx<R> u = sm1[i * BJ_LD + j];
                    reinterpret_cast<float2*>(U)[static_cast<size_t>(k) * BJ_S * BJ_S + e] = make_float2(u.x, u.y);
                }
                if (rot && tid == 0)
                    atomicExch(&flags[sweep % 3], 1);
                __syncthreads();
            }
            grid_barrier(bar);
            // phase 2: apply the unitaries of the step to A (pair groups P <= Q) and V (row chunks)
            for (int it = blockIdx.x; it < na + nrow * npb; it += gridDim.x)
            {
                const Cx<R>* Ug = U;
                if (it < na)
                {
                    int P = 0, rem = it;
                    while (rem >= npb - P)
                    {
                        rem -= npb - P;
                        ++P;
                    }
                    const int Q = P + rem;
                    int IP, JP, IQ, JQ;
                    bj_step_pair(step, P, nblk, IP, JP);
                    bj_step_pair(step, Q, nblk, IQ, JQ);
                    for (int e = tid; e < BJ_S * BJ_S; e += BJ_THREADS)
                    {
                        const int i = e / BJ_S, j = e % BJ_S;
                        sm0[i * BJ_LD + j] = ldcg(A + static_cast<size_t>(bj_index(IP, JP, i)) * Tp +
                                                  static_cast<size_t>(bj_index(IQ, JQ, j)));
                        sm1[i * BJ_LD + j] = ldcg(Ug + static_cast<size_t>(Q) * BJ_S * BJ_S + e);
                    }
                    __syncthreads();
                    bj_gemm<false>(sm0, sm1, sm2);  // X = A[P][Q] U_Q
                    __syncthreads();
                    if (P != Q)
                    {
                        for (int e = tid; e < BJ_S * BJ_S; e += BJ_THREADS)
                            sm1[(e / BJ_S) * BJ_LD + e % BJ_S] = ldcg(Ug + static_cast<size_t>(P) * BJ_S * BJ_S + e);
                        __syncthreads();
                    }
                    bj_gemm<true>(sm1, sm2, sm0);  // Y = U_P^H X
                    __syncthreads();
                    for (int e = tid; e < BJ_S * BJ_S; e += BJ_THREADS)
                    {
                        const int i = e / BJ_S, j = e % BJ_S;
                        const int gi = bj_index(IP, JP, i), gj = bj_index(IQ, JQ, j);
                        Cx<R> y = sm0[i * BJ_LD + j];
                        if (P == Q)
                        {
                            // exactly Hermitian diagonal group: average with the mirror element
                            const Cx<R> w = sm0[j * BJ_LD + i];
                            y = {R(0.5) * (y.x + w.x), i == j ? R(0) : R(0.5) * (y.y - w.y)};
                        }
                        An[static_cast<size_t>(gi) * Tp + gj] = y;
                        if (P != Q)
                            An[static_cast<size_t>(gj) * Tp + gi] = {y.x, -y.y};
                    }
                }
                else
                {
                    const int v = it - na, rc = v / npb, P = v % npb;
                    int IP, JP;
                    bj_step_pair(step, P, nblk, IP, JP);
                    for (int e = tid; e < BJ_S * BJ_S; e += BJ_THREADS)
                    {
                        const int i = e / BJ_S, j = e % BJ_S;
                        sm0[i * BJ_LD + j] =
                            ldcg(V + static_cast<size_t>(rc * BJ_S + i) * Tp + static_cast<size_t>(bj_index(IP, JP, j)));
                        sm1[i * BJ_LD + j] = ldcg(Ug + static_cast<size_t>(P) * BJ_S * BJ_S + e);
                    }
                    __syncthreads();
                    bj_gemm<false>(sm0, sm1, sm2);  // V[rows][P] U_P
                    __syncthreads();
                    for (int e = tid; e < BJ_S * BJ_S; e += BJ_THREADS)
                    {
                        const int i = e / BJ_S, j = e % BJ_S;
                        Vn[static_cast<size_t>(rc * BJ_S + i) * Tp + static_cast<size_t>(bj_index(IP, JP, j))] =
                            sm2[i * BJ_LD + j];
                    }
                }
                __syncthreads();
            }
            grid_barrier(bar);
            Cx<R>* t = A;
            A = An;
            An = t;
            t = V;
            V = Vn;
            Vn = t;
        }
        if (tid == 0)
            s_rot = *reinterpret_cast<volatile int*>(&flags[sweep % 3]);
        __syncthreads();
        if (!s_rot)
            break;  // the same value in every CTA: read after the sweep's last barrier
        if (reinterpret_cast<volatile int*>(&bar->err)[0])
            break;
    }
    for (size_t e = gtid; e < static_cast<size_t>(T) * T; e += gsz)
    {
        const int i = static_cast<int>(e / T), j = static_cast<int>(e % T);
        const Cx<R> v = ldcg(V + static_cast<size_t>(i) * Tp + j);
        Vout[e] = make_double2(static_cast<double>(v.x), static_cast<double>(v.y));
    }
    for (size_t i = gtid; i < static_cast<size_t>(T); i += gsz)
        evals[i] = static_cast<double>(ldcg(A + i * Tp + i).x) / scale;
}


// Finish of each eigenpair from the FP64 covariance (intact in the FP32-sweep paths): normalise
// the eigenvector column in FP64 and take its Rayleigh quotient v^H A v as the eigenvalue, whose
// error is second order in the eigenvector error. Acc = double: FP64 quotients; Acc = float: the
// quadratic form accumulated in FP32 (~1e-7 of the largest eigenvalue: enough to order the
// eigenvalues whose vectors are not refined afterwards, at a small fraction of the FP64 cost on
// this part). One CTA per eigenpair.
template <class Acc>
__global__ void k_eig_refine(const double2* __restrict__ A, double2* __restrict__ V, int T, double* __restrict__ evals)
{
    __shared__ double2 v[JC_MAX_T];
    __shared__ double red[4];
    __shared__ Acc redl[4];
    const int i = blockIdx.x, tid = threadIdx.x;
    double n2 = 0.0;
    for (int t = tid; t < T; t += blockDim.x)
    {
        const double2 x = V[t * T + i];
        v[t] = x;
        n2 += x.x * x.x + x.y * x.y;
    }
    for (int o = 16; o > 0; o >>= 1)
        n2 += __shfl_down_sync(0xffffffffu, n2, o);
    if ((tid & 31) == 0)
        red[tid >> 5] = n2;
    __syncthreads();
    const double inv = 1.0 / sqrt(red[0] + red[1] + red[2] + red[3]);
    __syncthreads();
    // v^H A v of the Hermitian A: sum_t a_tt |v_t|^2 + 2 Re sum_{t<s} conj(v_t) a_ts v_s (upper
    // triangle only: half the FP64 multiply-adds of the full product)
    Acc lam = 0;
    for (int t = tid; t < T; t += blockDim.x)
    {
        Acc ax = 0, ay = 0;
        for (int s2 = t + 1; s2 < T; ++s2)
        {
            const double2 a = A[t * T + s2], x = v[s2];
            const Acc arx = static_cast<Acc>(a.x), ary = static_cast<Acc>(a.y);
            const Acc xx = static_cast<Acc>(x.x), xy = static_cast<Acc>(x.y);
            ax += arx * xx - ary * xy;
            ay += arx * xy + ary * xx;
        }
        const double2 x = v[t];
        const Acc xx = static_cast<Acc>(x.x), xy = static_cast<Acc>(x.y);
        lam += (Acc(2) * (xx * ax + xy * ay) + static_cast<Acc>(A[t * T + t].x) * (xx * xx + xy * xy)) *
               static_cast<Acc>(inv * inv);
        V[t * T + i] = make_double2(x.x * inv, x.y * inv);
    }
    for (int o = 16; o > 0; o >>= 1)
        lam += __shfl_down_sync(0xffffffffu, lam, o);
    if ((tid & 31) == 0)
        redl[tid >> 5] = lam;
    __syncthreads();
    if (tid == 0)
        evals[i] = static_cast<double>(redl[0]) + redl[1] + redl[2] + redl[3];
}

// Sort eigenpairs ascending (rank = number of smaller values, ties by index), write the
// eigenvectors column-major like cusolverDnCheevd (evec[t + j*T]) and the PCA weights.
// One CTA per eigenpair: the rank is counted once, the column is copied by all threads.
__global__ void k_eig_sort(const double* evals_in, const double2* V, int T, double* evals, double2* evecs, int pmin,
                           int pmax, float2* weights)
{
    __shared__ int s_rank;
    const int i = blockIdx.x;
    const double ei = evals_in[i];
    if (threadIdx.x < 32)
    {
        int rank = 0;
        for (int j = threadIdx.x; j < T; j += 32)
        {
            const double ej = evals_in[j];
            rank += (ej < ei) || (ej == ei && j < i);
        }
        for (int o = 16; o > 0; o >>= 1)
            rank += __shfl_down_sync(0xffffffffu, rank, o);
        if (threadIdx.x == 0)
        {
            s_rank = rank;
            evals[rank] = ei;
        }
    }
    __syncthreads();
    const int rank = s_rank;
    for (int t = threadIdx.x; t < T; t += blockDim.x)
    {
        const double2 v = V[t * T + i];  // column i of V (row-major)
        evecs[static_cast<size_t>(rank) * T + t] = v;
        if (weights && rank >= pmin && rank <= pmax)
            weights[static_cast<size_t>(rank - pmin) * T + t] =
                make_float2(static_cast<float>(v.x), static_cast<float>(v.y));
    }
}

// ------------------------------------------------------------------ FP64 eigenvector refinement
// The FP32 sweeps leave each eigenvector with an error of the FP32 round-off of the matrix over
// the eigenvalue gap: when the gap is small against the largest eigenvalue (a dominant mean
// component, or close pairs of temporal modes), the kept components mix with their neighbours by
// up to 1e-3. The kept eigenvectors (ranks r0 .. r0 + K - 1, after the sort) are corrected in FP64
// against the FP64 covariance C with the first-order residual correction
//     lambda_j = v_j^H C v_j / v_j^H v_j,  r_j = C v_j - lambda_j v_j,
//     v_j <- v_j + sum_{i != j} v_i (v_i^H r_j) / (lambda_j - lambda_i),
// then normalised: an error of angle theta towards another eigenvector becomes O(theta^3) (and
// O(theta^2) against the FP32 error of the basis). Pairs closer than 1e-12 of the largest
// eigenvalue are numerically degenerate and left as they are. Kernels: y_j = C v_j (one warp per
// row), D = V^H Y and G = V^H V_kept (one warp per entry), the update (one thread per row), the
// normalisation (one CTA per kept vector).
constexpr int ER_MAX_K = 64;  // kept eigenvectors refined at most (wider ranges keep the FP32 vectors)

__device__ __forceinline__ double2 cfma_conj(double2 a, double2 b, double2 acc)
{
    // acc + conj(a) b
    acc.x += a.x * b.x + a.y * b.y;
    acc.y += a.x * b.y - a.y * b.x;
    return acc;
}

__device__ __forceinline__ double2 warp_sum2(double2 v)
{
    for (int o = 16; o > 0; o >>= 1)
    {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// Y[j][t] = sum_s C[t][s] v_{r0+j}[s]; grid (ceil(T / 8), K), 256 threads
__global__ void k_eigref_matvec(const double2* __restrict__ C, const double2* __restrict__ evecs, int T, int r0,
                                double2* __restrict__ Y)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * 8 + warp, j = blockIdx.y;
    if (t >= T)
        return;
    const double2* v = evecs + static_cast<size_t>(r0 + j) * T;
    const double2* c = C + static_cast<size_t>(t) * T;
    double2 acc = make_double2(0.0, 0.0);
    for (int s2 = lane; s2 < T; s2 += 32)
    {
        const double2 a = c[s2], x = v[s2];
        acc.x += a.x * x.x - a.y * x.y;
        acc.y += a.x * x.y + a.y * x.x;
    }
    acc = warp_sum2(acc);
    if (lane == 0)
        Y[static_cast<size_t>(j) * T + t] = acc;
}

// D[j][i] = v_i^H Y[j], G[j][i] = v_i^H v_{r0+j} for the basis vectors i = b0 .. T-1; grid (T - b0, K),
// 64 threads (FP64 throughput is a few operations per clock per SM on this part: one basis vector
// per CTA spreads the products over the SMs); the two warps' sums are added in warp order
constexpr int ER_PROJ_THREADS = 64;
__global__ void __launch_bounds__(ER_PROJ_THREADS) k_eigref_project(const double2* __restrict__ evecs,
                                                                   const double2* __restrict__ Y, int T, int r0,
                                                                   int b0, double2* __restrict__ D,
                                                                   double2* __restrict__ G)
{
    __shared__ double2 sd[ER_PROJ_THREADS / 32], sg[ER_PROJ_THREADS / 32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = b0 + blockIdx.x, j = blockIdx.y;
    const double2* vi = evecs + static_cast<size_t>(i) * T;
    const double2* vj = evecs + static_cast<size_t>(r0 + j) * T;
    const double2* y = Y + static_cast<size_t>(j) * T;
    double2 d = make_double2(0.0, 0.0), g = make_double2(0.0, 0.0);
    for (int t = threadIdx.x; t < T; t += ER_PROJ_THREADS)
    {
        const double2 a = vi[t];
        d = cfma_conj(a, y[t], d);
        g = cfma_conj(a, vj[t], g);
    }
    d = warp_sum2(d);
    g = warp_sum2(g);
    if (lane == 0)
    {
        sd[warp] = d;
        sg[warp] = g;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        for (int w = 1; w < ER_PROJ_THREADS / 32; ++w)
        {
            d.x += sd[w].x;
            d.y += sd[w].y;
            g.x += sg[w].x;
            g.y += sg[w].y;
        }
        D[static_cast<size_t>(j) * T + i] = d;
        G[static_cast<size_t>(j) * T + i] = g;
    }
}

// Rayleigh quotient of kept vector k (0-based in the kept range)
__device__ __forceinline__ double eigref_lambda(const double2* D, const double2* G, int T, int r0, int k)
{
    const size_t e = static_cast<size_t>(k) * T + r0 + k;
    return D[e].x / G[e].x;
}

// Vn[j][t] = v_j[t] + sum_{i != j} v_i[t] (D[j][i] - lambda_j G[j][i]) / (lambda_j - lambda_i), over
// the basis i = b0 .. T-1. With a partial basis (b0 > 0: the Ritz vectors of the largest
// eigenvalues) the part of the residual r = C v_j - lambda_j v_j outside the basis is added divided
// by lambda_j (the eigenvalues outside are the smaller ones; the factor lambda_i / lambda_j it
// neglects shrinks with each correction). grid (ceil(T / 32), K), ER_UPD_WARPS warps: lane = row t
// of the CTA's 32 rows (coalesced loads of v_i[t]), warp w sums the basis vectors i = b0 + w,
// b0 + w + ER_UPD_WARPS, ..., and the warps' sums are added in warp order. The coefficients of kept
// vector j are computed once per CTA into shared memory (FP64 divisions are slow on this part).
constexpr int ER_UPD_WARPS = 4;
__global__ void __launch_bounds__(32 * ER_UPD_WARPS) k_eigref_update(const double2* __restrict__ evecs,
                                                                    const double* __restrict__ evals,
                                                                    const double2* __restrict__ D,
                                                                    const double2* __restrict__ G,
                                                                    const double2* __restrict__ Y, int T, int r0,
                                                                    int K, int b0, double2* __restrict__ Vn)
{
    __shared__ double2 coef[JC_MAX_T];
    __shared__ double2 comp[JC_MAX_T];
    __shared__ double2 pacc[ER_UPD_WARPS][32], pproj[ER_UPD_WARPS][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * 32 + lane, j = blockIdx.y;
    const int rj = r0 + j;
    const double lj = eigref_lambda(D, G, T, r0, j);
    // pairs closer than 1e-12 of the largest eigenvalue (the last in ascending order) stay mixed
    const double degenerate = 1e-12 * fabs(evals[T - 1]);
    const double2* Dj = D + static_cast<size_t>(j) * T;
    const double2* Gj = G + static_cast<size_t>(j) * T;
    for (int i = b0 + threadIdx.x; i < T; i += blockDim.x)
    {
        const double li = (i >= r0 && i < r0 + K) ? eigref_lambda(D, G, T, r0, i - r0) : evals[i];
        const double gap = lj - li;
        const double2 d = Dj[i], g = Gj[i];
        const double2 cr = make_double2(d.x - lj * g.x, d.y - lj * g.y);  // component of r along v_i
        double2 c = make_double2(0.0, 0.0);
        if (i != rj && fabs(gap) > degenerate)
        {
            const double inv = 1.0 / gap;
            c = make_double2(cr.x * inv, cr.y * inv);
        }
        coef[i] = c;
        comp[i] = cr;
    }
    __syncthreads();
    double2 acc = make_double2(0.0, 0.0), proj = make_double2(0.0, 0.0);
    if (t < T)
        for (int i = b0 + warp; i < T; i += ER_UPD_WARPS)
        {
            const double2 c = coef[i];
            const double2 v = evecs[static_cast<size_t>(i) * T + t];
            acc.x += v.x * c.x - v.y * c.y;
            acc.y += v.x * c.y + v.y * c.x;
            if (b0 > 0)
            {
                const double2 cr = comp[i];
                proj.x += v.x * cr.x - v.y * cr.y;
                proj.y += v.x * cr.y + v.y * cr.x;
            }
        }
    pacc[warp][lane] = acc;
    pproj[warp][lane] = proj;
    __syncthreads();
    if (warp != 0 || t >= T)
        return;
    const double2 vj = evecs[static_cast<size_t>(rj) * T + t];
    acc = vj;
    proj = make_double2(0.0, 0.0);
    for (int w = 0; w < ER_UPD_WARPS; ++w)
    {
        acc.x += pacc[w][lane].x;
        acc.y += pacc[w][lane].y;
        proj.x += pproj[w][lane].x;
        proj.y += pproj[w][lane].y;
    }
    if (b0 > 0)
    {
        const double2 y = Y[static_cast<size_t>(j) * T + t];
        const double inv = 1.0 / lj;
        acc.x += (y.x - lj * vj.x - proj.x) * inv;
        acc.y += (y.y - lj * vj.y - proj.y) * inv;
    }
    Vn[static_cast<size_t>(j) * T + t] = acc;
}

// Normalise the corrected vectors into evecs (column r0 + j), their eigenvalues (the Rayleigh
// quotients of the vectors before the correction, second order in their error) and, for ranks
// pmin..pmax, the complex64 PCA weights. One CTA (128 threads) per kept vector.
__global__ void k_eigref_finish(double2* __restrict__ evecs, double* __restrict__ evals, const double2* __restrict__ Vn,
                                const double2* __restrict__ D, const double2* __restrict__ G, int T, int r0, int pmin,
                                int pmax, float2* __restrict__ weights)
{
    __shared__ double red[4];
    const int j = blockIdx.x, tid = threadIdx.x, rj = r0 + j;
    const double2* v = Vn + static_cast<size_t>(j) * T;
    double n2 = 0.0;
    for (int t = tid; t < T; t += blockDim.x)
        n2 += v[t].x * v[t].x + v[t].y * v[t].y;
    for (int o = 16; o > 0; o >>= 1)
        n2 += __shfl_xor_sync(0xffffffffu, n2, o);
    if ((tid & 31) == 0)
        red[tid >> 5] = n2;
    __syncthreads();
    const double inv = 1.0 / sqrt(red[0] + red[1] + red[2] + red[3]);
    for (int t = tid; t < T; t += blockDim.x)
    {
        const double2 x = make_double2(v[t].x * inv, v[t].y * inv);
        evecs[static_cast<size_t>(rj) * T + t] = x;
        if (weights && rj >= pmin && rj <= pmax)
            weights[static_cast<size_t>(rj - pmin) * T + t] = make_float2(static_cast<float>(x.x), static_cast<float>(x.y));
    }
    if (tid == 0)
        evals[rj] = eigref_lambda(D, G, T, r0, j);
}

// ------------------------------------------------------------------ top eigenpairs by subspace iteration
// When only the largest eigenpairs are used (PCA views of the dominant components, ranks T - 16 ..
// T - 1 at most) and T > 64, the block Jacobi's full diagonalisation (~1 ms per sweep at T = 512,
// 5 or more sweeps) is replaced by a block subspace iteration on TS_P = 32 vectors in FP32: Y = C V
// (all CTAs), V = orth(Y) (classical Gram-Schmidt with a second pass where needed, one CTA),
// repeated; then Rayleigh-Ritz (H = V^H C V, Jacobi on the 32 x 32 H in one CTA) gives the Ritz
// pairs, and the kept vectors are corrected in FP64 against the FP64 covariance with the Ritz
// vectors as the basis. The error towards an eigenvector outside the subspace falls by
// lambda_33 / lambda_m per iteration (m: the smallest kept rank from the top). The Ritz vectors of
// the previous window are the warm start (TS_ITERS_WARM iterations; TS_ITERS_COLD from the columns
// of C).
constexpr int TS_P = 32;          // subspace size
constexpr int TS_MAX_KEEP = 16;   // top ranks served (the other 16 vectors are the guard)
constexpr int TS_LD = TS_P + 1;   // shared-memory row pitch (float2) of the Rayleigh-Ritz matrices
constexpr int TS_ORTH_THREADS = 256;
constexpr int TS_ORTH_RPT = 2;    // rows per thread of the orthonormalisation (T <= 512)
constexpr int TS_MM_ROWS = 1;     // rows of C V per CTA
constexpr int TS_MM_SPLIT = 16;   // warps per row (warp q sums the terms s = q mod 16)
constexpr int TS_ITERS_COLD = 8, TS_ITERS_WARM = 1;
static_assert(TS_P == 32, "one lane per subspace vector");
static_assert(TS_ORTH_THREADS * TS_ORTH_RPT >= JC_MAX_T, "the orthonormalisation holds every row in registers");

// C32 (T x T), V, Y, Vw (T x TS_P each), then H and Q (TS_P x TS_P each) and the scale factor
static size_t ts_bytes(int T)
{
    return static_cast<size_t>(T) * T * sizeof(float2) + 3 * static_cast<size_t>(T) * TS_P * sizeof(float2) +
           2 * static_cast<size_t>(TS_P) * TS_P * sizeof(float2) + 512;
}

// C32 = 2^-e C (largest diagonal entry near 1); every CTA derives the factor from the diagonal, CTA
// 0 also stores it
__global__ void k_ts_convert(const double2* __restrict__ C, int T, float2* __restrict__ C32, double* __restrict__ scale)
{
    __shared__ double s_scale;
    if (threadIdx.x < 32)
    {
        double m = 0.0;
        for (int i = threadIdx.x; i < T; i += 32)
            m = fmax(m, fabs(C[static_cast<size_t>(i) * T + i].x));
        for (int o = 16; o > 0; o >>= 1)
            m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0)
        {
            s_scale = jac_scale(m);
            if (blockIdx.x == 0)
                *scale = s_scale;
        }
    }
    __syncthreads();
    const double sc = s_scale;
    const size_t n = static_cast<size_t>(T) * T;
    for (size_t e = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        const double2 a = C[e];
        C32[e] = make_float2(static_cast<float>(a.x * sc), static_cast<float>(a.y * sc));
    }
}

// cold start: Y[t][k] = C32[t][k T / TS_P] (columns of C span its dominant eigenvectors)
__global__ void k_ts_init(const float2* __restrict__ C32, int T, float2* __restrict__ Y)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= T * TS_P)
        return;
    const int t = e / TS_P, k = e % TS_P;
    Y[e] = C32[static_cast<size_t>(t) * T + (k * T) / TS_P];
}

// Y[t][k] = sum_s C32[t][s] V[s][k]. Warp (row t, part q) of a CTA sums the terms s = q,
// q + TS_MM_SPLIT, ... for the TS_P columns (lane k) in two interleaved chains; the parts are added
// in part order.
__global__ void __launch_bounds__(TS_MM_ROWS * TS_MM_SPLIT * 32)
    k_ts_matmul(const float2* __restrict__ C32, const float2* __restrict__ V, int T, float2* __restrict__ Y)
{
    __shared__ float2 part[TS_MM_ROWS * TS_MM_SPLIT][TS_P];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * TS_MM_ROWS + warp / TS_MM_SPLIT, q = warp % TS_MM_SPLIT;
    float re0 = 0.f, im0 = 0.f, re1 = 0.f, im1 = 0.f;
    if (t < T)
    {
        const float2* c = C32 + static_cast<size_t>(t) * T;
        int s2 = q;
#pragma unroll 4
        for (; s2 + TS_MM_SPLIT < T; s2 += 2 * TS_MM_SPLIT)
        {
            const float2 a0 = c[s2], v0 = V[static_cast<size_t>(s2) * TS_P + lane];
            const float2 a1 = c[s2 + TS_MM_SPLIT], v1 = V[static_cast<size_t>(s2 + TS_MM_SPLIT) * TS_P + lane];
            re0 = fmaf(a0.x, v0.x, fmaf(-a0.y, v0.y, re0));
            im0 = fmaf(a0.x, v0.y, fmaf(a0.y, v0.x, im0));
            re1 = fmaf(a1.x, v1.x, fmaf(-a1.y, v1.y, re1));
            im1 = fmaf(a1.x, v1.y, fmaf(a1.y, v1.x, im1));
        }
        if (s2 < T)
        {
            const float2 a0 = c[s2], v0 = V[static_cast<size_t>(s2) * TS_P + lane];
            re0 = fmaf(a0.x, v0.x, fmaf(-a0.y, v0.y, re0));
            im0 = fmaf(a0.x, v0.y, fmaf(a0.y, v0.x, im0));
        }
    }
    part[warp][lane] = make_float2(re0 + re1, im0 + im1);
    __syncthreads();
    if (q == 0 && t < T)
    {
        float2 y = part[warp][lane];
        for (int j = 1; j < TS_MM_SPLIT; ++j)
        {
            y.x += part[warp + j][lane].x;
            y.y += part[warp + j][lane].y;
        }
        Y[static_cast<size_t>(t) * TS_P + lane] = y;
    }
}

// Slot j's contribution of this thread's rows to the column sums of the orthonormalisation: slot 0
// holds |y_0|^2 (the column being processed), slot j > 0 the product y_j^H y_0.
__device__ __forceinline__ float2 ts_slot(const float2 (&y)[TS_ORTH_RPT][TS_P], int j)
{
    float re = 0.f, im = 0.f;
#pragma unroll
    for (int r = 0; r < TS_ORTH_RPT; ++r)
    {
        const float2 a = y[r][j], b = y[r][0];
        if (j == 0)
            re = fmaf(b.x, b.x, fmaf(b.y, b.y, re));
        else
        {
            re = fmaf(a.x, b.x, fmaf(a.y, b.y, re));
            im = fmaf(a.x, b.y, fmaf(-a.y, b.x, im));
        }
    }
    return make_float2(re, im);
}

// Sums of the 32 slots over the CTA: a reduce-scatter across each warp (lane l ends with the warp's
// sum of slot l), then a fixed-order sum over the warps in shared memory. Every warp returns the
// same totals (slot `lane` in its lane). `red` alternates between two buffers, so one barrier per
// reduction suffices.
__device__ __forceinline__ float2 ts_reduce_slots(const float2 (&y)[TS_ORTH_RPT][TS_P],
                                                  float2 (*red)[TS_ORTH_THREADS / 32][TS_P], int& buf)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float2 p[TS_P / 2];
    {
        const bool up = lane & 16;
#pragma unroll
        for (int j = 0; j < TS_P / 2; ++j)
        {
            const float2 a = ts_slot(y, j), b = ts_slot(y, j + TS_P / 2);
            const float2 send = up ? a : b, keep = up ? b : a;
            p[j] = make_float2(keep.x + __shfl_xor_sync(0xffffffffu, send.x, 16),
                               keep.y + __shfl_xor_sync(0xffffffffu, send.y, 16));
        }
    }
#pragma unroll
    for (int w = 8; w >= 1; w >>= 1)
    {
        const bool up = lane & w;
#pragma unroll
        for (int j = 0; j < w; ++j)
        {
            const float2 a = p[j], b = p[j + w];
            const float2 send = up ? a : b, keep = up ? b : a;
            p[j] = make_float2(keep.x + __shfl_xor_sync(0xffffffffu, send.x, w),
                               keep.y + __shfl_xor_sync(0xffffffffu, send.y, w));
        }
    }
    red[buf][warp][lane] = p[0];
    __syncthreads();
    float2 s2 = red[buf][0][lane];
#pragma unroll
    for (int w = 1; w < TS_ORTH_THREADS / 32; ++w)
    {
        s2.x += red[buf][w][lane].x;
        s2.y += red[buf][w][lane].y;
    }
    buf ^= 1;
    return s2;
}

// One Gram-Schmidt pass on register slot 0 against the processed columns (slots >= first), with
// the totals `s2` of ts_reduce_slots: y_0 -= sum_j (y_j^H y_0) y_j. Returns |y_0|^2 before the pass
// minus the removed squared norm.
__device__ __forceinline__ float ts_project(float2 (&y)[TS_ORTH_RPT][TS_P], float2 s2, int first)
{
    const float nn = __shfl_sync(0xffffffffu, s2.x, 0);
    float cc = 0.f;
#pragma unroll
    for (int j = 1; j < TS_P; ++j)
    {
        float cr = __shfl_sync(0xffffffffu, s2.x, j), ci = __shfl_sync(0xffffffffu, s2.y, j);
        if (j < first)
            cr = ci = 0.f;
        cc = fmaf(cr, cr, fmaf(ci, ci, cc));
#pragma unroll
        for (int r = 0; r < TS_ORTH_RPT; ++r)
        {
            const float2 v = y[r][j];
            y[r][0].x -= v.x * cr - v.y * ci;
            y[r][0].y -= v.x * ci + v.y * cr;
        }
    }
    return nn - cc;
}

// V = orth(Y), T x TS_P row-major (T <= TS_ORTH_THREADS * TS_ORTH_RPT): classical Gram-Schmidt from
// the last column (the largest Ritz value of the warm start) to the first, with a second pass when
// the first removed more than half of the column's squared norm ("twice is enough", Giraud et al.
// 2005). Thread i owns rows i + TS_ORTH_THREADS r in registers; the column being processed is
// always register slot 0 and the slots rotate by one after every column, so that registers are
// indexed by constants only. A column left without norm (Y of rank < TS_P) becomes the unit vector
// e_k, made orthogonal at the next iteration.
__global__ void __launch_bounds__(TS_ORTH_THREADS) k_ts_orth(const float2* __restrict__ Y, int T, float2* __restrict__ V,
                                                              const int* __restrict__ only_if = nullptr)
{
    if (only_if && *only_if == 0)  // the Cholesky-QR of the warm iteration succeeded
        return;
    __shared__ float2 red[2][TS_ORTH_THREADS / 32][TS_P];
    __shared__ float red1[2][TS_ORTH_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float2 y[TS_ORTH_RPT][TS_P];  // slot j: column TS_P - 1 - j (before the first and after the last rotation)
#pragma unroll
    for (int r = 0; r < TS_ORTH_RPT; ++r)
    {
        const int t = tid + r * TS_ORTH_THREADS;
#pragma unroll
        for (int j = 0; j < TS_P; ++j)
            y[r][j] = t < T ? Y[static_cast<size_t>(t) * TS_P + (TS_P - 1 - j)] : make_float2(0.f, 0.f);
    }
    int buf = 0, buf1 = 0;
#pragma unroll 1
    for (int k = 0; k < TS_P; ++k)
    {
        const int first = TS_P - k;  // the processed columns sit in slots first .. TS_P - 1
        const float2 s1 = ts_reduce_slots(y, red, buf);
        const float nn = __shfl_sync(0xffffffffu, s1.x, 0);
        float n2 = ts_project(y, s1, first);
        // the same totals in every warp: the branch is uniform over the CTA
        if (k > 0 && !(n2 >= 0.5f * nn))
        {
            ts_project(y, ts_reduce_slots(y, red, buf), first);
            float m = 0.f;
#pragma unroll
            for (int r = 0; r < TS_ORTH_RPT; ++r)
                m = fmaf(y[r][0].x, y[r][0].x, fmaf(y[r][0].y, y[r][0].y, m));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                m += __shfl_xor_sync(0xffffffffu, m, o);
            if (lane == 0)
                red1[buf1][warp] = m;
            __syncthreads();
            n2 = red1[buf1][0];
#pragma unroll
            for (int w = 1; w < TS_ORTH_THREADS / 32; ++w)
                n2 += red1[buf1][w];
            buf1 ^= 1;
        }
        const bool dead = !(n2 > 0.f) || !isfinite(n2);
        const float inv = dead ? 0.f : rsqrtf(n2);
        const int col = TS_P - 1 - k;
#pragma unroll
        for (int r = 0; r < TS_ORTH_RPT; ++r)
        {
            const int t = tid + r * TS_ORTH_THREADS;
            y[r][0] = dead ? make_float2(t == col ? 1.f : 0.f, 0.f) : make_float2(y[r][0].x * inv, y[r][0].y * inv);
            const float2 done = y[r][0];
#pragma unroll
            for (int j = 0; j < TS_P - 1; ++j)
                y[r][j] = y[r][j + 1];
            y[r][TS_P - 1] = done;
        }
    }
#pragma unroll
    for (int r = 0; r < TS_ORTH_RPT; ++r)
    {
        const int t = tid + r * TS_ORTH_THREADS;
        if (t < T)
        {
#pragma unroll
            for (int j = 0; j < TS_P; ++j)
                V[static_cast<size_t>(t) * TS_P + (TS_P - 1 - j)] = y[r][j];
        }
    }
}

// The warm iteration's V = orth(Y) as a Cholesky-QR: with G = Y^H Y (k_ts_gram) and D = diag(G)^-1/2,
// G' = D G D = L L^H and V = Y D L^-H (V^H V = L^-1 G' L^-H = I); k_ts_ritz applies M = D L^-H.
// The Cholesky runs from the last column down (the largest Ritz value of the warm start, as in
// k_ts_orth), so V's last column is Y's last column normalised and column j spans the columns
// j .. TS_P - 1 of Y. The warm start's C V has near-orthogonal columns (the previous window's Ritz
// vectors times a covariance that changed by one stride), so G' is near the identity and the FP32
// factorisation is well conditioned. A pivot below 1e-6 (Y of rank < TS_P, or columns too close to
// dependent) sets *fail and k_ts_orth recomputes V by Gram-Schmidt. One warp.
__global__ void __launch_bounds__(32) k_ts_cholqr(const float2* __restrict__ G, float2* __restrict__ M,
                                                  int* __restrict__ fail)
{
    __shared__ float2 L[TS_P][TS_P + 1];  // index a = TS_P - 1 - (column of Y); lower triangle = L
    __shared__ float2 X[TS_P][TS_P + 1];  // L^-1
    __shared__ float d[TS_P];
    const int lane = threadIdx.x;
    {
        const float g = G[(TS_P - 1 - lane) * TS_P + (TS_P - 1 - lane)].x;
        d[lane] = (g > 0.f && isfinite(g)) ? rsqrtf(g) : 0.f;
    }
    __syncwarp();
    for (int a = 0; a < TS_P; ++a)
    {
        const float2 v = G[(TS_P - 1 - a) * TS_P + (TS_P - 1 - lane)];
        const float sc = d[a] * d[lane];
        L[a][lane] = make_float2(v.x * sc, v.y * sc);
    }
    __syncwarp();
    bool ok = true;
    for (int j = 0; j < TS_P; ++j)
    {
        // every lane forms the same pivot from the same (broadcast) values
        float p = L[j][j].x;
        for (int k = 0; k < j; ++k)
        {
            const float2 l = L[j][k];
            p -= l.x * l.x + l.y * l.y;
        }
        ok = ok && p > 1e-6f && isfinite(p);
        const float ljj = sqrtf(fmaxf(p, 1e-6f));
        __syncwarp();
        if (lane > j)
        {
            float2 a = L[lane][j];
            for (int k = 0; k < j; ++k)
            {
                const float2 li = L[lane][k], lj = L[j][k];  // a -= li conj(lj)
                a.x -= li.x * lj.x + li.y * lj.y;
                a.y -= li.y * lj.x - li.x * lj.y;
            }
            L[lane][j] = make_float2(a.x / ljj, a.y / ljj);
        }
        if (lane == 0)
            L[j][j] = make_float2(ljj, 0.f);
        __syncwarp();
    }
    // X = L^-1 by forward substitution, lane = column
    for (int i = 0; i < TS_P; ++i)
    {
        float2 a = make_float2(i == lane ? 1.f : 0.f, 0.f);
        for (int k = 0; k < i; ++k)
        {
            const float2 l = L[i][k], x = X[k][lane];
            a.x -= l.x * x.x - l.y * x.y;
            a.y -= l.x * x.y + l.y * x.x;
        }
        const float inv = 1.f / L[i][i].x;
        X[i][lane] = make_float2(a.x * inv, a.y * inv);
    }
    __syncwarp();
    // M[k][r] (Y column k into V column r) = d_k conj(X[b][a]) with a = TS_P-1-k, b = TS_P-1-r, a <= b
    for (int k = 0; k < TS_P; ++k)
    {
        const int a = TS_P - 1 - k, b = TS_P - 1 - lane;
        const float2 x = X[b][a];
        M[k * TS_P + lane] = a <= b ? make_float2(d[a] * x.x, -d[a] * x.y) : make_float2(0.f, 0.f);
    }
    if (lane == 0)
        *fail = ok ? 0 : 1;
}

// Rayleigh-Ritz in three launches. k_ts_gram: H = V^H Y (Y = C32 V), one CTA per row i of H, warp w
// summing the rows t = w mod 8 in two chains, the warps added in warp order.
constexpr int TS_GRAM_WARPS = 8;
__global__ void __launch_bounds__(TS_GRAM_WARPS * 32) k_ts_gram(const float2* __restrict__ V,
                                                               const float2* __restrict__ Y, int T,
                                                               float2* __restrict__ H)
{
    __shared__ float2 part[TS_GRAM_WARPS][TS_P];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, i = blockIdx.x;
    float r0 = 0.f, i0 = 0.f, r1 = 0.f, i1 = 0.f;
    int t = warp;
#pragma unroll 4
    for (; t + TS_GRAM_WARPS < T; t += 2 * TS_GRAM_WARPS)
    {
        const float2 a0 = V[static_cast<size_t>(t) * TS_P + i], b0 = Y[static_cast<size_t>(t) * TS_P + lane];
        const float2 a1 = V[static_cast<size_t>(t + TS_GRAM_WARPS) * TS_P + i];
        const float2 b1 = Y[static_cast<size_t>(t + TS_GRAM_WARPS) * TS_P + lane];
        r0 = fmaf(a0.x, b0.x, fmaf(a0.y, b0.y, r0));
        i0 = fmaf(a0.x, b0.y, fmaf(-a0.y, b0.x, i0));
        r1 = fmaf(a1.x, b1.x, fmaf(a1.y, b1.y, r1));
        i1 = fmaf(a1.x, b1.y, fmaf(-a1.y, b1.x, i1));
    }
    if (t < T)
    {
        const float2 a0 = V[static_cast<size_t>(t) * TS_P + i], b0 = Y[static_cast<size_t>(t) * TS_P + lane];
        r0 = fmaf(a0.x, b0.x, fmaf(a0.y, b0.y, r0));
        i0 = fmaf(a0.x, b0.y, fmaf(-a0.y, b0.x, i0));
    }
    part[warp][lane] = make_float2(r0 + r1, i0 + i1);
    __syncthreads();
    if (warp == 0)
    {
        float2 h = part[0][lane];
        for (int w = 1; w < TS_GRAM_WARPS; ++w)
        {
            h.x += part[w][lane].x;
            h.y += part[w][lane].y;
        }
        H[i * TS_P + lane] = h;
    }
}

// k_ts_rr: H Q = Q diag(theta) by FP32 Jacobi on the Hermitian part of H (one CTA); the Ritz values
// (scaled back) into evals[T - TS_P ..] in ascending order, evals below set to 0, and Qo = the columns
// of Q in that order.
__global__ void __launch_bounds__(JS_THREADS) k_ts_rr(const float2* __restrict__ H, int T,
                                                     const double* __restrict__ scale, double* __restrict__ evals,
                                                     float2* __restrict__ Qo)
{
    constexpr int NW = JS_THREADS / 32;
    __shared__ Cx<float> Hs[TS_P * TS_LD], Qs[TS_P * TS_LD];
    __shared__ JacScratch<float> sc;
    __shared__ int order[TS_P];
    __shared__ float s_fro[NW];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // Hermitian part, real diagonal; round-off floor as in the other FP32 sweeps
    float f2 = 0.f;
    for (int e = tid; e < TS_P * TS_P; e += JS_THREADS)
    {
        const int i = e / TS_P, k = e % TS_P;
        const float2 a = H[i * TS_P + k], b = H[k * TS_P + i];
        const Cx<float> hh = {0.5f * (a.x + b.x), i == k ? 0.f : 0.5f * (a.y - b.y)};
        Hs[i * TS_LD + k] = hh;
        Qs[i * TS_LD + k] = {i == k ? 1.f : 0.f, 0.f};
        f2 += hh.x * hh.x + hh.y * hh.y;
    }
    for (int o = 16; o > 0; o >>= 1)
        f2 += __shfl_xor_sync(0xffffffffu, f2, o);
    if (lane == 0)
        s_fro[warp] = f2;
    __syncthreads();
    float tot = 0.f;
    for (int w = 0; w < NW; ++w)
        tot += s_fro[w];
    smem_sweeps<float, JS_THREADS>(Hs, Qs, TS_P, TS_P, TS_LD, sc, 5e-7f * sqrtf(tot), JAC_MAX_SWEEPS);
    __syncthreads();
    if (tid < TS_P)
    {
        const float th = Hs[tid * TS_LD + tid].x;
        int rank = 0;
        for (int j = 0; j < TS_P; ++j)
        {
            const float tj = Hs[j * TS_LD + j].x;
            rank += (tj < th) || (tj == th && j < tid);
        }
        order[rank] = tid;
        evals[T - TS_P + rank] = static_cast<double>(th) / *scale;
    }
    for (int i = tid; i < T - TS_P; i += JS_THREADS)
        evals[i] = 0.0;
    __syncthreads();
    for (int e = tid; e < TS_P * TS_P; e += JS_THREADS)
    {
        const int k = e / TS_P, r = e % TS_P;
        const Cx<float> q = Qs[k * TS_LD + order[r]];
        Qo[e] = make_float2(q.x, q.y);
    }
}

// k_ts_ritz: the Ritz vectors U = V Qo, TS_P rows of U per CTA (warp w: rows w, w + 8, ..., lane =
// column r): into the warm start Vw (row-major) and, when evecs is not null, evecs columns
// T - TS_P + r (FP64, through a shared-memory transpose so that each eigenvector's rows are written
// contiguously). Also the Cholesky-QR's V = Y M (evecs null).
__global__ void __launch_bounds__(256) k_ts_ritz(const float2* __restrict__ V, const float2* __restrict__ Qo, int T,
                                                 double2* __restrict__ evecs, float2* __restrict__ Vw)
{
    __shared__ float2 q[TS_P][TS_P];
    __shared__ float2 u[TS_P][TS_P + 1];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int t0 = blockIdx.x * TS_P;
    for (int e = tid; e < TS_P * TS_P; e += 256)
        q[e / TS_P][e % TS_P] = Qo[e];
    __syncthreads();
    for (int rr = warp; rr < TS_P; rr += 8)
    {
        const int t = t0 + rr;
        if (t >= T)
            break;
        const float2 v = V[static_cast<size_t>(t) * TS_P + lane];
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int k = 0; k < TS_P; ++k)
        {
            const float vx = __shfl_sync(0xffffffffu, v.x, k), vy = __shfl_sync(0xffffffffu, v.y, k);
            const float2 qq = q[k][lane];
            re += vx * qq.x - vy * qq.y;
            im += vx * qq.y + vy * qq.x;
        }
        u[rr][lane] = make_float2(re, im);
        Vw[static_cast<size_t>(t) * TS_P + lane] = make_float2(re, im);
    }
    __syncthreads();
    if (evecs && t0 + lane < T)
        for (int r = warp; r < TS_P; r += 8)
        {
            const float2 x = u[lane][r];
            evecs[static_cast<size_t>(T - TS_P + r) * T + t0 + lane] = make_double2(x.x, x.y);
        }
}

static std::atomic<int> g_eig_precision{HV_EIG_FP32};
static std::atomic<int> g_cholqr{1};

void set_eig_cholqr(int on) { g_cholqr = on ? 1 : 0; }
static bool cholqr_enabled() { return g_cholqr.load() != 0; }

void set_eig_precision(int p) { g_eig_precision = p; }

// bytes of the refinement buffers (Y, D, G, Vn: ER_MAX_K x T complex128 each) at the start of the
// workspace tail
static size_t eigref_bytes(int T) { return 4 * static_cast<size_t>(ER_MAX_K) * T * sizeof(double2) + 512; }

size_t pca_eigh_workspace(int T)
{
    const int Tp = (T % 2) ? T + 1 : T;
    size_t bytes = static_cast<size_t>(T) * T * sizeof(double2) + static_cast<size_t>(2 * Tp) * sizeof(double) +
                   static_cast<size_t>(T) * sizeof(double) + static_cast<size_t>(Tp) * sizeof(int) + 256 +
                   eigref_bytes(T) + (T > JS_MAX_T ? ts_bytes(T) : 0);
    if (T > JS_MAX_T && T <= JC_MAX_T)
    {
        // block Jacobi: FP32 A and V (two copies each) of the size rounded up to 64, the step's
        // unitaries, convergence flags and the grid barrier
        const size_t Tb = (static_cast<size_t>(T) + BJ_S - 1) / BJ_S * BJ_S;
        bytes += 256 + 4 * Tb * Tb * sizeof(float2) + (Tb / BJ_S) * BJ_S * BJ_S * sizeof(float2) + 256;
    }
    return bytes;
}

hv_status pca_eigh(double2* cov, int T, double* evals, double2* evecs, int pmin, int pmax, float2* weights, void* work,
                   cudaStream_t st, int refine_lo, int refine_hi, bool warm, bool kept_only, bool* cov_kept)
{
    if (cov_kept)
        *cov_kept = true;
    if (T <= 0 || !work)
        return HV_INVALID_VALUE;
    // kept_only: the caller uses the refined eigenvectors (ranks refine_lo..refine_hi) and the
    // order of the eigenvalues only, so the FP32 sweeps stop at a coarser floor and the other
    // eigenvalues are FP32 Rayleigh quotients (T = 512: 15 sweeps and 13.8 ms -> 5 sweeps, the view
    // unchanged at 3.5e-7 from FP64). The floor is relative to the whole matrix, so only kept ranks
    // among the TS_MAX_KEEP largest qualify: for smaller kept eigenvalues (ranks 175-178 of 192 at
    // ~1.5e-3 of the largest) the rotations skipped below it left errors the FP64 corrections did
    // not remove (view 1e-4 .. 4e-4 from FP64).
    const int Kr = refine_hi - refine_lo + 1;
    const bool loose = kept_only && refine_lo >= 0 && refine_hi < T && Kr >= 1 && Kr <= ER_MAX_K &&
                       refine_lo >= T - TS_MAX_KEEP;
    const float floor_rel = loose ? 2e-5f : 5e-7f;

    const int prec = g_eig_precision.load();  // one read: a concurrent switch cannot split the dispatch
    const int Tp = (T % 2) ? T + 1 : T;
    char* base = static_cast<char*>(work);
    double2* V = reinterpret_cast<double2*>(base);
    size_t off = static_cast<size_t>(T) * T * sizeof(double2);
    double* rot = reinterpret_cast<double*>(base + off);
    off += static_cast<size_t>(2 * Tp) * sizeof(double);
    double* ev_unsorted = reinterpret_cast<double*>(base + off);
    off += static_cast<size_t>(T) * sizeof(double);
    int* pairs = reinterpret_cast<int*>(base + off);
    // refinement buffers: after the pair list, before the subspace and block-Jacobi arrays
    char* er_base = base + ((off + static_cast<size_t>(Tp) * sizeof(int) + 255) & ~static_cast<size_t>(255));
    off += eigref_bytes(T);
    char* ts_base = base + ((off + static_cast<size_t>(Tp) * sizeof(int) + 255) & ~static_cast<size_t>(255));
    if (T > JS_MAX_T)
        off += ts_bytes(T);
    // FP64 correction of the kept eigenvectors (ranks refine_lo .. refine_hi) against the FP64
    // covariance, with the eigenvectors of ranks b0 .. T-1 as the basis; `iters` corrections (the
    // first leaves O(theta^2) against the FP32 error of the basis, the next bring that to the FP64
    // level)
    auto refine_kept = [&](int b0, int iters) -> hv_status {
        double2* Y = reinterpret_cast<double2*>(er_base);
        double2* D = Y + static_cast<size_t>(ER_MAX_K) * T;
        double2* G = D + static_cast<size_t>(ER_MAX_K) * T;
        double2* Vn = G + static_cast<size_t>(ER_MAX_K) * T;
        const dim3 gw((T + 7) / 8, Kr), gp(T - b0, Kr), gt((T + 31) / 32, Kr);
        for (int iter = 0; iter < iters; ++iter)
        {
            k_eigref_matvec<<<gw, 256, 0, st>>>(cov, evecs, T, refine_lo, Y);
            HV_LAUNCH_CHECK();
            k_eigref_project<<<gp, ER_PROJ_THREADS, 0, st>>>(evecs, Y, T, refine_lo, b0, D, G);
            HV_LAUNCH_CHECK();
            k_eigref_update<<<gt, 32 * ER_UPD_WARPS, 0, st>>>(evecs, evals, D, G, Y, T, refine_lo, Kr, b0, Vn);
            HV_LAUNCH_CHECK();
            k_eigref_finish<<<Kr, 128, 0, st>>>(evecs, evals, Vn, D, G, T, refine_lo, pmin, pmax, weights);
            HV_LAUNCH_CHECK();
            count_launch(4);
        }
        return HV_OK;
    };
    // the largest eigenpairs only: subspace iteration instead of the block Jacobi
    if (loose && prec == HV_EIG_FP32 && T > JS_MAX_T && T <= JC_MAX_T && refine_lo >= T - TS_MAX_KEEP)
    {
        float2* C32 = reinterpret_cast<float2*>(ts_base);
        float2* Vs = C32 + static_cast<size_t>(T) * T;
        float2* Ys = Vs + static_cast<size_t>(T) * TS_P;
        float2* Vw = Ys + static_cast<size_t>(T) * TS_P;
        float2* Hm = Vw + static_cast<size_t>(T) * TS_P;
        float2* Qo = Hm + TS_P * TS_P;
        double* scale = reinterpret_cast<double*>(Qo + TS_P * TS_P);
        const int gb = (T * TS_P + 255) / 256;
        const int gm = (T + TS_MM_ROWS - 1) / TS_MM_ROWS;
        constexpr int mm_threads = TS_MM_ROWS * TS_MM_SPLIT * 32;
        k_ts_convert<<<std::min(512, (T * T + 1023) / 1024), 256, 0, st>>>(cov, T, C32, scale);
        HV_LAUNCH_CHECK();
        // warm: the previous window's Ritz vectors are orthonormal (V Q with V orthonormal, Q unitary)
        // and start the iteration as they are
        if (!warm)
        {
            k_ts_init<<<gb, 256, 0, st>>>(C32, T, Ys);
            HV_LAUNCH_CHECK();
            k_ts_orth<<<1, TS_ORTH_THREADS, 0, st>>>(Ys, T, Vs);
            HV_LAUNCH_CHECK();
        }
        const int iters = warm ? TS_ITERS_WARM : TS_ITERS_COLD;
        int* chol_fail = reinterpret_cast<int*>(scale + 1);
        int extra = 0;
        for (int it = 0; it < iters; ++it)
        {
            k_ts_matmul<<<gm, mm_threads, 0, st>>>(C32, it == 0 && warm ? Vw : Vs, T, Ys);
            HV_LAUNCH_CHECK();
            if (warm && cholqr_enabled())
            {
                // Cholesky-QR (Gram, 32 x 32 factorisation, V = Y M), Gram-Schmidt only if it failed
                k_ts_gram<<<TS_P, TS_GRAM_WARPS * 32, 0, st>>>(Ys, Ys, T, Hm);
                HV_LAUNCH_CHECK();
                k_ts_cholqr<<<1, 32, 0, st>>>(Hm, Qo, chol_fail);
                HV_LAUNCH_CHECK();
                k_ts_ritz<<<(T + TS_P - 1) / TS_P, 256, 0, st>>>(Ys, Qo, T, nullptr, Vs);
                HV_LAUNCH_CHECK();
                k_ts_orth<<<1, TS_ORTH_THREADS, 0, st>>>(Ys, T, Vs, chol_fail);
                HV_LAUNCH_CHECK();
                extra += 3;
            }
            else
            {
                k_ts_orth<<<1, TS_ORTH_THREADS, 0, st>>>(Ys, T, Vs);
                HV_LAUNCH_CHECK();
            }
        }
        k_ts_matmul<<<gm, mm_threads, 0, st>>>(C32, Vs, T, Ys);
        HV_LAUNCH_CHECK();
        k_ts_gram<<<TS_P, TS_GRAM_WARPS * 32, 0, st>>>(Vs, Ys, T, Hm);
        HV_LAUNCH_CHECK();
        k_ts_rr<<<1, JS_THREADS, 0, st>>>(Hm, T, scale, evals, Qo);
        HV_LAUNCH_CHECK();
        k_ts_ritz<<<(T + TS_P - 1) / TS_P, 256, 0, st>>>(Vs, Qo, T, evecs, Vw);
        HV_LAUNCH_CHECK();
        count_launch(5 + 2 * iters + extra + (warm ? 0 : 2));
        // two corrections: on 512 x 512 frames with T = 512 and stride 64, one warm iteration and two
        // corrections reach the view error of three and three (3.5e-7 .. 1.9e-6 from FP64)
        return refine_kept(T - TS_P, 2);
    }
    if (T <= JS_MAX_T && prec == HV_EIG_FP32)
    {
        const size_t smem = jacobi_smem_bytes<float>(T, warm);
        if (smem > 48 * 1024)
            HV_CUDA_TRY(cudaFuncSetAttribute(k_jacobi_smem<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(jacobi_smem_bytes<float>(JS_MAX_T, true))));
        k_jacobi_smem<float><<<1, JS_THREADS, smem, st>>>(cov, V, T, Tp, ev_unsorted, warm ? 1 : 0, floor_rel);
    }
    else if (T <= JS_MAX_T)
    {
        const size_t smem = jacobi_smem_bytes<double>(T, false);
        if (smem > 48 * 1024)
            HV_CUDA_TRY(cudaFuncSetAttribute(k_jacobi_smem<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem)));
        k_jacobi_smem<double><<<1, JS_THREADS, smem, st>>>(cov, V, T, Tp, ev_unsorted, 0, 0.0f);
    }
    else if (T <= JC_MAX_T && prec == HV_EIG_FP32)
    {
        // FP32 block-cyclic sweeps over a cooperative grid (A and V copies in the workspace), then
        // the FP64 finish
        const int Tb = (T + BJ_S - 1) / BJ_S * BJ_S;
        const size_t tb2 = static_cast<size_t>(Tb) * Tb * sizeof(float2);
        size_t off2 = (off + static_cast<size_t>(Tp) * sizeof(int) + 255) & ~static_cast<size_t>(255);
        Cx<float>* A0 = reinterpret_cast<Cx<float>*>(base + off2);
        Cx<float>* A1 = reinterpret_cast<Cx<float>*>(base + off2 + tb2);
        Cx<float>* V0 = reinterpret_cast<Cx<float>*>(base + off2 + 2 * tb2);
        Cx<float>* V1 = reinterpret_cast<Cx<float>*>(base + off2 + 3 * tb2);
        off2 += 4 * tb2;
        Cx<float>* U = reinterpret_cast<Cx<float>*>(base + off2);
        off2 += static_cast<size_t>(Tb / BJ_S) * BJ_S * BJ_S * sizeof(float2);
        int* flags = reinterpret_cast<int*>(base + off2);  // three sweep flags (zeroed by the kernel)
        double* fro2 = reinterpret_cast<double*>(base + off2 + 32);
        GridBarrier* bar = reinterpret_cast<GridBarrier*>(base + off2 + 64);
        HV_CUDA_TRY(cudaMemsetAsync(base + off2, 0, 128, st));
        HV_CUDA_TRY(cudaFuncSetAttribute(k_jacobi_block, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(BJ_SMEM)));
        // co-resident CTAs per SM (the cooperative grid must fit); thread-safe one-time query
        static const int max_per_sm = [] {
            int v = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_jacobi_block, BJ_THREADS, BJ_SMEM) != cudaSuccess)
                v = 1;
            return v;
        }();
        int sms = 0;
        HV_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
        const int npb = Tb / BJ_S, na = npb * (npb + 1) / 2;
        int nb = na + (Tb / BJ_S) * npb;  // phase-2 items: A blocks and V blocks
        const int cap = sms * (max_per_sm > 0 ? max_per_sm : 1);
        nb = nb > cap ? cap : nb;
        int Ti = T, Tbi = Tb;
        const double2* cin = cov;
        double fr = floor_rel;
        void* args[] = {&cin, &Ti, &Tbi, &A0, &A1, &V0, &V1, &U, &flags, &fro2, &bar, &V, &ev_unsorted, &fr};
        HV_CUDA_TRY(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(k_jacobi_block), nb, BJ_THREADS, args, BJ_SMEM,
                                                st));
        count_launch();
    }
    if (T <= JS_MAX_T || (T <= JC_MAX_T && prec == HV_EIG_FP32))
    {
        HV_LAUNCH_CHECK();
        if (loose)
            k_eig_refine<float><<<T, 128, 0, st>>>(cov, V, T, ev_unsorted);
        else
            k_eig_refine<double><<<T, 128, 0, st>>>(cov, V, T, ev_unsorted);
        count_launch();
    }
    else
    {
        k_jacobi<<<1, JAC_THREADS, 0, st>>>(cov, V, T, Tp, ev_unsorted, pairs, rot);  // FP64 sweeps, in place
        if (cov_kept)
            *cov_kept = false;
    }
    HV_LAUNCH_CHECK();
    k_eig_sort<<<T, 128, 0, st>>>(ev_unsorted, V, T, evals, evecs, pmin, pmax, weights);
    HV_LAUNCH_CHECK();
    count_launch(2);
    // FP32 sweeps: the kept eigenvectors are corrected in FP64 (FP64 sweeps need no correction)
    const bool fp32_sweeps = T <= JS_MAX_T ? prec == HV_EIG_FP32 : (T <= JC_MAX_T && prec == HV_EIG_FP32);
    if (fp32_sweeps && refine_lo >= 0 && refine_hi < T && Kr >= 1 && Kr <= ER_MAX_K)
    {
        hv_status rr = refine_kept(0, loose ? 3 : 2);
        if (rr != HV_OK)
            return rr;
    }
    return HV_OK;
}

// ------------------------------------------------------------------------------ SSA_STFT
// p_acc = FFT_t(H V_q V_q^H) (fourier_transform.cc:379-444) restricted to the bins pmin..pmin+K-1
// is one more set of projection weights over the ring:
//   w[k][s] = sum_{j in q} V[s][j] c[j][k],   c[j][k] = sum_t conj(V[t][j]) exp(-2 pi i (pmin+k) t / T),
// computed in FP64 from the FP64 eigenvectors (column-major, evecs[j*T + t]); one CTA per bin.
__global__ void k_ssa_weights(const double2* __restrict__ evecs, int T, int qmin, int qn, int pmin, float2* w)
{
    extern __shared__ double2 s_c[];  // qn coefficients of this bin
    const int k = blockIdx.x;
    const long long p = pmin + k;
    for (int j = threadIdx.x; j < qn; j += blockDim.x)
    {
        const double2* v = evecs + static_cast<size_t>(qmin + j) * T;
        double cr = 0.0, ci = 0.0;
        for (int t = 0; t < T; ++t)
        {
            const long long m = (p * t) % T;
            double sn, cs;
            sincospi(-2.0 * static_cast<double>(m) / static_cast<double>(T), &sn, &cs);
            const double2 x = v[t];
            // conj(x) * (cs + i sn)
            cr += x.x * cs + x.y * sn;
            ci += x.x * sn - x.y * cs;
        }
        s_c[j] = make_double2(cr, ci);
    }
    __syncthreads();
    for (int s = threadIdx.x; s < T; s += blockDim.x)
    {
        double wr = 0.0, wi = 0.0;
        for (int j = 0; j < qn; ++j)
        {
            const double2 v = evecs[static_cast<size_t>(qmin + j) * T + s];
            const double2 c = s_c[j];
            wr += v.x * c.x - v.y * c.y;
            wi += v.x * c.y + v.y * c.x;
        }
        w[static_cast<size_t>(k) * T + s] = make_float2(static_cast<float>(wr), static_cast<float>(wi));
    }
}

hv_status ssa_weights(const double2* evecs, int T, int qmin, int qn, int pmin, int K, float2* weights, cudaStream_t st)
{
    if (T <= 0 || K <= 0 || qmin < 0 || qn < 1 || qmin + qn > T || pmin < 0 || pmin + K > T || !evecs || !weights)
        return HV_INVALID_VALUE;
    if (static_cast<size_t>(qn) * sizeof(double2) > 48 * 1024)
    {
        set_last_error_msg("ssa_weights: more than 3072 eigenvectors kept");
        return HV_ERR_UNSUPPORTED;
    }
    k_ssa_weights<<<K, 256, static_cast<size_t>(qn) * sizeof(double2), st>>>(evecs, T, qmin, qn, pmin, weights);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

// ------------------------------------------------------------------------------ phase increase
// The stored p plane X = sum_t ring[t] w[t] (fourier_transform.cc:446-460, w = the first row of
// the view's weights), d = arg(X conj(pred)) (kernel_compute_angle_mult), out = d + the previous
// d (a history of one frame: UnwrappingResources capacity 1, kernel_correct_angles), pred = X.
// `first` gives d = 0 (pred = X); `use_hist` is off until one d is stored. Per-CTA min / max of
// out go to mm[blockIdx.x] for the rescale.
constexpr int PI_THREADS = 256;

__global__ void __launch_bounds__(PI_THREADS) k_phase_increase(const float2* __restrict__ ring, int T, size_t HW,
                                                               const float2* __restrict__ w, float2* pred, float* hist,
                                                               int first, int use_hist, float* out, float2* mm)
{
    extern __shared__ float2 s_w[];
    __shared__ float s_mn[PI_THREADS / 32], s_mx[PI_THREADS / 32];
    for (int t = threadIdx.x; t < T; t += blockDim.x)
        s_w[t] = w[t];
    __syncthreads();
    const size_t i = static_cast<size_t>(blockIdx.x) * PI_THREADS + threadIdx.x;
    float mn = INFINITY, mx = -INFINITY;
    if (i < HW)
    {
        float xr = 0.f, xi = 0.f;
        for (int t = 0; t < T; ++t)
        {
            const float2 x = __ldcs(ring + static_cast<size_t>(t) * HW + i);
            const float2 c = s_w[t];
            xr = fmaf(x.x, c.x, fmaf(-x.y, c.y, xr));
            xi = fmaf(x.x, c.y, fmaf(x.y, c.x, xi));
        }
        // the first window compares the plane with itself: its increment is 0 (the reference takes
        // atan2 of the rounding residue of X conj(X) there)
        float d = 0.0f;
        if (!first)
        {
            const float2 pr = pred[i];
            const float re = xr * pr.x + xi * pr.y;
            const float im = xi * pr.x - xr * pr.y;
            d = atan2f(im, re);
        }
        const float o = use_hist ? d + hist[i] : d;
        hist[i] = d;
        pred[i] = make_float2(xr, xi);
        out[i] = o;
        mn = mx = o;
    }
    for (int off = 16; off > 0; off >>= 1)
    {
        mn = fminf(mn, __shfl_down_sync(0xffffffffu, mn, off));
        mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, off));
    }
    if ((threadIdx.x & 31) == 0)
    {
        s_mn[threadIdx.x >> 5] = mn;
        s_mx[threadIdx.x >> 5] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        for (int k = 1; k < PI_THREADS / 32; ++k)
        {
            mn = fminf(mn, s_mn[k]);
            mx = fmaxf(mx, s_mx[k]);
        }
        mm[blockIdx.x] = make_float2(mn, mx);
    }
}

// rescale_float (tools_conversion.cu:275-313): out = (in + |min|) * 65535 / (|max| + |min|), with
// min and max from the first 128 blocks of 128 pixels of the reference's reduction, i.e. over
// pixels [0, min(HW, 16384)) (the whole frame below that size, where the reference reads past its
// block results). Then the PCA scale (converts.cc:50-62) as a separate rounding. Every CTA
// reduces the min / max partials of the prefix itself.
__global__ void k_rescale_float(const float* __restrict__ in, size_t HW, const float2* __restrict__ mm, int nmm,
                                float post_scale, float* __restrict__ out)
{
    __shared__ float s_mn, s_mx;
    if (threadIdx.x < 32)
    {
        float mn = INFINITY, mx = -INFINITY;
        for (int k = threadIdx.x; k < nmm; k += 32)
        {
            const float2 v = mm[k];
            mn = fminf(mn, v.x);
            mx = fmaxf(mx, v.y);
        }
        for (int off = 16; off > 0; off >>= 1)
        {
            mn = fminf(mn, __shfl_down_sync(0xffffffffu, mn, off));
            mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, off));
        }
        if (threadIdx.x == 0)
        {
            s_mn = mn;
            s_mx = mx;
        }
    }
    __syncthreads();
    const float amin = fabsf(s_mn), den = __fadd_rn(fabsf(s_mx), amin);
    for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < HW;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        // an all-zero prefix (the first window) maps to 0 instead of the reference's 0 / 0
        float v = den > 0.0f ? __fdiv_rn(__fmul_rn(__fadd_rn(in[i], amin), 65535.0f), den) : 0.0f;
        if (post_scale != 1.0f)
            v = __fmul_rn(v, post_scale);
        out[i] = v;
    }
}

size_t phase_increase_minmax_count(size_t HW) { return (HW + PI_THREADS - 1) / PI_THREADS; }

hv_status phase_increase(const float2* ring, int T, size_t HW, const float2* w, float2* pred, float* hist, int first,
                         int use_hist, float* out, float2* mm, cudaStream_t st)
{
    if (T <= 0 || HW == 0 || !ring || !w || !pred || !hist || !out || !mm)
        return HV_INVALID_VALUE;
    const size_t grid = phase_increase_minmax_count(HW);
    if (grid > 0x7fffffffu)
        return HV_INVALID_VALUE;
    if (static_cast<size_t>(T) * sizeof(float2) > 40 * 1024)
    {
        set_last_error_msg("phase_increase: time window above 5120 frames");
        return HV_ERR_UNSUPPORTED;
    }
    k_phase_increase<<<static_cast<unsigned>(grid), PI_THREADS, static_cast<size_t>(T) * sizeof(float2), st>>>(
        ring, T, HW, w, pred, hist, first, use_hist, out, mm);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status rescale_float(const float* in, size_t HW, const float2* mm, float post_scale, float* out, cudaStream_t st)
{
    if (HW == 0 || !in || !mm || !out)
        return HV_INVALID_VALUE;
    const size_t prefix = HW < 16384 ? HW : 16384;
    const int nmm = static_cast<int>((prefix + PI_THREADS - 1) / PI_THREADS);
    size_t grid = (HW + 255) / 256;
    grid = grid < 152 * 16 ? grid : 152 * 16;
    k_rescale_float<<<static_cast<unsigned>(grid), 256, 0, st>>>(in, HW, mm, nmm, post_scale, out);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

}  // namespace hv
