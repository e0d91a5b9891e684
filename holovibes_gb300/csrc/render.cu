// Rendering stage on the float view frame: 2-D phase unwrap, renormalisation, fftshift,
// image accumulation, log10, percentile autocontrast and the contrast map to uint16.
//
// Reference behaviour (Holovibes):
//   unwrap_2d      Backend/cuda_sources/tools_unwrap.cu:79-95,269-369, tools.cu:50-68
//   rescale        Backend/cuda_sources/tools_conversion.cu:315-335
//   renorm         Backend/cuda_sources/tools_compute.cu:99-123, Backend/sources/compute/postprocessing.cc:135-155
//   fftshift       Backend/cuda_sources/shift_corners.cu:8-70
//   accumulation   Backend/cuda_sources/tools_conversion.cu:418-458, Backend/sources/compute/image_accumulation.cc:136-157
//   percentile     Backend/cuda_sources/percentile.cu:15-43,75-94,139-222, Backend/sources/api/contrast_api.cc:137-146
//   contrast       Backend/cuda_sources/contrast_correction.cu:5-17
//   float->ushort  Backend/cuda_sources/tools_conversion.cu:350-387
//
// GB300 design: the percentile is an exact three-pass radix select on order-preserving float keys
// (11/11/10 bits) instead of a full thrust sort, and the selected range never leaves the device:
// the contrast kernel reads it from device memory, so no host round trip or stream sync happens.
#include <float.h>
#include <math.h>

#include <mutex>
#include <string>

#include "hv_common.cuh"
#include "hv_internal.h"

namespace hv {

constexpr int EW_THREADS = 256;

static int ew_grid(size_t n)
{
    size_t g = (n + EW_THREADS - 1) / EW_THREADS;
    const size_t cap = 152 * 32;
    return static_cast<int>(g < cap ? (g > 0 ? g : 1) : cap);
}

// ====================================================================================== unwrap

// z = exp(i*phase) (kernel_init_unwrap_2d)
__global__ void k_unwrap_init(const float* in, float2* z, size_t n)
{
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        float s, c;
        sincosf(in[e], &s, &c);
        z[e] = make_float2(c, s);
    }
}

// Frequency index of flat element e after circ_shift(-W/2, -H/2) of the fx / fy grids:
// sfx[y][x] = ((x + W/2) % W) - W/2, sfy[y][x] = ((y + H/2) % H) - H/2.
__device__ __forceinline__ void shifted_freqs(size_t e, int W, int H, float& fx, float& fy)
{
    const int x = static_cast<int>(e % W), y = static_cast<int>(e / W);
    fx = static_cast<float>((x + (W >> 1)) % W - (W >> 1));
    fy = static_cast<float>((y + (H >> 1)) % H - (H >> 1));
}

// gx = Z * sfx, gy = Z * sfy (kernel_multiply_complexes_by_floats_)
__global__ void k_unwrap_grad_freq(const float2* Z, float2* gx, float2* gy, int W, int H)
{
    const size_t n = static_cast<size_t>(W) * H;
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        float fx, fy;
        shifted_freqs(e, W, H, fx, fy);
        const float2 v = Z[e];
        gx[e] = cscale(v, fx);
        gy[e] = cscale(v, fy);
    }
}

// g *= (i * 2pi) then g *= conj(i z) (kernel_multiply_complexes_by_single_complex, eq_unwrap_2d)
__global__ void k_unwrap_eq(float2* gx, float2* gy, const float2* z, size_t n, float two_pi)
{
    const float2 i2pi = make_float2(0.f, two_pi);
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        const float2 zc = cconj(cmul(z[e], make_float2(0.f, 1.f)));
        gx[e] = cmul(cmul(gx[e], i2pi), zc);
        gy[e] = cmul(cmul(gy[e], i2pi), zc);
    }
}

// acc = gx * sfx/(sfx^2+sfy^2) + gy * sfy/(...) (kernel_norm_ratio + kernel_add_complex_frames)
__global__ void k_unwrap_ratio(const float2* gx, const float2* gy, float2* acc, int W, int H)
{
    const size_t n = static_cast<size_t>(W) * H;
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        float fx, fy;
        shifted_freqs(e, W, H, fx, fy);
        const float norm = fx * fx + fy * fy;
        float2 r = make_float2(0.f, 0.f);
        if (norm != 0.f)
        {
            const float cx = fx / norm, cy = fy / norm;
            r = cadd(cscale(gx[e], cx), cscale(gy[e], cy));
        }
        acc[e] = r;
    }
}

// out = Im(acc) / -2pi (kernel_unwrap2d_last_step), plus FP64-free min/max via ordered keys
__device__ __forceinline__ unsigned int float_key(float f)
{
    const unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_float(unsigned int k)
{
    const unsigned int u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

__global__ void k_unwrap_last(const float2* acc, float* out, size_t n, float two_pi, unsigned int* minmax)
{
    unsigned int kmin = 0xffffffffu, kmax = 0u;
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        const float v = acc[e].y / -two_pi;
        out[e] = v;
        const unsigned int k = float_key(v);
        kmin = min(kmin, k);
        kmax = max(kmax, k);
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        kmin = min(kmin, __shfl_down_sync(0xffffffffu, kmin, o));
        kmax = max(kmax, __shfl_down_sync(0xffffffffu, kmax, o));
    }
    if ((threadIdx.x & 31) == 0)
    {
        atomicMin(minmax, kmin);
        atomicMax(minmax + 1, kmax);
    }
}

__global__ void k_init_minmax(unsigned int* minmax)
{
    minmax[0] = 0xffffffffu;
    minmax[1] = 0u;
}

// rescale_float_unwrap2d: (in + |min|)/(|min| + max)*65535 if min < 0 else (in - min)/(max - min)*65535
__global__ void k_unwrap_rescale(float* io, size_t n, const unsigned int* minmax)
{
    const float mn = key_float(minmax[0]), mx = key_float(minmax[1]);
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        const float in = io[e];
        float r;
        // a constant frame maps to 0 (the reference divides 0 by 0 there)
        if (mx == mn)
            r = 0.0f;
        else if (mn < 0.f)
            r = __fdiv_rn(__fadd_rn(in, fabsf(mn)), __fadd_rn(fabsf(mn), mx)) * 65535.0f;
        else
            r = __fdiv_rn(__fsub_rn(in, mn), __fsub_rn(mx, mn)) * 65535.0f;
        io[e] = r;
    }
}

size_t unwrap_workspace(int W, int H)
{
    const size_t n = static_cast<size_t>(W) * H;
    return 4 * n * sizeof(float2) + 256;
}

hv_status unwrap_2d(const float* in, float* out, int W, int H, void* work, cudaStream_t st)
{
    const size_t n = static_cast<size_t>(W) * H;
    // The reference plans its unwrap FFT with plan(width, height) (icompute.hh:140): the
    // row-major buffer is transformed as `width` rows of `height` samples.
    const int n0 = W, n1 = H;
    if (!fft_size_supported(n0) || !fft_size_supported(n1))
    {
        set_last_error_msg("unwrap_2d: frame size not supported by the shared-memory FFT");
        return HV_ERR_UNSUPPORTED;
    }
    float2* z = static_cast<float2*>(work);
    float2* g = z + n;  // gx, gy contiguous (batch of 2)
    float2* gx = g;
    float2* gy = g + n;
    float2* Z = g + 2 * n;
    unsigned int* minmax = reinterpret_cast<unsigned int*>(Z + n);
    const float two_pi = 6.28318530717959f;  // M_2PI of common.cuh:29
    const int grid = ew_grid(n);
    k_unwrap_init<<<grid, EW_THREADS, 0, st>>>(in, z, n);
    HV_LAUNCH_CHECK();
    hv_status s = fft2d(z, Z, n0, n1, 1, 0, 1.0f, st);
    if (s != HV_OK)
        return s;
    k_unwrap_grad_freq<<<grid, EW_THREADS, 0, st>>>(Z, gx, gy, W, H);
    HV_LAUNCH_CHECK();
    if ((s = fft2d(g, g, n0, n1, 2, 1, 1.0f, st)) != HV_OK)
        return s;
    k_unwrap_eq<<<grid, EW_THREADS, 0, st>>>(gx, gy, z, n, two_pi);
    HV_LAUNCH_CHECK();
    if ((s = fft2d(g, g, n0, n1, 2, 0, 1.0f, st)) != HV_OK)
        return s;
    k_unwrap_ratio<<<grid, EW_THREADS, 0, st>>>(gx, gy, Z, W, H);
    HV_LAUNCH_CHECK();
    if ((s = fft2d(Z, Z, n0, n1, 1, 1, 1.0f, st)) != HV_OK)
        return s;
    k_init_minmax<<<1, 1, 0, st>>>(minmax);
    HV_LAUNCH_CHECK();
    k_unwrap_last<<<grid, EW_THREADS, 0, st>>>(Z, out, n, two_pi, minmax);
    HV_LAUNCH_CHECK();
    k_unwrap_rescale<<<grid, EW_THREADS, 0, st>>>(out, n, minmax);
    HV_LAUNCH_CHECK();
    count_launch(7);
    return HV_OK;
}

// ---------------------------------------------------------------------- unwrap without allocation
// Some callers cannot allocate device memory at all: a frame-grabber or acquisition callback that
// runs on a driver thread with a real-time budget, or a host application whose memory policy
// forbids cudaMalloc once streaming has started. hv_unwrap_2d_noalloc serves them: its scratch
// (four complex frames and the min/max keys, the same layout hv_unwrap_2d takes from `work`) is
// this file-scope device array, sized for frames of at most HV_UNWRAP_NOALLOC_MAX_PIXELS pixels.
// Every GPU that loads the library keeps the array (8 MiB) until the process exits. With CUDA's
// lazy module loading the driver creates the array (and this module's other device data) when
// one of the module's kernels first runs on a device, so the first call on each device is the
// one that may allocate inside the driver: make it before streaming starts.

constexpr size_t kUnwrapNoallocMaxPixels = HV_UNWRAP_NOALLOC_MAX_PIXELS;
static __device__ __align__(256) float2 g_unwrap_scratch[4 * kUnwrapNoallocMaxPixels + 32];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};
}  // namespace

hv_status unwrap_2d_noalloc(const float* in, float* out, int W, int H, cudaStream_t st)
{
    if (W <= 0 || H <= 0)
    {
        set_last_error_msg("hv_unwrap_2d_noalloc: width and height must be positive");
        return HV_INVALID_VALUE;
    }
    const size_t n = static_cast<size_t>(W) * H;
    if (n > kUnwrapNoallocMaxPixels)
    {
        set_last_error_msg(("hv_unwrap_2d_noalloc: the frame's " + std::to_string(n) +
                            " pixels exceed the 262144-pixel static scratch").c_str());
        return HV_INVALID_VALUE;
    }
    int dev = 0;
    HV_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
    {
        set_last_error_msg(("hv_unwrap_2d_noalloc: device index " + std::to_string(dev) +
                            " beyond the 64 devices this entry point serves").c_str());
        return HV_INVALID_VALUE;
    }
    void* ptr = nullptr;
    {
        // set-up on the first call on each device (with that device current): the host-side name
        // of the array is not a device address, so fetch the address once and keep it
        std::lock_guard<std::mutex> g(g_scratch_mu);
        if (!g_scratch_ptr[dev])
        {
            void* p = nullptr;
            HV_CUDA_TRY(cudaGetSymbolAddress(&p, g_unwrap_scratch));
            g_scratch_ptr[dev] = p;
        }
        ptr = g_scratch_ptr[dev];
    }
    // every buffer of the scratch is fully written before it is read, and the min/max keys are
    // re-initialised by unwrap_2d itself, so the previous call's contents never leak into this one
    return unwrap_2d(in, out, W, H, ptr, st);
}

// ====================================================================================== renorm

size_t reduce_workspace(size_t n)
{
    return static_cast<size_t>(ew_grid(n)) * sizeof(double) + 64;
}

__global__ void k_partial_sums(const float* in, size_t n, double* partials, const CycleCtl* ctl)
{
    if (!ctl_render(ctl))
        return;
    __shared__ double red[EW_THREADS / 32];
    double s = 0.0;
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
        s += in[e];
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double t = 0.0;
        for (int i = 0; i < EW_THREADS / 32; ++i)
            t += red[i];
        partials[blockIdx.x] = t;
    }
}

// factors[0] = 2^c, factors[1] = (float)N / (float)sum; x' = (x * factors[0]) * factors[1]
__global__ void k_renorm_factors(const double* partials, int np, size_t n, int c, float* factors,
                                 const CycleCtl* ctl)
{
    if (!ctl_render(ctl))
        return;
    __shared__ double red[32];
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x)
        s += partials[i];
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double t = 0.0;
        for (int i = 0; i < (blockDim.x + 31) / 32; ++i)
            t += red[i];
        factors[0] = static_cast<float>(1 << c);
        // a zero-sum frame (all zero) stays zero instead of the reference's N / 0 = inf, 0 * inf = NaN
        factors[1] = t != 0.0 ? __fdiv_rn(static_cast<float>(n), static_cast<float>(t)) : 0.0f;
    }
}

hv_status renorm_factors(const float* frame, size_t n, int renorm_constant, const double* partials, int npartials,
                         float* factors, void* work, cudaStream_t st, const CycleCtl* ctl)
{
    if (!partials)
    {
        double* p = static_cast<double*>(work);
        const int grid = ew_grid(n);
        k_partial_sums<<<grid, EW_THREADS, 0, st>>>(frame, n, p, ctl);
        HV_LAUNCH_CHECK();
        count_launch();
        partials = p;
        npartials = grid;
    }
    k_renorm_factors<<<1, 1024, 0, st>>>(partials, npartials, n, renorm_constant, factors, ctl);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

// Fused: renormalise (factors may be null), optional quadrant swap (out of place), optional
// accumulation into an A-frame ring (write slot, mean of `count` frames from `start`), optional log10.
__global__ void k_renorm_shift_acc(const float* __restrict__ in, float* __restrict__ out, int W, int H,
                                   const float* __restrict__ factors, int shift, float* __restrict__ acc, int A,
                                   int slot, int start, int count, int log_enabled, float prescale,
                                   const CycleCtl* ctl)
{
    if (!ctl_render(ctl))
        return;
    if (ctl)
    {
        slot = ctl->acc_slot;
        start = ctl->acc_start;
        count = ctl->acc_count;
    }
    const size_t n = static_cast<size_t>(W) * H;
    float m0 = 1.f, m1 = 1.f;
    if (factors)
    {
        m0 = factors[0];
        m1 = factors[1];
    }
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        size_t src = e;
        if (shift)
        {
            const int x = static_cast<int>(e % W), y = static_cast<int>(e / W);
            src = static_cast<size_t>((y + H / 2) % H) * W + (x + W / 2) % W;
        }
        float v = in[src];
        if (prescale != 1.0f)
            v = v * prescale;
        if (factors)
            v = (v * m0) * m1;
        if (acc)
        {
            acc[static_cast<size_t>(slot) * n + e] = v;
            float s = 0.f;
            int pos = start;
            for (int i = 0; i < count; ++i)
            {
                s += (pos == slot) ? v : acc[static_cast<size_t>(pos) * n + e];
                pos = (pos + 1) % A;
            }
            v = s / static_cast<float>(count);
        }
        if (log_enabled)
            v = log10f(v);
        out[e] = v;
    }
}

hv_status renorm_shift_accumulate(const float* in, float* out, int W, int H, const float* factors, int shift,
                                  float* acc_ring, int A, int slot, int start, int count, int log_enabled,
                                  cudaStream_t st, float prescale, const CycleCtl* ctl)
{
    if (shift && ((W & 1) || (H & 1)))
    {
        set_last_error_msg("fftshift needs even width and height");
        return HV_INVALID_VALUE;
    }
    if (shift && in == out)
    {
        set_last_error_msg("renorm_shift_accumulate: shift must be out of place");
        return HV_INVALID_VALUE;
    }
    const size_t n = static_cast<size_t>(W) * H;
    k_renorm_shift_acc<<<ew_grid(n), EW_THREADS, 0, st>>>(in, out, W, H, factors, shift, acc_ring, A, slot, start,
                                                          count, log_enabled, prescale, ctl);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

// In-place quadrant swap: thread owns pixel (x, y) of the top half and swaps it with its partner.
__global__ void k_shift_corners(float* f, int W, int H)
{
    const size_t half = static_cast<size_t>(W) * (H / 2);
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < half;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        const int x = static_cast<int>(e % W), y = static_cast<int>(e / W);
        const int nx = x < W / 2 ? x + W / 2 : x - W / 2;
        const size_t a = static_cast<size_t>(y) * W + x;
        const size_t b = static_cast<size_t>(y + H / 2) * W + nx;
        const float t = f[b];
        f[b] = f[a];
        f[a] = t;
    }
}

hv_status shift_corners(float* frame, int W, int H, cudaStream_t st)
{
    if ((W & 1) || (H & 1))
    {
        set_last_error_msg("shift_corners needs even width and height");
        return HV_INVALID_VALUE;
    }
    k_shift_corners<<<ew_grid(static_cast<size_t>(W) * H / 2), EW_THREADS, 0, st>>>(frame, W, H);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status accumulate(const float* frame, float* acc_ring, int A, int slot, int start, int count, float* out, size_t n,
                     cudaStream_t st)
{
    if (A <= 0 || slot < 0 || slot >= A || start < 0 || start >= A || count <= 0 || count > A)
        return HV_INVALID_VALUE;
    // 1-row frame of n pixels: no shift, no renorm
    k_renorm_shift_acc<<<ew_grid(n), EW_THREADS, 0, st>>>(frame, out, static_cast<int>(n), 1, nullptr, 0, acc_ring, A,
                                                          slot, start, count, 0, 1.0f, nullptr);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

__global__ void k_log10(float* f, size_t n)
{
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
        f[e] = log10f(f[e]);
}

hv_status log10_map(float* frame, size_t n, cudaStream_t st)
{
    k_log10<<<ew_grid(n), EW_THREADS, 0, st>>>(frame, n);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

// ====================================================================================== percentile
// Exact k-th smallest selection for two ranks at once. Pass d (d = 0, 1, 2) histograms the
// digit d of the order-preserving key of the elements whose higher digits match the prefix
// selected so far for that rank; a single-CTA scan then picks the digit holding the rank.
// Digits: bits [31:21] (2048 bins), [20:10] (2048 bins), [9:0] (1024 bins).

constexpr int PCT_BINS = 2048;

struct PctState
{
    unsigned int prefix[2];  // selected high bits per rank
    unsigned int rank[2];    // remaining rank inside the prefix
    unsigned int count;      // number of candidate elements (frame or reticle disc)
};

__device__ __forceinline__ int digit_shift(int d) { return d == 0 ? 21 : (d == 1 ? 10 : 0); }
__device__ __forceinline__ unsigned int digit_mask(int d) { return d == 2 ? 1023u : 2047u; }
__device__ __forceinline__ unsigned int high_mask(int d) { return d == 0 ? 0u : (d == 1 ? 0xffe00000u : 0xfffffc00u); }

__device__ __forceinline__ bool in_reticle(size_t e, int W, int H, unsigned int r2, int use)
{
    if (!use)
        return true;
    const int x = static_cast<int>(e % W), y = static_cast<int>(e / W);
    const int dx = x - W / 2, dy = y - H / 2;
    return static_cast<unsigned int>(dx * dx + dy * dy) <= r2;
}

__global__ void k_pct_hist(const float* __restrict__ f, int W, int H, int pitch, unsigned int r2, int use_reticle,
                           const PctState* __restrict__ st, int d, unsigned int* __restrict__ hist,
                           const CycleCtl* ctl)
{
    if (ctl && !(ctl->render && ctl->pct_enable))
        return;
    __shared__ unsigned int sh[2][PCT_BINS];
    for (int i = threadIdx.x; i < 2 * PCT_BINS; i += blockDim.x)
        (&sh[0][0])[i] = 0u;
    __syncthreads();
    const size_t n = static_cast<size_t>(W) * H;
    const int sft = digit_shift(d);
    const unsigned int dm = digit_mask(d), hm = high_mask(d);
    const unsigned int pre0 = (d == 0) ? 0u : st->prefix[0];
    const unsigned int pre1 = (d == 0) ? 0u : st->prefix[1];
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        if (!in_reticle(e, W, H, r2, use_reticle))
            continue;
        const size_t a = pitch == W ? e : (e / W) * static_cast<size_t>(pitch) + e % W;
        const unsigned int k = float_key(f[a]);
        const unsigned int dig = (k >> sft) & dm;
        if ((k & hm) == pre0)
            atomicAdd(&sh[0][dig], 1u);
        if (d > 0 && (k & hm) == pre1)
            atomicAdd(&sh[1][dig], 1u);
    }
    __syncthreads();
    const int nh = d == 0 ? 1 : 2;
    for (int h = 0; h < nh; ++h)
        for (int i = threadIdx.x; i < PCT_BINS; i += blockDim.x)
            if (sh[h][i])
                atomicAdd(&hist[h * PCT_BINS + i], sh[h][i]);
}

// One CTA of 1024 threads: prefix scan of the histogram(s), choose the digit for each rank.
__global__ void k_pct_select(unsigned int* __restrict__ hist, PctState* __restrict__ st, int d, float lower,
                             float upper, float* __restrict__ range, const CycleCtl* ctl)
{
    if (ctl && !(ctl->render && ctl->pct_enable))
        return;
    __shared__ unsigned int scan[PCT_BINS];
    __shared__ unsigned int warp_tot[32];
    const int nb = (d == 2) ? 1024 : PCT_BINS;
    const int sft = digit_shift(d);
    for (int r = 0; r < 2; ++r)
    {
        const unsigned int* hh = hist + ((d == 0) ? 0 : r) * PCT_BINS;
        // inclusive scan of nb bins, two bins per thread
        const int i0 = threadIdx.x * 2;
        unsigned int a = (i0 < nb) ? hh[i0] : 0u, b = (i0 + 1 < nb) ? hh[i0 + 1] : 0u;
        unsigned int v = a + b;
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int o = 1; o < 32; o <<= 1)
        {
            const unsigned int t = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o)
                v += t;
        }
        if (lane == 31)
            warp_tot[w] = v;
        __syncthreads();
        if (w == 0)
        {
            unsigned int t = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1)
            {
                const unsigned int u = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o)
                    t += u;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        const unsigned int before = (w > 0 ? warp_tot[w - 1] : 0u) + v - (a + b);
        if (i0 < nb)
            scan[i0] = before + a;
        if (i0 + 1 < nb)
            scan[i0 + 1] = before + a + b;
        __syncthreads();
        if (threadIdx.x == 0)
        {
            unsigned int rank;
            if (d == 0)
            {
                // total candidates and the percentile index, float32 as percentile.cu:85, clamped
                const unsigned int total = scan[nb - 1];
                st->count = total;
                const float pct = r == 0 ? lower : upper;
                unsigned int idx = static_cast<unsigned int>(__fmul_rn(__fdiv_rn(pct, 100.0f), static_cast<float>(total)));
                if (total == 0)
                    idx = 0;
                else if (idx >= total)
                    idx = total - 1;
                rank = idx;
                st->prefix[r] = 0u;
            }
            else
            {
                rank = st->rank[r];
            }
            // first bin whose inclusive count exceeds rank
            int lo = 0, hi = nb - 1;
            while (lo < hi)
            {
                const int mid = (lo + hi) >> 1;
                if (scan[mid] > rank)
                    hi = mid;
                else
                    lo = mid + 1;
            }
            const unsigned int below = lo > 0 ? scan[lo - 1] : 0u;
            st->rank[r] = rank - below;
            st->prefix[r] |= static_cast<unsigned int>(lo) << sft;
            if (d == 2)
            {
                float val = st->count ? key_float(st->prefix[r]) : 0.f;
                // ContrastApi::update_contrast clamps both ends to >= 1
                range[r] = val > 1.0f ? val : 1.0f;
            }
        }
        __syncthreads();
        if (d == 0)
        {
            // both ranks use the same histogram in pass 0
        }
    }
}

size_t percentile_workspace(size_t n)
{
    (void)n;
    return 2 * PCT_BINS * sizeof(unsigned int) * 3 + sizeof(PctState) + 256;
}

hv_status percentile(const float* frame, int W, int H, float lower, float upper, float reticle_scale, float* range,
                     void* work, cudaStream_t st, const CycleCtl* ctl)
{
    return percentile_pitched(frame, W, H, W, lower, upper, reticle_scale, range, work, st, ctl);
}

// The W x H sub-image of rows `pitch` floats apart (the YZ cut's columns between the offsets,
// compute_percentile_yz_view's cudaMemcpy2DAsync, percentile.cu:230-250).
hv_status percentile_pitched(const float* frame, int W, int H, int pitch, float lower, float upper,
                             float reticle_scale, float* range, void* work, cudaStream_t st, const CycleCtl* ctl)
{
    const size_t n = static_cast<size_t>(W) * H;
    if (n == 0 || pitch < W)
        return HV_INVALID_VALUE;
    unsigned int* hist = static_cast<unsigned int*>(work);  // 3 passes x 2 ranks x PCT_BINS
    PctState* state = reinterpret_cast<PctState*>(hist + 3 * 2 * PCT_BINS);
    HV_CUDA_TRY(cudaMemsetAsync(hist, 0, 3 * 2 * PCT_BINS * sizeof(unsigned int), st));
    int use_reticle = 0;
    unsigned int r2 = 0;
    if (reticle_scale > 0.f)
    {
        // radius = (uint)(scale * min(W, H) / 2) (percentile.cu:113, 163)
        const unsigned int radius = static_cast<unsigned int>(reticle_scale * static_cast<float>(W < H ? W : H) / 2.0f);
        if (radius > 0)
        {
            use_reticle = 1;
            r2 = radius * radius;
        }
    }
    int grid = ew_grid(n);
    if (grid > 152 * 4)
        grid = 152 * 4;
    for (int d = 0; d < 3; ++d)
    {
        k_pct_hist<<<grid, EW_THREADS, 0, st>>>(frame, W, H, pitch, r2, use_reticle, state, d, hist + d * 2 * PCT_BINS,
                                                ctl);
        HV_LAUNCH_CHECK();
        k_pct_select<<<1, 1024, 0, st>>>(hist + d * 2 * PCT_BINS, state, d, lower, upper, range, ctl);
        HV_LAUNCH_CHECK();
    }
    count_launch(6);
    return HV_OK;
}

// ====================================================================================== contrast + ushort

__device__ __forceinline__ uint16_t to_ushort(float x)
{
    if (x <= 0.0f)
        return 0;
    const unsigned int u = static_cast<unsigned int>(x);
    if (u > 65535u)
        return 65535;
    return static_cast<uint16_t>(u);
}

__global__ void k_contrast_ushort(const float* __restrict__ in, const float* __restrict__ range, int invert, int apply,
                                  uint16_t* __restrict__ out, size_t n, const CycleCtl* ctl)
{
    if (!ctl_render(ctl))
        return;
    if (ctl)
        out += static_cast<size_t>(ctl->out_slot) * n;
    float mn = 0.f, factor = 1.f;
    if (apply)
    {
        float lo = range[0], hi = range[1];
        if (invert)
        {
            const float t = lo;
            lo = hi;
            hi = t;
        }
        mn = lo;
        factor = __fdiv_rn(65535.0f, __fadd_rn(__fsub_rn(hi, lo), FLT_EPSILON));
    }
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        float v = in[e];
        if (apply)
            v = __fmul_rn(factor, __fsub_rn(v, mn));
        out[e] = to_ushort(v);
    }
}

// ====================================================================================== filter2D view

// The filter2D view frame (Pipe::insert_filter2d_view, pipe.cc:526-546): the stored spectrum
// (spectrum x multiplier, FFT layout: apply_mask by the mask or by the masked transfer function)
// quadrant-swapped (shift_corners) and taken to its modulus (complex_to_modulus with one bin).
__global__ void k_f2d_view(const float2* __restrict__ spec, const float2* __restrict__ mult, int W, int H,
                           float* __restrict__ out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W)
        return;
    const size_t src = static_cast<size_t>((y + H / 2) % H) * W + (x + W / 2) % W;
    const float2 a = spec[src], m = mult[src];
    const float re = a.x * m.x - a.y * m.y, im = a.x * m.y + a.y * m.x;
    out[static_cast<size_t>(y) * W + x] = hypotf(re, im);
}

hv_status filter2d_view_frame(const float2* spec, const float2* mult, int W, int H, float* out, cudaStream_t st)
{
    if ((W & 1) || (H & 1))
        return HV_INVALID_VALUE;
    dim3 block(128), grid((W + 127) / 128, H);
    k_f2d_view<<<grid, block, 0, st>>>(spec, mult, W, H, out);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

// Contrast (apply_contrast_correction when `apply`) then float_to_ushort_normalized
// (tools_conversion.cu:389-393): trunc(x * 65535) saturated to [0, 65535] (NaN -> 0), the
// filter2D view's conversion.
__global__ void k_contrast_ushort_normalized(const float* __restrict__ in, const float* __restrict__ range, int invert,
                                             int apply, uint16_t* __restrict__ out, size_t n)
{
    float mn = 0.f, factor = 1.f;
    if (apply)
    {
        float lo = range[0], hi = range[1];
        if (invert)
        {
            const float t = lo;
            lo = hi;
            hi = t;
        }
        mn = lo;
        factor = __fdiv_rn(65535.0f, __fadd_rn(__fsub_rn(hi, lo), FLT_EPSILON));
    }
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        float v = in[e];
        if (apply)
            v = __fmul_rn(factor, __fsub_rn(v, mn));
        const float w = __fmul_rn(v, 65535.0f);
        out[e] = w >= 65535.0f ? static_cast<uint16_t>(65535) : (w > 0.0f ? static_cast<uint16_t>(w) : static_cast<uint16_t>(0));
    }
}

hv_status contrast_to_ushort_normalized(const float* frame, const float* range, int invert, int apply, uint16_t* out,
                                        size_t n, cudaStream_t st)
{
    k_contrast_ushort_normalized<<<ew_grid(n), EW_THREADS, 0, st>>>(frame, range, invert, apply, out, n);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status contrast_to_ushort(const float* frame, const float* range, int invert, int apply, uint16_t* out, size_t n,
                             cudaStream_t st, const CycleCtl* ctl)
{
    k_contrast_ushort<<<ew_grid(n), EW_THREADS, 0, st>>>(frame, range, invert, apply, out, n, ctl);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

}  // namespace hv
