// Time-transformation cuts: the XZ (T x W) and YZ (H x T) slices through the p_acc volume at a
// cursor position, with every one of the T bins or components.
//
// Reference behaviour (Holovibes):
//   slices         Backend/cuda_sources/stft.cu:17-115 (fill_32bit_slices: XZ[t][x] = mean over
//                  y in [ymin, ymax] of view(p_acc[t][y][x]), YZ[y][t] = mean over x in [xmin, xmax];
//                  view = hypotf (modulus, phase increase, composite), hypotf^2, or
//                  atanf(Im / Re) + pi/2 (argument), 0 otherwise)
//   call site      Backend/sources/compute/fourier_transform.cc:462-503 (x.start < W, y.start < H)
//   p_acc          STFT over all T bins (stft.cu:9-15), H V (PCA), FFT_t(H V_Q V_Q^H) (SSA_STFT),
//                  the ring itself (NONE, fourier_transform.cc:213-224)
//
// GB300 design: the reference keeps the whole T x HW p_acc volume to read two thin slices of it;
// here only the pixels of the two bands are transformed: a CTA stages the T samples of 32 band
// pixels in shared memory and its warps contract them with one weight row each (32 pixels, one
// bin: the weight is a broadcast), writing the view value of every (pixel, bin); a second kernel
// averages over the band width in the reference's order (float sum from the first column / row).
#include <math.h>

#include "hv_internal.h"

namespace hv {

constexpr int CUT_PX = 32;       // band pixels per CTA (one per lane)
constexpr int CUT_THREADS = 256; // 8 warps: bins strided over warps
constexpr int CUT_MAX_T = 512;   // 32 pixels x T samples x 8 B of shared memory <= 128 KB

struct CutGeom
{
    int W, H, T;
    int xmin, nx;  // YZ band columns
    int ymin, ny;  // XZ band rows
    long long n_xz, npix;  // XZ band pixels (W ny), all band pixels (W ny + H nx)
};

__device__ __forceinline__ size_t cut_pixel(const CutGeom& g, long long p)
{
    if (p < g.n_xz)
    {
        const long long j = p / g.W, x = p - j * g.W;
        return static_cast<size_t>(g.ymin + j) * g.W + static_cast<size_t>(x);
    }
    const long long q = p - g.n_xz;
    const long long y = q / g.nx, i = q - y * g.nx;
    return static_cast<size_t>(y) * g.W + static_cast<size_t>(g.xmin + i);
}

__device__ __forceinline__ float cut_view(float re, float im, int img_type)
{
    if (img_type == HV_IMG_MODULUS || img_type == HV_IMG_PHASE_INCREASE || img_type == 4)
        return hypotf(re, im);
    if (img_type == HV_IMG_SQUARED_MODULUS)
    {
        const float m = hypotf(re, im);
        return m * m;
    }
    if (img_type == HV_IMG_ARGUMENT)
        return static_cast<float>(static_cast<double>(atanf(__fdiv_rn(im, re))) + 1.57079632679489661923);
    return 0.0f;
}

// vals[p][t] = view(sum_s ring[s][pix(p)] w[t][s]) for the CUT_PX band pixels of this CTA.
__global__ void __launch_bounds__(CUT_THREADS) k_cut_values(const float2* __restrict__ ring, const float2* __restrict__ w,
                                                            CutGeom g, int img_type, float* __restrict__ vals)
{
    extern __shared__ float2 s_x[];  // [T][CUT_PX]
    const long long p0 = static_cast<long long>(blockIdx.x) * CUT_PX;
    const int T = g.T;
    const size_t HW = static_cast<size_t>(g.W) * g.H;
    for (int e = threadIdx.x; e < T * CUT_PX; e += CUT_THREADS)
    {
        const int s = e / CUT_PX, l = e - s * CUT_PX;
        const long long p = p0 + l;
        s_x[e] = p < g.npix ? ring[static_cast<size_t>(s) * HW + cut_pixel(g, p)] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long p = p0 + lane;
    for (int t = warp; t < T; t += CUT_THREADS / 32)
    {
        const float2* wt = w + static_cast<size_t>(t) * T;
        float xr = 0.f, xi = 0.f;
        for (int s = 0; s < T; ++s)
        {
            const float2 x = s_x[s * CUT_PX + lane];
            const float2 c = __ldg(wt + s);
            xr = fmaf(x.x, c.x, fmaf(-x.y, c.y, xr));
            xi = fmaf(x.x, c.y, fmaf(x.y, c.x, xi));
        }
        if (p < g.npix)
            vals[static_cast<size_t>(p) * T + t] = cut_view(xr, xi, img_type);
    }
}

// XZ[t][x] = (sum_{j < ny} vals[j W + x][t]) / ny, YZ[y][t] = (sum_{i < nx} vals[n_xz + y nx + i][t]) / nx
__global__ void k_cut_reduce(const float* __restrict__ vals, CutGeom g, float* __restrict__ xz, float* __restrict__ yz)
{
    const int T = g.T;
    const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const long long n_xz_out = static_cast<long long>(T) * g.W;
    if (e < n_xz_out)
    {
        const int t = static_cast<int>(e / g.W), x = static_cast<int>(e - static_cast<long long>(t) * g.W);
        float sum = 0.f;
        for (int j = 0; j < g.ny; ++j)
            sum += vals[(static_cast<size_t>(j) * g.W + x) * T + t];
        xz[e] = __fdiv_rn(sum, static_cast<float>(g.ny));
    }
    else if (e < n_xz_out + static_cast<long long>(g.H) * T)
    {
        const long long f = e - n_xz_out;
        const int y = static_cast<int>(f / T), t = static_cast<int>(f - static_cast<long long>(y) * T);
        float sum = 0.f;
        for (int i = 0; i < g.nx; ++i)
            sum += vals[(static_cast<size_t>(g.n_xz) + static_cast<size_t>(y) * g.nx + i) * T + t];
        yz[f] = __fdiv_rn(sum, static_cast<float>(g.nx));
    }
}

// PCA: the p_acc components are the eigenvector columns, evecs[j T + s] (complex128) -> w[j][s].
__global__ void k_c128_to_c64(const double2* __restrict__ in, float2* __restrict__ out, size_t n)
{
    for (size_t e = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < n;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
        out[e] = make_float2(static_cast<float>(in[e].x), static_cast<float>(in[e].y));
}

hv_status evecs_to_weights(const double2* evecs, int T, float2* w, cudaStream_t st)
{
    const size_t n = static_cast<size_t>(T) * T;
    const int grid = static_cast<int>((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
    k_c128_to_c64<<<grid, 256, 0, st>>>(evecs, w, n);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

static CutGeom cut_geom(int W, int H, int T, int xmin, int xmax, int ymin, int ymax)
{
    CutGeom g;
    g.W = W;
    g.H = H;
    g.T = T;
    g.xmin = xmin;
    g.nx = xmax - xmin + 1;
    g.ymin = ymin;
    g.ny = ymax - ymin + 1;
    g.n_xz = static_cast<long long>(W) * g.ny;
    g.npix = g.n_xz + static_cast<long long>(H) * g.nx;
    return g;
}

bool cuts_supported(int T) { return T >= 1 && T <= CUT_MAX_T; }

size_t cuts_workspace(int W, int H, int T, int nx, int ny)
{
    return (static_cast<size_t>(W) * ny + static_cast<size_t>(H) * nx) * T * sizeof(float) + 256;
}

hv_status time_cuts(const float2* ring, int T, int W, int H, const float2* weights_all, int xmin, int xmax, int ymin,
                    int ymax, int img_type, float* xz, float* yz, void* work, cudaStream_t st)
{
    if (!ring || !weights_all || !xz || !yz || !work || W <= 0 || H <= 0)
        return HV_INVALID_VALUE;
    if (xmin < 0 || xmax < xmin || xmax >= W || ymin < 0 || ymax < ymin || ymax >= H)
        return HV_INVALID_VALUE;
    if (!cuts_supported(T))
    {
        set_last_error_msg("time cuts: time window above 512 frames");
        return HV_ERR_UNSUPPORTED;
    }
    const CutGeom g = cut_geom(W, H, T, xmin, xmax, ymin, ymax);
    float* vals = static_cast<float*>(work);
    const size_t smem = static_cast<size_t>(T) * CUT_PX * sizeof(float2);
    if (smem > 48 * 1024)
        HV_CUDA_TRY(cudaFuncSetAttribute(k_cut_values, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem)));
    const long long blocks = (g.npix + CUT_PX - 1) / CUT_PX;
    k_cut_values<<<static_cast<unsigned>(blocks), CUT_THREADS, smem, st>>>(ring, weights_all, g, img_type, vals);
    HV_LAUNCH_CHECK();
    const long long outs = static_cast<long long>(T) * W + static_cast<long long>(H) * T;
    k_cut_reduce<<<static_cast<unsigned>((outs + 255) / 256), 256, 0, st>>>(vals, g, xz, yz);
    HV_LAUNCH_CHECK();
    count_launch(2);
    return HV_OK;
}

}  // namespace hv
