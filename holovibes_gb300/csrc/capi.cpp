// C ABI entry points for the compute steps, settings and library state.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>

#include "hv_internal.h"

namespace hv {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

void set_last_error(const char* msg, const char* file, int line)
{
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s (%s:%d)", msg ? msg : "error", file, line);
    g_last_error = buf;
}

void set_last_error_msg(const char* msg) { g_last_error = msg ? msg : ""; }

void count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

void settings_default(hv_settings* s);
hv_status settings_from_json(const char* text, hv_settings* s);
hv_status settings_validate(hv_settings* s, const hv_frame_desc* fd);

}  // namespace hv

using namespace hv;

static inline cudaStream_t S(void* s) { return static_cast<cudaStream_t>(s); }

extern "C" {

const char* hv_version(void) { return "holovibes_gb300 0.1.0 (sm_103a)"; }

const char* hv_last_error(void) { return g_last_error.c_str(); }

uint64_t hv_kernel_launches(void) { return launch_count(); }

void hv_settings_default(hv_settings* s)
{
    if (s)
        settings_default(s);
}

hv_status hv_settings_from_json(const char* json, hv_settings* s) { return settings_from_json(json, s); }

hv_status hv_settings_validate(hv_settings* s, const hv_frame_desc* fd) { return settings_validate(s, fd); }

int hv_fft_size_supported(int n) { return fft_size_supported(n) ? 1 : 0; }

void hv_fft_engine_mode(int mode) { set_fft_engine(mode); }

hv_status hv_fft_status(void) { return fft_status(); }

void hv_spatial_sub_batch_mb(int mb) { set_spatial_sub_batch_mb(mb); }

hv_status hv_fresnel_lens(void* lens_c64, int width, int height, float lambda, float z, float pixel_size_um,
                          int lens_mode, void* stream)
{
    if (!lens_c64 || width <= 0 || height <= 0)
        return HV_INVALID_VALUE;
    return make_fresnel_lens(static_cast<float2*>(lens_c64), width, height, lambda, z, pixel_size_um, lens_mode,
                             S(stream));
}

hv_status hv_angular_spectrum_lens(void* lens_c64, int width, int height, float lambda, float z,
                                   float pixel_size_um, int lens_mode, void* stream)
{
    if (!lens_c64 || width <= 0 || height <= 0 || (width & 1) || (height & 1))
        return HV_INVALID_VALUE;
    return make_spectral_lens(static_cast<float2*>(lens_c64), width, height, lambda, z, pixel_size_um, lens_mode,
                              S(stream));
}

hv_status hv_spatial_transform(const void* raw, int raw_bytes, int big_endian, int width, int height, int batch,
                               int space, const void* lens_c64, void* work_c64, void* ring_c64, int slot0,
                               int nslots, void* stream)
{
    const int kind = raw_kind(raw_bytes, big_endian);
    if (!raw || !ring_c64 || kind < 0 || width <= 0 || height <= 0 || batch < 0 || nslots <= 0 || slot0 < 0 ||
        slot0 >= nslots || batch > nslots)
        return HV_INVALID_VALUE;
    if (space != HV_SPACE_NONE && (!lens_c64 || !work_c64))
        return HV_INVALID_VALUE;
    return spatial_transform(raw, kind, width, height, batch, space, static_cast<const float2*>(lens_c64),
                             static_cast<float2*>(work_c64), static_cast<float2*>(ring_c64), slot0, nslots, S(stream));
}

hv_status hv_filter2d_mask(void* dst_c64, int width, int height, int n1, int n2, int smooth_low, int smooth_high,
                           int multiply, void* stream)
{
    return filter2d_mask(static_cast<float2*>(dst_c64), width, height, n1, n2, smooth_low, smooth_high, multiply,
                         S(stream));
}

hv_status hv_spatial_transform_filter2d(const void* raw, int raw_bytes, int big_endian, int width, int height,
                                        int batch, int space, const void* lens_c64, const void* mask_c64,
                                        void* work_c64, void* work2_c64, void* ring_c64, int slot0, int nslots,
                                        void* stream)
{
    const int kind = raw_kind(raw_bytes, big_endian);
    if (!raw || !ring_c64 || !work_c64 || kind < 0 || width <= 0 || height <= 0 || batch < 0 || nslots <= 0 ||
        slot0 < 0 || slot0 >= nslots || batch > nslots)
        return HV_INVALID_VALUE;
    if (space != HV_SPACE_ANGULARSP && !mask_c64)
        return HV_INVALID_VALUE;
    if (space != HV_SPACE_NONE && !lens_c64)
        return HV_INVALID_VALUE;
    return spatial_transform(raw, kind, width, height, batch, space, static_cast<const float2*>(lens_c64),
                             static_cast<float2*>(work_c64), static_cast<float2*>(ring_c64), slot0, nslots, S(stream),
                             nullptr, static_cast<const float2*>(mask_c64), static_cast<float2*>(work2_c64));
}

hv_status hv_fft2d(const void* in_c64, void* out_c64, int n0, int n1, int batch, int inverse, float scale,
                   void* stream)
{
    if (!in_c64 || !out_c64 || batch <= 0)
        return HV_INVALID_VALUE;
    return fft2d(static_cast<const float2*>(in_c64), static_cast<float2*>(out_c64), n0, n1, batch, inverse, scale,
                 S(stream));
}

hv_status hv_fft_rows(const void* in, int in_bytes, int big_endian, void* out_c64, int width, int height, int batch,
                      const void* premul_c64, int inverse, float scale, int slot0, int nslots, void* stream)
{
    const int kind = raw_kind(in_bytes, big_endian);
    if (!in || !out_c64 || kind < 0 || batch <= 0 || nslots <= 0 || slot0 < 0 || slot0 >= nslots || batch > nslots)
        return HV_INVALID_VALUE;
    return fft_rows_pass(in, kind, static_cast<float2*>(out_c64), width, height, batch,
                         static_cast<const float2*>(premul_c64), inverse, scale, slot0, nslots, S(stream));
}

hv_status hv_fft_cols(const void* in_c64, void* out_c64, int width, int height, int batch, const void* postmul_c64,
                      int mode, float scale, int slot0, int nslots, void* stream)
{
    if (!in_c64 || !out_c64 || batch <= 0 || mode < 0 || mode > 2 || (mode == 2 && !postmul_c64) || nslots <= 0 ||
        slot0 < 0 || slot0 >= nslots || batch > nslots)
        return HV_INVALID_VALUE;
    return fft_cols_pass(static_cast<const float2*>(in_c64), static_cast<float2*>(out_c64), width, height, batch,
                         static_cast<const float2*>(postmul_c64), mode, scale, slot0, nslots, S(stream));
}

hv_status hv_time_view(const void* ring_c64, int T, int width, int height, const void* weights_c64, int K,
                       int img_type, float scale, int shift, float* out_f32, double* partials_f64, void* stream)
{
    if (!ring_c64 || !weights_c64 || !out_f32 || img_type < 0 || img_type > HV_IMG_ARGUMENT)
        return HV_INVALID_VALUE;
    return time_view(static_cast<const float2*>(ring_c64), T, width, height, static_cast<const float2*>(weights_c64), K,
                     img_type, scale, shift, out_f32, partials_f64, S(stream));
}

hv_status hv_time_view_planes(const void* planes_u16, const void* ring_c64, int ring_slot0, int ring_n, int T,
                              int width, int height, const void* weights_c64, int K, int img_type, float scale,
                              int shift, float* out_f32, double* partials_f64, void* stream)
{
    if (!planes_u16 || (ring_n > 0 && !ring_c64) || !weights_c64 || !out_f32 || img_type < 0 ||
        img_type > HV_IMG_ARGUMENT)
        return HV_INVALID_VALUE;
    return time_view_planes(static_cast<const uint16_t*>(planes_u16), static_cast<const float2*>(ring_c64),
                            ring_slot0, ring_n, T, width, height, static_cast<const float2*>(weights_c64), K, img_type,
                            scale, shift, out_f32, partials_f64, S(stream));
}

int hv_time_view_partials(int width, int height) { return time_view_partials(width, height); }

void hv_time_view_mode(int mode) { set_view_mode(mode); }

hv_status hv_moment_bin_weights(float* bin_w_f32, int T, int pmin, int pmax, int img_type, float camera_fps,
                                void* stream)
{
    if (!is_moment(img_type))
        return HV_WRONG_IMG_TYPE;
    return moment_bin_weights(bin_w_f32, T, pmin, pmax, img_type - HV_IMG_MOMENTS_0, camera_fps, S(stream));
}

hv_status hv_time_moments(const void* ring_c64, int T, int width, int height, const void* weights_c64, int K,
                          const float* bin_w_f32, int shift, float* out_f32, double* partials_f64, void* stream)
{
    if (!ring_c64 || !weights_c64 || !bin_w_f32 || !out_f32)
        return HV_INVALID_VALUE;
    return time_view(static_cast<const float2*>(ring_c64), T, width, height, static_cast<const float2*>(weights_c64), K,
                     HV_IMG_MOMENTS_0, 1.0f, shift, out_f32, partials_f64, S(stream), nullptr, bin_w_f32);
}

hv_status hv_ssa_weights(const void* eigenvectors_c128, int T, int q_start, int q_width, int pmin, int pmax,
                         void* weights_c64, void* stream)
{
    if (!eigenvectors_c128 || !weights_c64 || T <= 0 || pmin < 0 || pmax < pmin || pmax >= T || q_width < 0 ||
        q_start < 0)
        return HV_INVALID_VALUE;
    // fourier_transform.cc:409-412: width 0 keeps every column
    const int qmin = q_width != 0 ? q_start : 0, qn = q_width != 0 ? q_width : T;
    if (qmin + qn > T)
        return HV_INVALID_VALUE;
    return ssa_weights(static_cast<const double2*>(eigenvectors_c128), T, qmin, qn, pmin, pmax - pmin + 1,
                       static_cast<float2*>(weights_c64), S(stream));
}

hv_status hv_phase_increase(const void* ring_c64, int T, int width, int height, const void* w_c64, void* pred_c64,
                            float* hist_f32, int first, int use_hist, float* out_f32, void* minmax, void* stream)
{
    if (width <= 0 || height <= 0)
        return HV_INVALID_VALUE;
    return phase_increase(static_cast<const float2*>(ring_c64), T, static_cast<size_t>(width) * height,
                          static_cast<const float2*>(w_c64), static_cast<float2*>(pred_c64), hist_f32, first, use_hist,
                          out_f32, static_cast<float2*>(minmax), S(stream));
}

size_t hv_phase_increase_workspace(size_t npix) { return phase_increase_minmax_count(npix) * sizeof(float2); }

hv_status hv_rescale_float(const float* in_f32, size_t npix, const void* minmax, float post_scale, float* out_f32,
                           void* stream)
{
    return rescale_float(in_f32, npix, static_cast<const float2*>(minmax), post_scale, out_f32, S(stream));
}

hv_status hv_time_cuts(const void* ring_c64, int T, int width, int height, const void* weights_c64, int xmin, int xmax,
                       int ymin, int ymax, int img_type, float* xz_f32, float* yz_f32, void* work, void* stream)
{
    return time_cuts(static_cast<const float2*>(ring_c64), T, width, height, static_cast<const float2*>(weights_c64),
                     xmin, xmax, ymin, ymax, img_type, xz_f32, yz_f32, work, S(stream));
}

size_t hv_time_cuts_workspace(int width, int height, int T, int xmin, int xmax, int ymin, int ymax)
{
    if (width <= 0 || height <= 0 || T <= 0 || xmax < xmin || ymax < ymin)
        return 0;
    return cuts_workspace(width, height, T, xmax - xmin + 1, ymax - ymin + 1);
}

hv_status hv_unpack_12_to_16(const void* in, size_t in_bytes, uint16_t* out, size_t out_count, void* stream)
{
    return unpack_packed(12, in, in_bytes, out, out_count, S(stream));
}

hv_status hv_unpack_10_to_16(const void* in, size_t in_bytes, uint16_t* out, size_t out_count, void* stream)
{
    return unpack_packed(10, in, in_bytes, out, out_count, S(stream));
}

size_t hv_time_view_tc_workspace(int K, int T) { return view_tc_supported(K) ? view_tc_workspace(K, T) : 0; }

hv_status hv_time_view_tc(const void* ring_c64, int T, int width, int height, const void* weights_c64, int K,
                          int img_type, float scale, int shift, float* out_f32, double* partials_f64, void* work,
                          void* stream)
{
    if (!ring_c64 || !weights_c64 || !out_f32 || !work || img_type < 0 || img_type > HV_IMG_ARGUMENT || T <= 0 ||
        width <= 0 || height <= 0)
        return HV_INVALID_VALUE;
    hv_status r = view_tc_prepare(static_cast<const float2*>(weights_c64), K, T, work, S(stream));
    if (r != HV_OK)
        return r;
    return view_tc(static_cast<const float2*>(ring_c64), T, width, height, K, img_type, scale, shift, out_f32,
                   partials_f64, work, S(stream));
}

hv_status hv_time_view_tc_prepare(const void* weights_c64, int K, int T, void* work, void* stream)
{
    if (!weights_c64 || !work || T <= 0)
        return HV_INVALID_VALUE;
    return view_tc_prepare(static_cast<const float2*>(weights_c64), K, T, work, S(stream));
}

hv_status hv_time_view_tc_run(const void* ring_c64, int T, int width, int height, int K, int img_type, float scale,
                              int shift, float* out_f32, double* partials_f64, void* work, void* stream)
{
    if (!ring_c64 || !out_f32 || !work || img_type < 0 || img_type > HV_IMG_ARGUMENT || T <= 0 || width <= 0 ||
        height <= 0)
        return HV_INVALID_VALUE;
    return view_tc(static_cast<const float2*>(ring_c64), T, width, height, K, img_type, scale, shift, out_f32,
                   partials_f64, work, S(stream));
}

hv_status hv_time_view_tc_status(const void* work)
{
    if (!work)
        return HV_INVALID_VALUE;
    int flag = 0;
    HV_CUDA_TRY(cudaMemcpy(&flag, work, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag)
    {
        set_last_error_msg("tensor-core time view: a bounded wait gave up");
        return HV_ERR_TIMEOUT;
    }
    return HV_OK;
}

hv_status hv_stft_weights(void* weights_c64, int T, int pmin, int pmax, void* stream)
{
    if (!weights_c64 || pmin < 0 || pmax < pmin || pmax >= T)
        return HV_INVALID_VALUE;
    return stft_weights(static_cast<float2*>(weights_c64), T, pmin, pmax, S(stream));
}

hv_status hv_pca_covariance(const void* ring_c64, int T, size_t npix, void* cov_c128, void* work, void* stream)
{
    if (!ring_c64 || !cov_c128 || !work)
        return HV_INVALID_VALUE;
    return pca_covariance(static_cast<const float2*>(ring_c64), T, npix, static_cast<double2*>(cov_c128), work,
                          S(stream));
}

size_t hv_pca_cov_workspace(int T, size_t npix) { return pca_cov_workspace(T, npix); }

void hv_pca_covariance_mode(int mode) { set_cov_mode(mode); }

void hv_pca_cov_incremental(int enable) { set_cov_incremental(enable != 0); }

size_t hv_pca_planes_bytes(int T, size_t npix, int real)
{
    return cov_planes_supported(T, npix) ? cov_planes_bytes(T, npix, real ? 1 : 0) : 0;
}

hv_status hv_pca_split_planes(const void* ring_c64, int T, size_t npix, int slot0, int n, int real, void* planes,
                              void* stream)
{
    if (!ring_c64 || !planes)
        return HV_INVALID_VALUE;
    return cov_split_planes(static_cast<const float2*>(ring_c64), T, npix, slot0, n, static_cast<uint16_t*>(planes),
                            real ? 1 : 0, S(stream));
}

hv_status hv_pca_covariance_planes(const void* planes, int T, size_t npix, int real, unsigned int blocks,
                                   void* cov_c128, void* work, void* stream)
{
    if (!planes || !cov_c128 || !work)
        return HV_INVALID_VALUE;
    return pca_covariance_planes(static_cast<const uint16_t*>(planes), T, npix, static_cast<double2*>(cov_c128), work,
                                 blocks, real ? 1 : 0, S(stream));
}

hv_status hv_pca_covariance_status(const void* work)
{
    if (!work)
        return HV_INVALID_VALUE;
    return pca_cov_status(work);
}

hv_status hv_pca_eigh(void* cov_c128, int T, double* eigenvalues, void* eigenvectors_c128, int pmin, int pmax,
                      void* weights_c64, void* work, void* stream)
{
    if (!cov_c128 || !eigenvalues || !eigenvectors_c128 || !work || T <= 0)
        return HV_INVALID_VALUE;
    if (weights_c64 && (pmin < 0 || pmax < pmin || pmax >= T))
        return HV_INVALID_VALUE;
    // the eigenvectors of ranks pmin..pmax (when that range is valid) are refined in FP64
    const bool range = pmin >= 0 && pmax >= pmin && pmax < T;
    return pca_eigh(static_cast<double2*>(cov_c128), T, eigenvalues, static_cast<double2*>(eigenvectors_c128), pmin,
                    pmax, static_cast<float2*>(weights_c64), work, S(stream), range ? pmin : 0, range ? pmax : -1);
}

size_t hv_pca_eigh_workspace(int T) { return pca_eigh_workspace(T); }

void hv_pca_eig_precision(int precision) { set_eig_precision(precision == HV_EIG_FP64 ? HV_EIG_FP64 : HV_EIG_FP32); }

void hv_pca_eig_cholqr(int enable) { set_eig_cholqr(enable); }

hv_status hv_unwrap_2d(const float* in, float* out, int width, int height, void* work, void* stream)
{
    if (!in || !out || !work)
        return HV_INVALID_VALUE;
    return unwrap_2d(in, out, width, height, work, S(stream));
}

size_t hv_unwrap_workspace(int width, int height) { return unwrap_workspace(width, height); }

hv_status hv_renormalize(float* frame, size_t n, int renorm_constant, const double* partials_f64, int npartials,
                         void* work, void* stream)
{
    if (!frame || !work || n == 0)
        return HV_INVALID_VALUE;
    float* factors = reinterpret_cast<float*>(static_cast<char*>(work) + reduce_workspace(n));
    hv_status r = renorm_factors(frame, n, renorm_constant, partials_f64, npartials, factors, work, S(stream));
    if (r != HV_OK)
        return r;
    // one-row frame: renormalise in place, no shift, no accumulation
    return renorm_shift_accumulate(frame, frame, static_cast<int>(n), 1, factors, 0, nullptr, 0, 0, 0, 0, 0, S(stream));
}

size_t hv_reduce_workspace(size_t n) { return reduce_workspace(n) + 64; }

hv_status hv_shift_corners(float* frame, int width, int height, void* stream)
{
    if (!frame)
        return HV_INVALID_VALUE;
    return shift_corners(frame, width, height, S(stream));
}

hv_status hv_accumulate(const float* frame, float* acc_ring, int A, int slot, int start, int count, float* out,
                        size_t n, void* stream)
{
    if (!frame || !acc_ring || !out)
        return HV_INVALID_VALUE;
    return accumulate(frame, acc_ring, A, slot, start, count, out, n, S(stream));
}

hv_status hv_log10(float* frame, size_t n, void* stream)
{
    if (!frame)
        return HV_INVALID_VALUE;
    return log10_map(frame, n, S(stream));
}

hv_status hv_percentile(const float* frame, int width, int height, float lower, float upper, float reticle_scale,
                        float* range_f32, void* work, void* stream)
{
    if (!frame || !range_f32 || !work || width <= 0 || height <= 0)
        return HV_INVALID_VALUE;
    return percentile(frame, width, height, lower, upper, reticle_scale, range_f32, work, S(stream));
}

size_t hv_percentile_workspace(size_t n) { return percentile_workspace(n); }

hv_status hv_contrast_to_ushort(const float* frame, const float* range_f32, int invert, int apply_contrast,
                                uint16_t* out, size_t n, void* stream)
{
    if (!frame || !out || (apply_contrast && !range_f32))
        return HV_INVALID_VALUE;
    return contrast_to_ushort(frame, range_f32, invert, apply_contrast, out, n, S(stream));
}

}  // extern "C"

namespace hv {
hv_status unwrap_2d_noalloc(const float* in, float* out, int W, int H, cudaStream_t st);
}

extern "C" hv_status hv_unwrap_2d_noalloc(const float* in, float* out, int width, int height, void* stream)
{
    if (!in || !out)
        return HV_INVALID_VALUE;
    return hv::unwrap_2d_noalloc(in, out, width, height, static_cast<cudaStream_t>(stream));
}
