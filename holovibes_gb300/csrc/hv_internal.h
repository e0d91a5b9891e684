// Internal declarations shared by the translation units of the library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "holovibes_gb300.h"

namespace hv {

// Per-cycle control block of a served stream, in device memory. The kernels of a served cycle read
// the values that change from cycle to cycle from here instead of from their launch arguments, so
// a stream's (or a shape bucket's) whole cycle is captured once in a CUDA graph and replayed; the
// host writes the blocks of a bucket with one copy before each launch. A null block means "use
// the launch arguments, always active".
struct CycleCtl
{
    long long raw_offset;  // byte offset of the batch in the stream's input ring
    int active;            // the batch is processed this cycle (spatial passes run)
    int render;            // the ring is full: the window is transformed and rendered
    int ring_begin;        // ring slot of the batch's first frame
    int acc_slot, acc_start, acc_count;  // accumulation queue (Queue::enqueue)
    int pct_enable;        // the autocontrast percentile runs this cycle
    int out_slot;          // output ring slot
    int pad[4];
};
static_assert(sizeof(CycleCtl) == 56, "CycleCtl layout");

#ifdef __CUDACC__
__device__ __forceinline__ bool ctl_active(const CycleCtl* c) { return !c || c->active; }
__device__ __forceinline__ bool ctl_render(const CycleCtl* c) { return !c || c->render; }
#endif

void set_last_error(const char* msg, const char* file, int line);
void set_last_error_msg(const char* msg);
void count_launch(uint64_t n = 1);
uint64_t launch_count();

// spatial.cu
bool fft_size_supported(int n);
int raw_kind(int raw_bytes, int big_endian);
hv_status make_fresnel_lens(float2* lens, int W, int H, float lam, float z, float ps, int mode, cudaStream_t st);
hv_status make_spectral_lens(float2* lens, int W, int H, float lam, float z, float ps, int mode, cudaStream_t st);
// real_planes (no spatial transform, frames of a multiple of 8 pixels): the real split-BF16 planes
// of the ring slots written are produced in the same pass (cov_tc.cu layout, real rows).
// reserve_sms: the persistent (TMA-fed) FFT passes leave that many SMs to kernels of other streams
// (a Pipe's render lanes).
hv_status spatial_transform(const void* raw, int kind, int W, int H, int batch, int space, const float2* lens,
                            float2* work, float2* ring, int slot0, int nslots, cudaStream_t st,
                            const CycleCtl* ctl = nullptr, const float2* f2d_mask = nullptr,
                            float2* work2 = nullptr, uint16_t* real_planes = nullptr, int reserve_sms = 0);
// Raw 8/16-bit frames (no spatial transform) -> the real split-BF16 planes of ring slots slot0 ..
// (mod T) only; and the ring slots back from those planes (exact for integer pixels below 2^16).
hv_status convert_to_planes(const void* raw, int kind, size_t HW, int batch, int slot0, int T, uint16_t* planes,
                            cudaStream_t st);
hv_status ring_from_planes(const uint16_t* planes, int T, size_t HW, int slot0, int n, float2* ring, cudaStream_t st);
// filter2D band-pass mask in FFT layout: written as complex (multiply = 0) or multiplied into dst.
hv_status filter2d_mask(float2* dst, int W, int H, int n1, int n2, int smooth_low, int smooth_high, int multiply,
                        cudaStream_t st);
hv_status fft2d(const float2* in, float2* out, int n0, int n1, int batch, int inverse, float scale, cudaStream_t st);
hv_status fft_rows_pass(const void* in, int kind, float2* out, int W, int H, int batch, const float2* premul,
                        int inverse, float scale, int slot0, int nslots, cudaStream_t st);
hv_status fft_cols_pass(const float2* in, float2* out, int W, int H, int batch, const float2* postmul, int mode,
                        float scale, int slot0, int nslots, cudaStream_t st);

// ingest.cu
hv_status unpack_packed(int bits, const void* in, size_t in_bytes, uint16_t* out, size_t out_count, cudaStream_t st);

// time_transform.cu
int time_view_partials(int W, int H);
hv_status time_view(const float2* ring, int T, int W, int H, const float2* weights, int K, int img_type, float scale,
                    int shift, float* out, double* partials, cudaStream_t st, const CycleCtl* ctl = nullptr,
                    const float* bin_w = nullptr);
// time_view on a real ring held as split-BF16 planes ([2][T][HW] bf16, hi then lo; HW % 8 == 0),
// the slots [ring_slot0, ring_slot0 + ring_n) mod T read from the complex ring instead.
hv_status time_view_planes(const uint16_t* planes, const float2* ring, int ring_slot0, int ring_n, int T, int W, int H,
                           const float2* weights, int K, int img_type, float scale, int shift, float* out,
                           double* partials, cudaStream_t st, const CycleCtl* ctl = nullptr,
                           const float* bin_w = nullptr);
hv_status moment_bin_weights(float* bin_w, int T, int pmin, int pmax, int order, float camera_fps, cudaStream_t st);
inline bool is_moment(int img_type) { return img_type >= HV_IMG_MOMENTS_0 && img_type <= HV_IMG_MOMENTS_2; }
hv_status stft_weights(float2* weights, int T, int pmin, int pmax, cudaStream_t st);
hv_status delta_weights(float2* weights, int T, int pmin, int pmax, cudaStream_t st);
// SSA_STFT projection weights of the bins pmin..pmin+K-1 from the eigenvector columns qmin..qmin+qn-1.
hv_status ssa_weights(const double2* evecs, int T, int qmin, int qn, int pmin, int K, float2* weights, cudaStream_t st);
// Phase increase of the p plane (weights row w) against the previous window's plane; per-CTA
// min / max partials in mm (phase_increase_minmax_count(HW) entries).
size_t phase_increase_minmax_count(size_t HW);
hv_status phase_increase(const float2* ring, int T, size_t HW, const float2* w, float2* pred, float* hist, int first,
                         int use_hist, float* out, float2* mm, cudaStream_t st);
hv_status rescale_float(const float* in, size_t HW, const float2* mm, float post_scale, float* out, cudaStream_t st);
size_t pca_cov_workspace(int T, size_t npix);
// the workspace of pca_covariance_planes (the caller keeps the planes) and of the SIMT engine
size_t pca_cov_workspace_planes(int T, size_t npix);
void set_cov_mode(int mode);
int cov_mode();
void set_cov_incremental(bool on);
bool cov_incremental();
hv_status pca_cov_status(const void* work);
// cov_tc.cu
bool cov_tc_supported(int T);
size_t cov_tc_workspace(int T, size_t npix);
hv_status cov_tc(const float2* ring, int T, size_t npix, double2* cov, void* work, int* err, cudaStream_t st);
// partial tiles of the tiled tensor-core covariance (T > 64): the workspace when the caller passes
// its own split planes
size_t cov_tc_partial_bytes(int T, size_t npix);
// Split-BF16 planes of the ring (T > 64): bytes, whether (T, npix) has them, the split of ring slots
// slot0 .. slot0 + n - 1 (mod T) into them, and the tiled covariance from them: `blocks` = ~0u for
// all of it, else only the rows and columns of the 64-frame slot blocks set (bit b: slots 64 b ..
// 64 b + 63), bit-identical to a full computation; cov_tc on a ring (T > 64) splits it into planes
// in its workspace first.
// `real`: the ring's imaginary parts are 0 (no spatial transform): real rows only, 128-frame blocks.
size_t cov_planes_bytes(int T, size_t npix, int real);
bool cov_planes_supported(int T, size_t npix);
hv_status cov_split_planes(const float2* ring, int T, size_t npix, int slot0, int n, uint16_t* planes, int real,
                           cudaStream_t st);
hv_status cov_tc_planes(const uint16_t* planes, int T, size_t npix, double2* cov, void* work, int* err,
                        uint32_t blocks, int real, cudaStream_t st);
hv_status pca_covariance(const float2* ring, int T, size_t npix, double2* cov, void* work, cudaStream_t st);
// The covariance from the split planes (engine modes 0 and 2; HV_ERR_UNSUPPORTED for the SIMT mode
// and shapes without planes).
hv_status pca_covariance_planes(const uint16_t* planes, int T, size_t npix, double2* cov, void* work, uint32_t blocks,
                                int real, cudaStream_t st);
size_t pca_eigh_workspace(int T);
void set_eig_precision(int p);
// 1 (default): the warm subspace iteration orthonormalises by Cholesky-QR (Gram-Schmidt when its
// factorisation fails); 0: Gram-Schmidt always.
void set_eig_cholqr(int on);
// Eigenvectors of ranks refine_lo..refine_hi (at most 64 of them) are refined in FP64 after FP32
// sweeps; an empty range (refine_hi < refine_lo) keeps the FP32 vectors. `warm`: `work` holds the
// eigenvectors of the previous successful call with the same T (a window of the same stream), from
// which the FP32 sweeps start (T <= 64). `kept_only`: the caller uses only the refined
// eigenvectors and the order of the eigenvalues (coarser sweeps, FP32 Rayleigh quotients for the
// others). `cov_kept` (optional): false when the eigensolve overwrote `cov` (the FP64 sweeps in
// global memory).
hv_status pca_eigh(double2* cov, int T, double* evals, double2* evecs, int pmin, int pmax, float2* weights, void* work,
                   cudaStream_t st, int refine_lo, int refine_hi, bool warm = false, bool kept_only = false,
                   bool* cov_kept = nullptr);

// view_tc.cu
bool view_tc_supported(int K);
void set_view_mode(int mode);
void set_fft_engine(int mode);
hv_status fft_status();
void set_spatial_sub_batch_mb(int mb);
bool view_engine_tc(int K, size_t HW);
size_t view_tc_workspace(int K, int T);
hv_status view_tc_prepare(const float2* weights, int K, int T, void* work, cudaStream_t st);
hv_status view_tc(const float2* ring, int T, int W, int H, int K, int img_type, float scale, int shift, float* out,
                  double* partials, void* work, cudaStream_t st, const CycleCtl* ctl = nullptr,
                  const float* bin_w = nullptr);

// render.cu
size_t unwrap_workspace(int W, int H);
hv_status unwrap_2d(const float* in, float* out, int W, int H, void* work, cudaStream_t st);
size_t reduce_workspace(size_t n);
hv_status renorm_factors(const float* frame, size_t n, int renorm_constant, const double* partials, int npartials,
                         float* factors, void* work, cudaStream_t st, const CycleCtl* ctl = nullptr);
hv_status renorm_shift_accumulate(const float* in, float* out, int W, int H, const float* factors, int shift,
                                  float* acc_ring, int A, int slot, int start, int count, int log_enabled,
                                  cudaStream_t st, float prescale = 1.0f, const CycleCtl* ctl = nullptr);
hv_status shift_corners(float* frame, int W, int H, cudaStream_t st);
hv_status accumulate(const float* frame, float* acc_ring, int A, int slot, int start, int count, float* out, size_t n,
                     cudaStream_t st);
hv_status log10_map(float* frame, size_t n, cudaStream_t st);
size_t percentile_workspace(size_t n);
hv_status percentile(const float* frame, int W, int H, float lower, float upper, float reticle_scale, float* range,
                     void* work, cudaStream_t st, const CycleCtl* ctl = nullptr);
hv_status percentile_pitched(const float* frame, int W, int H, int pitch, float lower, float upper,
                             float reticle_scale, float* range, void* work, cudaStream_t st,
                             const CycleCtl* ctl = nullptr);
// Time-transformation cuts (XZ: T x W, YZ: H x T) from all T weight rows; work: cuts_workspace bytes.
bool cuts_supported(int T);
size_t cuts_workspace(int W, int H, int T, int nx, int ny);
hv_status time_cuts(const float2* ring, int T, int W, int H, const float2* weights_all, int xmin, int xmax, int ymin,
                    int ymax, int img_type, float* xz, float* yz, void* work, cudaStream_t st);
hv_status evecs_to_weights(const double2* evecs, int T, float2* w, cudaStream_t st);
hv_status contrast_to_ushort(const float* frame, const float* range, int invert, int apply, uint16_t* out, size_t n,
                             cudaStream_t st, const CycleCtl* ctl = nullptr);
// filter2D view: |shift(spec x mult)| into out (W x H); contrast then trunc(x * 65535) saturated
hv_status filter2d_view_frame(const float2* spec, const float2* mult, int W, int H, float* out, cudaStream_t st);
hv_status contrast_to_ushort_normalized(const float* frame, const float* range, int invert, int apply, uint16_t* out,
                                        size_t n, cudaStream_t st);

}  // namespace hv

#define HV_CUDA_TRY(expr)                                                                                              \
    do                                                                                                                 \
    {                                                                                                                  \
        cudaError_t hv_err__ = (expr);                                                                                 \
        if (hv_err__ != cudaSuccess)                                                                                   \
        {                                                                                                              \
            hv::set_last_error(cudaGetErrorString(hv_err__), __FILE__, __LINE__);                                      \
            return (hv_err__ == cudaErrorMemoryAllocation) ? HV_ERR_OOM : HV_ERR_CUDA;                                \
        }                                                                                                              \
    } while (0)

#define HV_LAUNCH_CHECK() HV_CUDA_TRY(cudaGetLastError())
