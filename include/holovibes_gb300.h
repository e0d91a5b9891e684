/* holovibes_gb300 C ABI.
 *
 * A GB300-native (sm_103a) implementation of the Holovibes hologram path:
 * raw camera frames -> complex -> Fresnel / angular-spectrum propagation -> time ring ->
 * STFT bins / PCA -> modulus / squared modulus / argument (+ 2-D unwrap) -> renormalisation ->
 * fftshift -> image accumulation -> percentile contrast -> uint16.
 *
 * Two levels are exported:
 *   1. The Pipe (hv_pipe_*): the drop-in for the reference's Pipe/ICompute engine
 *      (Backend/includes/core/pipe.hh:70-125, Backend/sources/core/pipe.cc:255-387,650-676),
 *      fed like its BatchInputQueue and drained like its output Queue.
 *   2. Compute steps (hv_*): stream-ordered calls on caller-owned device buffers, one per
 *      reference CUDA-layer function they replace (cited per function).
 *
 * Conventions: plain pointers and sizes, no exceptions across the ABI, every call returns an
 * hv_status. Device pointers are CUDA device addresses; `stream` is a cudaStream_t passed as
 * void* (NULL = legacy default stream). All compute steps are asynchronous on `stream`.
 */
#ifndef HOLOVIBES_GB300_H
#define HOLOVIBES_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The first eight values are the reference's ApiCode
 * (Backend/includes/enum/enum_api_code.hh:13-23); the rest are device-side failures that the
 * reference turns into exit() / exceptions (Backend/cuda_includes/common.cuh:52-64). */
typedef enum hv_status
{
    HV_OK = 0,
    HV_NO_CHANGE = 1,
    HV_INVALID_VALUE = 2,
    HV_NO_IN_DATA = 3,
    HV_NOT_STARTED = 4,
    HV_WRONG_COMP_MODE = 5,
    HV_WRONG_IMG_TYPE = 6,
    HV_FAILURE = 7,
    HV_ERR_CUDA = 8,
    HV_ERR_OOM = 9,
    HV_ERR_TIMEOUT = 10,
    HV_ERR_ADMISSION = 11,
    HV_ERR_UNSUPPORTED = 12
} hv_status;

/* camera::FrameDescriptor (Camera/include/frame_desc.hh:13-48): depth in bytes per pixel
 * (1 = uint8, 2 = uint16, 4 = float32), byte_endian 0 = little, 1 = big. */
typedef struct hv_frame_desc
{
    uint16_t width;
    uint16_t height;
    uint32_t depth;
    uint32_t byte_endian;
} hv_frame_desc;

/* SpaceTransformation (Backend/includes/enum/enum_space_transformation.hh:17-22). */
enum { HV_SPACE_NONE = 0, HV_SPACE_FRESNELTR = 1, HV_SPACE_ANGULARSP = 2 };
/* TimeTransformation (Backend/includes/enum/enum_time_transformation.hh:16-22). */
enum { HV_TIME_NONE = 0, HV_TIME_STFT = 1, HV_TIME_PCA = 2, HV_TIME_SSA_STFT = 3 };
/* ImgType values of the reference (Backend/includes/enum/enum_img_type.hh:15-25); COMPOSITE (4)
 * is outside this path. Moments: sum over the selected bins of |X_k|^2 f_k^n (f_k the signed
 * FFT frequency in units of camera_fps / T), replacing the view frame. Phase increase: the phase
 * of the p plane against the previous window's (plus the previous increment), rescaled to
 * [0, 65535] (converts.cc:251-300). */
enum
{
    HV_IMG_MODULUS = 0,
    HV_IMG_SQUARED_MODULUS = 1,
    HV_IMG_ARGUMENT = 2,
    HV_IMG_PHASE_INCREASE = 3,
    HV_IMG_MOMENTS_0 = 5,
    HV_IMG_MOMENTS_1 = 6,
    HV_IMG_MOMENTS_2 = 7
};
/* Lens phase precision: FP64 (exact phase, reduced mod 2*pi) or the reference's float32 expression. */
enum { HV_LENS_FP64 = 0, HV_LENS_REF32 = 1 };
/* Memory kinds for hv_pipe_push_frames / hv_pipe_pull_output. */
enum { HV_MEM_HOST = 0, HV_MEM_DEVICE = 1 };

/* Flat settings record: the subset of the reference's typed settings that this path reads
 * (Backend/includes/core/holovibes.hh:370-450 defaults; compute-settings JSON keys in
 * Backend/includes/struct/*.hh). hv_settings_default() fills the reference defaults. */
typedef struct hv_settings
{
    int32_t space_transformation;    /* image_rendering.space_transformation */
    int32_t time_transformation;     /* image_rendering.time_transformation */
    int32_t time_transformation_size; /* image_rendering.time_transformation_size (T) */
    int32_t time_stride;             /* image_rendering.time_transformation_stride (S) */
    int32_t batch_size;              /* image_rendering.batch_size (B) */
    float lambda;                    /* image_rendering.lambda [m] */
    float z_distance;                /* image_rendering.propagation_distance [m] */
    float pixel_size;                /* input info pixel pitch [um] */
    int32_t image_type;              /* view.image_type */
    int32_t p_start;                 /* view.z.start */
    int32_t p_width;                 /* view.z.width */
    int32_t fft_shift;               /* view.fft_shift */
    int32_t renorm;                  /* view.renorm */
    int32_t renorm_constant;         /* advanced.renorm_constant */
    int32_t accumulation;            /* view.window.xy.output_image_accumulation */
    int32_t log_enabled;             /* view.window.xy.log_enabled */
    int32_t contrast_enabled;        /* view.window.xy.contrast.enabled */
    int32_t contrast_auto_refresh;   /* view.window.xy.contrast.auto_refresh */
    int32_t contrast_invert;         /* view.window.xy.contrast.invert */
    float contrast_min;              /* view.window.xy.contrast.min */
    float contrast_max;              /* view.window.xy.contrast.max */
    float contrast_lower;            /* advanced.contrast.lower [%] */
    float contrast_upper;            /* advanced.contrast.upper [%] */
    int32_t reticle_display;         /* view.reticle.display_enabled */
    float reticle_scale;             /* view.reticle.scale */
    int32_t unwrap_2d;               /* Unwrap2d setting */
    int32_t lens_mode;               /* HV_LENS_FP64 (default) or HV_LENS_REF32 */
    int32_t output_buffer_size;      /* advanced.buffer_size.output: output frames kept */
    int32_t input_buffer_size;       /* advanced.buffer_size.input: raw frames kept */
    int32_t camera_fps;              /* CameraFps input setting (.holo info.camera_fps): moment frequencies */
    int32_t q_start;                 /* view.z2.start: first eigenvector kept by SSA_STFT */
    int32_t q_width;                 /* view.z2.width: eigenvectors kept by SSA_STFT (0 = all) */
    int32_t filter2d_enabled;        /* image_rendering.filter2d.enabled */
    int32_t filter2d_n1;             /* image_rendering.filter2d.inner_radius (pixels, frequency domain) */
    int32_t filter2d_n2;             /* image_rendering.filter2d.outer_radius */
    int32_t filter2d_smooth_low;     /* advanced.filter2d_smooth.low: cosine roll-off of the inner edge */
    int32_t filter2d_smooth_high;    /* advanced.filter2d_smooth.high: cosine roll-off of the outer edge */
    int32_t cuts_enabled;            /* CutsViewEnabled: XZ (T x W) and YZ (H x T) time-transformation cuts */
    int32_t x_start;                 /* view.x.start: first column of the YZ cut's band */
    int32_t x_width;                 /* view.x.width: the band is columns x_start .. x_start + x_width */
    int32_t y_start;                 /* view.y.start: first row of the XZ cut's band */
    int32_t y_width;                 /* view.y.width */
    int32_t xz_accumulation;         /* view.window.xz.output_image_accumulation */
    int32_t yz_accumulation;         /* view.window.yz.output_image_accumulation */
    int32_t xz_log_enabled;          /* view.window.xz.log_enabled */
    int32_t yz_log_enabled;          /* view.window.yz.log_enabled */
    int32_t xz_contrast_enabled;     /* view.window.xz.contrast.enabled */
    int32_t xz_contrast_auto_refresh;
    int32_t xz_contrast_invert;
    float xz_contrast_min;
    float xz_contrast_max;
    int32_t yz_contrast_enabled;     /* view.window.yz.contrast.* */
    int32_t yz_contrast_auto_refresh;
    int32_t yz_contrast_invert;
    float yz_contrast_min;
    float yz_contrast_max;
    int32_t cuts_contrast_offset;    /* advanced.contrast.frame_index_offset: bins skipped at both ends */
    int32_t cuts_buffer_size;        /* advanced.buffer_size.time_transformation_cuts: cut outputs kept */
    int32_t filter2d_view_enabled;   /* Filter2dViewEnabled: queue the filter2D view (needs filter2d_enabled) */
    int32_t filter2d_log_enabled;    /* view.window.filter2d.log_enabled */
    int32_t filter2d_contrast_enabled; /* view.window.filter2d.contrast.* */
    int32_t filter2d_contrast_auto_refresh;
    int32_t filter2d_contrast_invert;
    float filter2d_contrast_min;
    float filter2d_contrast_max;
} hv_settings;

/* ------------------------------------------------------------------------------------------
 * Library
 * ---------------------------------------------------------------------------------------- */
const char* hv_version(void);
/* Last error message of the calling thread (empty string when none). */
const char* hv_last_error(void);
/* Kernels launched by this library in this process (all threads). */
uint64_t hv_kernel_launches(void);
void hv_settings_default(hv_settings* s);
/* Parses a compute-settings JSON document (the reference's ComputeSettings layout,
 * Backend/sources/core/compute_settings.cc:66-99) and merges it into *s. Unknown keys fail
 * with HV_FAILURE like merge_json (compute_settings.cc:24-36). */
hv_status hv_settings_from_json(const char* json, hv_settings* s);
/* Validates and adjusts settings like the reference's TransformApi setters
 * (Backend/sources/api/transform_api.cc:16-206): stride >= batch and a multiple of it,
 * z != 0, p range inside the time window. Returns HV_INVALID_VALUE for unsupported values. */
hv_status hv_settings_validate(hv_settings* s, const hv_frame_desc* fd);

/* ------------------------------------------------------------------------------------------
 * Pipe (drop-in for Pipe / ICompute; Backend/includes/core/pipe.hh:70-125)
 * ---------------------------------------------------------------------------------------- */
typedef struct hv_pipe hv_pipe;

/* Creates a pipe on the current CUDA device: allocates the spatial buffer, the time ring,
 * the view / accumulation / output buffers (ICompute ctor, Backend/includes/core/icompute.hh:123-171).
 * `stream` may be NULL, in which case the pipe creates and owns a non-blocking stream. */
hv_pipe* hv_pipe_create(const hv_frame_desc* fd, const hv_settings* settings, void* stream, hv_status* status);
void hv_pipe_destroy(hv_pipe* p);
/* Device bytes held by a pipe with these settings (admission by HBM footprint). */
size_t hv_pipe_footprint(const hv_frame_desc* fd, const hv_settings* settings);
/* Replaces BatchInputQueue::enqueue (Backend/sources/data_struct/batch_input_queue.cc:124-202)
 * followed by the compute cycles it unblocks (Pipe::exec, pipe.cc:650-676). `n` frames of
 * fd->depth bytes each; `mem` is HV_MEM_HOST or HV_MEM_DEVICE. Work is enqueued on the pipe's
 * stream; host memory is copied before the call returns only if it is pageable. */
hv_status hv_pipe_push_frames(hv_pipe* p, const void* frames, size_t n, int mem);
/* Number of uint16 output frames produced and not yet pulled. */
size_t hv_pipe_output_count(hv_pipe* p);
/* Replaces the output Queue dequeue: copies the oldest output frame (W*H uint16) into dst,
 * waiting at most timeout_us microseconds for it (HV_ERR_TIMEOUT otherwise). */
hv_status hv_pipe_pull_output(hv_pipe* p, uint16_t* dst, int mem, int64_t timeout_us);
/* Applies new settings at the next cycle boundary (pipe_refresh / pipe_cycle updates,
 * Backend/includes/core/pipe.hh:192-213). Returns HV_NO_CHANGE when nothing changed. */
hv_status hv_pipe_update_settings(hv_pipe* p, const hv_settings* settings);
/* Requests an autocontrast on the next output (Rendering::request_autocontrast,
 * Backend/sources/compute/rendering.cc:87-99). */
hv_status hv_pipe_request_autocontrast(hv_pipe* p);
/* Blocks until all work enqueued on the pipe's streams finished. */
hv_status hv_pipe_sync(hv_pipe* p);
/* Makes the pipe's stream (hv_pipe_stream) wait, on the device, for all rendering enqueued so
 * far. When batch == stride == time window the pipe double-buffers the ring and renders on a
 * second stream so the next batch's spatial passes overlap the current window's time transform;
 * work the caller chains on hv_pipe_stream after hv_pipe_join sees finished outputs. */
hv_status hv_pipe_join(hv_pipe* p);
/* Current XY contrast range (XYContrastRange setting) after the last autocontrast. */
hv_status hv_pipe_get_contrast_range(hv_pipe* p, float* min_out, float* max_out);
/* Copies the last float frame fed to the contrast stage (gpu_postprocess_frame) into dst (host). */
hv_status hv_pipe_get_float_frame(hv_pipe* p, float* dst);
/* Secondary views, each rendered window, each into its own output queue (pipe.cc:504-521):
 * the time-transformation cuts (CutsViewEnabled) XZ (T rows x W, row t = bin / component t) and
 * YZ (H rows x T), and the filter2D view (Filter2dViewEnabled: the modulus of the masked spectrum
 * of the batch's first frame, quadrant-swapped, W x H). */
enum { HV_VIEW_XZ = 0, HV_VIEW_YZ = 1, HV_VIEW_FILTER2D = 2 };
size_t hv_pipe_view_output_count(hv_pipe* p, int which);
/* Copies the oldest output of a secondary view (uint16) into dst; as hv_pipe_pull_output. */
hv_status hv_pipe_pull_view(hv_pipe* p, int which, uint16_t* dst, int mem, int64_t timeout_us);
/* The view's last float image fed to its contrast stage (host dst, may be NULL) and its contrast
 * range (range_out[2], may be NULL). */
hv_status hv_pipe_get_view_float_frame(hv_pipe* p, int which, float* dst, float* range_out);
/* Copies the time ring storage (T frames of complex64, slot order) and its start/size. */
hv_status hv_pipe_get_ring(hv_pipe* p, void* dst_host, int32_t* start, int32_t* size);
/* Number of kernels this pipe launched since creation. */
uint64_t hv_pipe_kernel_launches(hv_pipe* p);
void* hv_pipe_stream(hv_pipe* p);

/* ------------------------------------------------------------------------------------------
 * Compute steps (device buffers, stream-ordered)
 * ---------------------------------------------------------------------------------------- */

/* Supported transform lengths for the shared-memory FFT (each of width and height). */
int hv_fft_size_supported(int n);
/* Engine of the 512-, 768- and 1024-point spatial FFT passes (process-wide, read at every launch):
 * 0 = automatic (warp engine: 32 samples per thread, one transpose; the 1024-point forward /
 * inverse column passes and the 1024-point row passes of 8-/16-bit camera frames persistent and
 * fed by TMA), 1 = the shared-memory Stockham tile engine used for every other length, 2 = the
 * warp engine with register-loading passes only. All compute the same transform to FP32
 * round-off (0 and 2 bit-identically). */
void hv_fft_engine_mode(int mode);
/* HV_ERR_TIMEOUT when a bounded wait of a TMA-fed FFT pass gave up since the library was loaded
 * (its CTA stopped early; the pass's output is incomplete), HV_OK otherwise. Synchronous. */
hv_status hv_fft_status(void);
/* Batching of the spatial stage's passes (process-wide, read at every call): 0 = one launch per
 * pass over the whole batch (default: the fewest partial waves), n > 0 = sub-batches whose complex
 * intermediate fits in n MB (kept in L2 between the passes). Results are identical either way. */
void hv_spatial_sub_batch_mb(int mb);

/* Fresnel quadratic lens, H x W complex64, centre-cropped from the max(W,H) square.
 * Replaces fresnel_transform_lens + kernel_quadratic_lens (Backend/cuda_sources/fresnel_transform.cu:14-63,
 * masks.cu:7-29). */
hv_status hv_fresnel_lens(void* lens_c64, int width, int height, float lambda, float z, float pixel_size_um,
                          int lens_mode, void* stream);
/* Angular-spectrum transfer function in FFT layout (already quadrant-swapped).
 * Replaces angular_spectrum_lens + kernel_spectral_lens + shift_corners
 * (Backend/cuda_sources/angular_spectrum.cu:14-31, masks.cu:31-59, fourier_transform.cc:121-137). */
hv_status hv_angular_spectrum_lens(void* lens_c64, int width, int height, float lambda, float z,
                                   float pixel_size_um, int lens_mode, void* stream);

/* filter2D band-pass mask (kernel_update_filter2d_circles_mask + shift_corners, filter2D.cu:52-115):
 * m = A (1 - B), A = 1 for r < n2 with a cosine roll-off over smooth_high pixels, B the same for
 * n1 / smooth_low, r the distance to the frame centre; written in FFT layout as complex64 (m, 0)
 * when multiply == 0, or multiplied into the complex64 array (an FFT-layout transfer function)
 * when multiply != 0. Even width and height, 0 <= n1 < n2 (Filter2dApi::set_filter2d_n1/n2). */
hv_status hv_filter2d_mask(void* dst_c64, int width, int height, int n1, int n2, int smooth_low, int smooth_high,
                           int multiply, void* stream);
/* hv_spatial_transform with filter2D (fourier_transform.cc:30-72, filter2D.cu:28-46): for
 * FRESNELTR and NONE the frames first become IFFT2(FFT2(x) M) (unnormalised inverse), M = mask_c64
 * from hv_filter2d_mask; for ANGULARSP pass the transfer function multiplied by the mask and no
 * mask here. FRESNELTR also needs `work2_c64` (batch*W*H complex64). */
hv_status hv_spatial_transform_filter2d(const void* raw, int raw_bytes, int big_endian, int width, int height,
                                        int batch, int space, const void* lens_c64, const void* mask_c64,
                                        void* work_c64, void* work2_c64, void* ring_c64, int slot0, int nslots,
                                        void* stream);

/* Fused raw->complex convert + spatial propagation of `batch` frames, written into slots
 * (slot0 + b) % nslots of a ring of complex64 frames. Replaces input_queue_to_input_buffer
 * (tools_conversion.cu:120-171) + fresnel_transform (fresnel_transform.cu:65-83) /
 * angular_spectrum (angular_spectrum.cu:33-63) + Queue::enqueue_multiple (queue.cc:332-380).
 * `raw_kind`: bytes per pixel (1, 2, 4) or 8 for complex64 input; `big_endian` swaps 16-bit.
 * `work_c64` must hold batch*W*H complex64 (unused for space NONE). */
hv_status hv_spatial_transform(const void* raw, int raw_bytes, int big_endian, int width, int height, int batch,
                               int space, const void* lens_c64, void* work_c64, void* ring_c64, int slot0,
                               int nslots, void* stream);

/* Batched 2-D complex FFT over `batch` row-major n0 x n1 arrays (n0 rows of n1 samples),
 * forward (sign -1) or inverse (sign +1, unnormalised), multiplied by `scale`. */
hv_status hv_fft2d(const void* in_c64, void* out_c64, int n0, int n1, int batch, int inverse, float scale,
                   void* stream);

/* The two passes of the spatial stage, exposed separately (timing, custom pipelines).
 * Row pass: raw/complex input (in_bytes 1, 2, 4 or 8) converted, multiplied by premul (H x W, or
 * NULL), FFT along each row of `width` samples (inverse: conj in / conj out), times `scale`,
 * written to slots (slot0 + b) % nslots of out. Column pass: FFT along each column of `height`
 * samples; mode 0 forward, 1 inverse, 2 forward * postmul (H x W) then inverse (the angular
 * spectrum's middle pass). Together they replace cufftXtExec with the 2-D plan of
 * Backend/sources/core/icompute.cc:151-175 and the apply_mask / kernel_complex_divide passes. */
hv_status hv_fft_rows(const void* in, int in_bytes, int big_endian, void* out_c64, int width, int height, int batch,
                      const void* premul_c64, int inverse, float scale, int slot0, int nslots, void* stream);
hv_status hv_fft_cols(const void* in_c64, void* out_c64, int width, int height, int batch, const void* postmul_c64,
                      int mode, float scale, int slot0, int nslots, void* stream);

/* Fused time transform + view: for every pixel, X_k = sum_t ring[t] * W[k][t] for k < K,
 * then out = scale * mean_k f(X_k) with f = |.|, |.|^2 or atan2 (img_type), written at the
 * fftshift-ed position when `shift` is set. `weights_c64` is K x T complex64. Per-CTA partial
 * sums of the written values go to `partials_f64` (hv_time_view_partials entries) when not NULL.
 * Replaces stft (stft.cu:9-15) / matrix_multiply_complex (matrix_operations.cc:77-103) +
 * complex_to_modulus / _squared_modulus / _argument (tools_conversion.cu:11-103,199-232). */
hv_status hv_time_view(const void* ring_c64, int T, int width, int height, const void* weights_c64, int K,
                       int img_type, float scale, int shift, float* out_f32, double* partials_f64, void* stream);
int hv_time_view_partials(int width, int height);
/* hv_time_view of a real ring (zero imaginary parts: frames converted without a spatial
 * transform) from its split-BF16 planes (hv_pca_split_planes with real = 1: 4 bytes per sample
 * against the ring's 8). The slots [ring_slot0, ring_slot0 + ring_n) mod T are read from the
 * complex ring instead (ring_n = 0: the planes only, ring_c64 may be NULL): the pipe's slots that
 * the next batch overwrites in the planes while the view may still run. The view values equal
 * hv_time_view's on the ring for integer pixels below 2^16 (hi + lo is exact there); the partials
 * are the same 128-pixel sums. width x height a multiple of 8. */
hv_status hv_time_view_planes(const void* planes_u16, const void* ring_c64, int ring_slot0, int ring_n, int T,
                              int width, int height, const void* weights_c64, int K, int img_type, float scale,
                              int shift, float* out_f32, double* partials_f64, void* stream);
/* hv_time_view on the tensor cores (tcgen05, split-BF16 with FP32 accumulation): the K-bin
 * contraction runs as a 128-pixel x 2K x 2T GEMM per pixel tile. K <= 64, width * height even
 * and at most 2^29, ring and work 16-byte aligned (HV_ERR_UNSUPPORTED otherwise: the ring is
 * fetched with 2-D tensor copies). `work` needs hv_time_view_tc_workspace(K, T) bytes (pre-split
 * weights and an error flag; 0 when K is unsupported); hv_time_view_tc_status(work) reports
 * HV_ERR_TIMEOUT if a bounded device wait gave up. */
hv_status hv_time_view_tc(const void* ring_c64, int T, int width, int height, const void* weights_c64, int K,
                          int img_type, float scale, int shift, float* out_f32, double* partials_f64, void* work,
                          void* stream);
size_t hv_time_view_tc_workspace(int K, int T);
/* The two halves of hv_time_view_tc, for weights that stay fixed over many windows (the pipe's
 * use: once per settings refresh, like hv_stft_weights): _prepare splits the K x T weights into
 * the BF16 operand image in `work`; _run then contracts a ring with the prepared image (same
 * arguments and checks as hv_time_view_tc, without the weights). */
hv_status hv_time_view_tc_prepare(const void* weights_c64, int K, int T, void* work, void* stream);
hv_status hv_time_view_tc_run(const void* ring_c64, int T, int width, int height, int K, int img_type, float scale,
                              int shift, float* out_f32, double* partials_f64, void* work, void* stream);
/* Engine of the pipe's time view (process-wide, read when a pipe is built): 0 = automatic (tensor
 * cores for 8 <= K <= 64 selected bins, FP32 SIMT otherwise), 1 = SIMT, 2 = tensor cores wherever
 * hv_time_view_tc supports the shape. */
void hv_time_view_mode(int mode);
hv_status hv_time_view_tc_status(const void* work);
/* Packed camera data to 16-bit pixels (device buffers): 12-bit pairs in 3 bytes or 10-bit
 * quadruples in 5 bytes, MSB first, each value left-aligned in 16 bits; out_count pixels are
 * written where their bytes lie inside in_bytes. Replaces unpack_12_to_16bit / unpack_10_to_16bit
 * (unpack.cu:4-60, file_frame_read_worker.cc:220-240). */
hv_status hv_unpack_12_to_16(const void* in, size_t in_bytes, uint16_t* out, size_t out_count, void* stream);
hv_status hv_unpack_10_to_16(const void* in, size_t in_bytes, uint16_t* out, size_t out_count, void* stream);
/* Moments of order n = img_type - HV_IMG_MOMENTS_0: per-bin weights f_k^n of the bins pmin..pmax
 * with the Nyquist compensation (bin T/2 of an even window twice for n = 0, 2, not at all for
 * n = 1), written as pmax - pmin + 1 floats at bin_w_f32 (device); and the moment frame
 * out = sum_k |X_k|^2 bin_w[k] with the same ring / weights conventions as hv_time_view.
 * Replaces fft_freqs + tensor_multiply_vector_nyquist_compensation (icompute.cc:26-69,
 * tools_compute.cu:38-97, fourier_transform.cc:244-338). */
hv_status hv_moment_bin_weights(float* bin_w_f32, int T, int pmin, int pmax, int img_type, float camera_fps,
                                void* stream);
hv_status hv_time_moments(const void* ring_c64, int T, int width, int height, const void* weights_c64, int K,
                          const float* bin_w_f32, int shift, float* out_f32, double* partials_f64, void* stream);
/* SSA_STFT weights (fourier_transform.cc:379-444): with V the eigenvectors of hv_pca_eigh
 * (complex128, column-major, ascending eigenvalues) and Q the columns q_start..q_start+q_width-1
 * (all T columns when q_width == 0), p_acc = FFT_t(H V_Q V_Q^H), so bin pmin+k of p_acc is the
 * ring contracted with W[k][s] = sum_{j in Q} V[s][j] sum_t conj(V[t][j]) exp(-2*pi*i*(pmin+k)*t/T).
 * Writes W for k <= pmax-pmin (complex64, same layout as hv_stft_weights); FP64 arithmetic. */
hv_status hv_ssa_weights(const void* eigenvectors_c128, int T, int q_start, int q_width, int pmin, int pmax,
                         void* weights_c64, void* stream);
/* Phase increase (phase_increase, tools_unwrap.cu:210-267, with the one-frame history that
 * converts.cc:251-263 sets up): X = sum_t ring[t] w[t] (the stored p plane, w = one row of
 * weights), d = arg(X conj(pred)), out = d + hist when use_hist, then hist = d and pred = X.
 * first != 0 takes pred = X. pred (complex64) and hist (float) are W*H device buffers kept by the
 * caller between windows; `minmax` needs hv_phase_increase_workspace(W*H) bytes and feeds
 * hv_rescale_float. */
hv_status hv_phase_increase(const void* ring_c64, int T, int width, int height, const void* w_c64, void* pred_c64,
                            float* hist_f32, int first, int use_hist, float* out_f32, void* minmax, void* stream);
size_t hv_phase_increase_workspace(size_t npix);
/* rescale_float (tools_conversion.cu:275-313) of a frame written by hv_phase_increase:
 * out = (in + |min|) * 65535 / (|max| + |min|) * post_scale, min / max over the first
 * min(npix, 16384) pixels as the reference's block reduction reads them. */
hv_status hv_rescale_float(const float* in_f32, size_t npix, const void* minmax, float post_scale, float* out_f32,
                           void* stream);
/* XZ / YZ slices (fill_32bit_slices, stft.cu:17-115): with X_t(x, y) = sum_s ring[s][y W + x]
 * weights[t][s] for every t < T (weights: all T rows, e.g. hv_stft_weights(w, T, 0, T-1), the
 * eigenvector columns for PCA, hv_ssa_weights with pmin 0, pmax T-1),
 * xz[t][x] = mean over y in [ymin, ymax] of view(X_t(x, y)), yz[y][t] = mean over x in [xmin, xmax];
 * view: hypotf (modulus, phase increase), hypotf^2 (squared modulus), atanf(Im/Re) + pi/2
 * (argument), 0 for other types. T <= 512; `work` needs hv_time_cuts_workspace bytes. */
hv_status hv_time_cuts(const void* ring_c64, int T, int width, int height, const void* weights_c64, int xmin, int xmax,
                       int ymin, int ymax, int img_type, float* xz_f32, float* yz_f32, void* work, void* stream);
size_t hv_time_cuts_workspace(int width, int height, int T, int xmin, int xmax, int ymin, int ymax);
/* STFT weights W[k][t] = exp(-2*pi*i*(pmin+k)*t/T), k <= pmax-pmin, computed in FP64. */
hv_status hv_stft_weights(void* weights_c64, int T, int pmin, int pmax, void* stream);

/* PCA: covariance C = H^H H of the ring (H = HW x T column-major view), FP32 accumulation,
 * written as complex128 T x T (both triangles). Replaces cov_matrix (matrix_operations.cc:9-26).
 * `work` must hold hv_pca_cov_workspace(T, W*H) bytes (for the tensor-core engine at 64 < T: the
 * split-BF16 planes of the ring, 8 T npix bytes, and the partial tiles). */
hv_status hv_pca_covariance(const void* ring_c64, int T, size_t npix, void* cov_c128, void* work, void* stream);
size_t hv_pca_cov_workspace(int T, size_t npix);
/* Covariance engine: 0 = automatic (tcgen05 split-BF16 tensor cores for T <= 1024 and frames of a
 * multiple of 8 pixels: one tile for T <= 64, 128 x 128 tiles of the Gram matrix above; else FP32
 * SIMT), 1 = FP32 SIMT, 2 = tensor cores only. Process-wide. */
void hv_pca_covariance_mode(int mode);
/* Sliding windows (time stride < T) in a Pipe: 1 (default) = recompute only the covariance rows
 * and columns of the 64-frame ring-slot blocks rewritten since the last window (tensor-core tiled
 * engine, T > 64; the result is bit-identical to a full recomputation), 0 = recompute all of it
 * every window. Process-wide; read at each render. */
void hv_pca_cov_incremental(int enable);
/* After the covariance's stream work finished: HV_ERR_TIMEOUT when a bounded device wait in the
 * tensor-core kernel gave up (results invalid), HV_OK otherwise. Synchronous read of `work`. */
hv_status hv_pca_covariance_status(const void* work);
/* Split-BF16 planes of a ring for the tiled tensor-core covariance (64 < T <= 1024, npix a multiple
 * of 8): planes[p][2 s + c][px], p = 0: hi = bf16_rn(x), p = 1: lo = bf16_rn(x - hi), c = 0 / 1: real /
 * imaginary part of pixel px of ring slot s; with `real` != 0 (a ring whose imaginary parts are 0,
 * such as the converted frames without a spatial transform) planes[p][s][px] of the real parts only.
 * hv_pca_planes_bytes: their size (8 T npix bytes, 4 T npix for `real`; 0 when the shape has none).
 * hv_pca_split_planes: planes of ring slots slot0 .. slot0 + n - 1 (mod T), as a Pipe writes them when
 * frames enter its ring. hv_pca_covariance_planes: the covariance from the planes (the engine
 * hv_pca_covariance runs on planes it splits into `work`; `work` here needs only the partial tiles,
 * hv_pca_cov_workspace(T, npix) - hv_pca_planes_bytes(T, npix, 0) bytes at least), bit-identical to
 * hv_pca_covariance's tensor-core engine on the ring for complex planes; `blocks` = ~0u for all of
 * it, else only the rows and columns of the slot blocks set (bit b: slots 64 b .. 64 b + 63 for
 * complex planes, 128 b .. 128 b + 127 for real ones), the other entries of `cov_c128` left as they
 * are. HV_ERR_UNSUPPORTED for the SIMT engine mode and shapes without planes. */
size_t hv_pca_planes_bytes(int T, size_t npix, int real);
hv_status hv_pca_split_planes(const void* ring_c64, int T, size_t npix, int slot0, int n, int real, void* planes,
                              void* stream);
hv_status hv_pca_covariance_planes(const void* planes, int T, size_t npix, int real, unsigned int blocks,
                                   void* cov_c128, void* work, void* stream);
/* Eigensolve of the Hermitian T x T complex128 matrix (both triangles read): ascending
 * eigenvalues, eigenvectors as columns. Replaces cusolverDnCheevd (matrix_operations.cc:44-65).
 * Writes the columns pmin..pmax as PCA weights W[k][t] = V[t][pmin+k] (complex64) when weights_c64
 * != NULL. With the default precision (HV_EIG_FP32, T <= 512) the Jacobi sweeps run in FP32 on a
 * power-of-two-scaled copy, every eigenvalue is the FP64 Rayleigh quotient of its normalised
 * vector, and the eigenvectors of ranks pmin..pmax (when 0 <= pmin <= pmax < T, at most 64 of
 * them) are then corrected in FP64 against `cov_c128` (two first-order residual corrections): those
 * are accurate to the FP64 level, the others to the FP32 sweeps' (~1e-6). `cov_c128` is overwritten
 * in HV_EIG_FP64 mode. `work` needs hv_pca_eigh_workspace(T) bytes. */
hv_status hv_pca_eigh(void* cov_c128, int T, double* eigenvalues, void* eigenvectors_c128, int pmin, int pmax,
                      void* weights_c64, void* work, void* stream);
size_t hv_pca_eigh_workspace(int T);
/* Jacobi sweep precision (process-wide). HV_EIG_FP32 (default): FP32 sweeps (T <= 64: one CTA,
 * shared memory; 64 < T <= 512: block-cyclic Jacobi over a cooperative grid) stopping at the
 * round-off level of the matrix, FP64 Rayleigh quotients, FP64 correction of the kept eigenvectors
 * (GB300 runs FP64 far below its FP32 rate: FP64 sweeps take 1.7 ms at T = 32 and 87 ms at T = 128,
 * against 0.24 and 1.6 ms). HV_EIG_FP64, and any T above 512: the sweeps themselves in FP64. */
enum { HV_EIG_FP32 = 0, HV_EIG_FP64 = 1 };
void hv_pca_eig_precision(int precision);
/* Orthonormalisation of the warm subspace iteration (T > 64, dominant components): 1 (default) a
 * Cholesky-QR of the iterate (its Gram matrix, a 32 x 32 factorisation, one product), with the
 * Gram-Schmidt kernel run instead when the factorisation meets a pivot below 1e-6; 0 Gram-Schmidt
 * always. Both span the same subspace; the Ritz pairs agree to FP32 round-off. */
void hv_pca_eig_cholqr(int enable);

/* 2-D phase unwrap of a float phase image, then rescale to [0, 65535]. Replaces unwrap_2d +
 * rescale_float_unwrap2d (tools_unwrap.cu:269-369, tools_conversion.cu:315-335). `work` must hold
 * hv_unwrap_workspace(W, H) bytes. */
hv_status hv_unwrap_2d(const float* in, float* out, int width, int height, void* work, void* stream);
size_t hv_unwrap_workspace(int width, int height);

/* hv_unwrap_2d for callers that cannot allocate device memory (no counterpart in the reference).
 * Acquisition callbacks on a driver thread, or applications that forbid cudaMalloc once frames are
 * streaming, cannot provide `work`: this entry point takes none and calls no cudaMalloc, cudaFree or
 * allocating library routine. Its scratch is a static device array inside the library, sized for
 * frames of at most HV_UNWRAP_NOALLOC_MAX_PIXELS pixels; larger frames fail with HV_INVALID_VALUE.
 * Every GPU that loads the library keeps that array (8 MiB) until the process exits.
 * The first call on each device looks up the array's device address (with that device current),
 * and under CUDA's lazy module loading it is also when the driver creates the array on that
 * device: make that first call before streaming starts (and before any stream capture); later
 * calls allocate nothing. All calls share the one array: calls whose GPU
 * work overlaps (different streams, or different host threads) race and corrupt each other's
 * results, so serialise them on one stream. Results match hv_unwrap_2d. */
#define HV_UNWRAP_NOALLOC_MAX_PIXELS 262144
hv_status hv_unwrap_2d_noalloc(const float* in, float* out, int width, int height, void* stream);

/* Renormalisation x <- x * 2^c * N / sum(x), the sum being taken from `partials_f64`
 * (npartials entries) or computed here when partials_f64 is NULL. Replaces gpu_normalize
 * (tools_compute.cu:99-123). `work` needs hv_reduce_workspace(n) bytes. */
hv_status hv_renormalize(float* frame, size_t n, int renorm_constant, const double* partials_f64, int npartials,
                         void* work, void* stream);
size_t hv_reduce_workspace(size_t n);
/* In-place quadrant swap (fftshift for even sizes). Replaces shift_corners (shift_corners.cu:8-70). */
hv_status hv_shift_corners(float* frame, int width, int height, void* stream);
/* Writes `frame` into slot `slot` of an A-frame float ring and stores into `out` the mean of
 * `count` frames starting at slot `start` (circular). Replaces Queue::enqueue +
 * accumulate_images (tools_conversion.cu:418-458, image_accumulation.cc:136-157). */
hv_status hv_accumulate(const float* frame, float* acc_ring, int A, int slot, int start, int count, float* out,
                        size_t n, void* stream);
/* In-place log10 (map_log10, rendering.cc:127-138). */
hv_status hv_log10(float* frame, size_t n, void* stream);

/* Autocontrast: the values at percentiles `lower` and `upper` of the frame (or of the reticle
 * disc when reticle_scale > 0), clamped to >= 1, written to range_f32[0..1] on the device.
 * Exact selection (radix select), identical to sorting. Replaces compute_percentile_xy_view
 * + ContrastApi::update_contrast (percentile.cu:75-94,139-222; contrast_api.cc:137-146).
 * `work` needs hv_percentile_workspace(width*height) bytes. */
hv_status hv_percentile(const float* frame, int width, int height, float lower, float upper, float reticle_scale,
                        float* range_f32, void* work, void* stream);
size_t hv_percentile_workspace(size_t n);
/* Contrast map x <- 65535/(max-min+FLT_EPSILON)*(x-min) (min/max from range_f32 on the device,
 * swapped when invert) then float->ushort (clamp <=0 -> 0, >65535 -> 65535, truncation).
 * apply_contrast = 0 skips the map. Replaces apply_contrast_correction + float_to_ushort
 * (contrast_correction.cu:5-17, tools_conversion.cu:350-387). */
hv_status hv_contrast_to_ushort(const float* frame, const float* range_f32, int invert, int apply_contrast,
                                uint16_t* out, size_t n, void* stream);

/* ================================================================================ serving
 * No reference counterpart (the reference runs one Pipe per process on one compute thread,
 * Backend/sources/core/pipe.cc:650-676). A server runs many frame streams on one GPU: each
 * stream is a Pipe (same settings, kernels and outputs as hv_pipe_*) whose cycles are launched by
 * one persistent engine thread. Streams are admitted by device footprint against an HBM budget;
 * same-shape streams (width, height, depth, space / time transform, T, batch) share a bucket
 * whose steady streams are replayed from one CUDA graph per engine pass (one launch per bucket),
 * the others launched directly; buckets run on their own CUDA streams and overlap. Requirements
 * per stream: batch_size <= time_transformation_size. All calls are thread-safe; push and pull of
 * one stream from one thread each, and a stream is not closed while it is being pushed or pulled. */
typedef struct hv_server hv_server;
/* HV_SERVER_NO_GRAPHS: launch every cycle directly (for comparison).
 * HV_SERVER_STREAM_GRAPHS: every stream on its own CUDA stream, replaying its own graph (no
 * barrier between the streams' cycles) instead of one graph per bucket. */
enum { HV_SERVER_NO_GRAPHS = 1, HV_SERVER_STREAM_GRAPHS = 2 };
typedef struct hv_server_stats
{
    uint64_t batches;        /* stream cycles planned (batches consumed) */
    uint64_t outputs;        /* holograms rendered */
    uint64_t graph_launches; /* bucket graph launches */
    uint64_t graph_kernels;  /* kernel nodes executed by those launches */
    uint64_t eager_cycles;   /* stream cycles launched directly */
    uint64_t captures;       /* bucket graph captures */
    uint64_t latency_samples;
    double latency_p50_us;   /* batch complete (push) -> hologram ready, last 8192 outputs */
    double latency_p99_us;
    int32_t streams, buckets;
    size_t hbm_used, hbm_budget;
} hv_server_stats;
/* hbm_budget_bytes = 0: 90% of the currently free device memory. */
hv_server* hv_server_create(size_t hbm_budget_bytes, int flags, hv_status* status);
void hv_server_destroy(hv_server* server);
/* Device bytes a served stream holds (its admission cost); 0 for invalid settings. */
size_t hv_server_stream_footprint(const hv_frame_desc* fd, const hv_settings* settings);
/* Admits a stream: HV_ERR_ADMISSION when its footprint does not fit within admit_timeout_us
 * (0: do not wait) while other streams hold the budget. */
hv_status hv_server_open_stream(hv_server* server, const hv_frame_desc* fd, const hv_settings* settings,
                                int64_t admit_timeout_us, int32_t* stream_id);
hv_status hv_server_close_stream(hv_server* server, int32_t stream_id);
/* Stages n frames (host or device memory, like hv_pipe_push_frames); blocks (10 s bound) while
 * every input slot of the stream holds a batch not yet launched. */
hv_status hv_server_push(hv_server* server, int32_t stream_id, const void* frames, size_t n, int mem);
size_t hv_server_output_count(hv_server* server, int32_t stream_id);
/* Oldest rendered hologram of the stream (waits up to timeout_us for one; < 0 waits without bound). */
hv_status hv_server_pull(hv_server* server, int32_t stream_id, uint16_t* dst, int mem, int64_t timeout_us);
/* Float frame fed to the contrast stage by the stream's last rendered cycle (after hv_server_sync). */
hv_status hv_server_get_float_frame(hv_server* server, int32_t stream_id, float* dst);
/* Waits until every staged batch has been launched and the device work has finished. */
hv_status hv_server_sync(hv_server* server, int64_t timeout_us);
hv_status hv_server_get_stats(hv_server* server, hv_server_stats* stats);
hv_status hv_server_reset_stats(hv_server* server);
/* Continuous batching: a bucket whose graph-replayed streams are only partly ready waits up to
 * window_us (default 1500) after its oldest ready batch for the others, then launches the bucket
 * graph (at least half ready) or the ready streams' own graphs. 0 launches immediately. */
hv_status hv_server_set_batch_window(hv_server* server, int64_t window_us);

/* ================================================================================ .holo files
 * The reference's recording format (Backend/includes/io/holo_file.hh:1-81): a 64-byte header,
 * the raw frames, a JSON footer {"compute_settings": {...}, "info": {...}}. Reading replaces
 * InputHoloFile (input_holo_file.cc:18-157) and converts footers of versions 2..6 and compute
 * settings of version v0 to the current layout like HoloFileConverter / ComputeSettingsConverter
 * (holo_file_converter.cc, compute_settings_converter.cc), for the keys of this path; writing
 * replaces OutputHoloFile (output_holo_file.cc:10-131). Host-only: no GPU is used. Strings are
 * returned into caller buffers: *len receives the length; a call with buf = NULL, cap = 0 only
 * queries it. */
enum { HV_HOLO_RAW = 0, HV_HOLO_PROCESSED = 1, HV_HOLO_MOMENTS = 2 }; /* header data_type */
typedef struct hv_holo_header
{
    char magic[4];            /* "HOLO" */
    uint16_t version;         /* 7 when written here */
    uint16_t bits_per_pixel;  /* 8 * bytes per pixel */
    uint32_t width, height, img_nb;
    uint64_t total_data_size; /* width * height * img_nb * bytes per pixel */
    uint8_t endianness;       /* 1: big endian frames */
    uint8_t data_type;        /* HV_HOLO_*, 0 for files older than version 7 */
} hv_holo_header;
typedef struct hv_holo_file hv_holo_file;
hv_status hv_holo_open(const char* path, hv_holo_file** file);
void hv_holo_close(hv_holo_file* file);
hv_status hv_holo_get_header(const hv_holo_file* file, hv_holo_header* header, hv_frame_desc* fd);
/* n frames from frame `first` into host memory (n * frame bytes). */
hv_status hv_holo_read_frames(hv_holo_file* file, uint64_t first, uint64_t n, void* dst);
/* The footer converted to the current version (an empty object when the file has none). */
hv_status hv_holo_get_footer(const hv_holo_file* file, char* buf, size_t cap, size_t* len);
/* The footer's compute settings applied over *settings (keys this build does not use are skipped)
 * and the pixel size from info.pixel_pitch.x; HV_NO_IN_DATA when the file has no footer. */
hv_status hv_holo_get_settings(const hv_holo_file* file, hv_settings* settings);
typedef struct hv_holo_writer hv_holo_writer;
hv_status hv_holo_create(const char* path, const hv_frame_desc* fd, int data_type, hv_holo_writer** writer);
hv_status hv_holo_write_frames(hv_holo_writer* writer, const void* frames, uint64_t n);
/* Appends the footer (may be NULL), writes the final image count into the header, closes and frees. */
hv_status hv_holo_finish(hv_holo_writer* writer, const char* footer_json);
/* The footer the reference writes for these settings (OutputHoloFile::export_compute_settings). */
hv_status hv_holo_make_footer(const hv_settings* settings, int input_fps, int camera_fps, char* buf, size_t cap,
                              size_t* len);
/* A footer of `version` converted to the current version. */
hv_status hv_holo_convert_footer(const char* footer_json, int version, char* buf, size_t cap, size_t* len);
/* The compute-settings document (current layout, v1) of a settings record, and the conversion of
 * a compute-settings document to the current version. */
hv_status hv_settings_to_json(const hv_settings* settings, char* buf, size_t cap, size_t* len);
hv_status hv_settings_convert_json(const char* json, char* buf, size_t cap, size_t* len);

#ifdef __cplusplus
}
#endif

#endif /* HOLOVIBES_GB300_H */
