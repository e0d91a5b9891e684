// Cycle driver for the reference's own GPU build of the hologram path. TEST INFRASTRUCTURE ONLY.
//
// Compiled by oracle/ref_build.py together with the reference's unmodified hot-path translation
// units (Backend/cuda_sources/*.cu, Backend/sources/compute/matrix_operations.cc, the cuFFT / cuBLAS
// / cuSOLVER handle singletons). It replays one Pipe cycle in the order of Pipe::refresh
// (Backend/sources/core/pipe.cc:255-387) by calling the reference's functions with the arguments
// its compute classes pass:
//
//   wait_time_stride                      pipe.cc:400-416
//   input_queue_to_input_buffer           converts.cc:369-396
//   fresnel_transform_lens + transform    fourier_transform.cc:93-119 (lens once per refresh)
//   angular_spectrum_lens + shift_corners fourier_transform.cc:121-150
//   Queue::enqueue_multiple (ring)        queue.cc:332-380 (restated here: the Queue class needs the
//                                         whole data_struct layer), incl. its stream synchronisation
//   stft (plan of ICompute::update_stft)  fourier_transform.cc:231-242, icompute.cc:109-115
//   cov_matrix / eigen_values_vectors /
//   matrix_multiply_complex               fourier_transform.cc:340-377
//   p range, complex_to_*, x131071        converts.cc:20-92
//   unwrap_2d + rescale_float_unwrap2d    converts.cc:214-248
//   gpu_normalize                         postprocessing.cc:135-155
//   shift_corners                         rendering.cc:21-40
//   accumulate_images                     image_accumulation.cc:136-157 (Queue::enqueue restated,
//                                         queue.cc:149-189)
//   map_log10                             rendering.cc:127-138
//   compute_percentile_xy_view            rendering.cc:239-340 (gating of should_apply_contrast)
//   apply_contrast_correction             rendering.cc:185-237
//   float_to_ushort                       converts.cc:307-319
//   cudaStreamSynchronize                 pipe.cc:386
//
// It is never linked into the product. Tests and the bench load it through ctypes (hvref_*).

#include <cuComplex.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <cufftXt.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "angular_spectrum.cuh"
#include "compute_bundles_2d.hh"
#include "contrast_correction.cuh"
#include "cublas_handle.hh"
#include "cufft_handle.hh"
#include "cusolver_handle.hh"
#include "frame_desc.hh"
#include "fresnel_transform.cuh"
#include "map.cuh"
#include "matrix_operations.hh"
#include "percentile.cuh"
#include "shift_corners.cuh"
#include "stft.cuh"
#include "tools_compute.cuh"
#include "tools_conversion.cuh"
#include "tools_unwrap.cuh"

extern "C" {
struct hvref_config
{
    int width, height, depth;  // depth: bytes per raw pixel (1, 2, 4)
    int space;                 // 0 none, 1 Fresnel (FFT1), 2 angular spectrum (FFT2)
    int time;                  // 0 none, 1 STFT, 2 PCA
    int time_transformation_size, time_stride, batch_size;
    float lambda, z, pixel_size;  // metres, metres, micrometres (the settings' units)
    int img_type;                 // 0 modulus, 1 squared modulus, 2 argument
    int p_start, p_width;
    int fft_shift, renorm, renorm_constant;
    int accumulation;
    int log_enabled;
    int contrast_enabled, contrast_invert;
    float contrast_lower, contrast_upper;
    int unwrap_2d;
    int keep_float_frame;  // copy the frame fed to the contrast stage aside for hvref_float_frame
};
}

namespace
{
using holovibes::compute::cov_matrix;
using holovibes::compute::eigen_values_vectors;
using holovibes::compute::eigen_values_vectors_work_buffer_size;
using holovibes::compute::matrix_multiply_complex;

#define HVREF_CUDA(x)                                                                              \
    do                                                                                             \
    {                                                                                              \
        cudaError_t e_ = (x);                                                                      \
        if (e_ != cudaSuccess)                                                                     \
            throw std::runtime_error(std::string(#x) + ": " + cudaGetErrorString(e_));             \
    } while (0)

template <typename T>
T* dalloc(size_t n)
{
    void* p = nullptr;
    HVREF_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    return static_cast<T*>(p);
}

// A circular device queue of fixed-size frames with the reference Queue's slot arithmetic.
struct FrameRing
{
    char* data = nullptr;
    size_t frame_bytes = 0;
    unsigned max_size = 0, start = 0, size = 0;

    // queue.cc:332-380
    void enqueue_multiple(const char* elts, unsigned nb, cudaStream_t s)
    {
        if (nb > max_size)
        {
            elts += size_t(nb - max_size) * frame_bytes;
            start = (start + nb - max_size) % max_size;
            nb = max_size;
        }
        const unsigned begin = (start + size) % max_size;
        if (begin + nb > max_size)
        {
            const unsigned at_end = max_size - begin;
            HVREF_CUDA(cudaMemcpyAsync(data + size_t(begin) * frame_bytes, elts, size_t(at_end) * frame_bytes,
                                       cudaMemcpyDeviceToDevice, s));
            HVREF_CUDA(cudaMemcpyAsync(data, elts + size_t(at_end) * frame_bytes, size_t(nb - at_end) * frame_bytes,
                                       cudaMemcpyDeviceToDevice, s));
        }
        else
            HVREF_CUDA(cudaMemcpyAsync(data + size_t(begin) * frame_bytes, elts, size_t(nb) * frame_bytes,
                                       cudaMemcpyDeviceToDevice, s));
        HVREF_CUDA(cudaStreamSynchronize(s));
        size += nb;
        if (size > max_size)
        {
            start = (start + size - max_size) % max_size;
            size = max_size;
        }
    }

    // queue.cc:149-189
    void enqueue(const char* elt, cudaStream_t s)
    {
        const unsigned end = (start + size) % max_size;
        HVREF_CUDA(cudaMemcpyAsync(data + size_t(end) * frame_bytes, elt, frame_bytes, cudaMemcpyDeviceToDevice, s));
        HVREF_CUDA(cudaStreamSynchronize(s));
        if (size < max_size)
            ++size;
        else
            start = (start + 1) % max_size;
    }
};

struct RefPipe
{
    hvref_config c{};
    camera::FrameDescriptor fd{};
    size_t frame_res = 0;
    cudaStream_t stream = nullptr;
    holovibes::cuda_tools::CufftHandle spatial_plan, stft_plan, unwrap_plan;
    cuComplex* lens = nullptr;
    unsigned lens_side = 0;
    void* raw = nullptr;            // device copy of one raw batch
    cuComplex* spatial = nullptr;   // B x HW
    FrameRing ring;                 // T x HW complex
    cuComplex* p_acc = nullptr;     // T x HW complex
    cuComplex* cov = nullptr;       // T x T
    float* eig = nullptr;
    int* dev_info = nullptr;
    cuComplex* cusolver_work = nullptr;
    int cusolver_work_size = 0;
    float* post = nullptr;          // the post-processing float frame
    float* float_copy = nullptr;    // the frame fed to the contrast stage (kept aside on request)
    float* acc_avg = nullptr;
    FrameRing acc;                  // accumulation queue, A x HW float
    double* reduce_result = nullptr;
    unsigned short* out = nullptr;
    holovibes::UnwrappingResources_2d* unwrap = nullptr;
    unsigned batch_index = 0;
    bool autocontrast_pending = true;
    float contrast_min = 1.f, contrast_max = 65535.f;
    int outputs = 0;
    bool last_output_valid = false;

    explicit RefPipe(const hvref_config& cfg)
        : c(cfg)
    {
        fd.width = static_cast<unsigned short>(c.width);
        fd.height = static_cast<unsigned short>(c.height);
        fd.depth = static_cast<camera::PixelDepth>(c.depth);
        fd.byteEndian = camera::LittleEndian;
        frame_res = fd.get_frame_res();
        const size_t B = c.batch_size, T = c.time_transformation_size;
        HVREF_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        // compute_worker.cc:13-21: the library handles run on the pipe's stream
        holovibes::cuda_tools::CufftHandle::set_stream(stream);
        holovibes::cuda_tools::CublasHandle::set_stream(stream);
        holovibes::cuda_tools::CusolverHandle::set_stream(stream);

        raw = dalloc<char>(B * frame_res * c.depth);
        spatial = dalloc<cuComplex>(B * frame_res);
        ring.frame_bytes = frame_res * sizeof(cuComplex);
        ring.max_size = static_cast<unsigned>(T);
        ring.data = reinterpret_cast<char*>(dalloc<cuComplex>(T * frame_res));
        p_acc = dalloc<cuComplex>(T * frame_res);
        post = dalloc<float>(frame_res);
        float_copy = dalloc<float>(frame_res);
        acc_avg = dalloc<float>(frame_res);
        reduce_result = dalloc<double>(1);
        out = dalloc<unsigned short>(frame_res);
        if (c.accumulation > 1)
        {
            acc.frame_bytes = frame_res * sizeof(float);
            acc.max_size = static_cast<unsigned>(c.accumulation);
            acc.data = reinterpret_cast<char*>(dalloc<float>(size_t(c.accumulation) * frame_res));
        }
        autocontrast_pending = c.contrast_enabled != 0;

        // ICompute::update_spatial_transformation_parameters (icompute.cc:158-180)
        long long n[] = {fd.height, fd.width};
        spatial_plan.XtplanMany(2, n, n, 1, static_cast<long long>(frame_res), CUDA_C_32F, n, 1,
                                static_cast<long long>(frame_res), CUDA_C_32F, static_cast<long long>(B), CUDA_C_32F);
        if (c.time == 1)
        {
            // ICompute::update_stft (icompute.cc:109-115)
            int inembed[1] = {static_cast<int>(T)};
            const int zone = static_cast<int>(frame_res);
            stft_plan.planMany(1, inembed, inembed, zone, 1, inembed, zone, 1, CUFFT_C2C, zone);
        }
        if (c.time == 2)
        {
            cov = dalloc<cuComplex>(T * T);
            eig = dalloc<float>(T);
            dev_info = dalloc<int>(1);
            cusolver_work_size = eigen_values_vectors_work_buffer_size(static_cast<int>(T));
            cusolver_work = dalloc<cuComplex>(cusolver_work_size);
        }
        if (c.img_type == 2 && c.unwrap_2d)
        {
            unwrap_plan.plan(fd.width, fd.height, CUFFT_C2C);  // icompute.hh:140
            unwrap = new holovibes::UnwrappingResources_2d(frame_res, stream);
        }
        // lenses, once per refresh
        if (c.space == 1)
        {
            lens_side = std::max(fd.height, fd.width);
            lens = dalloc<cuComplex>(size_t(lens_side) * lens_side);
            fresnel_transform_lens(lens, lens_side, fd.height, fd.width, c.lambda, c.z, c.pixel_size, stream);
        }
        else if (c.space == 2)
        {
            lens = dalloc<cuComplex>(frame_res);
            angular_spectrum_lens(lens, fd.width, fd.height, c.z, c.lambda, c.pixel_size * 1e-6f,
                                  c.pixel_size * 1e-6f, stream);
            shift_corners(lens, 1, fd.width, fd.height, stream);
        }
        HVREF_CUDA(cudaStreamSynchronize(stream));
    }

    ~RefPipe()
    {
        cudaStreamSynchronize(stream);
        delete unwrap;
        for (void* p : std::initializer_list<void*>{lens, raw, spatial, ring.data, p_acc, cov, eig, dev_info,
                                                    cusolver_work, post, float_copy, acc_avg, acc.data, reduce_result,
                                                    out})
            if (p)
                cudaFree(p);
        spatial_plan.reset();
        stft_plan.reset();
        unwrap_plan.reset();
        cudaStreamDestroy(stream);
    }

    // One Pipe cycle for one batch already in `raw` (device). Returns 1 when a hologram was output.
    int cycle()
    {
        last_output_valid = false;
        const unsigned B = c.batch_size, T = c.time_transformation_size;
        // wait_time_stride
        batch_index += B;
        if (batch_index != static_cast<unsigned>(c.time_stride))
            return 0;
        batch_index = 0;
        // convert to complex
        input_queue_to_input_buffer(spatial, raw, frame_res, static_cast<int>(B), fd.depth, stream);
        // spatial transform
        if (c.space == 1)
            fresnel_transform(spatial, spatial, B, lens, spatial_plan, frame_res, stream);
        else if (c.space == 2)
            angular_spectrum(spatial, spatial, B, lens, nullptr, false, spatial_plan, fd, stream);
        // transfer into the time transformation queue
        ring.enqueue_multiple(reinterpret_cast<const char*>(spatial), B, stream);
        // wait_time_transformation_size (pipe.cc:418-431)
        if (ring.size < T)
            return 0;
        cuComplex* H = reinterpret_cast<cuComplex*>(ring.data);
        if (c.time == 1)
            stft(p_acc, H, stft_plan);
        else if (c.time == 2)
        {
            cuComplex* V = nullptr;
            cov_matrix(H, static_cast<int>(frame_res), static_cast<int>(T), cov);
            eigen_values_vectors(cov, static_cast<int>(T), eig, &V, cusolver_work, cusolver_work_size, dev_info);
            matrix_multiply_complex(H, V, static_cast<int>(frame_res), static_cast<int>(T), static_cast<int>(T), p_acc);
        }
        else
            HVREF_CUDA(cudaMemcpyAsync(p_acc, H, size_t(T) * frame_res * sizeof(cuComplex), cudaMemcpyDeviceToDevice,
                                       stream));
        // p range (converts.cc:76-92)
        const int pmin = c.p_start;
        const int pmax = c.p_width != 0 ? std::max(0, std::min<int>(pmin + c.p_width, static_cast<int>(T))) : pmin;
        if (c.img_type == 0)
            complex_to_modulus(post, p_acc, pmin, pmax, frame_res, stream);
        else if (c.img_type == 1)
            complex_to_squared_modulus(post, p_acc, pmin, pmax, frame_res, stream);
        else
        {
            complex_to_argument(post, p_acc, pmin, pmax, frame_res, stream);
            if (c.unwrap_2d)
            {
                unwrap_2d(unwrap->gpu_angle_, post, unwrap_plan, unwrap, fd, stream);
                rescale_float_unwrap2d(post, unwrap->gpu_angle_, unwrap->minmax_buffer_, frame_res, stream);
            }
        }
        if (c.time == 2)
            map_multiply(post, post, frame_res, static_cast<const float>((2 << 16) - 1), stream);
        if (c.renorm)
            gpu_normalize(post, reduce_result, frame_res, c.renorm_constant, stream);
        if (c.fft_shift)
            shift_corners(post, 1, fd.width, fd.height, stream);
        if (c.accumulation > 1)
        {
            acc.enqueue(reinterpret_cast<const char*>(post), stream);
            accumulate_images(acc_avg, reinterpret_cast<const float*>(acc.data), acc.start, acc.max_size, acc.size,
                              frame_res, stream);
            HVREF_CUDA(cudaMemcpyAsync(post, acc_avg, frame_res * sizeof(float), cudaMemcpyDeviceToDevice, stream));
        }
        if (c.log_enabled)
            map_log10(post, post, frame_res, stream);
        if (c.keep_float_frame)
            HVREF_CUDA(cudaMemcpyAsync(float_copy, post, frame_res * sizeof(float), cudaMemcpyDeviceToDevice, stream));
        if (c.contrast_enabled)
        {
            // the time queue is full here; should_apply_contrast (rendering.hh:168-181)
            const bool acc_gate = c.accumulation <= 1 || acc.size == acc.max_size || acc.size == 1;
            if (autocontrast_pending && acc_gate)
            {
                const float percent_in[2] = {c.contrast_lower, c.contrast_upper};
                float out_pct[2] = {0.f, 0.f};
                compute_percentile_xy_view(post, fd.width, fd.height, 0, percent_in, out_pct, 2, 0.5f, false, stream);
                // ContrastApi::update_contrast (contrast_api.cc:137-146) clamps both ends to >= 1
                contrast_min = out_pct[0] > 1.0f ? out_pct[0] : 1.0f;
                contrast_max = out_pct[1] > 1.0f ? out_pct[1] : 1.0f;
                if (c.accumulation <= 1 || acc.size == acc.max_size)
                    autocontrast_pending = false;
            }
            const float lo = c.contrast_invert ? contrast_max : contrast_min;
            const float hi = c.contrast_invert ? contrast_min : contrast_max;
            apply_contrast_correction(post, static_cast<unsigned>(frame_res), 65535, lo, hi, stream);
        }
        float_to_ushort(out, post, frame_res, stream);
        HVREF_CUDA(cudaStreamSynchronize(stream));  // end of the cycle (pipe.cc:386)
        ++outputs;
        last_output_valid = true;
        return 1;
    }
};

thread_local std::string g_error;

template <typename F>
int guarded(F&& f)
{
    try
    {
        return f();
    }
    catch (const std::exception& e)
    {
        g_error = e.what();
        return -1;
    }
}
}  // namespace

extern "C" {

const char* hvref_last_error() { return g_error.c_str(); }

void* hvref_create(const hvref_config* cfg)
{
    try
    {
        if (!cfg || cfg->width <= 0 || cfg->height <= 0 || cfg->batch_size <= 0 || cfg->time_transformation_size <= 0 ||
            cfg->time_stride <= 0)
            throw std::runtime_error("invalid configuration");
        return new RefPipe(*cfg);
    }
    catch (const std::exception& e)
    {
        g_error = e.what();
        return nullptr;
    }
}

void hvref_destroy(void* p) { delete static_cast<RefPipe*>(p); }

// One batch (batch_size raw frames) from host or device memory through one Pipe cycle.
// Returns 1 when a hologram was produced, 0 when the cycle was gated, -1 on error.
int hvref_push(void* h, const void* batch, int on_device)
{
    return guarded(
        [&]
        {
            RefPipe* p = static_cast<RefPipe*>(h);
            const size_t bytes = size_t(p->c.batch_size) * p->frame_res * p->c.depth;
            HVREF_CUDA(cudaMemcpyAsync(p->raw, batch, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                       p->stream));
            return p->cycle();
        });
}

// `count` consecutive cycles over `nbatches` device-resident batches (batch i % nbatches), each
// consumed in place; returns the elapsed milliseconds (host clock around the cycles, which end
// with the reference's stream synchronisation), or -1.
double hvref_run_device_batches(void* h, const void* const* batches, int nbatches, int count)
{
    RefPipe* p = static_cast<RefPipe*>(h);
    try
    {
        HVREF_CUDA(cudaStreamSynchronize(p->stream));
        cudaEvent_t e0, e1;
        HVREF_CUDA(cudaEventCreate(&e0));
        HVREF_CUDA(cudaEventCreate(&e1));
        HVREF_CUDA(cudaEventRecord(e0, p->stream));
        void* saved = p->raw;
        for (int i = 0; i < count; ++i)
        {
            p->raw = const_cast<void*>(batches[i % nbatches]);
            p->cycle();
        }
        p->raw = saved;
        HVREF_CUDA(cudaEventRecord(e1, p->stream));
        HVREF_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        HVREF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return ms;
    }
    catch (const std::exception& e)
    {
        g_error = e.what();
        return -1.0;
    }
}

int hvref_outputs(void* h) { return static_cast<RefPipe*>(h)->outputs; }

int hvref_output(void* h, unsigned short* host)
{
    return guarded(
        [&]
        {
            RefPipe* p = static_cast<RefPipe*>(h);
            HVREF_CUDA(cudaMemcpy(host, p->out, p->frame_res * sizeof(unsigned short), cudaMemcpyDeviceToHost));
            return 0;
        });
}

int hvref_float_frame(void* h, float* host)
{
    return guarded(
        [&]
        {
            RefPipe* p = static_cast<RefPipe*>(h);
            if (!p->c.keep_float_frame)
                throw std::runtime_error("keep_float_frame is off");
            HVREF_CUDA(cudaMemcpy(host, p->float_copy, p->frame_res * sizeof(float), cudaMemcpyDeviceToHost));
            return 0;
        });
}

int hvref_contrast_range(void* h, float* lo_hi)
{
    RefPipe* p = static_cast<RefPipe*>(h);
    lo_hi[0] = p->contrast_min;
    lo_hi[1] = p->contrast_max;
    return 0;
}

// The time transformation queue: storage (T x HW complex64, slot order), start index and size.
int hvref_ring(void* h, void* host, int* start, int* size)
{
    return guarded(
        [&]
        {
            RefPipe* p = static_cast<RefPipe*>(h);
            HVREF_CUDA(cudaMemcpy(host, p->ring.data, size_t(p->ring.max_size) * p->ring.frame_bytes,
                                  cudaMemcpyDeviceToHost));
            *start = static_cast<int>(p->ring.start);
            *size = static_cast<int>(p->ring.size);
            return 0;
        });
}

// The lens as the reference's transform reads it (H x W complex64: the Fresnel lens after the
// centre crop, the angular-spectrum transfer function after shift_corners). Returns H x W.
long long hvref_lens(void* h, void* host)
{
    RefPipe* p = static_cast<RefPipe*>(h);
    if (!p->lens)
        return 0;
    const size_t n = p->frame_res;
    if (host && cudaMemcpy(host, p->lens, n * sizeof(cuComplex), cudaMemcpyDeviceToHost) != cudaSuccess)
        return -1;
    return static_cast<long long>(n);
}

// PCA only: the eigenvalues of the last window (ascending, FP32 from cusolverDnCheevd).
int hvref_eigenvalues(void* h, float* host)
{
    return guarded(
        [&]
        {
            RefPipe* p = static_cast<RefPipe*>(h);
            if (!p->eig)
                throw std::runtime_error("not a PCA pipe");
            HVREF_CUDA(cudaMemcpy(host, p->eig, size_t(p->c.time_transformation_size) * sizeof(float),
                                  cudaMemcpyDeviceToHost));
            return 0;
        });
}
}
