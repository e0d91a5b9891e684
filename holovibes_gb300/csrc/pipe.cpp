// The Pipe: a GB300-native drop-in for the reference's Pipe / ICompute engine.
//
// Reference behaviour (Holovibes):
//   buffers / ctor       Backend/includes/core/icompute.hh:123-171, Backend/sources/core/icompute.cc:71-175
//   step list (refresh)  Backend/sources/core/pipe.cc:255-387
//   cycle (exec)         Backend/sources/core/pipe.cc:650-676
//   stride gate          Backend/sources/core/pipe.cc:400-416 (process the batch at which the batch
//                        counter reaches time_stride, drop the others)
//   wait T               Backend/sources/core/pipe.cc:418-427 (no output until the ring is full)
//   ring enqueue         Backend/sources/data_struct/queue.cc:332-380
//   accumulation queue   Backend/sources/data_struct/queue.cc:149-189, image_accumulation.cc:136-157
//   autocontrast gating  Backend/sources/compute/rendering.cc:239-299, rendering.hh:168-181
//   input queue          Backend/sources/data_struct/batch_input_queue.cc:124-235
//   output queue         Backend/sources/core/pipe.cc:491-524
//
// GB300 design: the host bookkeeping of a cycle (stride gate, ring indices, accumulation
// indices, autocontrast flags) is deterministic, so it runs at enqueue time on the caller's
// thread and every cycle is a stream of kernel launches with no host round trip (the reference
// synchronises the stream inside Queue::enqueue_multiple, on percentile D2H copies and at the
// end of each cycle). Raw frames arrive in a device ring of batch slots through a copy stream;
// outputs leave through a device ring of uint16 frames with one event each.
#include <chrono>
#include <cstring>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "pipe_internal.h"

namespace hv {
void settings_default(hv_settings* s);
hv_status settings_validate(hv_settings* s, const hv_frame_desc* fd);
}  // namespace hv

using namespace hv;

namespace {

template <class T>
hv_status dalloc(hv_pipe* p, T*& ptr, size_t bytes)
{
    void* v = nullptr;
    if (bytes == 0)
        bytes = 16;
    cudaError_t e = cudaMalloc(&v, bytes);
    if (e != cudaSuccess)
    {
        set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
        return e == cudaErrorMemoryAllocation ? HV_ERR_OOM : HV_ERR_CUDA;
    }
    p->allocs.push_back(v);
    ptr = static_cast<T*>(v);
    return HV_OK;
}

void free_buffers(hv_pipe* p)
{
    for (void* v : p->allocs)
        cudaFree(v);
    p->allocs.clear();
    for (hv_pipe::Lane& L : p->lanes)
    {
        for (cudaEvent_t* e : {&L.ready, &L.free})
            if (*e)
            {
                cudaEventDestroy(*e);
                *e = nullptr;
            }
        L = hv_pipe::Lane{};
    }
    for (cudaEvent_t* e : {&p->join_ev, &p->range_ev, &p->pp_cov_ev[0], &p->pp_cov_ev[1], &p->pp_eig_ev[0],
                           &p->pp_eig_ev[1], &p->pp_view_ev[0], &p->pp_view_ev[1], &p->pp_main_ev, &p->pp_ring_ev[0],
                           &p->pp_ring_ev[1], &p->pp_ring_ev[2], &p->pp_ring_ev[3]})
        if (*e)
        {
            cudaEventDestroy(*e);
            *e = nullptr;
        }
    p->pp = false;
    p->range_ev_set = false;
    for (auto* vec : {&p->in_filled, &p->in_consumed, &p->out_ready, &p->out_freed, &p->views[0].out_ready,
                      &p->views[0].out_freed, &p->views[1].out_ready, &p->views[1].out_freed, &p->views[2].out_ready,
                      &p->views[2].out_freed})
    {
        for (cudaEvent_t e : *vec)
            cudaEventDestroy(e);
        vec->clear();
    }
}

bool uses_pca(const hv_settings& s) { return s.time_transformation == HV_TIME_PCA; }
// PCA and SSA_STFT both run the covariance and the eigensolve every window
bool uses_eig(const hv_settings& s)
{
    return s.time_transformation == HV_TIME_PCA || s.time_transformation == HV_TIME_SSA_STFT;
}
bool uses_phase_increase(const hv_settings& s) { return s.image_type == HV_IMG_PHASE_INCREASE; }
bool use_view_tc(const hv_settings& s, int K, size_t HW) { return !uses_phase_increase(s) && view_engine_tc(K, HW); }
bool uses_unwrap(const hv_settings& s) { return s.image_type == HV_IMG_ARGUMENT && s.unwrap_2d; }
// filter2D outside the AS transfer function: its own mask and passes (fourier_transform.cc:55-58)
bool uses_f2d_mask(const hv_settings& s) { return s.filter2d_enabled && s.space_transformation != HV_SPACE_ANGULARSP; }
bool uses_spatial(const hv_settings& s) { return s.space_transformation != HV_SPACE_NONE || s.filter2d_enabled; }
// the filter2D view exists only with the filter (Pipe::insert_filter2d_view, pipe.cc:526-529)
bool uses_f2d_view(const hv_settings& s) { return s.filter2d_enabled && s.filter2d_view_enabled; }

struct Sizes
{
    size_t total = 0;
    void add(size_t b) { total += (b + 255) / 256 * 256; }
};

// Fast mode (batch == stride == window, plain pipes): how many lanes have their own render stream
// (eigensolve workloads without state carried from window to window), and how many rings are in
// flight.
int fast_renders(const hv_settings& s, bool served)
{
    if (served || s.batch_size != s.time_stride || s.batch_size != s.time_transformation_size)
        return 1;
    const bool own = uses_eig(s) && s.accumulation <= 1 && !s.cuts_enabled && !uses_f2d_view(s) &&
                     !uses_phase_increase(s) && !uses_unwrap(s);
    return own ? hv_pipe::kMaxLanes : 1;
}

int fast_lanes(const hv_settings& s, bool served)
{
    if (served || s.batch_size != s.time_stride || s.batch_size != s.time_transformation_size)
        return 0;
    return fast_renders(s, served) > 1 ? hv_pipe::kMaxLanes : 2;
}

// SMs the persistent spatial passes leave to the render lanes' kernels
constexpr int kLaneReserveSms = 8;

// The split-BF16 planes beside the ring (tiled covariance, T > 64): plain pipes whose ring slots the
// host tracks (not served, not the fast lanes)
// the ring holds the converted frames (imaginary parts 0): real planes
int planes_real(const hv_settings& s)
{
    return s.space_transformation == HV_SPACE_NONE && !s.filter2d_enabled ? 1 : 0;
}

bool uses_planes(const hv_frame_desc& fd, const hv_settings& s, bool served);

// PCA on the converted integer frames (no spatial transform) with sliding windows: the windows are
// pipelined over three streams (process_batch, render_view). The ring is rebuilt from the real
// split planes (exact for integer pixels), so only the conversion into the planes reads the input
// batch; a window's eigensolve then overlaps the next batch's conversion and covariance update and
// the previous window's view.
bool uses_pca_pipeline(const hv_frame_desc& fd, const hv_settings& s, bool served)
{
    const int T = s.time_transformation_size, B = s.batch_size;
    return uses_pca(s) && uses_planes(fd, s, served) && planes_real(s) && fd.depth <= 2 && !s.cuts_enabled &&
           !uses_phase_increase(s) && T >= 2 * B;
}

bool uses_planes(const hv_frame_desc& fd, const hv_settings& s, bool served)
{
    const size_t HW = static_cast<size_t>(fd.width) * fd.height;
    return uses_eig(s) && !served && fast_lanes(s, served) == 0 && cov_planes_supported(s.time_transformation_size, HW);
}

size_t footprint(const hv_frame_desc& fd, const hv_settings& s, bool served = false)
{
    const size_t HW = static_cast<size_t>(fd.width) * fd.height;
    const int B = s.batch_size, T = s.time_transformation_size;
    const int K = (s.p_width != 0 ? std::min(s.p_start + s.p_width, T) : s.p_start) - s.p_start + 1;
    Sizes z;
    z.add(HW * 8);                                                      // lens
    z.add(uses_spatial(s) ? HW * 8 * B : 16);  // spatial
    if (uses_f2d_mask(s))
        z.add(HW * 8);
    if (uses_f2d_mask(s) && s.space_transformation == HV_SPACE_FRESNELTR)
        z.add(HW * 8 * B);  // second spatial buffer
    z.add(HW * 8 * T);                                                  // ring
    const int lanes = fast_lanes(s, served), renders = fast_renders(s, served);
    for (int l = 1; l < lanes; ++l)
        z.add(HW * 8 * T);  // further rings of the fast mode
    for (int l = 1; l < renders; ++l)
    {
        // per-window buffers of a lane with its own render stream
        z.add(static_cast<size_t>(K > 0 ? K : 1) * T * 8);
        z.add(static_cast<size_t>(T) * T * 16 * 2 + T * 8);
        z.add(pca_cov_workspace(T, HW));
        z.add(pca_eigh_workspace(T));
        z.add(HW * 4 * 2);
        if (use_view_tc(s, K, HW))
            z.add(view_tc_workspace(K, T));
        z.add(static_cast<size_t>(time_view_partials(fd.width, fd.height)) * 8);
        z.add(reduce_workspace(HW));
        z.add(64);
    }
    z.add(static_cast<size_t>(K > 0 ? K : 1) * T * 8);                 // weights
    if (uses_eig(s))
    {
        z.add(static_cast<size_t>(T) * T * 16 * 2 + T * 8);
        z.add(uses_planes(fd, s, served) ? pca_cov_workspace_planes(T, HW) : pca_cov_workspace(T, HW));
        z.add(pca_eigh_workspace(T));
    }
    if (uses_planes(fd, s, served))
        z.add(cov_planes_bytes(T, HW, planes_real(s)));
    if (uses_pca_pipeline(fd, s, served))  // the second covariance and weights buffers
        z.add(static_cast<size_t>(T) * T * 16 + static_cast<size_t>(K > 0 ? K : 1) * T * 8);
    z.add(HW * 4 * 2);  // view + post
    if (is_moment(s.image_type))
        z.add(static_cast<size_t>(K > 0 ? K : 1) * sizeof(float));
    if (use_view_tc(s, K, HW))
        z.add(view_tc_workspace(K, T));
    if (uses_unwrap(s) || uses_phase_increase(s))
        z.add(HW * 4);
    if (uses_unwrap(s) || (uses_phase_increase(s) && s.unwrap_2d))
        z.add(unwrap_workspace(fd.width, fd.height));
    if (uses_phase_increase(s))
    {
        z.add(HW * 8);
        z.add(HW * 4);
        z.add(phase_increase_minmax_count(HW) * 8);
    }
    if (s.cuts_enabled)
    {
        const size_t ct = static_cast<size_t>(T) * (fd.width + fd.height);  // XZ + YZ pixels
        z.add(static_cast<size_t>(T) * T * 8);
        z.add(cuts_workspace(fd.width, fd.height, T, s.x_width + 1, s.y_width + 1));
        z.add(ct * 4);
        z.add(static_cast<size_t>(T) * fd.width * 4 * (s.xz_accumulation > 1 ? s.xz_accumulation : 0));
        z.add(static_cast<size_t>(T) * fd.height * 4 * (s.yz_accumulation > 1 ? s.yz_accumulation : 0));
        z.add(64);
        z.add(64);
        z.add(ct * 2 * static_cast<size_t>(std::max(1, s.cuts_buffer_size)));
        z.add(percentile_workspace(std::max(HW, static_cast<size_t>(T) * std::max(fd.width, fd.height))));
    }
    if (uses_f2d_view(s))
    {
        z.add(HW * 8 * 2);
        z.add(HW * 4);
        z.add(64);
        z.add(HW * 2 * static_cast<size_t>(std::max(1, s.output_buffer_size)));
    }
    z.add(static_cast<size_t>(time_view_partials(fd.width, fd.height)) * 8);
    z.add(reduce_workspace(HW));
    z.add(64);
    if (s.accumulation > 1)
        z.add(HW * 4 * s.accumulation);
    z.add(64);
    z.add(percentile_workspace(HW));
    const int in_slots = std::max(2, s.input_buffer_size / std::max(1, B));
    z.add(HW * fd.depth * B * static_cast<size_t>(in_slots));
    z.add(HW * 2 * static_cast<size_t>(std::max(1, s.output_buffer_size)));
    return z.total;
}

hv_status build(hv_pipe* p)
{
    free_buffers(p);
    const hv_settings& s = p->s;
    p->W = p->fd.width;
    p->H = p->fd.height;
    p->HW = static_cast<size_t>(p->W) * p->H;
    p->depth = static_cast<int>(p->fd.depth);
    p->kind = raw_kind(p->depth, p->fd.byte_endian != 0);
    p->B = s.batch_size;
    p->T = s.time_transformation_size;
    p->S = s.time_stride;
    // Converts::insert_compute_p_accu (converts.cc:76-92)
    p->pmin = s.p_start;
    p->pmax = s.p_width != 0 ? std::max(0, std::min(p->pmin + s.p_width, p->T)) : p->pmin;
    if (p->pmax > p->T - 1)
        p->pmax = p->T - 1;  // the reference reads past the buffer there; validation keeps p + width < T
    p->K = p->pmax - p->pmin + 1;
    // SSA_STFT eigenvector range (fourier_transform.cc:409-412): width 0 keeps every column
    p->qmin = s.q_width != 0 ? s.q_start : 0;
    p->qn = s.q_width != 0 ? s.q_width : p->T;
    p->A = s.accumulation > 1 ? s.accumulation : 0;
    const size_t HW = p->HW;
    hv_status st;
#define HV_ALLOC(ptr, bytes)                                                                                           \
    if ((st = dalloc(p, ptr, bytes)) != HV_OK)                                                                         \
        return st;
    HV_ALLOC(p->lens, HW * sizeof(float2));
    HV_ALLOC(p->spatial, (uses_spatial(s) ? HW * p->B : 1) * sizeof(float2));
    p->f2d_mask = nullptr;
    p->work2 = nullptr;
    if (uses_f2d_mask(s))
    {
        HV_ALLOC(p->f2d_mask, HW * sizeof(float2));
        if (s.space_transformation == HV_SPACE_FRESNELTR)
        {
            HV_ALLOC(p->work2, HW * p->B * sizeof(float2));
        }
    }
    p->nlanes = fast_lanes(s, p->served);
    p->nrender = fast_renders(s, p->served);
    p->fast = p->nlanes > 0;
    HV_ALLOC(p->ring, HW * p->T * sizeof(float2));
    p->lanes[0].ring = p->ring;
    for (int l = 1; l < p->nlanes; ++l)
    {
        HV_ALLOC(p->lanes[l].ring, HW * p->T * sizeof(float2));
    }
    HV_ALLOC(p->weights, static_cast<size_t>(p->K) * p->T * sizeof(float2));
    if (uses_eig(s))
    {
        HV_ALLOC(p->cov, static_cast<size_t>(p->T) * p->T * sizeof(double2));
        HV_ALLOC(p->evecs, static_cast<size_t>(p->T) * p->T * sizeof(double2));
        HV_ALLOC(p->evals, static_cast<size_t>(p->T) * sizeof(double));
        HV_ALLOC(p->cov_work, uses_planes(p->fd, s, p->served) ? pca_cov_workspace_planes(p->T, HW)
                                                                : pca_cov_workspace(p->T, HW));
        HV_ALLOC(p->eig_work, pca_eigh_workspace(p->T));
        // no warm start is read before an eigensolve wrote one; zeros if it ever is
        HV_CUDA_TRY(cudaMemsetAsync(p->eig_work, 0, pca_eigh_workspace(p->T), p->stream));
        p->eig_warm = false;
        p->cov_valid = false;
        p->cov_dirty = ~0u;
    }
    p->planes = nullptr;
    p->planes_ok = false;
    if (uses_planes(p->fd, s, p->served))
    {
        // zero like the ring
        p->planes_real = planes_real(s);
        HV_ALLOC(p->planes, cov_planes_bytes(p->T, HW, p->planes_real));
        HV_CUDA_TRY(cudaMemsetAsync(p->planes, 0, cov_planes_bytes(p->T, HW, p->planes_real), p->stream));
        p->planes_ok = true;
    }
    HV_ALLOC(p->view, HW * sizeof(float));
    p->bin_w = nullptr;
    if (is_moment(s.image_type))
    {
        HV_ALLOC(p->bin_w, static_cast<size_t>(p->K) * sizeof(float));
    }
    p->view_on_tc = use_view_tc(s, p->K, p->HW);
    if (p->view_on_tc)
    {
        HV_ALLOC(p->view_tc_work, view_tc_workspace(p->K, p->T));
    }
    HV_ALLOC(p->post, HW * sizeof(float));
    if (uses_unwrap(s) || uses_phase_increase(s))
    {
        HV_ALLOC(p->unwrapped, HW * sizeof(float));
    }
    if (uses_unwrap(s) || (uses_phase_increase(s) && s.unwrap_2d))
    {
        HV_ALLOC(p->unwrap_work, unwrap_workspace(p->W, p->H));
    }
    p->pi_count = 0;
    if (uses_phase_increase(s))
    {
        HV_ALLOC(p->pi_pred, HW * sizeof(float2));
        HV_ALLOC(p->pi_hist, HW * sizeof(float));
        HV_ALLOC(p->pi_minmax, phase_increase_minmax_count(HW) * sizeof(float2));
    }
    p->npartials = time_view_partials(p->W, p->H);
    HV_ALLOC(p->partials, static_cast<size_t>(p->npartials) * sizeof(double));
    HV_ALLOC(p->reduce_work, reduce_workspace(HW));
    HV_ALLOC(p->factors, 4 * sizeof(float));
    if (p->A > 0)
    {
        HV_ALLOC(p->acc_ring, HW * p->A * sizeof(float));
    }
    HV_ALLOC(p->range, 4 * sizeof(float));
    // lane 0 uses the buffers above; lanes with their own render stream get their own copies
    {
        hv_pipe::Lane& L0 = p->lanes[0];
        L0.weights = p->weights;
        L0.cov = p->cov;
        L0.evals = p->evals;
        L0.evecs = p->evecs;
        L0.cov_work = p->cov_work;
        L0.eig_work = p->eig_work;
        L0.eig_warm = false;
        L0.view = p->view;
        L0.post = p->post;
        L0.partials = p->partials;
        L0.reduce_work = p->reduce_work;
        L0.factors = p->factors;
        L0.view_tc_work = p->view_tc_work;
        for (int l = 1; l < p->nrender; ++l)
        {
            hv_pipe::Lane& L = p->lanes[l];
            HV_ALLOC(L.weights, static_cast<size_t>(p->K) * p->T * sizeof(float2));
            HV_ALLOC(L.cov, static_cast<size_t>(p->T) * p->T * sizeof(double2));
            HV_ALLOC(L.evecs, static_cast<size_t>(p->T) * p->T * sizeof(double2));
            HV_ALLOC(L.evals, static_cast<size_t>(p->T) * sizeof(double));
            HV_ALLOC(L.cov_work, pca_cov_workspace(p->T, HW));
            HV_ALLOC(L.eig_work, pca_eigh_workspace(p->T));
            HV_CUDA_TRY(cudaMemsetAsync(L.eig_work, 0, pca_eigh_workspace(p->T), p->stream));
            HV_ALLOC(L.view, HW * sizeof(float));
            HV_ALLOC(L.post, HW * sizeof(float));
            HV_ALLOC(L.partials, static_cast<size_t>(p->npartials) * sizeof(double));
            HV_ALLOC(L.reduce_work, reduce_workspace(HW));
            HV_ALLOC(L.factors, 4 * sizeof(float));
            if (p->view_on_tc)
            {
                HV_ALLOC(L.view_tc_work, view_tc_workspace(p->K, p->T));
            }
        }
    }
    p->cuts = s.cuts_enabled != 0;
    size_t pct_n = HW;
    if (p->cuts)
    {
        HV_ALLOC(p->w_all, static_cast<size_t>(p->T) * p->T * sizeof(float2));
        HV_ALLOC(p->cut_work, cuts_workspace(p->W, p->H, p->T, s.x_width + 1, s.y_width + 1));
        const int accs[2] = {s.xz_accumulation, s.yz_accumulation};
        for (int v = 0; v < 2; ++v)
        {
            hv_pipe::SecondaryView& c = p->views[v];
            c.w = v == 0 ? p->W : p->T;
            c.h = v == 0 ? p->T : p->H;
            const size_t px = static_cast<size_t>(c.w) * c.h;
            pct_n = std::max(pct_n, px);
            HV_ALLOC(c.post, px * sizeof(float));
            HV_CUDA_TRY(cudaMemsetAsync(c.post, 0, px * sizeof(float), p->stream));
            c.A = accs[v] > 1 ? accs[v] : 0;
            c.acc_ring = nullptr;
            if (c.A > 0)
            {
                HV_ALLOC(c.acc_ring, px * c.A * sizeof(float));
            }
            HV_ALLOC(c.range, 4 * sizeof(float));
            c.out_cap = std::max(1, s.cuts_buffer_size);
            HV_ALLOC(c.out_ring, px * sizeof(uint16_t) * c.out_cap);
        }
    }
    p->f2d_view = uses_f2d_view(s);
    if (p->f2d_view)
    {
        hv_pipe::SecondaryView& c = p->views[HV_VIEW_FILTER2D];
        c.w = p->W;
        c.h = p->H;
        HV_ALLOC(p->f2d_spec[0], HW * sizeof(float2));
        HV_ALLOC(p->f2d_spec[1], HW * sizeof(float2));
        HV_ALLOC(c.post, HW * sizeof(float));
        HV_CUDA_TRY(cudaMemsetAsync(c.post, 0, HW * sizeof(float), p->stream));
        c.A = 0;
        c.acc_ring = nullptr;
        HV_ALLOC(c.range, 4 * sizeof(float));
        c.out_cap = std::max(1, s.output_buffer_size);  // gpu_filter2d_view_queue (pipe.cc:222)
        HV_ALLOC(c.out_ring, HW * sizeof(uint16_t) * c.out_cap);
    }
    HV_ALLOC(p->pct_work, percentile_workspace(pct_n));
    p->in_slots = std::max(2, s.input_buffer_size / std::max(1, p->B));
    p->batch_bytes = HW * p->depth * p->B;
    HV_ALLOC(p->in_ring, p->batch_bytes * p->in_slots);
    p->out_cap = std::max(1, s.output_buffer_size);
    HV_ALLOC(p->out_ring, HW * sizeof(uint16_t) * p->out_cap);
#undef HV_ALLOC
    auto mk_events = [&](std::vector<cudaEvent_t>& v, int n) -> hv_status {
        v.resize(n);
        for (int i = 0; i < n; ++i)
            HV_CUDA_TRY(cudaEventCreateWithFlags(&v[i], cudaEventDisableTiming));
        return HV_OK;
    };
    if ((st = mk_events(p->in_filled, p->in_slots)) != HV_OK || (st = mk_events(p->in_consumed, p->in_slots)) != HV_OK ||
        (st = mk_events(p->out_ready, p->out_cap)) != HV_OK || (st = mk_events(p->out_freed, p->out_cap)) != HV_OK)
        return st;
    for (int v = 0; v < 3; ++v)
    {
        if ((v < 2 && !p->cuts) || (v == HV_VIEW_FILTER2D && !p->f2d_view))
            continue;
        if ((st = mk_events(p->views[v].out_ready, p->views[v].out_cap)) != HV_OK ||
            (st = mk_events(p->views[v].out_freed, p->views[v].out_cap)) != HV_OK)
            return st;
    }

    // ring starts zeroed like Queue::resize (queue.cc:131-134)
    HV_CUDA_TRY(cudaMemsetAsync(p->ring, 0, HW * p->T * sizeof(float2), p->stream));
    for (int l = 0; l < p->nlanes; ++l)
    {
        hv_pipe::Lane& L = p->lanes[l];
        if (l > 0)
            HV_CUDA_TRY(cudaMemsetAsync(L.ring, 0, HW * p->T * sizeof(float2), p->stream));
        HV_CUDA_TRY(cudaEventCreateWithFlags(&L.ready, cudaEventDisableTiming));
        HV_CUDA_TRY(cudaEventCreateWithFlags(&L.free, cudaEventDisableTiming));
        L.st = (p->nrender > 1 && l > 0) ? p->render_extra[l - 1] : p->render_stream_owned;
        if (l >= p->nrender)
        {
            // lanes sharing lane 0's render stream share its buffers
            const float2* ring = L.ring;
            const cudaEvent_t ready = L.ready, fr = L.free;
            L = p->lanes[0];
            L.ring = const_cast<float2*>(ring);
            L.ready = ready;
            L.free = fr;
        }
    }
    HV_CUDA_TRY(cudaEventCreateWithFlags(&p->join_ev, cudaEventDisableTiming));
    HV_CUDA_TRY(cudaEventCreateWithFlags(&p->range_ev, cudaEventDisableTiming));
    p->range_ev_set = false;
    p->render_stream = p->fast ? p->render_stream_owned : p->stream;
    p->windows = 0;
    // PCA windows over three streams (the tensor-core view's prepared weights are not double-buffered)
    p->pp = uses_pca_pipeline(p->fd, s, p->served) && p->planes_ok && !p->view_on_tc && !p->fast;
    p->pp_w = p->pp_b = 0;
    if (p->pp)
    {
        p->render_stream = p->render_stream_owned;
        p->pp_cov[0] = p->cov;
        if ((st = dalloc(p, p->pp_cov[1], static_cast<size_t>(p->T) * p->T * sizeof(double2))) != HV_OK)
            return st;
        p->pp_weights[0] = p->weights;
        if ((st = dalloc(p, p->pp_weights[1], static_cast<size_t>(p->K) * p->T * sizeof(float2))) != HV_OK)
            return st;
        for (cudaEvent_t* e : {&p->pp_cov_ev[0], &p->pp_cov_ev[1], &p->pp_eig_ev[0], &p->pp_eig_ev[1],
                               &p->pp_view_ev[0], &p->pp_view_ev[1], &p->pp_main_ev, &p->pp_ring_ev[0],
                               &p->pp_ring_ev[1], &p->pp_ring_ev[2], &p->pp_ring_ev[3]})
            HV_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    // lens (computed once per refresh, fourier_transform.cc:93-137)
    if (s.space_transformation == HV_SPACE_FRESNELTR)
        st = make_fresnel_lens(p->lens, p->W, p->H, s.lambda, s.z_distance, s.pixel_size, s.lens_mode, p->stream);
    else if (s.space_transformation == HV_SPACE_ANGULARSP)
        st = make_spectral_lens(p->lens, p->W, p->H, s.lambda, s.z_distance, s.pixel_size, s.lens_mode, p->stream);
    if (st != HV_OK)
        return st;
    // filter2D mask (fourier_transform.cc:36-58): multiplied into G for AS, else used by its passes
    if (s.filter2d_enabled)
    {
        if (s.space_transformation == HV_SPACE_ANGULARSP)
            st = filter2d_mask(p->lens, p->W, p->H, s.filter2d_n1, s.filter2d_n2, s.filter2d_smooth_low,
                               s.filter2d_smooth_high, 1, p->stream);
        else
            st = filter2d_mask(p->f2d_mask, p->W, p->H, s.filter2d_n1, s.filter2d_n2, s.filter2d_smooth_low,
                               s.filter2d_smooth_high, 0, p->stream);
        if (st != HV_OK)
            return st;
    }
    if (s.time_transformation == HV_TIME_STFT)
        st = stft_weights(p->weights, p->T, p->pmin, p->pmax, p->stream);
    else if (s.time_transformation == HV_TIME_NONE)
        st = delta_weights(p->weights, p->T, p->pmin, p->pmax, p->stream);
    if (st != HV_OK)
        return st;
    if (p->view_on_tc && !uses_eig(s) && (st = view_tc_prepare(p->weights, p->K, p->T, p->view_tc_work, p->stream)) != HV_OK)
        return st;
    if (p->bin_w && (st = moment_bin_weights(p->bin_w, p->T, p->pmin, p->pmax, s.image_type - HV_IMG_MOMENTS_0,
                                             static_cast<float>(s.camera_fps), p->stream)) != HV_OK)
        return st;
    float r0[4] = {s.contrast_min, s.contrast_max, 0.f, 0.f};
    HV_CUDA_TRY(cudaMemcpyAsync(p->range, r0, sizeof(r0), cudaMemcpyHostToDevice, p->stream));
    if (p->cuts)
    {
        // p_acc rows for the cuts: every STFT bin, or the ring itself without a time transform;
        // PCA / SSA_STFT rows are rebuilt from each window's eigenvectors
        if (s.time_transformation == HV_TIME_STFT)
            st = stft_weights(p->w_all, p->T, 0, p->T - 1, p->stream);
        else if (s.time_transformation == HV_TIME_NONE)
            st = delta_weights(p->w_all, p->T, 0, p->T - 1, p->stream);
        if (st != HV_OK)
            return st;
        const float rxz[4] = {s.xz_contrast_min, s.xz_contrast_max, 0.f, 0.f};
        const float ryz[4] = {s.yz_contrast_min, s.yz_contrast_max, 0.f, 0.f};
        HV_CUDA_TRY(cudaMemcpyAsync(p->views[0].range, rxz, sizeof(rxz), cudaMemcpyHostToDevice, p->stream));
        HV_CUDA_TRY(cudaMemcpyAsync(p->views[1].range, ryz, sizeof(ryz), cudaMemcpyHostToDevice, p->stream));
        // Rendering::request_autocontrast (rendering.cc:87-99)
        p->views[0].autocontrast_pending = s.xz_contrast_enabled && s.xz_contrast_auto_refresh;
        p->views[1].autocontrast_pending = s.yz_contrast_enabled && s.yz_contrast_auto_refresh;
        for (int v = 0; v < 2; ++v)
        {
            p->views[v].acc_start = p->views[v].acc_size = 0;
            p->views[v].out_head = p->views[v].out_count = 0;
            p->views[v].valid = false;
        }
    }
    if (p->f2d_view)
    {
        hv_pipe::SecondaryView& c = p->views[HV_VIEW_FILTER2D];
        const float rf[4] = {s.filter2d_contrast_min, s.filter2d_contrast_max, 0.f, 0.f};
        HV_CUDA_TRY(cudaMemcpyAsync(c.range, rf, sizeof(rf), cudaMemcpyHostToDevice, p->stream));
        // Rendering::request_autocontrast (rendering.cc:87-99): once per refresh
        c.autocontrast_pending = s.filter2d_contrast_enabled && s.filter2d_contrast_auto_refresh;
        c.out_head = c.out_count = 0;
        c.valid = false;
        p->f2d_buf = 0;
    }
    HV_CUDA_TRY(cudaStreamSynchronize(p->stream));

    p->ring_start = p->ring_size = 0;
    p->batch_index = 0;
    p->acc_start = p->acc_size = 0;
    p->autocontrast_pending = s.contrast_enabled && s.contrast_auto_refresh;
    p->in_slot = 0;
    p->in_fill = 0;
    {
        std::lock_guard<std::mutex> g(p->mu);
        p->ready.clear();
        p->in_free = p->in_slots;
    }
    p->out_head = p->out_count = 0;
    p->last_frame_valid = false;
    return HV_OK;
}

// Time transform and view of one full ring, up to the renormalisation factors
// (fourier_transform.cc:194-242,340-460, converts.cc:19-62,251-300, postprocessing.cc:135-155):
// sets *frame to the float frame that the fused renorm / shift / accumulation pass reads and
// *shift_after when that pass applies the fftshift (the view kernels apply it themselves
// otherwise). `ctl` gates the kernels of a served cycle (null for the plain pipe).
hv_status render_view(hv_pipe* p, cudaStream_t st, const CycleCtl* ctl, const float** frame, int* shift_after);

// The covariance and eigensolve of a PCA window of the three-stream pipeline (p->pp): the update
// of covariance buffer w % 2 on the pipe stream (from the other buffer, the previous window's),
// the eigensolve into weights buffer w % 2 on the eigensolve stream, then the view on the render
// stream `st` (render_view's view part, with p->weights bound to the window's buffer).
hv_status render_view_pp(hv_pipe* p, cudaStream_t st, uint32_t dirty, uint32_t all, const float** frame,
                         int* shift_after)
{
    const int w = p->pp_w++, i = w & 1;
    double2* cov = p->pp_cov[i];
    cudaStream_t es = p->eig_stream;
    hv_status r;
    if (w >= 2)  // window w - 2's eigensolve read this buffer
        HV_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->pp_eig_ev[i], 0));
    const bool inc = w >= 1 && p->cov_valid && p->cov_mode == cov_mode() && dirty != all && cov_incremental();
    if (inc)
        HV_CUDA_TRY(cudaMemcpyAsync(cov, p->pp_cov[i ^ 1], static_cast<size_t>(p->T) * p->T * sizeof(double2),
                                    cudaMemcpyDeviceToDevice, p->stream));
    if (!inc || dirty)
    {
        uint32_t blocks = inc ? dirty : ~0u;
        if (inc)
        {
            uint32_t b2 = 0;  // real planes: 128-frame blocks
            for (int b = 0; b < 16; ++b)
                if ((dirty >> (2 * b)) & 3u)
                    b2 |= 1u << b;
            blocks = b2;
        }
        r = pca_covariance_planes(p->planes, p->T, p->HW, cov, p->cov_work, blocks, 1, p->stream);
        if (r == HV_ERR_UNSUPPORTED)  // the SIMT engine mode: from the ring, which the render stream writes
        {
            HV_CUDA_TRY(cudaEventRecord(p->pp_main_ev, st));
            HV_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->pp_main_ev, 0));
            r = pca_covariance(p->ring, p->T, p->HW, cov, p->cov_work, p->stream);
        }
        if (r != HV_OK)
            return r;
    }
    p->cov_dirty = 0;
    p->cov_mode = cov_mode();
    HV_CUDA_TRY(cudaEventRecord(p->pp_cov_ev[i], p->stream));
    HV_CUDA_TRY(cudaStreamWaitEvent(es, p->pp_cov_ev[i], 0));
    if (w >= 2)  // window w - 2's view read this weights buffer
        HV_CUDA_TRY(cudaStreamWaitEvent(es, p->pp_view_ev[i], 0));
    bool kept = false;
    if ((r = pca_eigh(cov, p->T, p->evals, p->evecs, p->pmin, p->pmax, p->pp_weights[i], p->eig_work, es, p->pmin,
                      p->pmax, p->eig_warm, true, &kept)) != HV_OK)
        return r;
    p->eig_warm = true;
    p->cov_valid = kept;
    HV_CUDA_TRY(cudaEventRecord(p->pp_eig_ev[i], es));
    HV_CUDA_TRY(cudaStreamWaitEvent(st, p->pp_eig_ev[i], 0));
    p->weights = p->pp_weights[i];
    p->pp_nested = true;
    r = render_view(p, st, nullptr, frame, shift_after);
    p->pp_nested = false;
    if (r != HV_OK)
        return r;
    HV_CUDA_TRY(cudaEventRecord(p->pp_view_ev[i], st));
    return HV_OK;
}

// The FP32 SIMT time view of the ring into p->view. The pipelined PCA windows (p->pp: a real
// ring) read the real split planes instead, half the bytes; the slots that the next batch's
// planes overwrite while this view may still run (the next batch waits only for the views
// enqueued before the previous batch) are read from the ring, which holds every slot.
hv_status ring_view(hv_pipe* p, cudaStream_t st, float scale, int shift, double* partials, const CycleCtl* ctl,
                    bool bins = true)
{
    const hv_settings& s = p->s;
    const float* bin_w = bins ? p->bin_w : nullptr;
    if (p->pp)
        return time_view_planes(p->planes, p->ring, (p->ring_start + p->ring_size) % p->T, std::min(p->B, p->T),
                                p->T, p->W, p->H, p->weights, p->K, s.image_type, scale, shift, p->view, partials, st,
                                ctl, bin_w);
    return time_view(p->ring, p->T, p->W, p->H, p->weights, p->K, s.image_type, scale, shift, p->view, partials, st,
                     ctl, bin_w);
}

hv_status render_view(hv_pipe* p, cudaStream_t st, const CycleCtl* ctl, const float** frame, int* shift_after)
{
    const hv_settings& s = p->s;
    hv_status r;
    const bool pca = uses_pca(s);
    const bool unwrap = uses_unwrap(s);
    const bool pinc = uses_phase_increase(s);
    if (uses_eig(s) && !p->pp_nested)
    {
        // not gated by the block: served PCA / SSA_STFT cycles are launched eagerly (render cycles only).
        // A sliding window (stride < T) rewrites S of the T ring slots between renders: only the
        // covariance rows and columns of those slots change, and those are recomputed (the other
        // entries are the previous window's, computed from the same samples: bit-identical to a
        // full recomputation).
        const int nblk = (p->T + 63) / 64;
        const uint32_t all = nblk >= 32 ? ~0u : ((1u << nblk) - 1u);
        const uint32_t dirty = p->cov_dirty & all;
        if (p->pp && !ctl)
            return render_view_pp(p, st, dirty, all, frame, shift_after);
        bool done = false;
        const bool inc = !ctl && p->nrender <= 1 && p->cov_valid && p->cov_mode == cov_mode() && dirty != all &&
                         cov_incremental();
        if (!ctl && p->planes_ok)
        {
            // real planes: 128-frame blocks (pairs of the 64-frame blocks)
            uint32_t blocks = inc ? dirty : ~0u;
            if (p->planes_real && inc)
            {
                uint32_t b2 = 0;
                for (int b = 0; b < 16; ++b)
                    if ((dirty >> (2 * b)) & 3u)
                        b2 |= 1u << b;
                blocks = b2;
            }
            r = inc && !dirty ? HV_OK
                              : pca_covariance_planes(p->planes, p->T, p->HW, p->cov, p->cov_work, blocks,
                                                      p->planes_real, st);
            if (r == HV_OK)
                done = true;
            else if (r != HV_ERR_UNSUPPORTED)
                return r;
        }
        if (!done && (r = pca_covariance(p->ring, p->T, p->HW, p->cov, p->cov_work, st)) != HV_OK)
            return r;
        p->cov_dirty = 0;
        p->cov_mode = cov_mode();
        // refined in FP64: the viewed components (PCA) or the kept range of SSA_STFT (all columns
        // kept: the projector is the identity, nothing to refine)
        const int rlo = pca ? p->pmin : p->qmin;
        const int rhi = pca ? p->pmax : (p->qn < p->T ? p->qmin + p->qn - 1 : -1);
        // the sweeps start from the previous window's eigenvectors once there is one
        // PCA views read only the refined weights (the cuts read every eigenvector)
        bool kept = false;
        if ((r = pca_eigh(p->cov, p->T, p->evals, p->evecs, p->pmin, p->pmax, pca ? p->weights : nullptr,
                          p->eig_work, st, rlo, rhi, p->eig_warm, pca && !p->cuts, &kept)) != HV_OK)
            return r;
        p->eig_warm = true;
        p->cov_valid = kept && !ctl;
        if (!pca && (r = ssa_weights(p->evecs, p->T, p->qmin, p->qn, p->pmin, p->K, p->weights, st)) != HV_OK)
            return r;
        if (p->view_on_tc && (r = view_tc_prepare(p->weights, p->K, p->T, p->view_tc_work, st)) != HV_OK)
            return r;
    }
    // PCA views are scaled by (2 << 16) - 1 (converts.cc:50-62); a moment replaces the frame after
    // that scaling (pipe.cc:346, fourier_transform.cc:317-338) and is not scaled
    const float scale = (pca && !p->bin_w) ? static_cast<float>((2 << 16) - 1) : 1.0f;
    const bool renorm = s.renorm != 0;
    *frame = p->view;
    *shift_after = 0;
    if (pinc)
    {
        // phase increase of the p plane (weights row 0), not gated by the block: its history makes
        // every served cycle an eager one
        const bool first = p->pi_count == 0;
        if ((r = phase_increase(p->ring, p->T, p->HW, p->weights, p->pi_pred, p->pi_hist, first ? 1 : 0,
                                first ? 0 : 1, p->view, p->pi_minmax, st)) != HV_OK)
            return r;
        ++p->pi_count;
        if (s.unwrap_2d && first)
        {
            // the first window's increments are all 0: its unwrapped frame is the zero frame (the
            // reference unwraps and rescales rounding residues there)
            HV_CUDA_TRY(cudaMemsetAsync(p->unwrapped, 0, p->HW * sizeof(float), st));
        }
        else if (s.unwrap_2d)
        {
            if ((r = unwrap_2d(p->view, p->unwrapped, p->W, p->H, p->unwrap_work, st)) != HV_OK)
                return r;
            if (pca && (r = renorm_shift_accumulate(p->unwrapped, p->unwrapped, p->W, p->H, nullptr, 0, nullptr, 0, 0,
                                                    0, 0, 0, st, scale, ctl)) != HV_OK)
                return r;
        }
        else if ((r = rescale_float(p->view, p->HW, p->pi_minmax, scale, p->unwrapped, st)) != HV_OK)
            return r;
        *frame = p->unwrapped;
        *shift_after = s.fft_shift ? 1 : 0;
        if (renorm && (r = renorm_factors(*frame, p->HW, s.renorm_constant, nullptr, 0, p->factors, p->reduce_work, st,
                                          ctl)) != HV_OK)
            return r;
        return HV_OK;
    }
    if (!unwrap)
    {
        const int shift_in_view = s.fft_shift ? 1 : 0;
        if ((r = p->view_on_tc ? view_tc(p->ring, p->T, p->W, p->H, p->K, s.image_type, scale, shift_in_view, p->view,
                                         renorm ? p->partials : nullptr, p->view_tc_work, st, ctl, p->bin_w)
                               : ring_view(p, st, scale, shift_in_view, renorm ? p->partials : nullptr, ctl)) !=
            HV_OK)
            return r;
        if (renorm && (r = renorm_factors(p->view, p->HW, s.renorm_constant, p->partials, p->npartials, p->factors,
                                          p->reduce_work, st, ctl)) != HV_OK)
            return r;
        return HV_OK;
    }
    // not gated by the block: served unwrap cycles are launched eagerly (render cycles only)
    if ((r = p->view_on_tc ? view_tc(p->ring, p->T, p->W, p->H, p->K, s.image_type, 1.0f, 0, p->view, nullptr,
                                     p->view_tc_work, st, ctl)
                           : ring_view(p, st, 1.0f, 0, nullptr, ctl, false)) != HV_OK)
        return r;
    if ((r = unwrap_2d(p->view, p->unwrapped, p->W, p->H, p->unwrap_work, st)) != HV_OK)
        return r;
    if (pca && (r = renorm_shift_accumulate(p->unwrapped, p->unwrapped, p->W, p->H, nullptr, 0, nullptr, 0, 0, 0, 0, 0,
                                            st, scale, ctl)) != HV_OK)
        return r;
    *frame = p->unwrapped;
    *shift_after = s.fft_shift ? 1 : 0;
    if (renorm && (r = renorm_factors(*frame, p->HW, s.renorm_constant, nullptr, 0, p->factors, p->reduce_work, st,
                                      ctl)) != HV_OK)
        return r;
    return HV_OK;
}

// Queues one output of a secondary view from its float image (the oldest output is overwritten
// when the queue is full, like Queue::enqueue).
template <class Convert>
hv_status queue_view_output(hv_pipe* p, hv_pipe::SecondaryView& c, cudaStream_t st, Convert convert)
{
    const size_t px = static_cast<size_t>(c.w) * c.h;
    int slot_out;
    {
        std::lock_guard<std::mutex> g(p->mu);
        if (c.out_count == c.out_cap)
        {
            c.out_head = (c.out_head + 1) % c.out_cap;
            --c.out_count;
            ++c.out_overwritten;
        }
        slot_out = (c.out_head + c.out_count) % c.out_cap;
    }
    HV_CUDA_TRY(cudaStreamWaitEvent(st, c.out_freed[slot_out], 0));
    hv_status r = convert(c.out_ring + slot_out * px, px);
    if (r != HV_OK)
        return r;
    HV_CUDA_TRY(cudaEventRecord(c.out_ready[slot_out], st));
    {
        std::lock_guard<std::mutex> g(p->mu);
        ++c.out_count;
    }
    c.valid = true;
    return HV_OK;
}

// XZ / YZ cuts of the window just rendered (fourier_transform.cc:462-503, image_accumulation.cc:159-257,
// rendering.cc:75-340, converts.cc:321-350, pipe.cc:504-514): slices at the cursor band, then per
// view accumulation, log10, autocontrast (bins frame_index_offset .. T-1-offset, or the reticle
// disc for XZ), contrast and uint16 into the view's own output queue.
hv_status render_cuts(hv_pipe* p, cudaStream_t st)
{
    const hv_settings& s = p->s;
    hv_status r;
    if (s.time_transformation == HV_TIME_PCA && (r = evecs_to_weights(p->evecs, p->T, p->w_all, st)) != HV_OK)
        return r;
    if (s.time_transformation == HV_TIME_SSA_STFT &&
        (r = ssa_weights(p->evecs, p->T, p->qmin, p->qn, 0, p->T, p->w_all, st)) != HV_OK)
        return r;
    if (s.x_start < p->W && s.y_start < p->H &&
        (r = time_cuts(p->ring, p->T, p->W, p->H, p->w_all, s.x_start, s.x_start + s.x_width, s.y_start,
                       s.y_start + s.y_width, s.image_type, p->views[0].post, p->views[1].post, p->cut_work, st)) != HV_OK)
        return r;
    for (int v = 0; v < 2; ++v)
    {
        hv_pipe::SecondaryView& c = p->views[v];
        const int log_on = v == 0 ? s.xz_log_enabled : s.yz_log_enabled;
        const int contrast_on = v == 0 ? s.xz_contrast_enabled : s.yz_contrast_enabled;
        const int invert = v == 0 ? s.xz_contrast_invert : s.yz_contrast_invert;
        int slot = 0, start = 0, count = 0;
        if (c.A > 0)
        {
            slot = (c.acc_start + c.acc_size) % c.A;
            if (c.acc_size < c.A)
                ++c.acc_size;
            else
                c.acc_start = (c.acc_start + 1) % c.A;
            start = c.acc_start;
            count = c.acc_size;
        }
        if ((c.A > 0 || log_on) &&
            (r = renorm_shift_accumulate(c.post, c.post, c.w, c.h, nullptr, 0, c.A > 0 ? c.acc_ring : nullptr, c.A,
                                         slot, start, count, log_on, st, 1.0f)) != HV_OK)
            return r;
        if (contrast_on && c.autocontrast_pending)
        {
            const bool apply = c.A == 0 || c.acc_size == c.A || c.acc_size == 1;
            if (apply)
            {
                // percentile.cu:139-250: bins offset .. T-1-offset (the whole window when that is empty)
                int off = s.cuts_contrast_offset;
                if (2 * off >= p->T)
                    off = 0;
                if (v == 0 && s.reticle_display)
                    r = percentile(c.post, c.w, c.h, s.contrast_lower, s.contrast_upper, s.reticle_scale, c.range,
                                   p->pct_work, st);
                else if (v == 0)
                    r = percentile(c.post + static_cast<size_t>(off) * c.w, c.w, c.h - 2 * off, s.contrast_lower,
                                   s.contrast_upper, 0.0f, c.range, p->pct_work, st);
                else
                    r = percentile_pitched(c.post + off, c.w - 2 * off, c.h, c.w, s.contrast_lower, s.contrast_upper,
                                           0.0f, c.range, p->pct_work, st);
                if (r != HV_OK)
                    return r;
                if (c.A == 0 || c.acc_size == c.A)
                    c.autocontrast_pending = false;
            }
        }
        if ((r = queue_view_output(p, c, st, [&](uint16_t* dst, size_t n) {
                 return contrast_to_ushort(c.post, c.range, invert, contrast_on, dst, n, st);
             })) != HV_OK)
            return r;
    }
    return HV_OK;
}

// The filter2D view of the window just rendered (pipe.cc:526-546, rendering.cc:75-340,
// converts.cc:355-367): |shift(stored spectrum)|, log10, autocontrast once per refresh over the
// whole frame, contrast, then float_to_ushort_normalized.
hv_status render_f2d_view(hv_pipe* p, cudaStream_t st)
{
    const hv_settings& s = p->s;
    hv_pipe::SecondaryView& c = p->views[HV_VIEW_FILTER2D];
    hv_status r;
    const float2* mult = s.space_transformation == HV_SPACE_ANGULARSP ? p->lens : p->f2d_mask;
    if ((r = filter2d_view_frame(p->f2d_spec[p->f2d_buf], mult, p->W, p->H, c.post, st)) != HV_OK)
        return r;
    if (s.filter2d_log_enabled &&
        (r = renorm_shift_accumulate(c.post, c.post, c.w, c.h, nullptr, 0, nullptr, 0, 0, 0, 0, 1, st, 1.0f)) != HV_OK)
        return r;
    if (s.filter2d_contrast_enabled && c.autocontrast_pending)
    {
        if ((r = percentile(c.post, c.w, c.h, s.contrast_lower, s.contrast_upper, 0.0f, c.range, p->pct_work, st)) !=
            HV_OK)
            return r;
        c.autocontrast_pending = false;
    }
    return queue_view_output(p, c, st, [&](uint16_t* dst, size_t px) {
        return contrast_to_ushort_normalized(c.post, c.range, s.filter2d_contrast_invert, s.filter2d_contrast_enabled,
                                             dst, px, st);
    });
}

// Rendering of one output from a full ring (pipe.cc:334-374).
hv_status render(hv_pipe* p)
{
    const hv_settings& s = p->s;
    cudaStream_t st = p->render_stream;
    hv_status r;
    const bool renorm = s.renorm != 0;
    const float* frame = nullptr;
    int shift_after = 0;
    if ((r = render_view(p, st, nullptr, &frame, &shift_after)) != HV_OK)
        return r;
    // accumulation queue bookkeeping (Queue::enqueue, queue.cc:149-189)
    int slot = 0, start = 0, count = 0;
    if (p->A > 0)
    {
        slot = (p->acc_start + p->acc_size) % p->A;
        if (p->acc_size < p->A)
            ++p->acc_size;
        else
            p->acc_start = (p->acc_start + 1) % p->A;
        start = p->acc_start;
        count = p->acc_size;
    }
    if ((r = renorm_shift_accumulate(frame, p->post, p->W, p->H, renorm ? p->factors : nullptr, shift_after,
                                     p->A > 0 ? p->acc_ring : nullptr, p->A, slot, start, count, s.log_enabled, st,
                                     1.0f)) != HV_OK)
        return r;
    // autocontrast (rendering.cc:239-299): first frame without accumulation, or at accumulation
    // size 1 and when the accumulation queue is full
    if (s.contrast_enabled && p->autocontrast_pending)
    {
        const bool apply = p->A == 0 || p->acc_size == p->A || p->acc_size == 1;
        if (apply)
        {
            if (p->nrender > 1)
            {
                // earlier windows on the other lanes read the range being replaced: wait for them
                for (int l = 0; l < p->nlanes; ++l)
                    if (p->lanes[l].st != st)
                        HV_CUDA_TRY(cudaStreamWaitEvent(st, p->lanes[l].free, 0));
            }
            if ((r = percentile(p->post, p->W, p->H, s.contrast_lower, s.contrast_upper,
                                s.reticle_display ? s.reticle_scale : 0.0f, p->range, p->pct_work, st)) != HV_OK)
                return r;
            if (p->nrender > 1)
            {
                HV_CUDA_TRY(cudaEventRecord(p->range_ev, st));
                p->range_ev_set = true;
            }
            if (p->A == 0 || p->acc_size == p->A)
                p->autocontrast_pending = false;
        }
    }
    // output slot (overwrite the oldest when the queue is full, like Queue::enqueue)
    int slot_out;
    {
        std::lock_guard<std::mutex> g(p->mu);
        if (p->out_count == p->out_cap)
        {
            p->out_head = (p->out_head + 1) % p->out_cap;
            --p->out_count;
            ++p->out_overwritten;
        }
        slot_out = (p->out_head + p->out_count) % p->out_cap;
    }
    HV_CUDA_TRY(cudaStreamWaitEvent(st, p->out_freed[slot_out], 0));
    if ((r = contrast_to_ushort(p->post, p->range, s.contrast_invert, s.contrast_enabled, p->out_ring + slot_out * p->HW,
                                p->HW, st)) != HV_OK)
        return r;
    HV_CUDA_TRY(cudaEventRecord(p->out_ready[slot_out], st));
    {
        std::lock_guard<std::mutex> g(p->mu);
        ++p->out_count;
    }
    p->last_frame_valid = true;
    if (p->cuts && (r = render_cuts(p, st)) != HV_OK)
        return r;
    return p->f2d_view ? render_f2d_view(p, st) : HV_OK;
}

// Masked spectrum of the batch's first frame (filter2D's store_frame: FFT2(x0) then the mask, or
// the masked transfer function for AS; filter2D.cu:36-44, angular_spectrum.cu:50-55): the forward
// FFT of frame 0 into f2d_spec[buf] (the mask is applied by the view kernel). Runs on the pipe's
// stream right after the batch's spatial passes, with the spatial buffer as scratch.
hv_status capture_f2d_spectrum(hv_pipe* p, const uint8_t* raw0, int buf)
{
    hv_status r = fft_rows_pass(raw0, p->kind, p->spatial, p->W, p->H, 1, nullptr, 0, 1.0f, 0, 1, p->stream);
    if (r != HV_OK)
        return r;
    return fft_cols_pass(p->spatial, p->f2d_spec[buf], p->W, p->H, 1, nullptr, 0, 1.0f, 0, 1, p->stream);
}

// One batch of B raw frames at device address `raw` (pipe.cc:295-334).
hv_status process_batch(hv_pipe* p, const uint8_t* raw)
{
    // insert_wait_time_stride (pipe.cc:400-416)
    p->batch_index += p->B;
    if (p->batch_index != p->S)
        return HV_OK;
    p->batch_index = 0;
    if (p->fast)
    {
        // batch == stride == window: every batch refills the whole ring in batch order (with B = T,
        // Queue::enqueue_multiple always lands frame j in slot j), so the lanes' rings alternate.
        // The spatial passes of batch k+1 run on `stream` while window k (and, with a render stream
        // per lane, windows k-1 and k-2) are transformed and rendered; ring k % nlanes is reused
        // only after window k - nlanes finished with it.
        const int r = static_cast<int>(p->windows % static_cast<uint64_t>(p->nlanes));
        hv_pipe::Lane& L = p->lanes[r];
        HV_CUDA_TRY(cudaStreamWaitEvent(p->stream, L.free, 0));
        // with render lanes of their own, the persistent spatial passes leave SMs to the lanes'
        // covariance / eigensolve / view kernels (1024 x 1024 8-bit Fresnel + PCA, T = 32: 88.8k -> 99.5k
        // frames/s with 8 of 152)
        hv_status st = spatial_transform(raw, p->kind, p->W, p->H, p->T, p->s.space_transformation, p->lens,
                                         p->spatial, L.ring, 0, p->T, p->stream, nullptr, p->f2d_mask, p->work2,
                                         nullptr, p->nrender > 1 ? kLaneReserveSms : 0);
        if (st != HV_OK)
            return st;
        p->cov_dirty = ~0u;  // every slot rewritten
        p->f2d_buf = r;  // one spectrum per ring: window k's render reads it while batch k+1 runs
        if (p->f2d_view && (st = capture_f2d_spectrum(p, raw, r)) != HV_OK)
            return st;
        HV_CUDA_TRY(cudaEventRecord(L.ready, p->stream));
        HV_CUDA_TRY(cudaStreamWaitEvent(L.st, L.ready, 0));
        // the lane's ring, render stream and (with its own stream) per-window buffers
        p->ring = L.ring;
        p->render_stream = L.st;
        if (p->nrender > 1)
        {
            p->weights = L.weights;
            p->cov = L.cov;
            p->evals = L.evals;
            p->evecs = L.evecs;
            p->cov_work = L.cov_work;
            p->eig_work = L.eig_work;
            p->eig_warm = L.eig_warm;
            p->view = L.view;
            p->post = L.post;
            p->partials = L.partials;
            p->reduce_work = L.reduce_work;
            p->factors = L.factors;
            p->view_tc_work = L.view_tc_work;
            // the contrast range of the last autocontrast (computed on another lane)
            if (p->range_ev_set)
                HV_CUDA_TRY(cudaStreamWaitEvent(L.st, p->range_ev, 0));
        }
        p->ring_start = 0;
        p->ring_size = p->T;
        ++p->windows;
        st = render(p);
        if (st != HV_OK)
            return st;
        if (p->nrender > 1)
            L.eig_warm = p->eig_warm;
        HV_CUDA_TRY(cudaEventRecord(L.free, L.st));
        return HV_OK;
    }
    // Queue::enqueue_multiple (queue.cc:332-380)
    int nb = p->B;
    const int T = p->T;
    const size_t frame_bytes = p->HW * p->depth;
    const uint8_t* raw0 = raw;  // the batch's first frame (filter2D view)
    if (nb > T)
    {
        raw += static_cast<size_t>(nb - T) * frame_bytes;
        p->ring_start = (p->ring_start + nb - T) % T;
        nb = T;
    }
    const int begin = (p->ring_start + p->ring_size) % T;
    hv_status r = HV_OK;
    if (p->pp)
    {
        // the batch is read once, into its slots' planes (pipe stream: the covariance update reads
        // them next); the render stream writes the ring slots from the planes after the previous
        // window's view. The views read the planes: batch b waits for the ring copy of batch b - 1,
        // which the render stream runs after every view enqueued before batch b - 1. A view
        // enqueued since (it may run while batch b is converted) reads the slots of batch b from
        // the ring (ring_view).
        const int b = p->pp_b++;
        if (b >= 1)
            HV_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->pp_ring_ev[(b - 1) & 3], 0));
        r = convert_to_planes(raw, p->kind, p->HW, nb, begin, T, p->planes, p->stream);
        if (r == HV_OK)
        {
            HV_CUDA_TRY(cudaEventRecord(p->pp_main_ev, p->stream));
            HV_CUDA_TRY(cudaStreamWaitEvent(p->render_stream, p->pp_main_ev, 0));
            if ((r = ring_from_planes(p->planes, T, p->HW, begin, nb, p->ring, p->render_stream)) != HV_OK)
                return r;
        }
        else if (r == HV_ERR_UNSUPPORTED)
        {
            // a batch off 16-byte alignment: converted into the ring on the pipe stream once the
            // render stream is idle, then split
            HV_CUDA_TRY(cudaEventRecord(p->pp_main_ev, p->render_stream));
            HV_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->pp_main_ev, 0));
            if ((r = spatial_transform(raw, p->kind, p->W, p->H, nb, p->s.space_transformation, p->lens, p->spatial,
                                       p->ring, begin, T, p->stream, nullptr, p->f2d_mask, p->work2)) != HV_OK ||
                (r = cov_split_planes(p->ring, T, p->HW, begin, nb, p->planes, 1, p->stream)) != HV_OK)
                return r;
            HV_CUDA_TRY(cudaEventRecord(p->pp_main_ev, p->stream));
            HV_CUDA_TRY(cudaStreamWaitEvent(p->render_stream, p->pp_main_ev, 0));
        }
        else
            return r;
        HV_CUDA_TRY(cudaEventRecord(p->pp_ring_ev[b & 3], p->render_stream));
    }
    // real planes (no spatial transform) come out of the conversion pass itself
    const bool fused_split = !p->pp && p->planes_ok && p->planes_real && p->HW % 8 == 0 &&
                             (reinterpret_cast<uintptr_t>(raw) & 15) == 0;
    if (!p->pp && (r = spatial_transform(raw, p->kind, p->W, p->H, nb, p->s.space_transformation, p->lens,
                                         p->spatial, p->ring, begin, T, p->stream, nullptr, p->f2d_mask, p->work2,
                                         fused_split ? p->planes : nullptr)) != HV_OK)
        return r;
    // the 64-frame slot blocks whose covariance rows change, and their split planes
    for (int f = 0; f < nb; f += 1)
        p->cov_dirty |= 1u << (((begin + f) % T) / 64 & 31);
    if (p->planes_ok && !fused_split && !p->pp &&
        (r = cov_split_planes(p->ring, T, p->HW, begin, nb, p->planes, p->planes_real, p->stream)) != HV_OK)
        return r;
    p->ring_size += nb;
    if (p->ring_size > T)
    {
        p->ring_start = (p->ring_start + p->ring_size - T) % T;
        p->ring_size = T;
    }
    // insert_wait_time_transformation_size (pipe.cc:418-427)
    if (p->ring_size < T)
        return HV_OK;
    if (p->f2d_view && (r = capture_f2d_spectrum(p, raw0, 0)) != HV_OK)
        return r;
    return render(p);
}

}  // namespace

// ==================================================================================== served mode
// The serving engine (server.cpp) drives these pipes: push stages complete batches in the input
// ring and queues them; the engine plans each cycle on the host (the same bookkeeping as
// process_batch / render) into a device-side control block and launches the cycle's kernels,
// replayed from a CUDA graph where every kernel of the cycle is gated by the block.

namespace {

int64_t now_us()
{
    return std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// Copies frames into input slots; a complete slot is queued for the engine. Blocks (bounded) while
// every slot holds a queued or in-flight batch.
hv_status served_push(hv_pipe* p, const uint8_t* src, size_t n, cudaMemcpyKind kind)
{
    const size_t frame_bytes = p->HW * p->depth;
    while (n > 0)
    {
        const int slot = p->in_slot;
        if (p->in_fill == 0)
        {
            // claim the slot: wait until the engine released one (backpressure, 10 s bound)
            const auto t0 = std::chrono::steady_clock::now();
            for (;;)
            {
                {
                    std::lock_guard<std::mutex> g(p->mu);
                    if (p->in_free > 0)
                    {
                        --p->in_free;
                        break;
                    }
                }
                if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(10))
                {
                    set_last_error_msg("served push: no input slot freed within 10 s");
                    return HV_ERR_TIMEOUT;
                }
                std::this_thread::sleep_for(std::chrono::microseconds(20));
            }
            HV_CUDA_TRY(cudaStreamWaitEvent(p->copy_stream, p->in_consumed[slot], 0));
        }
        const size_t take = std::min(n, static_cast<size_t>(p->B - p->in_fill));
        uint8_t* dst = p->in_ring + slot * p->batch_bytes + static_cast<size_t>(p->in_fill) * frame_bytes;
        HV_CUDA_TRY(cudaMemcpyAsync(dst, src, take * frame_bytes, kind, p->copy_stream));
        p->in_fill += static_cast<int>(take);
        src += take * frame_bytes;
        n -= take;
        if (p->in_fill == p->B)
        {
            HV_CUDA_TRY(cudaEventRecord(p->in_filled[slot], p->copy_stream));
            {
                std::lock_guard<std::mutex> g(p->mu);
                p->ready.push_back({slot, now_us()});
            }
            p->in_fill = 0;
            p->in_slot = (slot + 1) % p->in_slots;
            if (p->notify)
                p->notify(p->notify_ctx);
        }
    }
    // the caller may reuse host memory on return
    if (kind == cudaMemcpyHostToDevice)
        HV_CUDA_TRY(cudaStreamSynchronize(p->copy_stream));
    return HV_OK;
}

}  // namespace

namespace hv {

size_t served_footprint(const hv_frame_desc& fd, const hv_settings& s) { return footprint(fd, s, true); }

hv_pipe* pipe_create_served(const hv_frame_desc* fd, const hv_settings* settings, cudaStream_t stream,
                            void (*notify)(void*), void* ctx, hv_status* status)
{
    hv_status dummy;
    hv_status& out = status ? *status : dummy;
    if (!fd || !settings || !stream)
    {
        out = HV_INVALID_VALUE;
        return nullptr;
    }
    hv_pipe* p = new (std::nothrow) hv_pipe();
    if (!p)
    {
        out = HV_FAILURE;
        return nullptr;
    }
    p->served = true;
    p->notify = notify;
    p->notify_ctx = ctx;
    p->fd = *fd;
    p->s = *settings;
    if ((out = settings_validate(&p->s, fd)) != HV_OK)
    {
        delete p;
        return nullptr;
    }
    if (p->s.cuts_enabled || (p->s.filter2d_enabled && p->s.filter2d_view_enabled))
    {
        set_last_error_msg("served streams render the XY view only (time cuts, filter2D view: use a Pipe)");
        out = HV_ERR_UNSUPPORTED;
        delete p;
        return nullptr;
    }
    if (p->s.batch_size > p->s.time_transformation_size)
    {
        set_last_error_msg("served streams need batch_size <= time_transformation_size");
        out = HV_INVALID_VALUE;
        delete p;
        return nullptr;
    }
    cudaGetDevice(&p->device);
    p->stream = stream;
    if (cudaStreamCreateWithFlags(&p->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
    {
        out = HV_ERR_CUDA;
        delete p;
        return nullptr;
    }
    p->launches0 = launch_count();
    if ((out = build(p)) != HV_OK)
    {
        hv_pipe_destroy(p);
        return nullptr;
    }
    return p;
}

bool served_graphable(const hv_pipe* p)
{
    return !uses_eig(p->s) && !uses_unwrap(p->s) && !uses_phase_increase(p->s);
}

bool served_plan(hv_pipe* p, CycleCtl* ctl, ServedCycle* c)
{
    *c = ServedCycle{};
    std::memset(ctl, 0, sizeof(*ctl));
    {
        std::lock_guard<std::mutex> g(p->mu);
        if (p->ready.empty())
            return false;
        c->in_slot = p->ready.front().slot;
        c->t_push_us = p->ready.front().t_push_us;
        p->ready.pop_front();
    }
    ctl->raw_offset = static_cast<long long>(c->in_slot) * static_cast<long long>(p->batch_bytes);
    // insert_wait_time_stride (pipe.cc:400-416): only the batch completing the stride is processed
    p->batch_index += p->B;
    if (p->batch_index != p->S)
        return true;
    p->batch_index = 0;
    c->active = true;
    ctl->active = 1;
    // Queue::enqueue_multiple (queue.cc:332-380), B <= T
    const int T = p->T;
    ctl->ring_begin = (p->ring_start + p->ring_size) % T;
    p->ring_size += p->B;
    if (p->ring_size > T)
    {
        p->ring_start = (p->ring_start + p->ring_size - T) % T;
        p->ring_size = T;
    }
    // insert_wait_time_transformation_size (pipe.cc:418-427)
    if (p->ring_size < T)
        return true;
    c->render = true;
    ctl->render = 1;
    // accumulation queue (queue.cc:149-189)
    if (p->A > 0)
    {
        ctl->acc_slot = (p->acc_start + p->acc_size) % p->A;
        if (p->acc_size < p->A)
            ++p->acc_size;
        else
            p->acc_start = (p->acc_start + 1) % p->A;
        ctl->acc_start = p->acc_start;
        ctl->acc_count = p->acc_size;
    }
    // autocontrast gating (rendering.cc:239-299)
    const hv_settings& s = p->s;
    if (s.contrast_enabled && p->autocontrast_pending)
    {
        const bool apply = p->A == 0 || p->acc_size == p->A || p->acc_size == 1;
        if (apply)
        {
            ctl->pct_enable = 1;
            if (p->A == 0 || p->acc_size == p->A)
                p->autocontrast_pending = false;
        }
    }
    // output slot (the oldest output is overwritten when the queue is full)
    {
        std::lock_guard<std::mutex> g(p->mu);
        if (p->out_count == p->out_cap)
        {
            p->out_head = (p->out_head + 1) % p->out_cap;
            --p->out_count;
            ++p->out_overwritten;
        }
        c->out_slot = (p->out_head + p->out_count) % p->out_cap;
    }
    ctl->out_slot = c->out_slot;
    return true;
}

hv_status served_prepare(hv_pipe* p, const ServedCycle& c, cudaStream_t st)
{
    HV_CUDA_TRY(cudaStreamWaitEvent(st, p->in_filled[c.in_slot], 0));
    if (c.render)
        HV_CUDA_TRY(cudaStreamWaitEvent(st, p->out_freed[c.out_slot], 0));
    return HV_OK;
}

hv_status served_record(hv_pipe* p, const CycleCtl* ctl, const ServedCycle& c, bool gated, cudaStream_t st)
{
    const hv_settings& s = p->s;
    hv_status r;
    if (gated || c.active)
    {
        if ((r = spatial_transform(p->in_ring, p->kind, p->W, p->H, p->B, s.space_transformation, p->lens, p->spatial,
                                   p->ring, 0, p->T, st, ctl, p->f2d_mask, p->work2)) != HV_OK)
            return r;
        // ring slots chosen on the device: no record of which covariance rows changed
        p->cov_valid = false;
        p->planes_ok = false;
    }
    if (!gated && !c.render)
        return HV_OK;
    const bool renorm = s.renorm != 0;
    const float* frame = nullptr;
    int shift_after = 0;
    if ((r = render_view(p, st, ctl, &frame, &shift_after)) != HV_OK)
        return r;
    if ((r = renorm_shift_accumulate(frame, p->post, p->W, p->H, renorm ? p->factors : nullptr, shift_after,
                                     p->A > 0 ? p->acc_ring : nullptr, p->A, 0, 0, 0, s.log_enabled, st, 1.0f, ctl)) !=
        HV_OK)
        return r;
    if (s.contrast_enabled && (gated || (ctl && c.render)))
    {
        // gated per cycle by ctl->pct_enable (autocontrast requests)
        if ((r = percentile(p->post, p->W, p->H, s.contrast_lower, s.contrast_upper,
                            s.reticle_display ? s.reticle_scale : 0.0f, p->range, p->pct_work, st, ctl)) != HV_OK)
            return r;
    }
    return contrast_to_ushort(p->post, p->range, s.contrast_invert, s.contrast_enabled, p->out_ring, p->HW, st, ctl);
}

hv_status served_complete(hv_pipe* p, const ServedCycle& c, cudaStream_t st)
{
    HV_CUDA_TRY(cudaEventRecord(p->in_consumed[c.in_slot], st));
    if (c.render)
    {
        HV_CUDA_TRY(cudaEventRecord(p->out_ready[c.out_slot], st));
        p->last_frame_valid = true;
    }
    std::lock_guard<std::mutex> g(p->mu);
    ++p->in_free;
    if (c.render)
        ++p->out_count;
    return HV_OK;
}

}  // namespace hv

// ==================================================================================== C ABI

extern "C" {

size_t hv_pipe_footprint(const hv_frame_desc* fd, const hv_settings* settings)
{
    if (!fd || !settings)
        return 0;
    hv_settings s = *settings;
    if (settings_validate(&s, fd) != HV_OK)
        return 0;
    return footprint(*fd, s);
}

hv_pipe* hv_pipe_create(const hv_frame_desc* fd, const hv_settings* settings, void* stream, hv_status* status)
{
    hv_status dummy;
    hv_status& out = status ? *status : dummy;
    if (!fd || !settings)
    {
        out = HV_INVALID_VALUE;
        return nullptr;
    }
    hv_pipe* p = new (std::nothrow) hv_pipe();
    if (!p)
    {
        out = HV_FAILURE;
        return nullptr;
    }
    p->fd = *fd;
    p->s = *settings;
    if ((out = settings_validate(&p->s, fd)) != HV_OK)
    {
        delete p;
        return nullptr;
    }
    if (cudaGetDevice(&p->device) != cudaSuccess)
    {
        set_last_error_msg("no CUDA device");
        out = HV_ERR_CUDA;
        delete p;
        return nullptr;
    }
    if (stream)
        p->stream = static_cast<cudaStream_t>(stream);
    else
    {
        if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess)
        {
            out = HV_ERR_CUDA;
            delete p;
            return nullptr;
        }
        p->own_stream = true;
    }
    // the eigensolve chain of a pipelined PCA window is latency bound and on the critical path: its
    // small grids go first when SMs free up
    int least_prio = 0, greatest_prio = 0;
    if (cudaStreamCreateWithFlags(&p->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p->render_stream_owned, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p->render_extra[0], cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&p->render_extra[1], cudaStreamNonBlocking) != cudaSuccess ||
        cudaDeviceGetStreamPriorityRange(&least_prio, &greatest_prio) != cudaSuccess ||
        cudaStreamCreateWithPriority(&p->eig_stream, cudaStreamNonBlocking, greatest_prio) != cudaSuccess)
    {
        out = HV_ERR_CUDA;
        hv_pipe_destroy(p);
        return nullptr;
    }
    p->launches0 = launch_count();
    if ((out = build(p)) != HV_OK)
    {
        hv_pipe_destroy(p);
        return nullptr;
    }
    return p;
}

void hv_pipe_destroy(hv_pipe* p)
{
    if (!p)
        return;
    if (p->stream)
        cudaStreamSynchronize(p->stream);
    if (p->copy_stream)
        cudaStreamSynchronize(p->copy_stream);
    if (p->render_stream_owned)
        cudaStreamSynchronize(p->render_stream_owned);
    for (cudaStream_t e : p->render_extra)
        if (e)
            cudaStreamSynchronize(e);
    if (p->eig_stream)
        cudaStreamSynchronize(p->eig_stream);
    free_buffers(p);
    if (p->copy_stream)
        cudaStreamDestroy(p->copy_stream);
    if (p->render_stream_owned)
        cudaStreamDestroy(p->render_stream_owned);
    for (cudaStream_t e : p->render_extra)
        if (e)
            cudaStreamDestroy(e);
    if (p->eig_stream)
        cudaStreamDestroy(p->eig_stream);
    if (p->own_stream && p->stream)
        cudaStreamDestroy(p->stream);
    delete p;
}

hv_status hv_pipe_push_frames(hv_pipe* p, const void* frames, size_t n, int mem)
{
    if (!p || (!frames && n))
        return HV_INVALID_VALUE;
    const size_t frame_bytes = p->HW * p->depth;
    const uint8_t* src = static_cast<const uint8_t*>(frames);
    const cudaMemcpyKind kind = mem == HV_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    hv_status r;
    if (p->served)
        return served_push(p, src, n, kind);
    while (n > 0)
    {
        if (mem == HV_MEM_DEVICE && p->in_fill == 0 && n >= static_cast<size_t>(p->B))
        {
            // zero-copy: the batch is consumed in place, stream-ordered on the pipe's stream
            if ((r = process_batch(p, src)) != HV_OK)
                return r;
            src += frame_bytes * p->B;
            n -= p->B;
            continue;
        }
        const int slot = p->in_slot;
        const size_t take = std::min(n, static_cast<size_t>(p->B - p->in_fill));
        uint8_t* dst = p->in_ring + slot * p->batch_bytes + static_cast<size_t>(p->in_fill) * frame_bytes;
        if (p->in_fill == 0)
            HV_CUDA_TRY(cudaStreamWaitEvent(p->copy_stream, p->in_consumed[slot], 0));
        HV_CUDA_TRY(cudaMemcpyAsync(dst, src, take * frame_bytes, kind, p->copy_stream));
        p->in_fill += static_cast<int>(take);
        src += take * frame_bytes;
        n -= take;
        if (p->in_fill == p->B)
        {
            HV_CUDA_TRY(cudaEventRecord(p->in_filled[slot], p->copy_stream));
            HV_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->in_filled[slot], 0));
            if ((r = process_batch(p, p->in_ring + slot * p->batch_bytes)) != HV_OK)
                return r;
            HV_CUDA_TRY(cudaEventRecord(p->in_consumed[slot], p->stream));
            p->in_fill = 0;
            p->in_slot = (slot + 1) % p->in_slots;
        }
    }
    // the caller may reuse host memory on return: wait for its copies only
    if (mem == HV_MEM_HOST)
        HV_CUDA_TRY(cudaStreamSynchronize(p->copy_stream));
    return HV_OK;
}

size_t hv_pipe_output_count(hv_pipe* p)
{
    if (!p)
        return 0;
    std::lock_guard<std::mutex> g(p->mu);
    return static_cast<size_t>(p->out_count);
}

hv_status hv_pipe_pull_output(hv_pipe* p, uint16_t* dst, int mem, int64_t timeout_us)
{
    if (!p || !dst)
        return HV_INVALID_VALUE;
    int slot;
    {
        std::lock_guard<std::mutex> g(p->mu);
        if (p->out_count == 0)
            return timeout_us > 0 ? HV_ERR_TIMEOUT : HV_NO_IN_DATA;
        slot = p->out_head;
    }
    // bounded wait for the frame's kernels
    const auto t0 = std::chrono::steady_clock::now();
    for (;;)
    {
        const cudaError_t e = cudaEventQuery(p->out_ready[slot]);
        if (e == cudaSuccess)
            break;
        if (e != cudaErrorNotReady)
        {
            set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
            return HV_ERR_CUDA;
        }
        const auto us =
            std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_us >= 0 && us > timeout_us)
            return HV_ERR_TIMEOUT;
        std::this_thread::yield();
    }
    HV_CUDA_TRY(cudaMemcpyAsync(dst, p->out_ring + slot * p->HW, p->HW * sizeof(uint16_t),
                                mem == HV_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                p->copy_stream));
    HV_CUDA_TRY(cudaEventRecord(p->out_freed[slot], p->copy_stream));
    HV_CUDA_TRY(cudaStreamSynchronize(p->copy_stream));
    {
        std::lock_guard<std::mutex> g(p->mu);
        if (p->out_head == slot && p->out_count > 0)
        {
            p->out_head = (p->out_head + 1) % p->out_cap;
            --p->out_count;
        }
    }
    return HV_OK;
}

// Waits for the rendering of every window enqueued so far (all lanes' render streams).
static hv_status sync_render(hv_pipe* p)
{
    HV_CUDA_TRY(cudaStreamSynchronize(p->render_stream));
    if (p->pp)
        HV_CUDA_TRY(cudaStreamSynchronize(p->eig_stream));
    if (p->nrender > 1)
        for (int l = 0; l < p->nrender; ++l)
            HV_CUDA_TRY(cudaStreamSynchronize(p->lanes[l].st));
    return HV_OK;
}

hv_status hv_pipe_update_settings(hv_pipe* p, const hv_settings* settings)
{
    if (!p || !settings)
        return HV_INVALID_VALUE;
    hv_settings ns = *settings;
    hv_status r = settings_validate(&ns, &p->fd);
    if (r != HV_OK)
        return r;
    if (std::memcmp(&ns, &p->s, sizeof(ns)) == 0)
        return HV_NO_CHANGE;
    HV_CUDA_TRY(cudaStreamSynchronize(p->stream));
    HV_CUDA_TRY(cudaStreamSynchronize(p->copy_stream));
    {
        const hv_status rs = sync_render(p);
        if (rs != HV_OK)
            return rs;
    }
    p->s = ns;
    return build(p);
}

hv_status hv_pipe_request_autocontrast(hv_pipe* p)
{
    if (!p)
        return HV_INVALID_VALUE;
    p->autocontrast_pending = p->s.contrast_enabled != 0;
    if (p->cuts)
    {
        p->views[0].autocontrast_pending = p->s.xz_contrast_enabled != 0;
        p->views[1].autocontrast_pending = p->s.yz_contrast_enabled != 0;
    }
    if (p->f2d_view)
        p->views[HV_VIEW_FILTER2D].autocontrast_pending = p->s.filter2d_contrast_enabled != 0;
    return HV_OK;
}

hv_status hv_pipe_sync(hv_pipe* p)
{
    if (!p)
        return HV_INVALID_VALUE;
    HV_CUDA_TRY(cudaStreamSynchronize(p->copy_stream));
    HV_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return sync_render(p);
}

hv_status hv_pipe_join(hv_pipe* p)
{
    if (!p)
        return HV_INVALID_VALUE;
    if (p->render_stream != p->stream)
    {
        // one event, recorded and waited on per render stream in turn (a wait takes the event's
        // state at the time of the call)
        const int n = p->nrender > 1 ? p->nrender : 1;
        for (int l = 0; l < n; ++l)
        {
            HV_CUDA_TRY(cudaEventRecord(p->join_ev, n > 1 ? p->lanes[l].st : p->render_stream));
            HV_CUDA_TRY(cudaStreamWaitEvent(p->stream, p->join_ev, 0));
        }
    }
    return HV_OK;
}

hv_status hv_pipe_get_contrast_range(hv_pipe* p, float* min_out, float* max_out)
{
    if (!p)
        return HV_INVALID_VALUE;
    float r[2];
    HV_CUDA_TRY(cudaStreamSynchronize(p->stream));
    {
        const hv_status rs = sync_render(p);
        if (rs != HV_OK)
            return rs;
    }
    HV_CUDA_TRY(cudaMemcpy(r, p->range, sizeof(r), cudaMemcpyDeviceToHost));
    if (min_out)
        *min_out = r[0];
    if (max_out)
        *max_out = r[1];
    return HV_OK;
}

hv_status hv_pipe_get_float_frame(hv_pipe* p, float* dst)
{
    if (!p || !dst)
        return HV_INVALID_VALUE;
    if (!p->last_frame_valid)
        return HV_NO_IN_DATA;
    HV_CUDA_TRY(cudaStreamSynchronize(p->stream));
    {
        const hv_status rs = sync_render(p);
        if (rs != HV_OK)
            return rs;
    }
    HV_CUDA_TRY(cudaMemcpy(dst, p->post, p->HW * sizeof(float), cudaMemcpyDeviceToHost));
    return HV_OK;
}

// a secondary view exists: the cuts (0, 1) or the filter2D view (2)
static bool has_view(const hv_pipe* p, int which)
{
    return (which == HV_VIEW_XZ || which == HV_VIEW_YZ) ? p->cuts : (which == HV_VIEW_FILTER2D && p->f2d_view);
}

size_t hv_pipe_view_output_count(hv_pipe* p, int which)
{
    if (!p || which < 0 || which > 2 || !has_view(p, which))
        return 0;
    std::lock_guard<std::mutex> g(p->mu);
    return static_cast<size_t>(p->views[which].out_count);
}

hv_status hv_pipe_pull_view(hv_pipe* p, int which, uint16_t* dst, int mem, int64_t timeout_us)
{
    if (!p || !dst || which < 0 || which > 2)
        return HV_INVALID_VALUE;
    if (!has_view(p, which))
        return HV_NO_IN_DATA;
    hv_pipe::SecondaryView& c = p->views[which];
    int slot;
    {
        std::lock_guard<std::mutex> g(p->mu);
        if (c.out_count == 0)
            return timeout_us > 0 ? HV_ERR_TIMEOUT : HV_NO_IN_DATA;
        slot = c.out_head;
    }
    const auto t0 = std::chrono::steady_clock::now();
    for (;;)
    {
        const cudaError_t e = cudaEventQuery(c.out_ready[slot]);
        if (e == cudaSuccess)
            break;
        if (e != cudaErrorNotReady)
        {
            set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
            return HV_ERR_CUDA;
        }
        const auto us =
            std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_us >= 0 && us > timeout_us)
            return HV_ERR_TIMEOUT;
        std::this_thread::yield();
    }
    const size_t px = static_cast<size_t>(c.w) * c.h;
    HV_CUDA_TRY(cudaMemcpyAsync(dst, c.out_ring + slot * px, px * sizeof(uint16_t),
                                mem == HV_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                p->copy_stream));
    HV_CUDA_TRY(cudaEventRecord(c.out_freed[slot], p->copy_stream));
    HV_CUDA_TRY(cudaStreamSynchronize(p->copy_stream));
    {
        std::lock_guard<std::mutex> g(p->mu);
        if (c.out_head == slot && c.out_count > 0)
        {
            c.out_head = (c.out_head + 1) % c.out_cap;
            --c.out_count;
        }
    }
    return HV_OK;
}

hv_status hv_pipe_get_view_float_frame(hv_pipe* p, int which, float* dst, float* range_out)
{
    if (!p || which < 0 || which > 2)
        return HV_INVALID_VALUE;
    if (!has_view(p, which) || !p->views[which].valid)
        return HV_NO_IN_DATA;
    const hv_pipe::SecondaryView& c = p->views[which];
    HV_CUDA_TRY(cudaStreamSynchronize(p->stream));
    {
        const hv_status rs = sync_render(p);
        if (rs != HV_OK)
            return rs;
    }
    if (dst)
        HV_CUDA_TRY(cudaMemcpy(dst, c.post, static_cast<size_t>(c.w) * c.h * sizeof(float), cudaMemcpyDeviceToHost));
    if (range_out)
        HV_CUDA_TRY(cudaMemcpy(range_out, c.range, 2 * sizeof(float), cudaMemcpyDeviceToHost));
    return HV_OK;
}

hv_status hv_pipe_get_ring(hv_pipe* p, void* dst_host, int32_t* start, int32_t* size)
{
    if (!p)
        return HV_INVALID_VALUE;
    HV_CUDA_TRY(cudaStreamSynchronize(p->stream));
    {
        const hv_status rs = sync_render(p);
        if (rs != HV_OK)
            return rs;
    }
    if (dst_host)
        HV_CUDA_TRY(cudaMemcpy(dst_host, p->ring, p->HW * p->T * sizeof(float2), cudaMemcpyDeviceToHost));
    if (start)
        *start = p->ring_start;
    if (size)
        *size = p->ring_size;
    return HV_OK;
}

uint64_t hv_pipe_kernel_launches(hv_pipe* p)
{
    return p ? launch_count() - p->launches0 : 0;
}

void* hv_pipe_stream(hv_pipe* p) { return p ? static_cast<void*>(p->stream) : nullptr; }

}  // extern "C"
