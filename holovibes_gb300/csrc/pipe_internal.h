// Internal view of the Pipe for the serving engine (server.cpp): the pipe's state and the
// served-mode entry points. Not part of the ABI.
#pragma once

#include <deque>
#include <mutex>
#include <vector>

#include "hv_internal.h"

struct hv_pipe
{
    hv_frame_desc fd{};
    hv_settings s{};
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaStream_t render_stream = nullptr;  // == stream unless the double-buffered fast mode is on
    cudaStream_t render_stream_owned = nullptr;
    bool own_stream = false;

    int W = 0, H = 0;
    size_t HW = 0;
    int depth = 2, kind = 0;
    int B = 1, T = 1, S = 1, K = 1, pmin = 0, pmax = 0, A = 0;
    int qmin = 0, qn = 1;  // SSA_STFT eigenvector columns kept

    // device buffers
    std::vector<void*> allocs;
    float2* lens = nullptr;
    float2* spatial = nullptr;
    float2* f2d_mask = nullptr;  // filter2D mask in FFT layout (Fresnel / no propagation)
    float2* work2 = nullptr;     // second spatial buffer of the filtered Fresnel passes
    float2* ring = nullptr;
    // fast mode (batch == stride == window): window k fills the ring of lane k % nlanes on
    // `stream` while earlier windows are transformed and rendered. With nrender == 1 the lanes
    // share `render_stream` and the per-window buffers; with nrender == nlanes (eigensolve
    // workloads, whose covariance -> eigensolve -> projection chain per window is longer than the
    // spatial passes) every lane has its own render stream and per-window buffers, so the time
    // transforms of consecutive windows overlap too.
    static constexpr int kMaxLanes = 3;
    struct Lane
    {
        float2* ring = nullptr;
        cudaEvent_t ready = nullptr, free = nullptr;
        cudaStream_t st = nullptr;
        float2* weights = nullptr;
        double2* cov = nullptr;
        double* evals = nullptr;
        double2* evecs = nullptr;
        void* cov_work = nullptr;
        void* eig_work = nullptr;
        bool eig_warm = false;
        float* view = nullptr;
        float* post = nullptr;
        double* partials = nullptr;
        void* reduce_work = nullptr;
        float* factors = nullptr;
        void* view_tc_work = nullptr;
    };
    bool fast = false;
    Lane lanes[kMaxLanes];
    int nlanes = 0, nrender = 1;
    cudaStream_t render_extra[kMaxLanes - 1] = {nullptr, nullptr};  // render streams of lanes 1, 2
    cudaStream_t eig_stream = nullptr;  // the pipelined PCA windows' eigensolves (greatest priority)
    cudaEvent_t range_ev = nullptr;  // after the last autocontrast (lanes with their own streams)
    bool range_ev_set = false;
    cudaEvent_t join_ev = nullptr;
    uint64_t windows = 0;
    float2* weights = nullptr;
    double2* cov = nullptr;
    double* evals = nullptr;
    double2* evecs = nullptr;
    void* cov_work = nullptr;
    void* eig_work = nullptr;
    bool eig_warm = false;  // eig_work holds the eigenvectors of the previous window (same T)
    // `cov` holds the covariance of the ring as it was at the last render, computed with engine
    // mode `cov_mode`; the 64-frame slot blocks rewritten since then are set in `cov_dirty`
    bool cov_valid = false;
    int cov_mode = -1;
    uint32_t cov_dirty = ~0u;
    // split-BF16 planes of the ring for the tiled covariance; planes_ok: they mirror every slot
    uint16_t* planes = nullptr;
    bool planes_ok = false;
    int planes_real = 0;  // the ring's imaginary parts are 0: real rows only
    // PCA windows pipelined over three streams (pipe.cpp, `pp`): the pipe stream converts each
    // batch into the split planes and updates the covariance, the eigensolve stream solves it,
    // the render stream writes the ring from the planes and renders; covariance and weights
    // alternate between two buffers by window parity
    bool pp = false, pp_nested = false;
    int pp_w = 0, pp_b = 0;
    double2* pp_cov[2] = {nullptr, nullptr};
    float2* pp_weights[2] = {nullptr, nullptr};
    cudaEvent_t pp_cov_ev[2] = {nullptr, nullptr}, pp_eig_ev[2] = {nullptr, nullptr};
    cudaEvent_t pp_view_ev[2] = {nullptr, nullptr}, pp_main_ev = nullptr;
    cudaEvent_t pp_ring_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    float* view = nullptr;
    float* unwrapped = nullptr;
    void* unwrap_work = nullptr;
    double* partials = nullptr;
    int npartials = 0;
    void* reduce_work = nullptr;
    float* factors = nullptr;
    float* post = nullptr;
    float* acc_ring = nullptr;
    float* range = nullptr;
    void* pct_work = nullptr;
    bool view_on_tc = false;  // K-bin contraction on the tensor cores (hv_time_view_tc)
    float* bin_w = nullptr;   // moments: per-bin weights f_k^n (null for the other views)
    void* view_tc_work = nullptr;
    // phase increase: previous p plane, previous increment, min / max partials, windows rendered
    float2* pi_pred = nullptr;
    float* pi_hist = nullptr;
    float2* pi_minmax = nullptr;
    uint64_t pi_count = 0;

    // secondary views, each with its float image, accumulation ring, contrast range and output
    // queue: the time-transformation cuts (XZ: T x W, YZ: H x T; gpu_output_queue_xz / _yz,
    // icompute.cc:195-213) and the filter2D view (W x H, gpu_filter2d_view_queue, pipe.cc:215-224)
    struct SecondaryView
    {
        int w = 0, h = 0;  // image width and height (XZ: W x T, YZ: T x H)
        float* post = nullptr;
        float* acc_ring = nullptr;
        int A = 0, acc_start = 0, acc_size = 0;
        float* range = nullptr;
        bool autocontrast_pending = false;
        uint16_t* out_ring = nullptr;
        int out_cap = 0, out_head = 0, out_count = 0;
        uint64_t out_overwritten = 0;
        std::vector<cudaEvent_t> out_ready, out_freed;
        bool valid = false;
    };
    bool cuts = false;
    float2* w_all = nullptr;  // all T weight rows: bins (STFT / SSA_STFT), components (PCA), identity (NONE)
    void* cut_work = nullptr;
    bool f2d_view = false;
    float2* f2d_spec[2] = {nullptr, nullptr};  // masked spectrum of the batch's first frame (per fast-mode ring)
    int f2d_buf = 0;
    SecondaryView views[3];   // HV_VIEW_XZ, HV_VIEW_YZ, HV_VIEW_FILTER2D

    // input ring of batch slots
    uint8_t* in_ring = nullptr;
    int in_slots = 0;
    size_t batch_bytes = 0;
    std::vector<cudaEvent_t> in_filled, in_consumed;
    int in_slot = 0;
    int in_fill = 0;  // frames already in the current slot

    // output ring
    uint16_t* out_ring = nullptr;
    int out_cap = 0;
    std::vector<cudaEvent_t> out_ready, out_freed;
    int out_head = 0, out_count = 0;
    uint64_t out_overwritten = 0;

    // cycle state
    int ring_start = 0, ring_size = 0;
    int batch_index = 0;
    int acc_start = 0, acc_size = 0;
    bool autocontrast_pending = false;
    bool last_frame_valid = false;
    uint64_t launches0 = 0;

    std::mutex mu;

    // served mode (driven by an hv_server): inputs are only staged by push; the server plans and
    // launches the cycles (one per ready batch) with a device-side control block
    bool served = false;
    struct ReadyBatch
    {
        int slot;          // input ring slot
        int64_t t_push_us; // steady-clock time the batch was complete
    };
    std::deque<ReadyBatch> ready;  // guarded by mu
    int in_free = 0;               // input slots not holding a queued or in-flight batch (mu)
    void (*notify)(void*) = nullptr;
    void* notify_ctx = nullptr;
};

namespace hv {

// One planned served cycle (host side of the control block).
struct ServedCycle
{
    int in_slot = -1;
    int64_t t_push_us = 0;
    bool active = false;  // spatial passes run (stride gate passed)
    bool render = false;  // the window is rendered into output slot out_slot
    int out_slot = -1;
};

// Creates a pipe for a server: cycles are launched by the server on `stream` (no double-buffered
// fast mode); push only stages batches. B <= T and S a multiple of B are required.
hv_pipe* pipe_create_served(const hv_frame_desc* fd, const hv_settings* s, cudaStream_t stream,
                            void (*notify)(void*), void* ctx, hv_status* status);
// Device footprint of a served pipe.
size_t served_footprint(const hv_frame_desc& fd, const hv_settings& s);
// Whether the pipe's cycle can be captured in a CUDA graph (every kernel of its cycle is gated by the
// control block): STFT or no time transform, no 2-D unwrap, no phase increase.
bool served_graphable(const hv_pipe* p);
// Takes the oldest ready batch (if any) and advances the host bookkeeping of the cycle (stride gate,
// ring, accumulation queue, autocontrast gating, output slot); fills the control block.
bool served_plan(hv_pipe* p, CycleCtl* ctl, ServedCycle* c);
// Enqueues the cycle's kernels, reading the cycle's values from `ctl_dev`. With `gated`, the whole
// cycle is recorded (for a graph) and the control block gates it; otherwise only the planned part.
hv_status served_record(hv_pipe* p, const CycleCtl* ctl_dev, const ServedCycle& c, bool gated, cudaStream_t st);
// After the cycle's launch on `st`: input slot release and output publication.
hv_status served_complete(hv_pipe* p, const ServedCycle& c, cudaStream_t st);
// Before the cycle's launch on `st`: wait for the batch's upload and for the output slot's reader.
hv_status served_prepare(hv_pipe* p, const ServedCycle& c, cudaStream_t st);

}  // namespace hv
