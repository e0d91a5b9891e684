// Serving engine: many frame streams of different resolutions and time windows on one GPU.
//
// No reference counterpart: the reference runs one Pipe per Holovibes instance on one compute
// thread (Backend/sources/core/pipe.cc:650-676, one cudaStream_t per Pipe, compute_worker.cc:13-21).
// Each served stream here is a served-mode Pipe (the same kernels, buffers and cycle semantics as
// hv_pipe, pipe.cc:255-524) whose cycles are planned and launched by one persistent engine thread:
//
//   admission   a stream is admitted when its device footprint fits the server's HBM budget;
//               an open request waits (bounded) until closed streams free enough memory
//   buckets     streams are grouped by shape (width, height, depth, space / time transform, T, B);
//               a bucket owns one CUDA stream, so buckets overlap on the device
//   cycles      each engine pass takes at most one ready batch per stream and plans its cycle on
//               the host into a device-side control block (ring slot, accumulation slot,
//               autocontrast gate, output slot, active / render flags); one copy uploads the
//               blocks of a bucket
//   graphs      the cycles of a bucket's steady streams (ring full, first render done eagerly)
//               are captured once as parallel branches of one CUDA graph, replayed every pass:
//               one graph launch per bucket; streams without a batch in that pass are gated off
//               by their control block. Streams whose cycle is not fully gated (PCA, 2-D unwrap)
//               and streams still filling their ring are launched eagerly on the bucket stream.
//   latency     batch complete (push) -> hologram ready (host callback after the launch)
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "pipe_internal.h"

using namespace hv;

namespace {

constexpr int kMaxMembers = 32;  // streams per bucket (graph branches)
constexpr int kCtlRing = 4;      // pinned control-block upload buffers per bucket
constexpr size_t kLatencyKeep = 8192;

int64_t now_us()
{
    return std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct Bucket;

struct Member
{
    int32_t id = 0;
    hv_pipe* p = nullptr;
    Bucket* bucket = nullptr;
    size_t footprint = 0;
    bool steady = false;  // ring full and one render done eagerly: eligible for the bucket graph
    cudaGraphExec_t solo = nullptr;  // this stream's cycle alone (launched when few streams are ready)
    size_t solo_kernels = 0;
    // per-stream launches (HV_SERVER_STREAM_GRAPHS): the stream's own CUDA stream and control block
    cudaStream_t own = nullptr;
    CycleCtl* ctl_dev = nullptr;
    CycleCtl* ctl_host = nullptr;  // pinned ring of kCtlRing blocks
    cudaEvent_t ctl_ev[kCtlRing] = {};
    int ctl_i = 0;
};

void destroy_member_stream(Member* m)
{
    if (m->own)
        cudaStreamSynchronize(m->own);
    for (cudaEvent_t& e : m->ctl_ev)
        if (e)
        {
            cudaEventDestroy(e);
            e = nullptr;
        }
    if (m->ctl_dev)
        cudaFree(m->ctl_dev);
    if (m->ctl_host)
        cudaFreeHost(m->ctl_host);
    if (m->own)
        cudaStreamDestroy(m->own);
    m->own = nullptr;
    m->ctl_dev = nullptr;
    m->ctl_host = nullptr;
}

hv_status make_member_stream(Member* m)
{
    cudaError_t e = cudaStreamCreateWithFlags(&m->own, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaMalloc(&m->ctl_dev, sizeof(CycleCtl));
    if (e == cudaSuccess)
        e = cudaMemset(m->ctl_dev, 0, sizeof(CycleCtl));
    if (e == cudaSuccess)
        e = cudaMallocHost(&m->ctl_host, kCtlRing * sizeof(CycleCtl));
    for (int i = 0; i < kCtlRing && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&m->ctl_ev[i], cudaEventDisableTiming);
    if (e != cudaSuccess)
    {
        set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
        destroy_member_stream(m);
        return e == cudaErrorMemoryAllocation ? HV_ERR_OOM : HV_ERR_CUDA;
    }
    return HV_OK;
}

struct Bucket
{
    std::string key;
    cudaStream_t stream = nullptr;
    std::vector<Member*> members;  // member i uses control block i
    CycleCtl* ctl_dev = nullptr;   // kMaxMembers blocks
    CycleCtl* ctl_host = nullptr;  // pinned, kCtlRing x kMaxMembers
    cudaEvent_t ctl_ev[kCtlRing] = {};
    int ctl_i = 0;
    bool graphable = true;
    cudaGraphExec_t exec = nullptr;
    std::vector<Member*> graph_members;  // members captured in `exec`, in capture order
    size_t graph_kernels = 0;
    int pending = 0;  // streams being opened into this bucket (keeps it alive)
};

}  // namespace

struct hv_server
{
    size_t budget = 0, used = 0;
    int flags = 0;
    int64_t batch_window_us = 1500;  // how long a partly ready bucket waits for its other streams
    std::mutex mu;      // membership, buckets, admission (held by the engine during a pass)
    std::mutex map_mu;  // the id -> stream map (push / pull lookups do not wait for the engine)
    std::condition_variable admit_cv;
    std::mutex work_mu;
    std::condition_variable work_cv;
    uint64_t work_seq = 0;  // guarded by work_mu
    std::map<int32_t, Member*> members;
    std::vector<Bucket*> buckets;
    int32_t next_id = 1;
    std::thread engine;
    std::atomic<bool> stop{false};
    std::atomic<bool> idle{true};
    hv_status engine_error = HV_OK;
    std::string engine_error_msg;
    cudaStream_t capture_stream = nullptr;
    std::vector<cudaStream_t> branch;  // kMaxMembers capture branches
    cudaEvent_t fork_ev = nullptr;
    std::vector<cudaEvent_t> join_ev;
    // statistics
    std::atomic<uint64_t> batches{0}, outputs{0}, graph_launches{0}, eager_cycles{0}, captures{0},
        graph_kernels{0};
    std::mutex lat_mu;
    std::vector<int64_t> latencies;  // ring of the last kLatencyKeep values (us)
    size_t lat_next = 0;
};

namespace {

void notify_engine(void* ctx)
{
    hv_server* s = static_cast<hv_server*>(ctx);
    {
        std::lock_guard<std::mutex> g(s->work_mu);
        ++s->work_seq;
    }
    s->work_cv.notify_one();
}

struct LatencyRecord
{
    hv_server* s;
    std::vector<int64_t> t_push;
};

void CUDART_CB record_latencies(void* data)
{
    LatencyRecord* r = static_cast<LatencyRecord*>(data);
    const int64_t t = now_us();
    {
        std::lock_guard<std::mutex> g(r->s->lat_mu);
        for (int64_t tp : r->t_push)
        {
            const int64_t v = t - tp;
            if (r->s->latencies.size() < kLatencyKeep)
                r->s->latencies.push_back(v);
            else
                r->s->latencies[r->s->lat_next] = v;
            r->s->lat_next = (r->s->lat_next + 1) % kLatencyKeep;
        }
    }
    r->s->outputs += r->t_push.size();
    delete r;
}

std::string bucket_key(const hv_frame_desc& fd, const hv_settings& s)
{
    char buf[160];
    std::snprintf(buf, sizeof(buf), "%dx%d:d%d:e%d:sp%d:tt%d:T%d:B%d", fd.width, fd.height, fd.depth, fd.byte_endian,
                  s.space_transformation, s.time_transformation, s.time_transformation_size, s.batch_size);
    return buf;
}

hv_status destroy_bucket(Bucket* b)
{
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    for (cudaEvent_t& e : b->ctl_ev)
        if (e)
            cudaEventDestroy(e);
    if (b->ctl_dev)
        cudaFree(b->ctl_dev);
    if (b->ctl_host)
        cudaFreeHost(b->ctl_host);
    if (b->stream)
        cudaStreamDestroy(b->stream);
    delete b;
    return HV_OK;
}

hv_status make_bucket(const std::string& key, bool graphable, Bucket** out)
{
    Bucket* b = new (std::nothrow) Bucket();
    if (!b)
        return HV_FAILURE;
    b->key = key;
    b->graphable = graphable;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaMalloc(&b->ctl_dev, kMaxMembers * sizeof(CycleCtl));
    if (e == cudaSuccess)
        e = cudaMemset(b->ctl_dev, 0, kMaxMembers * sizeof(CycleCtl));
    if (e == cudaSuccess)
        e = cudaMallocHost(&b->ctl_host, kCtlRing * kMaxMembers * sizeof(CycleCtl));
    for (int i = 0; i < kCtlRing && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&b->ctl_ev[i], cudaEventDisableTiming);
    if (e != cudaSuccess)
    {
        set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
        destroy_bucket(b);
        return e == cudaErrorMemoryAllocation ? HV_ERR_OOM : HV_ERR_CUDA;
    }
    *out = b;
    return HV_OK;
}

// Captures the cycles of `ms` (members of `b`) as parallel branches of one graph.
hv_status capture_members(hv_server* s, Bucket* b, const std::vector<Member*>& ms, cudaGraphExec_t* exec,
                          size_t* kernels_out, bool own_blocks = false)
{
    *exec = nullptr;
    *kernels_out = 0;
    HV_CUDA_TRY(cudaStreamBeginCapture(s->capture_stream, cudaStreamCaptureModeThreadLocal));
    hv_status r = HV_OK;
    cudaError_t e = cudaEventRecord(s->fork_ev, s->capture_stream);
    for (size_t k = 0; k < ms.size() && e == cudaSuccess && r == HV_OK; ++k)
    {
        Member* m = ms[k];
        const size_t idx = std::find(b->members.begin(), b->members.end(), m) - b->members.begin();
        const CycleCtl* ctl = own_blocks ? m->ctl_dev : b->ctl_dev + idx;
        e = cudaStreamWaitEvent(s->branch[k], s->fork_ev, 0);
        if (e == cudaSuccess)
            r = served_record(m->p, ctl, ServedCycle{}, true, s->branch[k]);
        if (e == cudaSuccess && r == HV_OK)
            e = cudaEventRecord(s->join_ev[k], s->branch[k]);
        if (e == cudaSuccess)
            e = cudaStreamWaitEvent(s->capture_stream, s->join_ev[k], 0);
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(s->capture_stream, &graph);
    if (r != HV_OK || e != cudaSuccess || e2 != cudaSuccess)
    {
        if (graph)
            cudaGraphDestroy(graph);
        if (r == HV_OK)
        {
            set_last_error(cudaGetErrorString(e != cudaSuccess ? e : e2), __FILE__, __LINE__);
            r = HV_ERR_CUDA;
        }
        return r;
    }
    size_t nnodes = 0;
    cudaGraphGetNodes(graph, nullptr, &nnodes);
    std::vector<cudaGraphNode_t> nodes(nnodes);
    if (nnodes)
        cudaGraphGetNodes(graph, nodes.data(), &nnodes);
    size_t kernels = 0;
    for (cudaGraphNode_t n : nodes)
    {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(n, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
            ++kernels;
    }
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
    {
        *exec = nullptr;
        set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
        return HV_ERR_CUDA;
    }
    *kernels_out = kernels;
    ++s->captures;
    return HV_OK;
}

void drop_graphs(Bucket* b)
{
    if (b->exec)
    {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    b->graph_members.clear();
    b->graph_kernels = 0;
    for (Member* m : b->members)
        if (m->solo)
        {
            cudaGraphExecDestroy(m->solo);
            m->solo = nullptr;
        }
}

// (Re)captures the bucket graph over its steady members (one branch per member) and the solo
// graphs of steady members that have none.
hv_status capture_bucket(hv_server* s, Bucket* b)
{
    std::vector<Member*> steady;
    for (Member* m : b->members)
        if (m->steady)
            steady.push_back(m);
    HV_CUDA_TRY(cudaStreamSynchronize(b->stream));
    if (b->exec)
    {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    b->graph_members.clear();
    b->graph_kernels = 0;
    hv_status r;
    for (Member* m : steady)
        if (!m->solo && (r = capture_members(s, b, {m}, &m->solo, &m->solo_kernels)) != HV_OK)
            return r;
    if (steady.size() > 1 && (r = capture_members(s, b, steady, &b->exec, &b->graph_kernels)) != HV_OK)
        return r;
    b->graph_members = steady;
    return HV_OK;
}

// One engine pass over a bucket: plan, upload the control blocks, launch. A bucket whose steady
// streams are only partly ready waits up to batch_window_us (from its oldest ready batch) for the
// others; then the bucket graph is launched when at least half of them are ready, else the solo
// graphs of the ready ones. *wait_us receives the time left in a window that is still open.
hv_status run_bucket(hv_server* s, Bucket* b, bool* did_work, int64_t* wait_us)
{
    const size_t n = b->members.size();
    if (n == 0)
        return HV_OK;
    const bool use_graph = b->graphable && !(s->flags & HV_SERVER_NO_GRAPHS);
    if (use_graph)
    {
        size_t n_steady = 0, ready_steady = 0, ready_other = 0;
        int64_t oldest = INT64_MAX;
        for (Member* m : b->members)
        {
            std::lock_guard<std::mutex> g(m->p->mu);
            n_steady += m->steady ? 1 : 0;
            if (!m->p->ready.empty())
            {
                (m->steady ? ready_steady : ready_other) += 1;
                oldest = std::min(oldest, m->p->ready.front().t_push_us);
            }
        }
        if (ready_other == 0 && ready_steady > 0 && ready_steady < n_steady)
        {
            const int64_t left = oldest + s->batch_window_us - now_us();
            if (left > 0)
            {
                *wait_us = std::min(*wait_us, left);
                return HV_OK;
            }
        }
    }
    const int ci = b->ctl_i;
    CycleCtl* host = b->ctl_host + static_cast<size_t>(ci) * kMaxMembers;
    // the pinned buffer is reused after its previous upload finished
    HV_CUDA_TRY(cudaEventSynchronize(b->ctl_ev[ci]));
    std::vector<ServedCycle> cyc(n);
    bool any = false;
    for (size_t i = 0; i < n; ++i)
    {
        const bool planned = served_plan(b->members[i]->p, &host[i], &cyc[i]);
        if (!planned)
            cyc[i].in_slot = -1;
        any = any || planned;
    }
    if (!any)
        return HV_OK;
    *did_work = true;
    b->ctl_i = (ci + 1) % kCtlRing;
    HV_CUDA_TRY(cudaMemcpyAsync(b->ctl_dev, host, n * sizeof(CycleCtl), cudaMemcpyHostToDevice, b->stream));
    HV_CUDA_TRY(cudaEventRecord(b->ctl_ev[ci], b->stream));
    hv_status r;
    for (size_t i = 0; i < n; ++i)
        if (cyc[i].in_slot >= 0 && (r = served_prepare(b->members[i]->p, cyc[i], b->stream)) != HV_OK)
            return r;
    std::vector<char> launched(n, 0);
    if (use_graph)
    {
        std::vector<Member*> steady;
        for (Member* m : b->members)
            if (m->steady)
                steady.push_back(m);
        if (steady != b->graph_members && (r = capture_bucket(s, b)) != HV_OK)
            return r;
        size_t k = 0;
        for (size_t i = 0; i < n; ++i)
            k += (cyc[i].in_slot >= 0 && b->members[i]->steady) ? 1 : 0;
        if (k > 0 && b->exec && 2 * k >= steady.size())
        {
            HV_CUDA_TRY(cudaGraphLaunch(b->exec, b->stream));
            ++s->graph_launches;
            s->graph_kernels += b->graph_kernels;
            for (size_t i = 0; i < n; ++i)
                launched[i] = b->members[i]->steady ? 1 : 0;
        }
        else
        {
            for (size_t i = 0; i < n; ++i)
            {
                Member* m = b->members[i];
                if (cyc[i].in_slot >= 0 && m->steady && m->solo)
                {
                    HV_CUDA_TRY(cudaGraphLaunch(m->solo, b->stream));
                    ++s->graph_launches;
                    s->graph_kernels += m->solo_kernels;
                    launched[i] = 1;
                }
            }
        }
    }
    auto rec = std::make_unique<LatencyRecord>();
    rec->s = s;
    for (size_t i = 0; i < n; ++i)
    {
        if (cyc[i].in_slot < 0)
            continue;
        Member* m = b->members[i];
        if (!launched[i])
        {
            if ((r = served_record(m->p, b->ctl_dev + i, cyc[i], false, b->stream)) != HV_OK)
                return r;
            if (cyc[i].active)
                ++s->eager_cycles;
            if (cyc[i].render)
                m->steady = served_graphable(m->p);  // joins the graphs from the next pass
        }
        if ((r = served_complete(m->p, cyc[i], b->stream)) != HV_OK)
            return r;
        ++s->batches;
        if (cyc[i].render)
            rec->t_push.push_back(cyc[i].t_push_us);
    }
    if (!rec->t_push.empty())
    {
        HV_CUDA_TRY(cudaLaunchHostFunc(b->stream, record_latencies, rec.get()));
        rec.release();
    }
    return HV_OK;
}

// HV_SERVER_STREAM_GRAPHS: every stream runs on its own CUDA stream like independent Pipes (no
// barrier between the streams' cycles); per ready batch: the stream's control block is uploaded
// on its stream, then its own graph (steady) or its kernels (warm-up, PCA, unwrap) are launched.
hv_status run_bucket_streams(hv_server* s, Bucket* b, bool* did_work)
{
    hv_status r;
    for (Member* m : b->members)
    {
        CycleCtl* host = m->ctl_host + m->ctl_i;
        HV_CUDA_TRY(cudaEventSynchronize(m->ctl_ev[m->ctl_i]));
        ServedCycle cyc;
        if (!served_plan(m->p, host, &cyc))
            continue;
        *did_work = true;
        cudaStream_t st = m->own;
        HV_CUDA_TRY(cudaMemcpyAsync(m->ctl_dev, host, sizeof(CycleCtl), cudaMemcpyHostToDevice, st));
        HV_CUDA_TRY(cudaEventRecord(m->ctl_ev[m->ctl_i], st));
        m->ctl_i = (m->ctl_i + 1) % kCtlRing;
        if ((r = served_prepare(m->p, cyc, st)) != HV_OK)
            return r;
        const bool graph = b->graphable && !(s->flags & HV_SERVER_NO_GRAPHS);
        if (graph && m->steady && !m->solo && (r = capture_members(s, b, {m}, &m->solo, &m->solo_kernels, true)) != HV_OK)
            return r;
        if (graph && m->steady && m->solo)
        {
            HV_CUDA_TRY(cudaGraphLaunch(m->solo, st));
            ++s->graph_launches;
            s->graph_kernels += m->solo_kernels;
        }
        else
        {
            if ((r = served_record(m->p, m->ctl_dev, cyc, false, st)) != HV_OK)
                return r;
            if (cyc.active)
                ++s->eager_cycles;
            if (cyc.render)
                m->steady = served_graphable(m->p);
        }
        if ((r = served_complete(m->p, cyc, st)) != HV_OK)
            return r;
        ++s->batches;
        if (cyc.render)
        {
            auto rec = std::make_unique<LatencyRecord>();
            rec->s = s;
            rec->t_push.push_back(cyc.t_push_us);
            HV_CUDA_TRY(cudaLaunchHostFunc(st, record_latencies, rec.get()));
            rec.release();
        }
    }
    return HV_OK;
}

void engine_main(hv_server* s)
{
    uint64_t seen = 0;
    int64_t wait_us = 1000;
    while (!s->stop.load())
    {
        {
            std::unique_lock<std::mutex> lk(s->work_mu);
            s->work_cv.wait_for(lk, std::chrono::microseconds(std::max<int64_t>(20, wait_us)),
                                [&] { return s->work_seq != seen || s->stop.load(); });
            seen = s->work_seq;
        }
        // keep passing while any bucket found work (one batch per stream per pass)
        for (;;)
        {
            bool did = false;
            wait_us = 1000;
            s->idle = false;
            {
                std::lock_guard<std::mutex> g(s->mu);
                for (Bucket* b : s->buckets)
                {
                    const hv_status r = (s->flags & HV_SERVER_STREAM_GRAPHS) ? run_bucket_streams(s, b, &did)
                                                                             : run_bucket(s, b, &did, &wait_us);
                    if (r != HV_OK && s->engine_error == HV_OK)
                    {
                        s->engine_error = r;
                        s->engine_error_msg = hv_last_error();
                    }
                }
            }
            if (!did)
                break;
        }
        s->idle = wait_us >= 1000;
    }
}

Member* find_member(hv_server* s, int32_t id)
{
    std::lock_guard<std::mutex> g(s->map_mu);
    auto it = s->members.find(id);
    return it == s->members.end() ? nullptr : it->second;
}

}  // namespace

extern "C" {

size_t hv_server_stream_footprint(const hv_frame_desc* fd, const hv_settings* settings)
{
    if (!fd || !settings)
        return 0;
    hv_settings s = *settings;
    if (hv_settings_validate(&s, fd) != HV_OK)
        return 0;
    return served_footprint(*fd, s);
}

hv_server* hv_server_create(size_t hbm_budget_bytes, int flags, hv_status* status)
{
    hv_status dummy;
    hv_status& out = status ? *status : dummy;
    hv_server* s = new (std::nothrow) hv_server();
    if (!s)
    {
        out = HV_FAILURE;
        return nullptr;
    }
    s->flags = flags;
    if (hbm_budget_bytes == 0)
    {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess)
        {
            out = HV_ERR_CUDA;
            delete s;
            return nullptr;
        }
        hbm_budget_bytes = free_b / 10 * 9;
    }
    s->budget = hbm_budget_bytes;
    s->branch.resize(kMaxMembers, nullptr);
    s->join_ev.resize(kMaxMembers, nullptr);
    cudaError_t e = cudaStreamCreateWithFlags(&s->capture_stream, cudaStreamNonBlocking);
    for (int i = 0; i < kMaxMembers && e == cudaSuccess; ++i)
    {
        e = cudaStreamCreateWithFlags(&s->branch[i], cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&s->join_ev[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&s->fork_ev, cudaEventDisableTiming);
    if (e != cudaSuccess)
    {
        set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
        out = HV_ERR_CUDA;
        hv_server_destroy(s);
        return nullptr;
    }
    s->engine = std::thread(engine_main, s);
    out = HV_OK;
    return s;
}

void hv_server_destroy(hv_server* s)
{
    if (!s)
        return;
    s->stop = true;
    s->work_cv.notify_all();
    if (s->engine.joinable())
        s->engine.join();
    for (Bucket* b : s->buckets)
        cudaStreamSynchronize(b->stream);
    for (auto& kv : s->members)
    {
        if (kv.second->solo)
            cudaGraphExecDestroy(kv.second->solo);
        hv_pipe_destroy(kv.second->p);
        destroy_member_stream(kv.second);
        delete kv.second;
    }
    s->members.clear();
    for (Bucket* b : s->buckets)
        destroy_bucket(b);
    s->buckets.clear();
    for (cudaStream_t st : s->branch)
        if (st)
            cudaStreamDestroy(st);
    for (cudaEvent_t ev : s->join_ev)
        if (ev)
            cudaEventDestroy(ev);
    if (s->fork_ev)
        cudaEventDestroy(s->fork_ev);
    if (s->capture_stream)
        cudaStreamDestroy(s->capture_stream);
    delete s;
}

hv_status hv_server_open_stream(hv_server* s, const hv_frame_desc* fd, const hv_settings* settings,
                                int64_t admit_timeout_us, int32_t* stream_id)
{
    if (!s || !fd || !settings || !stream_id)
        return HV_INVALID_VALUE;
    hv_settings vs = *settings;
    hv_status r = hv_settings_validate(&vs, fd);
    if (r != HV_OK)
        return r;
    const size_t fp = served_footprint(*fd, vs);
    if (fp > s->budget)
    {
        set_last_error_msg("stream footprint exceeds the server's HBM budget");
        return HV_ERR_ADMISSION;
    }
    // admission: reserve the footprint, waiting (bounded) for closed streams to free memory
    {
        std::unique_lock<std::mutex> lk(s->mu);
        const auto deadline = std::chrono::steady_clock::now() + std::chrono::microseconds(std::max<int64_t>(0, admit_timeout_us));
        while (s->used + fp > s->budget)
        {
            if (admit_timeout_us <= 0 || s->admit_cv.wait_until(lk, deadline) == std::cv_status::timeout)
            {
                if (s->used + fp <= s->budget)
                    break;
                set_last_error_msg("not admitted: the server's HBM budget is in use");
                return HV_ERR_ADMISSION;
            }
        }
        s->used += fp;
    }
    // the bucket (created on first use, kept alive by `pending`) and the served pipe on its stream
    const std::string key = bucket_key(*fd, vs);
    Bucket* bucket = nullptr;
    {
        std::lock_guard<std::mutex> g(s->mu);
        for (Bucket* b : s->buckets)
            if (b->key == key && b->members.size() + b->pending < static_cast<size_t>(kMaxMembers))
            {
                bucket = b;
                break;
            }
        if (!bucket)
        {
            // the key fixes the time transformation; members whose own cycle is not fully gated
            // (unwrap, phase increase) never become steady and stay eager
            const bool graphable = vs.time_transformation != HV_TIME_PCA && vs.time_transformation != HV_TIME_SSA_STFT;
            if ((r = make_bucket(key, graphable, &bucket)) != HV_OK)
            {
                s->used -= fp;
                return r;
            }
            s->buckets.push_back(bucket);
        }
        ++bucket->pending;
    }
    Member* m = new (std::nothrow) Member();
    hv_pipe* p = nullptr;
    if (!m)
        r = HV_FAILURE;
    else if ((s->flags & HV_SERVER_STREAM_GRAPHS) && (r = make_member_stream(m)) != HV_OK)
    {
        delete m;
        m = nullptr;
    }
    if (m)
    {
        p = pipe_create_served(fd, &vs, m->own ? m->own : bucket->stream, notify_engine, s, &r);
        if (!p)
        {
            destroy_member_stream(m);
            delete m;
            m = nullptr;
        }
    }
    Bucket* drop = nullptr;
    {
        std::lock_guard<std::mutex> g(s->mu);
        --bucket->pending;
        if (m)
        {
            m->p = p;
            m->bucket = bucket;
            m->footprint = fp;
            m->id = s->next_id++;
            {
                std::lock_guard<std::mutex> g2(s->map_mu);
                s->members[m->id] = m;
            }
            bucket->members.push_back(m);
        }
        else
        {
            s->used -= fp;
            if (bucket->members.empty() && bucket->pending == 0)
            {
                s->buckets.erase(std::find(s->buckets.begin(), s->buckets.end(), bucket));
                drop = bucket;
            }
        }
    }
    if (!m)
    {
        if (drop)
            destroy_bucket(drop);
        s->admit_cv.notify_all();
        return r;
    }
    *stream_id = m->id;
    return HV_OK;
}

hv_status hv_server_close_stream(hv_server* s, int32_t id)
{
    if (!s)
        return HV_INVALID_VALUE;
    Member* m = nullptr;
    Bucket* empty_bucket = nullptr;
    {
        std::lock_guard<std::mutex> g(s->mu);
        {
            std::lock_guard<std::mutex> g2(s->map_mu);
            auto it = s->members.find(id);
            if (it == s->members.end())
                return HV_INVALID_VALUE;
            m = it->second;
            s->members.erase(it);
        }
        Bucket* b = m->bucket;
        b->members.erase(std::find(b->members.begin(), b->members.end(), m));
        // the graphs referenced this member's buffers and control-block indices: drop them
        // (recaptured on the next pass); per-stream graphs of the others use their own blocks
        cudaStreamSynchronize(b->stream);
        if (m->own)
            cudaStreamSynchronize(m->own);
        if (m->solo)
        {
            cudaGraphExecDestroy(m->solo);
            m->solo = nullptr;
        }
        if (!(s->flags & HV_SERVER_STREAM_GRAPHS))
            drop_graphs(b);
        if (b->members.empty() && b->pending == 0)
        {
            s->buckets.erase(std::find(s->buckets.begin(), s->buckets.end(), b));
            empty_bucket = b;
        }
    }
    // the pipe synchronises the bucket's stream: destroy it while the stream exists
    hv_pipe_destroy(m->p);
    destroy_member_stream(m);
    if (empty_bucket)
        destroy_bucket(empty_bucket);
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->used -= m->footprint;
    }
    delete m;
    s->admit_cv.notify_all();
    return HV_OK;
}

hv_status hv_server_push(hv_server* s, int32_t id, const void* frames, size_t n, int mem)
{
    if (!s)
        return HV_INVALID_VALUE;
    if (s->engine_error != HV_OK)
    {
        set_last_error_msg(s->engine_error_msg.c_str());
        return s->engine_error;
    }
    Member* m = find_member(s, id);
    if (!m)
        return HV_INVALID_VALUE;
    return hv_pipe_push_frames(m->p, frames, n, mem);
}

size_t hv_server_output_count(hv_server* s, int32_t id)
{
    Member* m = s ? find_member(s, id) : nullptr;
    return m ? hv_pipe_output_count(m->p) : 0;
}

hv_status hv_server_pull(hv_server* s, int32_t id, uint16_t* dst, int mem, int64_t timeout_us)
{
    Member* m = s ? find_member(s, id) : nullptr;
    if (!m)
        return HV_INVALID_VALUE;
    // outputs appear when the engine plans their cycle: wait (bounded) for one
    const int64_t t0 = now_us();
    while (hv_pipe_output_count(m->p) == 0)
    {
        if (s->engine_error != HV_OK)
            return s->engine_error;
        if (timeout_us >= 0 && now_us() - t0 > timeout_us)
            return HV_ERR_TIMEOUT;
        std::this_thread::sleep_for(std::chrono::microseconds(10));
    }
    const int64_t left = timeout_us < 0 ? -1 : std::max<int64_t>(0, timeout_us - (now_us() - t0));
    return hv_pipe_pull_output(m->p, dst, mem, left);
}

hv_status hv_server_get_float_frame(hv_server* s, int32_t id, float* dst)
{
    Member* m = s ? find_member(s, id) : nullptr;
    if (!m)
        return HV_INVALID_VALUE;
    return hv_pipe_get_float_frame(m->p, dst);
}

hv_status hv_server_sync(hv_server* s, int64_t timeout_us)
{
    if (!s)
        return HV_INVALID_VALUE;
    const int64_t t0 = now_us();
    for (;;)
    {
        bool pending = false;
        {
            std::lock_guard<std::mutex> g(s->mu);
            for (auto& kv : s->members)
            {
                std::lock_guard<std::mutex> g2(kv.second->p->mu);
                pending = pending || !kv.second->p->ready.empty();
            }
        }
        if (!pending && s->idle.load())
            break;
        if (s->engine_error != HV_OK)
            return s->engine_error;
        if (timeout_us >= 0 && now_us() - t0 > timeout_us)
            return HV_ERR_TIMEOUT;
        notify_engine(s);
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    std::lock_guard<std::mutex> g(s->mu);
    for (Bucket* b : s->buckets)
    {
        HV_CUDA_TRY(cudaStreamSynchronize(b->stream));
        for (Member* m : b->members)
            if (m->own)
                HV_CUDA_TRY(cudaStreamSynchronize(m->own));
    }
    return s->engine_error;
}

hv_status hv_server_get_stats(hv_server* s, hv_server_stats* out)
{
    if (!s || !out)
        return HV_INVALID_VALUE;
    std::memset(out, 0, sizeof(*out));
    out->batches = s->batches.load();
    out->outputs = s->outputs.load();
    out->graph_launches = s->graph_launches.load();
    out->graph_kernels = s->graph_kernels.load();
    out->eager_cycles = s->eager_cycles.load();
    out->captures = s->captures.load();
    std::vector<int64_t> lat;
    {
        std::lock_guard<std::mutex> g(s->lat_mu);
        lat = s->latencies;
    }
    if (!lat.empty())
    {
        auto pct = [&](double q) {
            const size_t k = std::min(lat.size() - 1, static_cast<size_t>(q * static_cast<double>(lat.size() - 1) + 0.5));
            std::nth_element(lat.begin(), lat.begin() + static_cast<std::ptrdiff_t>(k), lat.end());
            return static_cast<double>(lat[k]);
        };
        out->latency_p50_us = pct(0.50);
        out->latency_p99_us = pct(0.99);
        out->latency_samples = lat.size();
    }
    std::lock_guard<std::mutex> g(s->mu);
    out->streams = static_cast<int32_t>(s->members.size());
    out->buckets = static_cast<int32_t>(s->buckets.size());
    out->hbm_used = s->used;
    out->hbm_budget = s->budget;
    return s->engine_error;
}

hv_status hv_server_set_batch_window(hv_server* s, int64_t window_us)
{
    if (!s || window_us < 0)
        return HV_INVALID_VALUE;
    s->batch_window_us = window_us;
    return HV_OK;
}

hv_status hv_server_reset_stats(hv_server* s)
{
    if (!s)
        return HV_INVALID_VALUE;
    std::lock_guard<std::mutex> g(s->lat_mu);
    s->latencies.clear();
    s->lat_next = 0;
    return HV_OK;
}

}  // extern "C"
