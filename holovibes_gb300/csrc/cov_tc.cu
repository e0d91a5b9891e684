// PCA covariance on the 5th-generation tensor cores (tcgen05, TMEM accumulator), split-BF16.
//
// Reference: cov = H^H H with cublasCgemm3m (Backend/sources/compute/matrix_operations.cc:9-26),
// H the HW x T column-major view of the time ring.
//
// Formulation: Y is the 2T x HW real matrix with rows 2t = Re(ring[t]) and 2t+1 = Im(ring[t]);
// G = Y Y^T (2T x 2T) gives C_re[i][j] = G[2i][2j] + G[2i+1][2j+1] and
// C_im[i][j] = G[2i][2j+1] - G[2i+1][2j]. Each FP32 sample is split y = yh + yl with yh, yl in
// BF16, and G ~= Yh Yh^T + Yh Yl^T + Yl Yh^T (the Yl Yl^T term is below FP32 resolution), so
// three BF16 MMAs with FP32 accumulation per K step recover ~16-bit-mantissa accuracy.
//
// Kernel: one CTA per SM-slot walks a contiguous range of 64-pixel chunks. All warps load a chunk
// (coalesced float2), split it and write Yh / Yl into shared memory in the no-swizzle K-major
// canonical layout (8-row x 16-byte core matrices); one thread issues the MMAs
// (M = 128 rows of Y, rows >= 2T are zero; N = 2T rounded to 16; K = 16) into a TMEM
// accumulator; tcgen05.commit signals an mbarrier per buffer so loads of chunk c+2 wait only
// for the MMAs of chunk c (two buffers). Every wait is bounded and reports through an error flag.
// Per-CTA partial G tiles are summed in FP64 by k_cov_tc_reduce.
#include <cuda_bf16.h>

#include "hv_common.cuh"
#include "hv_internal.h"
#include "tc_common.cuh"

namespace hv {

namespace {

constexpr int TC_PRODUCERS = 256;            // 8 producer warps
constexpr int TC_MMA_WARP = TC_PRODUCERS / 32;  // warp 8 issues the MMAs
constexpr int TC_THREADS = TC_PRODUCERS + 32;
constexpr int TC_STAGES = 3;
constexpr int TC_KC = 64;           // pixels (K elements) per chunk
constexpr int TC_ROWS = 128;        // M rows of the operand tile (2T <= 128, zero padded)
constexpr int TILE_BYTES = TC_ROWS * TC_KC * 2;  // one BF16 tile: 16 KB
using tc::fence_async_smem;
using tc::mbar_arrive;
using tc::mbar_init;
using tc::mbar_wait;
using tc::mma_bf16;
using tc::mma_commit;
using tc::smem_u32;
using tc::tmem_ld16;
__device__ __forceinline__ void tc_fence_before() { tc::fence_before(); }
__device__ __forceinline__ void tc_fence_after() { tc::fence_after(); }
__device__ __forceinline__ uint32_t tile_offset(int r, int kgroup) { return tc::sw128_offset(r, kgroup); }
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) { return tc::sw128_desc(addr); }
using tc::instr_desc;

// part: [gridDim.x][2T][2T] FP32 partial G; err: set to 1 when a bounded wait gave up.
// Warps 0-7 produce (load with one chunk of register prefetch, split to BF16 hi/lo, store the
// canonical tiles of stage it % TC_STAGES, arrive on full[s]); warp 8 lane 0 consumes (wait
// full[s], 12 MMAs, commit to empty[s]); after the last chunk a commit to `done` releases the
// epilogue (warps 0-3 read the TMEM accumulator lanes 32w..32w+31).
__global__ void __launch_bounds__(TC_THREADS) k_cov_tc(const float2* __restrict__ ring, int T, size_t npix,
                                                       size_t chunks_per_cta, int N, uint32_t tmem_cols,
                                                       float* __restrict__ part, int* __restrict__ err)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    // [stage][hi/lo] tiles on a 1024-byte boundary (the swizzle atom); the launch adds 1 KB of slack
    uint8_t* tiles = smem + ((1024u - (smem_u32(smem) & 1023u)) & 1023u);
    __shared__ __align__(8) uint64_t full[TC_STAGES];
    __shared__ __align__(8) uint64_t empty[TC_STAGES];
    __shared__ __align__(8) uint64_t done;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int rows = 2 * T;
    const size_t nchunks = (npix + TC_KC - 1) / TC_KC;
    const size_t c_begin = blockIdx.x * chunks_per_cta;
    size_t c_end = c_begin + chunks_per_cta;
    if (c_end > nchunks)
        c_end = nchunks;
    const size_t nmine = c_end > c_begin ? c_end - c_begin : 0;

    // zero all tiles once (rows >= 2T stay zero)
    for (int i = tid; i < TC_STAGES * 2 * TILE_BYTES / 16; i += TC_THREADS)
        reinterpret_cast<uint4*>(tiles)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0)
    {
        for (int s2 = 0; s2 < TC_STAGES; ++s2)
        {
            mbar_init(&full[s2], TC_PRODUCERS / 32);  // one arrival per producer warp
            mbar_init(&empty[s2], 1);
        }
        mbar_init(&done, 1);
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == TC_MMA_WARP)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    bool fail = false;

    if (warp < TC_MMA_WARP)
    {
        // ------------------------------------------------------------------ producers
        const int items = T * (TC_KC / 8);  // T rows x 8 k-groups of 8 pixels; <= 2 per thread (T <= 64)
        float2 nxt[2][8];
        auto load_chunk = [&](size_t c) {
            const size_t p0 = c * TC_KC;
#pragma unroll
            for (int q = 0; q < 2; ++q)
            {
                const int w = tid + q * TC_PRODUCERS;
                if (w >= items)
                    continue;
                const int g = w & 7, t = w >> 3;  // 8 threads read one frame's 512 contiguous bytes
                const size_t p = p0 + static_cast<size_t>(g) * 8;
                const float2* src = ring + static_cast<size_t>(t) * npix + p;
                if (p + 8 <= npix)
                {
                    const float4* s4 = reinterpret_cast<const float4*>(src);
#pragma unroll
                    for (int h = 0; h < 4; ++h)
                    {
                        const float4 f = __ldcs(s4 + h);
                        nxt[q][2 * h] = make_float2(f.x, f.y);
                        nxt[q][2 * h + 1] = make_float2(f.z, f.w);
                    }
                }
                else
                {
#pragma unroll
                    for (int h = 0; h < 8; ++h)
                        nxt[q][h] = (p + h < npix) ? __ldg(src + h) : make_float2(0.f, 0.f);
                }
            }
        };
        if (nmine)
            load_chunk(c_begin);
        for (size_t it = 0; it < nmine; ++it)
        {
            const int st = static_cast<int>(it % TC_STAGES);
            const size_t use = it / TC_STAGES;
            float2 cur[2][8];
#pragma unroll
            for (int q = 0; q < 2; ++q)
#pragma unroll
                for (int h = 0; h < 8; ++h)
                    cur[q][h] = nxt[q][h];
            if (it + 1 < nmine)
                load_chunk(c_begin + it + 1);
            if (use >= 1 && !mbar_wait(&empty[st], static_cast<uint32_t>((use - 1) & 1)))
                fail = true;
            uint8_t* th = tiles + st * 2 * TILE_BYTES;
            uint8_t* tl = th + TILE_BYTES;
#pragma unroll
            for (int q = 0; q < 2; ++q)
            {
                const int w = tid + q * TC_PRODUCERS;
                if (w >= items)
                    continue;
                const int g = w & 7, t = w >> 3;
                const float2* v = cur[q];
                uint32_t rh[4], rl[4], ih[4], il[4];
#pragma unroll
                for (int h = 0; h < 4; ++h)
                {
                    tc::split2(v[2 * h].x, v[2 * h + 1].x, rh[h], rl[h]);
                    tc::split2(v[2 * h].y, v[2 * h + 1].y, ih[h], il[h]);
                }
                const uint32_t ore = tile_offset(2 * t, g), oim = tile_offset(2 * t + 1, g);
                *reinterpret_cast<uint4*>(th + ore) = make_uint4(rh[0], rh[1], rh[2], rh[3]);
                *reinterpret_cast<uint4*>(th + oim) = make_uint4(ih[0], ih[1], ih[2], ih[3]);
                *reinterpret_cast<uint4*>(tl + ore) = make_uint4(rl[0], rl[1], rl[2], rl[3]);
                *reinterpret_cast<uint4*>(tl + oim) = make_uint4(il[0], il[1], il[2], il[3]);
            }
            fence_async_smem();
            __syncwarp();
            if (lane == 0)
                mbar_arrive(&full[st]);
        }
    }
    else if (lane == 0)
    {
        // ------------------------------------------------------------------ MMA issuer
        const uint32_t idesc = instr_desc(TC_ROWS, N);
        for (size_t it = 0; it < nmine; ++it)
        {
            const int st = static_cast<int>(it % TC_STAGES);
            if (!mbar_wait(&full[st], static_cast<uint32_t>((it / TC_STAGES) & 1)))
                fail = true;
            tc_fence_after();
            const uint32_t ah = smem_u32(tiles + st * 2 * TILE_BYTES), al = ah + TILE_BYTES;
#pragma unroll
            for (int s2 = 0; s2 < TC_KC / 16; ++s2)
            {
                const uint64_t dh = smem_desc(ah + s2 * 32), dl = smem_desc(al + s2 * 32);
                mma_bf16(tmem, dh, dh, idesc, (it > 0 || s2 > 0) ? 1u : 0u);  // Yh Yh^T
                mma_bf16(tmem, dh, dl, idesc, 1u);                            // Yh Yl^T
                mma_bf16(tmem, dl, dh, idesc, 1u);                            // Yl Yh^T
            }
            mma_commit(&empty[st]);
        }
        mma_commit(&done);
    }
    // epilogue: wait for the last MMAs, warps 0-3 read row r = 32w + lane of G, columns 0..N-1
    if (warp < 4)
    {
        if (!mbar_wait(&done, 0))
            fail = true;
        tc_fence_after();
        const int r = warp * 32 + lane;
        float* dst = part + static_cast<size_t>(blockIdx.x) * rows * rows;
        for (int c0 = 0; c0 < N; c0 += 16)
        {
            float v[16];
            const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c0);
            tmem_ld16(taddr, v);
            if (r < rows)
            {
#pragma unroll
                for (int i = 0; i < 16; ++i)
                    if (c0 + i < rows)
                        dst[static_cast<size_t>(r) * rows + c0 + i] = nmine ? v[i] : 0.f;
            }
        }
    }
    if (fail)
        atomicExch(&s_fail, 1);
    tc_fence_before();
    __syncthreads();
    if (warp == TC_MMA_WARP)
    {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols) : "memory");
    }
    if (tid == 0 && s_fail)
        atomicExch(err, 1);
}

// cov[i][j] (complex128, row-major, both triangles, zeroed before) += a slice of the FP32
// partial G tiles, summed in FP64.
__global__ void k_cov_tc_reduce(const float* __restrict__ part, int T, int nparts, int per_slice,
                                double2* __restrict__ cov)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= T * T)
        return;
    // the upper triangle is summed and mirrored, so the result is exactly Hermitian
    const int ei = e / T, ej = e % T;
    const bool mirror = ei > ej;
    const int i = mirror ? ej : ei, j = mirror ? ei : ej;
    const int R = 2 * T;
    double g00 = 0, g11 = 0, g01 = 0, g10 = 0;
    const int c0 = blockIdx.y * per_slice;
    const int c1 = min(nparts, c0 + per_slice);
#pragma unroll 4
    for (int c = c0; c < c1; ++c)
    {
        const float* G = part + static_cast<size_t>(c) * R * R;
        g00 += G[(2 * i) * R + 2 * j];
        g11 += G[(2 * i + 1) * R + 2 * j + 1];
        g01 += G[(2 * i) * R + 2 * j + 1];
        g10 += G[(2 * i + 1) * R + 2 * j];
    }
    atomicAdd(&cov[e].x, g00 + g11);
    if (i != j)
        atomicAdd(&cov[e].y, mirror ? -(g01 - g10) : (g01 - g10));
}

struct TcPlan
{
    int ctas;
    size_t chunks_per_cta;
    int N;
    uint32_t cols;
};

TcPlan tc_plan(int T, size_t npix)
{
    TcPlan p;
    const size_t nchunks = (npix + TC_KC - 1) / TC_KC;
    int ctas = 152 * 2;
    if (static_cast<size_t>(ctas) > nchunks)
        ctas = static_cast<int>(nchunks);
    if (ctas < 1)
        ctas = 1;
    p.chunks_per_cta = (nchunks + ctas - 1) / ctas;
    p.ctas = static_cast<int>((nchunks + p.chunks_per_cta - 1) / p.chunks_per_cta);
    p.N = (2 * T + 15) / 16 * 16;
    uint32_t cols = 32;
    while (cols < static_cast<uint32_t>(p.N))
        cols <<= 1;
    p.cols = cols;
    return p;
}

}  // namespace

bool cov_tc_supported(int T) { return T >= 1 && 2 * T <= TC_ROWS; }

size_t cov_tc_workspace(int T, size_t npix)
{
    const TcPlan p = tc_plan(T, npix);
    return static_cast<size_t>(p.ctas) * 4 * T * T * sizeof(float) + 256;
}

hv_status cov_tc(const float2* ring, int T, size_t npix, double2* cov, void* work, int* err, cudaStream_t st)
{
    if (!cov_tc_supported(T) || npix == 0)
        return HV_ERR_UNSUPPORTED;
    if (npix % 8 != 0 || (reinterpret_cast<uintptr_t>(ring) & 15) != 0)
    {
        set_last_error_msg("tensor-core covariance needs 16-byte aligned frames of a multiple of 8 pixels");
        return HV_ERR_UNSUPPORTED;
    }
    const TcPlan p = tc_plan(T, npix);
    const size_t smem = static_cast<size_t>(TC_STAGES) * 2 * TILE_BYTES + 1024;
    HV_CUDA_TRY(cudaFuncSetAttribute(k_cov_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    float* part = static_cast<float*>(work);
    k_cov_tc<<<p.ctas, TC_THREADS, smem, st>>>(ring, T, npix, p.chunks_per_cta, p.N, p.cols, part, err);
    HV_LAUNCH_CHECK();
    const int slices = p.ctas < 16 ? p.ctas : 16;
    const int per = (p.ctas + slices - 1) / slices;
    k_cov_tc_reduce<<<dim3((T * T + 255) / 256, (p.ctas + per - 1) / per), 256, 0, st>>>(part, T, p.ctas, per, cov);
    HV_LAUNCH_CHECK();
    count_launch(2);
    return HV_OK;
}

}  // namespace hv
