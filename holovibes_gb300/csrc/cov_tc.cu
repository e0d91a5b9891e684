// PCA covariance on the 5th-generation tensor cores (tcgen05, TMEM accumulator), split-BF16.
//
// Reference: cov = H^H H with cublasCgemm3m (Backend/sources/compute/matrix_operations.cc:9-26),
// H the HW x T column-major view of the time ring.
//
// Formulation: Y is the 2T x HW real matrix with rows 2t = Re(ring[t]) and 2t+1 = Im(ring[t]);
// G = Y Y^T (2T x 2T) gives C_re[i][j] = G[2i][2j] + G[2i+1][2j+1] and
// C_im[i][j] = G[2i][2j+1] - G[2i+1][2j]. Each FP32 sample is split y = yh + yl with yh, yl in
// BF16, and G ~= Yh Yh^T + Yh Yl^T + Yl Yh^T (+ Yl Yl^T where it is free: the packed form for
// 2T <= 64), so three (four) BF16 MMAs with FP32 accumulation per K step recover ~16-bit-mantissa
// accuracy.
//
// Kernel: one CTA per SM walks a contiguous range of 64-pixel chunks (K slices of Y):
//   warp 17    loader: one 2-D tensor copy (TMA) per pair of chunks (T x 128 complex samples, rows
//              of 1 KB) into a ring of R raw stages (zero fill past the frame)
//   warps 0-15 converters: raw samples -> Yh / Yl tiles of an A stage (128-byte-swizzled K-major,
//              rows >= 2T stay zero), each warp releasing its part of the raw and A stages
//   warp 16    MMA issuer (M = 128 rows of Y, N = 2T rounded to 16, K = 16) into three TMEM
//              accumulators (Yh Yh^T, Yh Yl^T, Yl Yh^T: independent chains, summed by the
//              epilogue), tcgen05.commit frees the A stage; after the last chunk a commit to
//              `done` releases the epilogue (warps 0-3 read the accumulator lanes 32w..32w+31)
// Every wait is bounded in time and reports through the error flag. Per-CTA partial G tiles are
// summed in FP64 by k_cov_tc_reduce.
#include <algorithm>
#include <cstring>
#include <cuda_bf16.h>

#include "hv_common.cuh"
#include "hv_internal.h"
#include "tc_common.cuh"

namespace hv {

namespace {

constexpr int TC_CONVERTERS = 256;              // warps 0-7
constexpr int TC_MMA_WARP = TC_CONVERTERS / 32;  // warp 8 issues the MMAs
constexpr int TC_LOAD_WARP = TC_MMA_WARP + 1;    // warp 9 issues the tensor copies
constexpr int TC_THREADS = TC_CONVERTERS + 64;
constexpr int TC_A_STAGES = 2;
constexpr int TC_A_STAGES_PACKED = 2;
constexpr int TC_MAX_RAW = 8;
constexpr int TC_KC = 64;           // pixels (K elements) per chunk
constexpr int TC_ROWS = 128;        // M rows of the operand tile (2T <= 128, zero padded)
constexpr int TILE_BYTES = TC_ROWS * TC_KC * 2;  // one BF16 tile: 16 KB
constexpr int COV_TC_MAX_T = 1024;               // tiled kernel: (T / 64)^2 / 2 tiles of 128 x 128
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
__global__ void __launch_bounds__(TC_THREADS, 2) k_cov_tc(const __grid_constant__ CUtensorMap ring_map, int T,
                                                          size_t npix, size_t chunks_per_cta, int N, uint32_t tmem_cols,
                                                          int raw_stages, int packed, float* __restrict__ part,
                                                          int* __restrict__ err)
{
    // packed (2T <= 64): one 128-row tile per stage, Yh in rows 0..63 and Yl in rows 64..127, and
    // one 128 x 128 MMA per K step gives [[Yh Yh^T, Yh Yl^T], [Yl Yh^T, Yl Yl^T]];
    // otherwise two tiles (Yh, Yl) and three MMAs into three accumulators
    const int A_STAGES = packed ? TC_A_STAGES_PACKED : TC_A_STAGES;
    const uint32_t a_stage_bytes = packed ? TILE_BYTES : 2 * TILE_BYTES;
    extern __shared__ __align__(1024) uint8_t smem[];
    // A stages ([hi | lo] tiles) then the raw stages, on 1024-byte boundaries; 1 KB of launch slack
    uint8_t* tiles = smem + ((1024u - (smem_u32(smem) & 1023u)) & 1023u);
    const uint32_t raw_bytes = static_cast<uint32_t>(T) * TC_KC * 16;  // a pair of chunks: T rows of 1 KB
    uint8_t* raw_base = tiles + A_STAGES * a_stage_bytes;
    __shared__ __align__(8) uint64_t raw_full[TC_MAX_RAW], raw_empty[TC_MAX_RAW];
    __shared__ __align__(8) uint64_t a_full[TC_A_STAGES_PACKED], a_empty[TC_A_STAGES_PACKED];
    __shared__ __align__(8) uint64_t done, drain;
    __shared__ uint32_t tmem_base;
    __shared__ int s_abort;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int rows = 2 * T, R = raw_stages;
    const size_t nchunks = (npix + TC_KC - 1) / TC_KC;
    const size_t c_begin = blockIdx.x * chunks_per_cta;
    size_t c_end = c_begin + chunks_per_cta;
    if (c_end > nchunks)
        c_end = nchunks;
    const int nmine = static_cast<int>(c_end > c_begin ? c_end - c_begin : 0);
    volatile int* abort = &s_abort;

    // zero the A tiles once (rows >= 2T stay zero)
    for (int i = tid; i < A_STAGES * static_cast<int>(a_stage_bytes) / 16; i += TC_THREADS)
        reinterpret_cast<uint4*>(tiles)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0)
    {
        for (int i = 0; i < R; ++i)
        {
            mbar_init(&raw_full[i], 1);
            mbar_init(&raw_empty[i], TC_CONVERTERS / 32);
        }
        for (int i = 0; i < A_STAGES; ++i)
        {
            mbar_init(&a_full[i], TC_CONVERTERS / 32);
            mbar_init(&a_empty[i], 1);
        }
        mbar_init(&done, 1);
        mbar_init(&drain, 1);
        s_abort = 0;
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

    if (warp == TC_LOAD_WARP)
    {
        // ------------------------------------------------------------------ loader (TMA)
        if (lane == 0)
        {
            asm volatile("prefetch.tensormap [%0];" ::"l"(&ring_map) : "memory");
            const int npairs = (nmine + 1) / 2;
            for (int m = 0; m < npairs; ++m)
            {
                const int r = m % R;
                if (m >= R)
                    mbar_wait(&raw_empty[r], static_cast<uint32_t>(((m / R) - 1) & 1), abort);
                tc::mbar_arrive_expect_tx(&raw_full[r], raw_bytes);
                tc::tma_load_2d(raw_base + r * raw_bytes, &ring_map, static_cast<int>(2 * TC_KC * (c_begin + 2 * m)), 0,
                                &raw_full[r]);
            }
        }
        __syncwarp();
    }
    else if (warp < TC_MMA_WARP)
    {
        // ------------------------------------------------------------------ converters
        // one raw row (frame t: 64 complex samples, 512 B) per warp iteration: lane l reads 16 B
        // (pixels 2l, 2l+1), splits Re and Im into BF16 hi / lo pairs and writes 32-bit words
        // j = l & 3 of chunk g = l >> 2 in rows 2t (Re) and 2t+1 (Im): conflict-free reads and writes
        for (int it = 0; it < nmine; ++it)
        {
            const int m = it >> 1, half = it & 1;  // chunk it is half `half` of raw pair m
            const int r = m % R, st = it % A_STAGES;
            if (half == 0)
                mbar_wait(&raw_full[r], static_cast<uint32_t>((m / R) & 1), abort);
            if (it >= A_STAGES)
                mbar_wait(&a_empty[st], static_cast<uint32_t>(((it / A_STAGES) - 1) & 1), abort);
            const uint8_t* raw = raw_base + r * raw_bytes + half * (TC_KC * 8);
            uint8_t* th = tiles + st * a_stage_bytes;
            uint8_t* tl = packed ? th : th + TILE_BYTES;
            const int lo_row = packed ? 64 : 0;  // Yl rows: 64.. of the same tile, or the lo tile
            const int g = lane >> 2;
            const uint32_t j4 = static_cast<uint32_t>(lane & 3) * 4u;
            for (int t = warp; t < T; t += TC_CONVERTERS / 32)
            {
                const float4 f = reinterpret_cast<const float4*>(raw + t * (TC_KC * 16))[lane];
                uint32_t reh, rel, imh, iml;
                tc::split2(f.x, f.z, reh, rel);
                tc::split2(f.y, f.w, imh, iml);
                const uint32_t ore = tile_offset(2 * t, g) + j4, oim = tile_offset(2 * t + 1, g) + j4;
                const uint32_t lre = tile_offset(lo_row + 2 * t, g) + j4, lim = tile_offset(lo_row + 2 * t + 1, g) + j4;
                *reinterpret_cast<uint32_t*>(th + ore) = reh;
                *reinterpret_cast<uint32_t*>(th + oim) = imh;
                *reinterpret_cast<uint32_t*>(tl + lre) = rel;
                *reinterpret_cast<uint32_t*>(tl + lim) = iml;
            }
            fence_async_smem();
            __syncwarp();
            if (lane == 0)
            {
                if (half == 1 || it == nmine - 1)
                    mbar_arrive(&raw_empty[r]);  // both halves of the pair converted
                mbar_arrive(&a_full[st]);
            }
        }
    }
    else if (lane == 0)
    {
        // ------------------------------------------------------------------ MMA issuer
        const uint32_t idesc = instr_desc(TC_ROWS, packed ? TC_ROWS : N);
        for (int it = 0; it < nmine; ++it)
        {
            const int st = it % A_STAGES;
            mbar_wait(&a_full[st], static_cast<uint32_t>((it / A_STAGES) & 1), abort);
            tc_fence_after();
            const uint32_t ah = smem_u32(tiles + st * a_stage_bytes), al = ah + TILE_BYTES;
            if (packed)
            {
#pragma unroll
                for (int s2 = 0; s2 < TC_KC / 16; ++s2)
                {
                    const uint64_t d = smem_desc(ah + s2 * 32);
                    mma_bf16(tmem, d, d, idesc, (it > 0 || s2 > 0) ? 1u : 0u);  // [Yh; Yl] [Yh; Yl]^T
                }
                mma_commit(&a_empty[st]);
                continue;
            }
#pragma unroll
            for (int s2 = 0; s2 < TC_KC / 16; ++s2)
            {
                const uint64_t dh = smem_desc(ah + s2 * 32), dl = smem_desc(al + s2 * 32);
                const uint32_t acc = (it > 0 || s2 > 0) ? 1u : 0u;
                // three independent accumulator chains (consecutive MMAs do not wait on each other)
                mma_bf16(tmem, dh, dh, idesc, acc);                                      // Yh Yh^T
                mma_bf16(tmem + static_cast<uint32_t>(N), dh, dl, idesc, acc);           // Yh Yl^T
                mma_bf16(tmem + static_cast<uint32_t>(2 * N), dl, dh, idesc, acc);       // Yl Yh^T
            }
            mma_commit(&a_empty[st]);
        }
        mma_commit(&done);
    }
    // epilogue: wait for the last MMAs, warps 0-3 read row r = 32w + lane of G, columns 0..N-1
    if (warp < 4)
    {
        mbar_wait(&done, 0, abort);
        tc_fence_after();
        const int r = warp * 32 + lane;
        if (packed)
        {
            // partial layout [128][64]: row i < 64 holds Yh Yh^T + Yh Yl^T, row 64 + i holds
            // Yl Yh^T + Yl Yl^T (the packed MMA computes all four blocks, so the fourth product
            // costs nothing here: with it, samples whose hi + lo split is exact, such as integer
            // camera values below 2^16, give exact products before the FP32 accumulation)
            float* dstp = part + static_cast<size_t>(blockIdx.x) * TC_ROWS * 64 + static_cast<size_t>(r) * 64;
            for (int c0 = 0; c0 < 64; c0 += 16)
            {
                float v[16], w1[16];
                const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c0);
                tmem_ld16(taddr, v);
                tmem_ld16(taddr + 64u, w1);
#pragma unroll
                for (int i = 0; i < 16; ++i)
                {
                    v[i] += w1[i];
                    dstp[c0 + i] = nmine ? v[i] : 0.f;
                }
            }
        }
        float* dst = part + static_cast<size_t>(blockIdx.x) * rows * rows;
        for (int c0 = 0; c0 < (packed ? 0 : N); c0 += 16)
        {
            float v[16], w1[16], w2[16];
            const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c0);
            tmem_ld16(taddr, v);
            tmem_ld16(taddr + static_cast<uint32_t>(N), w1);
            tmem_ld16(taddr + static_cast<uint32_t>(2 * N), w2);
#pragma unroll
            for (int i = 0; i < 16; ++i)
                v[i] += w1[i] + w2[i];
            if (r < rows)
            {
#pragma unroll
                for (int i = 0; i < 16; ++i)
                    if (c0 + i < rows)
                        dst[static_cast<size_t>(r) * rows + c0 + i] = nmine ? v[i] : 0.f;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (s_abort)
    {
        // a wait gave up: let the copies and MMAs already issued finish before shared and tensor
        // memory are released (bounded waits)
        if (warp == TC_LOAD_WARP && lane == 0)
        {
            const int npairs = (nmine + 1) / 2;
            for (int m = npairs - R > 0 ? npairs - R : 0; m < npairs; ++m)
                mbar_wait(&raw_full[m % R], static_cast<uint32_t>((m / R) & 1));
            atomicExch(err, 1);
        }
        if (warp == TC_MMA_WARP && lane == 0)
        {
            mma_commit(&drain);
            mbar_wait(&drain, 0);
        }
        __syncthreads();
    }
    if (warp == TC_MMA_WARP)
    {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tmem_cols) : "memory");
    }
}

// cov[i][j] (complex128, row-major, both triangles, zeroed before) += a slice of the FP32
// partial G tiles, summed in FP64.
__device__ __forceinline__ float cov_g(const float* P, int R, int packed, int a, int b)
{
    // element (a, b) of G from one CTA's partial: packed [128][64] rows a and 64 + a, else [R][R]
    return packed ? P[a * 64 + b] + P[(64 + a) * 64 + b] : P[a * R + b];
}

__global__ void k_cov_tc_reduce(const float* __restrict__ part, int T, int nparts, int per_slice, int packed,
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
    const size_t stride = packed ? static_cast<size_t>(TC_ROWS) * 64 : static_cast<size_t>(R) * R;
#pragma unroll 4
    for (int c = c0; c < c1; ++c)
    {
        const float* G = part + static_cast<size_t>(c) * stride;
        g00 += cov_g(G, R, packed, 2 * i, 2 * j);
        g11 += cov_g(G, R, packed, 2 * i + 1, 2 * j + 1);
        g01 += cov_g(G, R, packed, 2 * i, 2 * j + 1);
        g10 += cov_g(G, R, packed, 2 * i + 1, 2 * j);
    }
    atomicAdd(&cov[e].x, g00 + g11);
    if (i != j)
        atomicAdd(&cov[e].y, mirror ? -(g01 - g10) : (g01 - g10));
}

int sm_count();

// ------------------------------------------------------------------------------ tiled (T > 64)
// G (2T x 2T) in 128 x 128 tiles (bm, bn), bm <= bn: operand A = Y rows of frames 64 bm .. 64 bm + 63,
// B = frames 64 bn .. (the same as A on diagonal tiles; frames >= T are zero-filled by the tensor
// copy), from the split-BF16 planes of the ring (below). CTA (split ks, tile tp) walks the 64-pixel
// chunks of split ks (tiled_plan); the MMA warp issues Ah Bh^T, Ah Bl^T, Al Bh^T
// (M = N = 128, K = 16) into three TMEM accumulators in chains of at most kMaxChainChunks chunks,
// whose sums the epilogue warps add in FP32 registers. The CTAs of one split stream the same
// chunks at about the same time, so each chunk comes from HBM about once and the other tiles read
// it from L2.
constexpr int TT_FRAMES = 64;                          // frames per operand tile (128 rows of Y)

// Longest accumulation chain (64-pixel chunks, 4 MMA K-steps each) one TMEM accumulator takes.
// The FP32 accumulation of a tcgen05.mma into its accumulator does not round to nearest: summing
// 262144 pixels (4096 K-steps) into one accumulator drifted by 3.4e-4 relative to the FP64 sum on
// 512 x 512 frames (measured), about one unit of the last place per step in one direction; with
// chains of 64 chunks the drift was 1e-5 (a uniform scale: 9e-7 left after it). Chain sums are
// added in FP32 registers (round to nearest) within a split, the splits' partial tiles in FP64.
// The packed kernel (T <= 32) keeps one wave up to 128 chunks per CTA (1024 x 1024 frames: 108),
// where its extra waves cost more time than the drift costs accuracy.
constexpr size_t kMaxChainChunks = 64;
constexpr size_t kMaxChainChunksPacked = 128;
constexpr int TT_MAX_BLOCKS = COV_TC_MAX_T / TT_FRAMES;  // 64-frame blocks of a ring (16)
constexpr int TT_MAX_PAIRS = TT_MAX_BLOCKS * (TT_MAX_BLOCKS + 1) / 2;

// The tiles (bm <= bn) one launch computes, and the index of tile (bm, bn) in that list (-1: not
// computed): every tile of G, or the tiles touching the 64-frame blocks whose ring slots were
// rewritten since the covariance was last computed.
struct TileList
{
    int n;
    unsigned char bm[TT_MAX_PAIRS], bn[TT_MAX_PAIRS];
    signed char index[TT_MAX_BLOCKS][TT_MAX_BLOCKS];
};

// cov[i][j] from the tiled partials: row 2i of G is row 2 (i % 64) of tile row i / 64; the upper
// triangle (i <= j) is read from tile (i / 64, j / 64) and mirrored. Sums in FP64 over the splits:
// a CTA holds TR_ENTRIES consecutive entries, group q of its threads sums the splits q, q + TR_GROUPS,
// ..., and the group sums are added in group order. Entries of tiles outside the list are left as
// they are.
constexpr int TR_ENTRIES = 64, TR_GROUPS = 4;
__global__ void __launch_bounds__(TR_ENTRIES * TR_GROUPS) k_cov_tc_tiled_reduce(const float* __restrict__ part, int T,
                                                                               const __grid_constant__ TileList tiles,
                                                                               int nsplit, int real,
                                                                               double2* __restrict__ cov)
{
    __shared__ double red[TR_GROUPS - 1][4][TR_ENTRIES];
    const int q = threadIdx.x / TR_ENTRIES, el = threadIdx.x % TR_ENTRIES;
    const int e = blockIdx.x * TR_ENTRIES + el;
    int tp = -1, ri = 0, cj = 0;
    bool mirror = false, diag = false;
    if (e < T * T)
    {
        const int ei = e / T, ej = e % T;
        mirror = ei > ej;
        diag = ei == ej;
        const int i = mirror ? ej : ei, j = mirror ? ei : ej;
        // complex planes: 64 frames (128 rows: Re, Im) per block; real planes: 128 frames
        const int fb = real ? TC_ROWS : TT_FRAMES;
        tp = tiles.index[i / fb][j / fb];
        ri = real ? i % fb : 2 * (i % fb);
        cj = real ? j % fb : 2 * (j % fb);
    }
    double g00 = 0, g11 = 0, g01 = 0, g10 = 0;
    if (tp >= 0)
    {
        const int npairs = tiles.n;
        for (int k = q; k < nsplit; k += TR_GROUPS)
        {
            const float* G = part + (static_cast<size_t>(k) * npairs + tp) * TC_ROWS * TC_ROWS;
            g00 += G[ri * TC_ROWS + cj];
            if (!real)
            {
                g11 += G[(ri + 1) * TC_ROWS + cj + 1];
                g01 += G[ri * TC_ROWS + cj + 1];
                g10 += G[(ri + 1) * TC_ROWS + cj];
            }
        }
    }
    if (q > 0)
    {
        red[q - 1][0][el] = g00;
        red[q - 1][1][el] = g11;
        red[q - 1][2][el] = g01;
        red[q - 1][3][el] = g10;
    }
    __syncthreads();
    if (q > 0 || tp < 0)
        return;
    for (int w = 0; w < TR_GROUPS - 1; ++w)
    {
        g00 += red[w][0][el];
        g11 += red[w][1][el];
        g01 += red[w][2][el];
        g10 += red[w][3][el];
    }
    const double im = diag ? 0.0 : (g01 - g10);
    cov[e] = make_double2(g00 + g11, mirror ? -im : im);
}

// ------------------------------------------------------------------ split-BF16 planes of the ring
// planes[p][2 s + c][px] (p = 0: hi = bf16_rn(x), p = 1: lo = bf16_rn(x - hi); c = 0: real, c = 1:
// imaginary part of pixel px of ring slot s), written once per frame when it enters the ring. The
// tiled covariance streams the four operand tiles of a chunk (Ah, Al, Bh, Bl: 128 rows x 64 pixels
// each) from them by 3-D tensor copies straight into the swizzled K-major layout the MMAs read, so
// that a chunk is split once instead of once per tile it takes part in. A real ring (no spatial
// transform: imaginary parts exactly 0) keeps the real rows only (planes[p][s][px]): half the bytes,
// and C = Re Re^T from tiles of 128 frames, a quarter of the products.

// Thread: 8 consecutive pixels of one frame of slots slot0 .. slot0 + n - 1 (mod T).
__global__ void k_ring_split(const float2* __restrict__ ring, int T, size_t npix, int slot0, int n, int real,
                             uint16_t* __restrict__ planes)
{
    const size_t groups = npix / 8;
    const size_t total = static_cast<size_t>(n) * groups;
    const size_t plane = (real ? 1 : 2) * static_cast<size_t>(T) * npix;
    for (size_t e = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
         e += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        const int f = static_cast<int>(e / groups);
        const size_t g = e % groups;
        const size_t slot = static_cast<size_t>((slot0 + f) % T);
        const float4* src = reinterpret_cast<const float4*>(ring + slot * npix + 8 * g);
        const float4 a = src[0], b = src[1], c = src[2], d = src[3];
        uint4 rh, rl, ih, il;
        tc::split2(a.x, a.z, rh.x, rl.x);
        tc::split2(b.x, b.z, rh.y, rl.y);
        tc::split2(c.x, c.z, rh.z, rl.z);
        tc::split2(d.x, d.z, rh.w, rl.w);
        tc::split2(a.y, a.w, ih.x, il.x);
        tc::split2(b.y, b.w, ih.y, il.y);
        tc::split2(c.y, c.w, ih.z, il.z);
        tc::split2(d.y, d.w, ih.w, il.w);
        uint16_t* re = planes + (real ? 1 : 2) * slot * npix + 8 * g;
        *reinterpret_cast<uint4*>(re) = rh;
        *reinterpret_cast<uint4*>(re + plane) = rl;
        if (!real)
        {
            *reinterpret_cast<uint4*>(re + npix) = ih;
            *reinterpret_cast<uint4*>(re + plane + npix) = il;
        }
    }
}

constexpr int TP_STAGES = 3;
constexpr int TP_EPI_WARPS = 4;               // warps 0-3 read the accumulators
constexpr int TP_MMA_WARP = TP_EPI_WARPS;     // warp 4 issues the MMAs
constexpr int TP_LOAD_WARP = TP_EPI_WARPS + 1;  // warp 5 issues the tensor copies
constexpr int TP_THREADS = (TP_EPI_WARPS + 2) * 32;
constexpr uint32_t TP_STAGE_BYTES = 4 * TILE_BYTES;  // Ah, Al, Bh, Bl

// part: [gridDim.x][128][128] FP32 partial tiles (CTA index = ks * tiles.n + tp)
__global__ void __launch_bounds__(TP_THREADS, 1) k_cov_tc_tiled(const __grid_constant__ CUtensorMap planes_map,
                                                                size_t npix, const __grid_constant__ TileList tiles_in,
                                                                size_t chunks_per_split, float* __restrict__ part,
                                                                int* __restrict__ err)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* stages = smem + ((1024u - (smem_u32(smem) & 1023u)) & 1023u);
    __shared__ __align__(8) uint64_t full[TP_STAGES], empty[TP_STAGES];
    __shared__ __align__(8) uint64_t acc_full, acc_empty, drain;
    __shared__ uint32_t tmem_base;
    __shared__ int s_abort, s_issued;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tp = static_cast<int>(blockIdx.x % static_cast<unsigned>(tiles_in.n));
    const int ks = static_cast<int>(blockIdx.x / static_cast<unsigned>(tiles_in.n));
    const int bm = tiles_in.bm[tp], bn = tiles_in.bn[tp];
    const bool diag = bm == bn;
    const size_t nchunks = (npix + TC_KC - 1) / TC_KC;
    const size_t c_begin = static_cast<size_t>(ks) * chunks_per_split;
    size_t c_end = c_begin + chunks_per_split;
    if (c_end > nchunks)
        c_end = nchunks;
    const int nmine = static_cast<int>(c_end > c_begin ? c_end - c_begin : 0);
    constexpr int CHAIN = static_cast<int>(kMaxChainChunks);
    const int nchains = (nmine + CHAIN - 1) / CHAIN;
    volatile int* abort = &s_abort;
    constexpr uint32_t N = TC_ROWS;

    if (tid == 0)
    {
        for (int i = 0; i < TP_STAGES; ++i)
        {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        mbar_init(&acc_full, 1);
        mbar_init(&acc_empty, TP_EPI_WARPS);
        mbar_init(&drain, 1);
        s_abort = 0;
        s_issued = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == TP_MMA_WARP)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(512u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    if (warp == TP_LOAD_WARP)
    {
        // ------------------------------------------------------------------ loader (TMA)
        if (lane == 0)
        {
            asm volatile("prefetch.tensormap [%0];" ::"l"(&planes_map) : "memory");
            int m = 0;
            for (; m < nmine; ++m)
            {
                const int st = m % TP_STAGES;
                if (m >= TP_STAGES)
                    mbar_wait(&empty[st], static_cast<uint32_t>(((m / TP_STAGES) - 1) & 1), abort);
                if (*abort)
                    break;
                const int x = static_cast<int>(TC_KC * (c_begin + m));
                uint8_t* dst = stages + st * TP_STAGE_BYTES;
                tc::mbar_arrive_expect_tx(&full[st], diag ? 2 * TILE_BYTES : 4 * TILE_BYTES);
                tc::tma_load_3d(dst, &planes_map, x, bm * TC_ROWS, 0, &full[st]);
                tc::tma_load_3d(dst + TILE_BYTES, &planes_map, x, bm * TC_ROWS, 1, &full[st]);
                if (!diag)
                {
                    tc::tma_load_3d(dst + 2 * TILE_BYTES, &planes_map, x, bn * TC_ROWS, 0, &full[st]);
                    tc::tma_load_3d(dst + 3 * TILE_BYTES, &planes_map, x, bn * TC_ROWS, 1, &full[st]);
                }
            }
            s_issued = m;
        }
        __syncwarp();
    }
    else if (warp == TP_MMA_WARP)
    {
        // ------------------------------------------------------------------ MMA issuer
        if (lane == 0)
        {
            const uint32_t idesc = instr_desc(TC_ROWS, TC_ROWS);
            for (int it = 0; it < nmine; ++it)
            {
                const int pos = it % CHAIN;
                if (pos == 0 && it > 0)
                {
                    // chain it / CHAIN - 1 done: the epilogue reads the accumulators before the next starts
                    mma_commit(&acc_full);
                    mbar_wait(&acc_empty, static_cast<uint32_t>((it / CHAIN - 1) & 1), abort);
                }
                const int st = it % TP_STAGES;
                mbar_wait(&full[st], static_cast<uint32_t>((it / TP_STAGES) & 1), abort);
                if (*abort)
                    break;
                tc_fence_after();
                const uint32_t ah = smem_u32(stages + st * TP_STAGE_BYTES), al = ah + TILE_BYTES;
                const uint32_t bh = diag ? ah : ah + 2 * TILE_BYTES, bl = diag ? al : ah + 3 * TILE_BYTES;
#pragma unroll
                for (int s2 = 0; s2 < TC_KC / 16; ++s2)
                {
                    const uint64_t dah = smem_desc(ah + s2 * 32), dal = smem_desc(al + s2 * 32);
                    const uint64_t dbh = smem_desc(bh + s2 * 32), dbl = smem_desc(bl + s2 * 32);
                    const uint32_t acc = (pos > 0 || s2 > 0) ? 1u : 0u;
                    mma_bf16(tmem, dah, dbh, idesc, acc);          // Ah Bh^T
                    mma_bf16(tmem + N, dah, dbl, idesc, acc);      // Ah Bl^T
                    mma_bf16(tmem + 2 * N, dal, dbh, idesc, acc);  // Al Bh^T
                }
                mma_commit(&empty[st]);
            }
            mma_commit(&acc_full);
        }
        __syncwarp();
    }
    else
    {
        // ------------------------------------------------------------------ epilogue
        // thread r (warp w, lane l: r = 32w + l) keeps row r of the split's tile: the sum over the
        // chains of the three products' accumulators
        const int r = warp * 32 + lane;
        float sum[TC_ROWS];
#pragma unroll
        for (int i = 0; i < TC_ROWS; ++i)
            sum[i] = 0.f;
        for (int c = 0; c < nchains; ++c)
        {
            mbar_wait(&acc_full, static_cast<uint32_t>(c & 1), abort);
            if (*abort)
                break;
            tc_fence_after();
#pragma unroll
            for (int c0 = 0; c0 < TC_ROWS; c0 += 16)
            {
                float v[16], w1[16], w2[16];
                const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c0);
                tmem_ld16(taddr, v);
                tmem_ld16(taddr + N, w1);
                tmem_ld16(taddr + 2 * N, w2);
#pragma unroll
                for (int i = 0; i < 16; ++i)
                    sum[c0 + i] += v[i] + w1[i] + w2[i];
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0)
                mbar_arrive(&acc_empty);
        }
        float* dst = part + static_cast<size_t>(blockIdx.x) * TC_ROWS * TC_ROWS + static_cast<size_t>(r) * TC_ROWS;
#pragma unroll
        for (int i = 0; i < TC_ROWS; i += 4)
            *reinterpret_cast<float4*>(dst + i) = make_float4(sum[i], sum[i + 1], sum[i + 2], sum[i + 3]);
    }
    tc_fence_before();
    __syncthreads();
    if (s_abort)
    {
        // a wait gave up: the copies and MMAs already issued finish before shared and tensor memory
        // are released (bounded waits)
        if (warp == TP_LOAD_WARP && lane == 0)
        {
            const int issued = s_issued;
            for (int m = issued - TP_STAGES > 0 ? issued - TP_STAGES : 0; m < issued; ++m)
                mbar_wait(&full[m % TP_STAGES], static_cast<uint32_t>((m / TP_STAGES) & 1));
            atomicExch(err, 1);
        }
        if (warp == TP_MMA_WARP && lane == 0)
        {
            mma_commit(&drain);
            mbar_wait(&drain, 0);
        }
        __syncthreads();
    }
    if (warp == TP_MMA_WARP)
    {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512u) : "memory");
    }
}

struct TiledPlan
{
    int nb, npairs, nsplit;
    size_t chunks_per_split;
};


// The pixel splits depend on (T, npix) only, never on which tiles a launch computes, so that a
// recomputed entry equals the full computation's bit for bit. Their count fills one wave for the
// tiles of one block (nb tiles: the update after one stride of <= 64 frames), with at least
// kMaxChainChunks chunks per split. Blocks: 64 frames (complex planes), 128 frames (real planes).
TiledPlan tiled_plan(int T, size_t npix, int real = 0)
{
    TiledPlan p;
    p.nb = real ? (T + TC_ROWS - 1) / TC_ROWS : (T + TT_FRAMES - 1) / TT_FRAMES;
    p.npairs = p.nb * (p.nb + 1) / 2;
    const size_t nchunks = (npix + TC_KC - 1) / TC_KC;
    size_t ns = static_cast<size_t>(sm_count() / p.nb);
    const size_t max_ns = (nchunks + kMaxChainChunks - 1) / kMaxChainChunks;
    if (ns > max_ns)
        ns = max_ns;
    if (ns < 1)
        ns = 1;
    p.chunks_per_split = (nchunks + ns - 1) / ns;
    p.nsplit = static_cast<int>((nchunks + p.chunks_per_split - 1) / p.chunks_per_split);
    return p;
}

struct TcPlan
{
    int ctas;
    size_t chunks_per_cta;
    int N;
    int packed;
    uint32_t cols;
};

int sm_count()
{
    static const int sms = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
            v = 152;
        return v;
    }();
    return sms;
}

TcPlan tc_plan(int T, size_t npix)
{
    TcPlan p;
    const size_t nchunks = (npix + TC_KC - 1) / TC_KC;
    // two persistent CTAs per SM (96 KB of shared memory each: two handoff pipelines per SM, 85.9
    // -> 76.3 us at T = 32 on 1024 x 1024 frames against one CTA with 200 KB), or whole waves of
    // them when a CTA's chain would exceed the limit
    const size_t sms = 2 * static_cast<size_t>(sm_count());
    const size_t chain = 2 * T <= 64 ? kMaxChainChunksPacked : kMaxChainChunks;
    size_t waves = (nchunks + sms * chain - 1) / (sms * chain);
    if (waves < 1)
        waves = 1;
    int ctas = static_cast<int>(sms * waves);
    if (static_cast<size_t>(ctas) > nchunks)
        ctas = static_cast<int>(nchunks);
    if (ctas < 1)
        ctas = 1;
    p.chunks_per_cta = (nchunks + ctas - 1) / ctas;
    p.ctas = static_cast<int>((nchunks + p.chunks_per_cta - 1) / p.chunks_per_cta);
    p.N = (2 * T + 15) / 16 * 16;
    p.packed = 2 * T <= 64 ? 1 : 0;
    uint32_t cols = 32;  // packed: one 128-column accumulator; else three accumulators of N columns
    while (cols < static_cast<uint32_t>(p.packed ? TC_ROWS : 3 * p.N))
        cols <<= 1;
    p.cols = cols;
    return p;
}

}  // namespace

bool cov_tc_supported(int T) { return T >= 1 && T <= COV_TC_MAX_T; }

// partial tiles of the tiled kernel (every tile), rounded to 256 bytes: the planes of a ring passed
// to cov_tc follow them in the workspace
static size_t tiled_part_bytes(int T, size_t npix)
{
    const TiledPlan q = tiled_plan(T, npix);
    return (static_cast<size_t>(q.nsplit) * q.npairs * TC_ROWS * TC_ROWS * sizeof(float) + 255) & ~static_cast<size_t>(255);
}

size_t cov_tc_workspace(int T, size_t npix)
{
    if (2 * T > TC_ROWS)
        return tiled_part_bytes(T, npix) + cov_planes_bytes(T, npix, 0) + 256;
    const TcPlan p = tc_plan(T, npix);
    const size_t per = p.packed ? static_cast<size_t>(TC_ROWS) * 64 : static_cast<size_t>(4) * T * T;
    return static_cast<size_t>(p.ctas) * per * sizeof(float) + 256;
}

size_t cov_planes_bytes(int T, size_t npix, int real) { return (real ? 4 : 8) * static_cast<size_t>(T) * npix; }

size_t cov_tc_partial_bytes(int T, size_t npix) { return 2 * T > TC_ROWS ? tiled_part_bytes(T, npix) + 256 : 0; }

bool cov_planes_supported(int T, size_t npix)
{
    return cov_tc_supported(T) && 2 * T > TC_ROWS && npix > 0 && npix % 8 == 0 && npix <= (1ull << 29);
}

hv_status cov_split_planes(const float2* ring, int T, size_t npix, int slot0, int n, uint16_t* planes, int real,
                           cudaStream_t st)
{
    if (!cov_planes_supported(T, npix) || (reinterpret_cast<uintptr_t>(ring) & 15) != 0 ||
        (reinterpret_cast<uintptr_t>(planes) & 15) != 0)
        return HV_ERR_UNSUPPORTED;
    if (n <= 0)
        return HV_OK;
    if (slot0 < 0 || slot0 >= T || n > T)
        return HV_INVALID_VALUE;
    const size_t total = static_cast<size_t>(n) * (npix / 8);
    const size_t cap = static_cast<size_t>(sm_count()) * 8;
    const int grid = static_cast<int>(std::min((total + 255) / 256, cap));
    k_ring_split<<<grid, 256, 0, st>>>(ring, T, npix, slot0, n, real ? 1 : 0, planes);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status cov_tc_planes(const uint16_t* planes, int T, size_t npix, double2* cov, void* work, int* err,
                        uint32_t blocks, int real, cudaStream_t st)
{
    if (!cov_planes_supported(T, npix) || (reinterpret_cast<uintptr_t>(planes) & 15) != 0)
        return HV_ERR_UNSUPPORTED;
    const TiledPlan q = tiled_plan(T, npix, real);
    TileList tl{};
    std::memset(tl.index, -1, sizeof(tl.index));
    for (int bm = 0; bm < q.nb; ++bm)
        for (int bn = bm; bn < q.nb; ++bn)
            if (((blocks >> bm) & 1u) || ((blocks >> bn) & 1u))
            {
                tl.bm[tl.n] = static_cast<unsigned char>(bm);
                tl.bn[tl.n] = static_cast<unsigned char>(bn);
                tl.index[bm][bn] = static_cast<signed char>(tl.n);
                ++tl.n;
            }
    if (tl.n == 0)
        return HV_OK;
    CUtensorMap tmap;
    const uint64_t rows = (real ? 1 : 2) * static_cast<uint64_t>(T);
    if (!tc::encode_tmap_3d_bf16_sw128(&tmap, planes, npix, rows, 2, npix * 2, rows * npix * 2, TC_KC, TC_ROWS))
    {
        set_last_error_msg("tensor-core covariance: cuTensorMapEncodeTiled failed for the split planes");
        return HV_ERR_CUDA;
    }
    const size_t smem = static_cast<size_t>(TP_STAGES) * TP_STAGE_BYTES + 1024;
    static const cudaError_t attr = cudaFuncSetAttribute(k_cov_tc_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         static_cast<int>(smem));
    HV_CUDA_TRY(attr);
    float* tpart = static_cast<float*>(work);
    k_cov_tc_tiled<<<q.nsplit * tl.n, TP_THREADS, smem, st>>>(tmap, npix, tl, q.chunks_per_split, tpart, err);
    HV_LAUNCH_CHECK();
    k_cov_tc_tiled_reduce<<<(T * T + TR_ENTRIES - 1) / TR_ENTRIES, TR_ENTRIES * TR_GROUPS, 0, st>>>(tpart, T, tl,
                                                                                                  q.nsplit, real ? 1 : 0,
                                                                                                  cov);
    HV_LAUNCH_CHECK();
    count_launch(2);
    return HV_OK;
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
    if (npix > (1ull << 29))
    {
        set_last_error_msg("tensor-core covariance: at most 2^29 pixels per frame");
        return HV_ERR_UNSUPPORTED;
    }
    if (2 * T > TC_ROWS)
    {
        // the ring's split planes in the workspace after the partial tiles
        uint16_t* planes = reinterpret_cast<uint16_t*>(static_cast<char*>(work) + tiled_part_bytes(T, npix));
        hv_status r = cov_split_planes(ring, T, npix, 0, T, planes, 0, st);
        if (r != HV_OK)
            return r;
        return cov_tc_planes(planes, T, npix, cov, work, err, ~0u, 0, st);
    }
    const TcPlan p = tc_plan(T, npix);
    // raw stages: T x 64 complex samples (T x 512 B) each, as many as fit beside the A stages in 96 KB
    const size_t raw_bytes = static_cast<size_t>(T) * TC_KC * 16;  // pairs of 64-pixel chunks
    const size_t a_bytes = p.packed ? static_cast<size_t>(TC_A_STAGES_PACKED) * TILE_BYTES
                                    : static_cast<size_t>(TC_A_STAGES) * 2 * TILE_BYTES;
    int raw = static_cast<int>((96 * 1024 - a_bytes) / raw_bytes);
    raw = raw > TC_MAX_RAW ? TC_MAX_RAW : (raw < 2 ? 2 : raw);
    const size_t smem = a_bytes + raw * raw_bytes + 1024;
    CUtensorMap map;
    if (!tc::encode_tmap_2d_f32(&map, ring, 2 * npix, static_cast<uint64_t>(T), npix * 8, 4 * TC_KC,
                                static_cast<uint32_t>(T)))
    {
        set_last_error_msg("tensor-core covariance: cuTensorMapEncodeTiled failed");
        return HV_ERR_CUDA;
    }
    HV_CUDA_TRY(cudaFuncSetAttribute(k_cov_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    float* part = static_cast<float*>(work);
    k_cov_tc<<<p.ctas, TC_THREADS, smem, st>>>(map, T, npix, p.chunks_per_cta, p.N, p.cols, raw, p.packed, part, err);
    HV_LAUNCH_CHECK();
    // four partials per thread (independent loads), the slices combined by FP64 atomics
    const int per = p.ctas < 4 ? p.ctas : 4;
    k_cov_tc_reduce<<<dim3((T * T + 255) / 256, (p.ctas + per - 1) / per), 256, 0, st>>>(part, T, p.ctas, per,
                                                                                       p.packed, cov);
    HV_LAUNCH_CHECK();
    count_launch(2);
    return HV_OK;
}

}  // namespace hv
