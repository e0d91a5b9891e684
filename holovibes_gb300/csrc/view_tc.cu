// Time transform + view on the 5th-generation tensor cores (tcgen05, TMEM), split-BF16.
//
// Reference: the STFT bins (stft.cu:9-15, plan icompute.cc:109-115) or the PCA projection
// (matrix_operations.cc:77-103) followed by the bin-averaged modulus / squared modulus / argument
// (tools_conversion.cu:11-103,199-232). Here only the K selected bins are computed:
// X[k][pix] = sum_t W[k][t] ring[t][pix] for a 128-pixel tile is the real GEMM
//   D[pix][n] = sum_kd A[pix][kd] B[n][kd],  kd = 2t + c (c = re/im of sample t),
//   row n = 2k holds (wr, -wi) pairs (X_re), row n = 2k+1 holds (wi, wr) pairs (X_im),
// with A and B split into BF16 hi + lo and D = Ah Bh + Ah Bl + Al Bh accumulated in FP32.
//
// Persistent kernel, one CTA per SM, 14 warps. Two shared-memory rings:
//   raw ring (R stages of 32 KB): one 2-D tensor copy (TMA, box 128 pixels x 32 samples of FP32
//     complex, zero fill past the frame and past T) per (tile, 32-sample chunk)
//   A ring (2 stages): the chunk's hi and lo A tiles (128 x 64 BF16, 128-byte-swizzled K-major)
//     and the chunk's pre-split B image (bulk copy)
//   warp 13    loader: the tensor copies, up to R chunks (R x 32 KB of ring data) in flight per SM
//   warps 0-7  converters: raw samples -> BF16 hi / lo A tiles; each warp releases its part of the
//              raw stage and of the A stage on its own (no lock-step between the warps)
//   warp 8     MMA issuer (tcgen05.mma kind::f16, M = 128, K = 16) into two independent
//              accumulator chains so consecutive MMAs do not wait on each other:
//                2N <= 256 and 3N <= 256: D1 (2N cols) += Ah [Bh; Bl] (one N = 2N MMA), D2 += Al Bh
//                otherwise (N <= 128):    D1 += Ah Bh + Al Bh,  D2 += Ah Bl
//              accumulators double-buffered in TMEM so the epilogue of a tile overlaps the next
//   warps 9-12 epilogue: tcgen05.ld of the accumulator parts (X = sum of the parts), view + bin
//              mean + scale, fftshift placement, per-tile renormalisation partial sum
// All waits are bounded in time; a wait that gives up stops every role and sets the error flag.
#include "hv_common.cuh"
#include <atomic>

#include "hv_internal.h"
#include "tc_common.cuh"

namespace hv {

namespace {

constexpr int V_M = 128;               // pixels per tile
constexpr int V_TC = 32;               // time samples per chunk (64 K values = one 128 B line)
constexpr int V_CONVERTERS = 256;      // warps 0-7
constexpr int V_MMA_WARP = 8;
constexpr int V_EPI_WARP0 = 9;         // warps 9-12
constexpr int V_LOAD_WARP = 13;
constexpr int V_THREADS = 14 * 32;
constexpr int V_A_TILE = V_M * 128;    // 16 KB (hi or lo)
constexpr int V_RAW = V_TC * V_M * 8;  // 32 KB of raw samples per chunk
constexpr int V_MAX_RAW = 4;
constexpr int V_A_STAGES = 2;
constexpr uint32_t V_ACC_COLS = 256;   // TMEM columns per accumulator buffer (two buffers)

__device__ __forceinline__ float view_value_tc(float xr, float xi, int img_type)
{
    if (img_type == HV_IMG_MODULUS)
        return hypotf(xr, xi);
    if (img_type == HV_IMG_SQUARED_MODULUS)
    {
        const float t = hypotf(xr, xi);
        return t * t;
    }
    return atan2f(xi, xr);
}

struct ViewTcArgs
{
    int T, W, H, K, N, nchunks;
    size_t HW;
    int ntiles;
    int img_type, shift;
    float scale;
    const uint8_t* bimg;  // [chunk][hi N*128 | lo N*128]
    float* out;
    double* partials;     // one per tile, or null
    int* err;
    int raw_stages;
    const CycleCtl* ctl;  // served cycle gate (render), or null
    const float* bin_w;   // moments: out = sum_k |X_k|^2 bin_w[k] (else the mean of the view)
    int stacked;          // 1: D1 = Ah [Bh; Bl] (2N cols) + D2 = Al Bh;  0: D1 = Ah Bh + Al Bh, D2 = Ah Bl
};

// MOM: moments epilogue (sum_k |X_k|^2 bin_w[k]); a compile-time instantiation, because the
// epilogue is on the kernel's critical path and a runtime branch there cost about 20% in time.
template <bool MOM>
__global__ void __launch_bounds__(V_THREADS, 1) k_view_tc(const __grid_constant__ CUtensorMap ring_map, ViewTcArgs a)
{
    if (!ctl_render(a.ctl))
        return;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
    __shared__ __align__(8) uint64_t raw_full[V_MAX_RAW], raw_empty[V_MAX_RAW];
    __shared__ __align__(8) uint64_t a_full[V_A_STAGES], a_empty[V_A_STAGES];
    __shared__ __align__(8) uint64_t acc_full[2], acc_empty[2], mma_drain;
    __shared__ uint32_t tmem_base;
    __shared__ int s_abort;
    __shared__ double epi_red[4];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = a.N, R = a.raw_stages;
    const uint32_t b_bytes = static_cast<uint32_t>(2 * N * 128);
    const uint32_t a_stage_bytes = static_cast<uint32_t>(2 * V_A_TILE) + ((b_bytes + 1023u) & ~1023u);
    uint8_t* raw_base = smem;
    uint8_t* a_base = smem + R * V_RAW;
    // tiles of this CTA: blockIdx.x, blockIdx.x + gridDim.x, ...; chunk g = ti * nchunks + c
    const int my_tiles = a.ntiles > static_cast<int>(blockIdx.x)
                             ? (a.ntiles - 1 - static_cast<int>(blockIdx.x)) / static_cast<int>(gridDim.x) + 1
                             : 0;
    const int total = my_tiles * a.nchunks;
    volatile int* abort = &s_abort;

    if (tid == 0)
    {
        for (int i = 0; i < R; ++i)
        {
            tc::mbar_init(&raw_full[i], 1);                  // loader's expect_tx arrival + the box bytes
            tc::mbar_init(&raw_empty[i], V_CONVERTERS / 32); // one arrival per converter warp
        }
        for (int i = 0; i < V_A_STAGES; ++i)
        {
            tc::mbar_init(&a_full[i], V_CONVERTERS / 32 + 1); // converter warps + the B image's expect_tx
            tc::mbar_init(&a_empty[i], 1);                    // tcgen05.commit of the chunk's MMAs
        }
        for (int i = 0; i < 2; ++i)
        {
            tc::mbar_init(&acc_full[i], 1);
            tc::mbar_init(&acc_empty[i], 4);  // one arrival per epilogue warp
        }
        tc::mbar_init(&mma_drain, 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == V_MMA_WARP)
        tc::tmem_alloc(&tmem_base, 2 * V_ACC_COLS);
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = tmem_base;

    if (warp == V_LOAD_WARP)
    {
        // ---------------------------------------------------------------- loader (TMA)
        if (lane == 0)
        {
            asm volatile("prefetch.tensormap [%0];" ::"l"(&ring_map) : "memory");
            int ti = 0, c = 0;
            for (int g = 0; g < total; ++g)
            {
                const int r = g % R;
                if (g >= R)
                    tc::mbar_wait(&raw_empty[r], static_cast<uint32_t>(((g / R) - 1) & 1), abort);
                const int pix0 = (static_cast<int>(blockIdx.x) + ti * static_cast<int>(gridDim.x)) * V_M;
                tc::mbar_arrive_expect_tx(&raw_full[r], static_cast<uint32_t>(V_RAW));
                tc::tma_load_2d(raw_base + r * V_RAW, &ring_map, 2 * pix0, c * V_TC, &raw_full[r]);
                if (++c == a.nchunks)
                {
                    c = 0;
                    ++ti;
                }
            }
        }
        __syncwarp();
    }
    else if (warp < V_MMA_WARP)
    {
        // ---------------------------------------------------------------- converters
        int c = 0;
        for (int g = 0; g < total; ++g)
        {
            const int r = g % R, s = g % V_A_STAGES;
            const uint8_t* raw = raw_base + r * V_RAW;
            uint8_t* as = a_base + s * a_stage_bytes;
            tc::mbar_wait(&raw_full[r], static_cast<uint32_t>((g / R) & 1), abort);
            if (g >= V_A_STAGES)
                tc::mbar_wait(&a_empty[s], static_cast<uint32_t>(((g / V_A_STAGES) - 1) & 1), abort);
            if (tid == 0)
            {
                tc::mbar_arrive_expect_tx(&a_full[s], b_bytes);
                tc::bulk_g2s(as + 2 * V_A_TILE, a.bimg + static_cast<size_t>(c) * b_bytes, b_bytes, &a_full[s]);
            }
            // items (pixel, 8-sample group): a warp reads 32 consecutive pixels of one sample row
            // (256 contiguous bytes) and writes one 16-byte chunk of 32 swizzled rows
#pragma unroll
            for (int q = 0; q < 2; ++q)
            {
                const int w = tid + q * V_CONVERTERS;
                const int pix = w & (V_M - 1), tg = w >> 7;
                uint32_t h[8], l[8];
#pragma unroll
                for (int u = 0; u < 8; ++u)
                {
                    const float2 v = *reinterpret_cast<const float2*>(raw + ((tg * 8 + u) * V_M + pix) * 8);
                    tc::split2(v.x, v.y, h[u], l[u]);
                }
                const uint32_t o0 = tc::sw128_offset(pix, 2 * tg), o1 = tc::sw128_offset(pix, 2 * tg + 1);
                *reinterpret_cast<uint4*>(as + o0) = make_uint4(h[0], h[1], h[2], h[3]);
                *reinterpret_cast<uint4*>(as + o1) = make_uint4(h[4], h[5], h[6], h[7]);
                *reinterpret_cast<uint4*>(as + V_A_TILE + o0) = make_uint4(l[0], l[1], l[2], l[3]);
                *reinterpret_cast<uint4*>(as + V_A_TILE + o1) = make_uint4(l[4], l[5], l[6], l[7]);
            }
            tc::fence_async_smem();
            __syncwarp();
            if (lane == 0)
            {
                tc::mbar_arrive(&raw_empty[r]);
                tc::mbar_arrive(&a_full[s]);
            }
            if (++c == a.nchunks)
                c = 0;
        }
    }
    else if (warp == V_MMA_WARP)
    {
        // ---------------------------------------------------------------- MMA issuer
        if (lane == 0)
        {
            const uint32_t idesc_n = tc::instr_desc(V_M, N);
            const uint32_t idesc_2n = a.stacked ? tc::instr_desc(V_M, 2 * N) : idesc_n;
            int g = 0;
            for (int ti = 0; ti < my_tiles; ++ti)
            {
                const int buf = ti & 1;
                const uint32_t d1 = tmem + static_cast<uint32_t>(buf) * V_ACC_COLS;
                const uint32_t d2 = d1 + static_cast<uint32_t>(a.stacked ? 2 * N : N);
                if (ti >= 2)
                    tc::mbar_wait(&acc_empty[buf], static_cast<uint32_t>(((ti >> 1) - 1) & 1), abort);
                tc::fence_after();
                for (int c = 0; c < a.nchunks; ++c, ++g)
                {
                    const int s = g % V_A_STAGES;
                    tc::mbar_wait(&a_full[s], static_cast<uint32_t>((g / V_A_STAGES) & 1), abort);
                    tc::fence_after();
                    const uint32_t sb = tc::smem_u32(a_base + s * a_stage_bytes);
                    const uint32_t ah = sb, al = sb + V_A_TILE, bh = sb + 2 * V_A_TILE, bl = bh + N * 128;
#pragma unroll
                    for (int ks = 0; ks < 4; ++ks)
                    {
                        const uint32_t acc = (c > 0 || ks > 0) ? 1u : 0u;
                        const uint64_t dah = tc::sw128_desc(ah + ks * 32), dal = tc::sw128_desc(al + ks * 32);
                        const uint64_t dbh = tc::sw128_desc(bh + ks * 32);
                        if (a.stacked)
                        {
                            tc::mma_bf16(d1, dah, dbh, idesc_2n, acc);  // rows [Bh; Bl]: 2N columns
                            tc::mma_bf16(d2, dal, dbh, idesc_n, acc);
                        }
                        else
                        {
                            const uint64_t dbl = tc::sw128_desc(bl + ks * 32);
                            tc::mma_bf16(d1, dah, dbh, idesc_n, acc);
                            tc::mma_bf16(d2, dah, dbl, idesc_n, acc);
                            tc::mma_bf16(d1, dal, dbh, idesc_n, 1u);
                        }
                    }
                    tc::mma_commit(&a_empty[s]);
                }
                tc::mma_commit(&acc_full[buf]);
            }
        }
        __syncwarp();
    }
    else
    {
        // ---------------------------------------------------------------- epilogue
        const int quarter = warp & 3;  // TMEM lanes 32*quarter .. +31
        const int r = quarter * 32 + lane;
        const uint32_t part2 = static_cast<uint32_t>(a.stacked ? 2 * N : N);
        for (int ti = 0; ti < my_tiles; ++ti)
        {
            const int buf = ti & 1;
            tc::mbar_wait(&acc_full[buf], static_cast<uint32_t>((ti >> 1) & 1), abort);
            tc::fence_after();
            const uint32_t acc = tmem + static_cast<uint32_t>(buf) * V_ACC_COLS + (static_cast<uint32_t>(quarter * 32) << 16);
            float sum = 0.f;
            for (int c0 = 0; c0 < N; c0 += 16)
            {
                float d[16], e[16];
                tc::tmem_ld16(acc + static_cast<uint32_t>(c0), d);
                tc::tmem_ld16(acc + part2 + static_cast<uint32_t>(c0), e);
#pragma unroll
                for (int i = 0; i < 16; ++i)
                    d[i] += e[i];
                if (a.stacked)
                {
                    tc::tmem_ld16(acc + static_cast<uint32_t>(N + c0), e);
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        d[i] += e[i];
                }
#pragma unroll
                for (int i = 0; i < 8; ++i)
                {
                    const int k = c0 / 2 + i;
                    if (k < a.K)
                    {
                        if constexpr (MOM)
                            sum += (d[2 * i] * d[2 * i] + d[2 * i + 1] * d[2 * i + 1]) * __ldg(a.bin_w + k);
                        else
                            sum += view_value_tc(d[2 * i], d[2 * i + 1], a.img_type);
                    }
                }
            }
            tc::fence_before();
            __syncwarp();
            if (lane == 0)
                tc::mbar_arrive(&acc_empty[buf]);
            const size_t P = static_cast<size_t>(blockIdx.x + static_cast<size_t>(ti) * gridDim.x) * V_M + r;
            float v = 0.f;
            if (P < a.HW)
            {
                v = MOM ? sum : sum / static_cast<float>(a.K);
                if (a.scale != 1.0f)
                    v = v * a.scale;
                size_t dst = P;
                if (a.shift)
                {
                    const int x = static_cast<int>(P % a.W), y = static_cast<int>(P / a.W);
                    dst = static_cast<size_t>((y + a.H / 2) % a.H) * a.W + (x + a.W / 2) % a.W;
                }
                a.out[dst] = v;
            }
            if (a.partials)
            {
                double dsum = v;
                for (int o = 16; o > 0; o >>= 1)
                    dsum += __shfl_down_sync(0xffffffffu, dsum, o);
                if (lane == 0)
                    epi_red[quarter] = dsum;
                asm volatile("bar.sync 1, 128;" ::: "memory");
                if (warp == V_EPI_WARP0 && lane == 0)
                    a.partials[blockIdx.x + static_cast<size_t>(ti) * gridDim.x] =
                        epi_red[0] + epi_red[1] + epi_red[2] + epi_red[3];
                asm volatile("bar.sync 1, 128;" ::: "memory");
            }
        }
    }
    tc::fence_before();
    __syncthreads();
    if (s_abort)
    {
        // a wait gave up: let the copies and MMAs already issued finish before the CTA's shared
        // and tensor memory are released (each wait bounded, without the abort shortcut)
        if (warp == V_LOAD_WARP && lane == 0)
        {
            for (int g = total - R > 0 ? total - R : 0; g < total; ++g)
                tc::mbar_wait(&raw_full[g % R], static_cast<uint32_t>((g / R) & 1));
            for (int g = total - V_A_STAGES > 0 ? total - V_A_STAGES : 0; g < total; ++g)
                tc::mbar_wait(&a_full[g % V_A_STAGES], static_cast<uint32_t>((g / V_A_STAGES) & 1));
            atomicExch(a.err, 1);
        }
        if (warp == V_MMA_WARP && lane == 0)
        {
            tc::mma_commit(&mma_drain);
            tc::mbar_wait(&mma_drain, 0);
        }
        __syncthreads();
    }
    if (warp == V_MMA_WARP)
    {
        tc::fence_after();
        tc::tmem_dealloc(tmem, 2 * V_ACC_COLS);
    }
}

// B images for every 32-sample chunk: row n = 2k: (wr, -wi) per sample, row 2k+1: (wi, wr);
// rows >= 2K and samples >= T are zero. Split into BF16 hi / lo in the swizzled layout.
__global__ void k_view_tc_weights(const float2* __restrict__ W, int K, int T, int N, int nchunks, uint8_t* bimg)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;  // over nchunks * N * 8 chunks of 8 K values
    if (e >= nchunks * N * 8)
        return;
    const int c = e / (N * 8), rem = e % (N * 8), n = rem / 8, ch = rem % 8;
    const int k = n / 2, part = n & 1;
    float vals[8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
        const int t = c * V_TC + ch * 4 + i;  // K values 8*ch + 2i, +1 -> sample 4*ch + i
        float2 w = make_float2(0.f, 0.f);
        if (k < K && t < T)
            w = W[static_cast<size_t>(k) * T + t];
        if (part == 0)
        {
            vals[2 * i] = w.x;
            vals[2 * i + 1] = -w.y;
        }
        else
        {
            vals[2 * i] = w.y;
            vals[2 * i + 1] = w.x;
        }
    }
    uint32_t h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        tc::split2(vals[2 * i], vals[2 * i + 1], h[i], l[i]);
    uint8_t* img = bimg + static_cast<size_t>(c) * 2 * N * 128;
    const uint32_t off = tc::sw128_offset(n, ch);
    *reinterpret_cast<uint4*>(img + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(img + N * 128 + off) = make_uint4(l[0], l[1], l[2], l[3]);
}

int view_tc_n(int K) { return ((2 * K + 15) / 16) * 16; }

size_t view_tc_a_stage_bytes(int N)
{
    return 2 * V_A_TILE + ((static_cast<size_t>(2) * N * 128 + 1023) & ~static_cast<size_t>(1023));
}

}  // namespace

// N = 2K rounded up to 16 must fit the two accumulator parts in 256 TMEM columns (K <= 64).
bool view_tc_supported(int K) { return K >= 1 && view_tc_n(K) <= 128; }

static std::atomic<int> g_view_mode{0};  // 0 automatic (tensor cores for K >= 8), 1 SIMT, 2 tensor cores

void set_view_mode(int mode) { g_view_mode = mode; }

bool view_engine_tc(int K, size_t HW)
{
    if (!view_tc_supported(K) || (HW & 1))
        return false;
    if (g_view_mode == 1)
        return false;
    if (g_view_mode == 2)
        return true;
    return K >= 8;
}

size_t view_tc_workspace(int K, int T)
{
    const int N = view_tc_n(K);
    const int nchunks = (T + V_TC - 1) / V_TC;
    return static_cast<size_t>(nchunks) * 2 * N * 128 + 256;
}

hv_status view_tc_prepare(const float2* weights, int K, int T, void* work, cudaStream_t st)
{
    if (!view_tc_supported(K))
        return HV_ERR_UNSUPPORTED;
    const int N = view_tc_n(K);
    const int nchunks = (T + V_TC - 1) / V_TC;
    uint8_t* bimg = static_cast<uint8_t*>(work) + 256;  // [0, 256): error flag
    const int total = nchunks * N * 8;
    k_view_tc_weights<<<(total + 255) / 256, 256, 0, st>>>(weights, K, T, N, nchunks, bimg);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

hv_status view_tc(const float2* ring, int T, int W, int H, int K, int img_type, float scale, int shift, float* out,
                  double* partials, void* work, cudaStream_t st, const CycleCtl* ctl, const float* bin_w)
{
    if (!view_tc_supported(K))
        return HV_ERR_UNSUPPORTED;
    if (shift && ((W & 1) || (H & 1)))
    {
        set_last_error_msg("fftshift needs even width and height");
        return HV_INVALID_VALUE;
    }
    const size_t HW = static_cast<size_t>(W) * H;
    // tensor copies: 16-byte aligned base and row pitch (HW even); x = 2 * pixel index stays in int
    if ((HW & 1) || HW > (1u << 29) || (reinterpret_cast<uintptr_t>(ring) & 15) ||
        (reinterpret_cast<uintptr_t>(work) & 15))
    {
        set_last_error_msg("tensor-core time view: needs an even pixel count (at most 2^29) and 16-byte aligned "
                           "ring and workspace");
        return HV_ERR_UNSUPPORTED;
    }
    CUtensorMap map;
    if (!tc::encode_tmap_2d_f32(&map, ring, 2 * HW, static_cast<uint64_t>(T), HW * 8, 2 * V_M, V_TC))
    {
        set_last_error_msg("tensor-core time view: cuTensorMapEncodeTiled failed");
        return HV_ERR_CUDA;
    }
    ViewTcArgs a;
    a.T = T;
    a.W = W;
    a.H = H;
    a.K = K;
    a.N = view_tc_n(K);
    a.nchunks = (T + V_TC - 1) / V_TC;
    a.HW = HW;
    a.ntiles = static_cast<int>((a.HW + V_M - 1) / V_M);
    a.img_type = img_type;
    a.shift = shift;
    a.scale = scale;
    a.err = static_cast<int*>(work);
    a.bimg = static_cast<const uint8_t*>(work) + 256;
    a.out = out;
    a.partials = partials;
    a.ctl = ctl;
    a.bin_w = bin_w;
    a.stacked = (3 * a.N <= static_cast<int>(V_ACC_COLS)) ? 1 : 0;
    const size_t a_bytes = V_A_STAGES * view_tc_a_stage_bytes(a.N);
    const size_t budget = 220 * 1024;
    int raw = static_cast<int>((budget - a_bytes) / V_RAW);
    if (raw > V_MAX_RAW)
        raw = V_MAX_RAW;
    if (raw < 2)
        return HV_ERR_UNSUPPORTED;
    a.raw_stages = raw;
    const size_t smem = raw * static_cast<size_t>(V_RAW) + a_bytes + 1024;
    auto kern = bin_w ? k_view_tc<true> : k_view_tc<false>;
    HV_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int sms = 0;
    HV_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
    int grid = a.ntiles < sms ? a.ntiles : sms;
    if (grid < 1)
        grid = 1;
    HV_CUDA_TRY(cudaMemsetAsync(a.err, 0, sizeof(int), st));
    kern<<<grid, V_THREADS, smem, st>>>(map, a);
    HV_LAUNCH_CHECK();
    count_launch();
    return HV_OK;
}

}  // namespace hv
