// Learned warm start: a message-passing network over the face adjacency graph,
// trained and evaluated with hand-written tcgen05 BF16 kernels (FP32
// accumulation in tensor memory).  It has no counterpart in the reference; it
// predicts the initial guess of each Krylov solve (the solve itself is the
// unchanged FP64 BiCGStab).
//
// Network (hidden width 64), per face E with neighbours N(E) = the faces that
// share a cell with E (the off-diagonal pattern of the face system):
//     h1 = relu(x W0 + b0)                          x: 16 features
//     a_l = mean_{E' in N(E)} h_l(E')               l = 1, 2, 3
//     h_{l+1} = relu([h_l, a_l] W_l + b_l) + h_l
//     out = h4 . wd + bd
//
// Kernels (128 faces per tile, 128 threads per CTA, persistent grids):
//  - k_mpnn_layer<KIN>: each thread stages one face row of the A tile
//    [h_l | mean of neighbours] (the gather is fused into the staging) in the
//    canonical K-major layout; one thread issues KIN/16 tcgen05.mma
//    (M=128, N=64, K=16) into a 64-column TMEM accumulator; the epilogue
//    (tcgen05.ld, bias, ReLU, residual) writes h_{l+1} in BF16.
//  - k_mpnn_bwd_dx: dX = dZ W^T (M=128, N=128, K=64) with dZ = dH * (Z > 0)
//    formed while staging (dH gathers the layer above's neighbour
//    gradients there); writes dH_self + dH_next and the scaled neighbour
//    gradient (BF16).
//  - k_mpnn_bwd_dw: dW = X^T dZ, split over faces: each CTA accumulates its
//    faces' contribution in TMEM (M=128 features, N=64, K=128 faces per
//    tile) and writes one FP32 partial; partials are summed in a fixed order.
//  - decode + loss, the encoder's dZ, Adam: CUDA-core kernels.
#include <cuda_bf16.h>

#include "mhfem_internal.h"
#include "mpnn.h"
#include "tcgen05.cuh"

namespace mhfem {

namespace {

constexpr int H = kMpnnHidden;  // 64
constexpr int TB = 128;         // faces per tile
constexpr int NT = 512;         // threads per CTA of the tensor-core kernels (4 per face)

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ float2 unpack_bf16(uint32_t u)
{
    __nv_bfloat162 v = *reinterpret_cast<__nv_bfloat162*>(&u);
    return __bfloat1622float2(v);
}

// Stores 8 consecutive bf16 (one uint4) of row `r`, columns k0..k0+7, of a K-major tile.
__device__ __forceinline__ void st_tile(uint8_t* tile, int r, int k0, int K, uint4 v)
{
    *reinterpret_cast<uint4*>(tile + tc::kmajor_offset(r, k0, K)) = v;
}

// Bulk L2 prefetch of a contiguous range (16-byte aligned start, size a
// multiple of 16 bytes): the next tile's rows and neighbour indices are on
// their way to L2 while the current tile is processed.
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(p), "r"(bytes) : "memory");
}

struct TileSync {
    uint64_t* mbar;
    uint32_t phase;
};

// MMA over a staged tile pair; thread 0 issues, every thread waits.
template <int M, int N, int K>
__device__ __forceinline__ bool tile_mma(uint8_t* sA, uint8_t* sB, uint32_t taddr, TileSync& ts, bool accumulate)
{
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x == 0) {
        constexpr uint32_t idesc = tc::make_idesc_bf16(M, N);
#pragma unroll
        for (int ks = 0; ks < K / 16; ++ks) {
            const uint64_t ad = tc::make_desc(tc::smem_addr(sA) + ks * 256, 128, K * 16);
            const uint64_t bd = tc::make_desc(tc::smem_addr(sB) + ks * 256, 128, K * 16);
            tc::mma_bf16(taddr, ad, bd, idesc, accumulate || ks > 0);
        }
        tc::mma_commit(ts.mbar);
    }
    const bool ok = tc::mbar_wait(ts.mbar, ts.phase);
    ts.phase ^= 1u;
    tc::fence_after_sync();
    return ok;
}

__device__ __forceinline__ void tile_done()
{
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
}

// ---- forward layer ----------------------------------------------------------

// Row stride (bytes) of the output staging tile: 128 bytes of BF16 plus 16
// bytes of padding, so the epilogue's per-row 16-byte stores spread over all
// banks.
constexpr int kOutStride = 2 * H + 16;

// Global <-> tile traffic is row-coalesced: thread t moves the 16-byte chunk
// c = t % 8 (columns 8c .. 8c + 7) of the rows t / 8 and t / 8 + 64, so a warp
// reads or writes four whole 128-byte rows per instruction (for the
// neighbour gather too: the four rows' k-th neighbours).  The epilogue is
// row-per-thread: thread (r, qs) = (t % 128, t / 128) reads columns
// 16 qs .. 16 qs + 15 of row r from TMEM (warp % 4 == r / 32 is its TMEM lane
// quarter) and writes them to the staging tile.
// Inference keeps 3 CTAs per SM resident (registers capped at 42; the
// staging of the three CTAs' tiles overlaps the others' MMA and epilogue);
// training also stages the pre-activations and fits 2.  DEC (inference, last
// layer): the decoder runs in the epilogue -- each thread's 16 columns of
// h4 (as stored in BF16) dotted with wd, the four slices of a row summed in
// shared memory -- and the guess is written instead of h4.
template <int KIN, bool TRAIN, bool DEC = false>
__global__ void __launch_bounds__(NT, TRAIN ? 2 : 3) k_mpnn_layer(const MpnnView V, int layer)
{
    extern __shared__ __align__(128) uint8_t smem[];
    uint8_t* sA = smem;                            // 128 x KIN (K-major)
    uint8_t* sB = sA + TB * KIN * 2;               // 64 x KIN (K-major)
    uint8_t* sO = sB + H * KIN * 2;                // 128 rows x kOutStride: h_{l+1}
    uint8_t* sZ = sO + TB * kOutStride;            // 128 rows x kOutStride: z_l (training)
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    __shared__ float sbias[H];
    __shared__ float swd[DEC ? H : 1];
    __shared__ float sdec[DEC ? 4 : 1][DEC ? TB : 1];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int r = tid & (TB - 1), qs = tid >> 7;  // epilogue mapping
    const int c8 = tid & 7, slot = tid >> 3;      // row-coalesced mapping
    static_assert(!(DEC && TRAIN), "the fused decoder is an inference path");
    const int64_t F = V.F;

    const __nv_bfloat16* Wf = V.w_fwd[layer];  // [64][KIN]
    for (int idx = tid; idx < H * KIN / 8; idx += NT) {
        const int rr = idx / (KIN / 8), k0 = (idx % (KIN / 8)) * 8;
        st_tile(sB, rr, k0, KIN, *reinterpret_cast<const uint4*>(Wf + rr * KIN + k0));
    }
    if (tid < H) sbias[tid] = V.bias[layer][tid];
    if constexpr (DEC)
        if (tid < H) swd[tid] = V.wd[tid];
    if (warp == 0) {
        tc::tmem_alloc(&tbase, H);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(&mbar, 1);
    tile_done();
    const uint32_t taddr = tbase + ((uint32_t)(32 * (warp & 3)) << 16) + 16 * qs;
    TileSync ts{&mbar, 0};
    const __nv_bfloat16* hin = (KIN == 16) ? V.x0 : V.h[layer];
    __nv_bfloat16* hout = V.h[layer + 1];
    const int64_t ntiles = (F + TB - 1) / TB;

    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t row0 = tile * TB;
        // the next tile of this CTA: its input rows and (hidden layers) its
        // neighbour index slices; whole 16-byte multiples inside the arrays
        if (tid == 0 && tile + gridDim.x < ntiles) {
            const int64_t nr0 = (tile + gridDim.x) * TB;
            const int64_t nrows = (F - nr0) < TB ? (F - nr0) : TB;
            prefetch_l2(hin + nr0 * (KIN == 16 ? 16 : H), (uint32_t)(nrows * (KIN == 16 ? 32 : 2 * H)));
            if constexpr (KIN != 16) {
                const uint32_t ib = (uint32_t)((nrows * 4) & ~15);
                if (ib > 0)
                    for (int k = 0; k < V.W; ++k)
                        if ((((uint64_t)(V.nbr + (int64_t)k * F + nr0)) & 15) == 0) prefetch_l2(V.nbr + (int64_t)k * F + nr0, ib);
            }
        }
        if constexpr (KIN == 16) {
            // 128 rows x 32 bytes: two chunks per row
            if (tid < 2 * TB) {
                const int rr = tid >> 1, ch = tid & 1;
                uint4 v = make_uint4(0, 0, 0, 0);
                if (row0 + rr < F) v = __ldg(reinterpret_cast<const uint4*>(hin + (row0 + rr) * 16 + 8 * ch));
                st_tile(sA, rr, 8 * ch, 16, v);
            }
        }
        else {
            // neighbour indices of both rows first (padding entries point at
            // the row itself); the eight lanes of a row read the same words
            int32_t nbs[2][kMpnnMaxWidth];
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int64_t row = row0 + slot + 64 * j;
#pragma unroll
                for (int k = 0; k < kMpnnMaxWidth; ++k) {
                    int32_t c = -1;
                    if (row < F && k < V.W) c = __ldg(V.nbr + (int64_t)k * F + row);
                    nbs[j][k] = (c == (int32_t)row) ? -1 : c;
                }
            }
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int rr = slot + 64 * j;
                const int64_t row = row0 + rr;
                const bool valid = row < F;
                const int32_t* nb = nbs[j];
                uint4 self = make_uint4(0, 0, 0, 0);
                if (valid) self = __ldg(reinterpret_cast<const uint4*>(hin + row * H + 8 * c8));
                const int d = valid ? (int)V.deg[row] : 0;
                uint4 g[kMpnnMaxWidth];
#pragma unroll
                for (int k = 0; k < kMpnnMaxWidth; ++k) {
                    g[k] = make_uint4(0, 0, 0, 0);
                    if (nb[k] >= 0) g[k] = __ldg(reinterpret_cast<const uint4*>(hin + (int64_t)nb[k] * H + 8 * c8));
                }
                st_tile(sA, rr, 8 * c8, KIN, self);
                float acc[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) acc[q] = 0.f;
#pragma unroll
                for (int k = 0; k < kMpnnMaxWidth; ++k) {
                    const uint32_t w4[4] = {g[k].x, g[k].y, g[k].z, g[k].w};
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        const float2 f = unpack_bf16(w4[t]);
                        acc[2 * t] += f.x;
                        acc[2 * t + 1] += f.y;
                    }
                }
                const float inv = d > 0 ? 1.0f / (float)d : 0.0f;
                uint4 v;
                v.x = pack_bf16(acc[0] * inv, acc[1] * inv);
                v.y = pack_bf16(acc[2] * inv, acc[3] * inv);
                v.z = pack_bf16(acc[4] * inv, acc[5] * inv);
                v.w = pack_bf16(acc[6] * inv, acc[7] * inv);
                st_tile(sA, rr, H + 8 * c8, KIN, v);
                if (TRAIN && valid) *reinterpret_cast<uint4*>(V.a[layer] + row * H + 8 * c8) = v;
            }
        }
        if (!tile_mma<TB, H, KIN>(sA, sB, tbase, ts, false)) {
            if (tid == 0) atomicOr(V.err, 4);
            break;
        }
        {
            float acc[16];
            tc::tmem_ld_x16(taddr, acc);
            uint32_t sw[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if constexpr (KIN != 16) {
                const uint4 s0 = *reinterpret_cast<const uint4*>(sA + tc::kmajor_offset(r, 16 * qs, KIN));
                const uint4 s1 = *reinterpret_cast<const uint4*>(sA + tc::kmajor_offset(r, 16 * qs + 8, KIN));
                sw[0] = s0.x; sw[1] = s0.y; sw[2] = s0.z; sw[3] = s0.w;
                sw[4] = s1.x; sw[5] = s1.y; sw[6] = s1.z; sw[7] = s1.w;
            }
            uint32_t zo[8], ho[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int q = 2 * t;
                const float z0 = acc[q] + sbias[16 * qs + q], z1 = acc[q + 1] + sbias[16 * qs + q + 1];
                float o0 = fmaxf(z0, 0.f), o1 = fmaxf(z1, 0.f);
                if constexpr (KIN != 16) {
                    const float2 sv = unpack_bf16(sw[t]);
                    o0 += sv.x;
                    o1 += sv.y;
                }
                zo[t] = pack_bf16(z0, z1);
                ho[t] = pack_bf16(o0, o1);
            }
            if constexpr (DEC) {
                float part = 0.f;
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const float2 hv = unpack_bf16(ho[t]);
                    part = fmaf(hv.x, swd[16 * qs + 2 * t], part);
                    part = fmaf(hv.y, swd[16 * qs + 2 * t + 1], part);
                }
                sdec[qs][r] = part;
            }
            else {
                uint4* so = reinterpret_cast<uint4*>(sO + r * kOutStride + 32 * qs);
                so[0] = make_uint4(ho[0], ho[1], ho[2], ho[3]);
                so[1] = make_uint4(ho[4], ho[5], ho[6], ho[7]);
            }
            if (TRAIN) {
                uint4* sz = reinterpret_cast<uint4*>(sZ + r * kOutStride + 32 * qs);
                sz[0] = make_uint4(zo[0], zo[1], zo[2], zo[3]);
                sz[1] = make_uint4(zo[4], zo[5], zo[6], zo[7]);
            }
        }
        tile_done();
        if constexpr (DEC) {
            if (tid < TB && row0 + tid < F) {
                const int64_t row = row0 + tid;
                const float out = sdec[0][tid] + sdec[1][tid] + sdec[2][tid] + sdec[3][tid] + V.bd[0];
                V.dec_guess[row] = V.fixed[row] ? V.dec_rhs[row] : V.dec_base[row] + V.dec_scal[10] * (double)out;
            }
        }
        else {
            // row-coalesced write-out of the staged tile
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int rr = slot + 64 * j;
                const int64_t row = row0 + rr;
                if (row < F) {
                    *reinterpret_cast<uint4*>(hout + row * H + 8 * c8) =
                        *reinterpret_cast<const uint4*>(sO + rr * kOutStride + 16 * c8);
                    if (TRAIN)
                        *reinterpret_cast<uint4*>(V.z[layer] + row * H + 8 * c8) =
                            *reinterpret_cast<const uint4*>(sZ + rr * kOutStride + 16 * c8);
                }
            }
        }
    }
    tile_done();
    if (warp == 0) tc::tmem_dealloc(tbase, H);
}

// ---- decoder, loss and the start of the backward pass --------------------------

// Training decoder: out = h4 . wd + bd, the loss, dout, dh4 = dout wd and
// the decoder gradients (one partial per block).
__global__ void __launch_bounds__(256) k_mpnn_decode(const MpnnView V, const double* target, double inv_nt)
{
    __shared__ float swd[H];
    __shared__ double red[256 / 32][H + 2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < H) swd[tid] = V.wd[tid];
    __syncthreads();
    const float bd = V.bd[0];
    double acc_l = 0, acc_db = 0;
    float acc_w[H];
#pragma unroll
    for (int q = 0; q < H; ++q) acc_w[q] = 0.f;
    const __nv_bfloat16* h4 = V.h[kMpnnLayers + 1];
    for (int64_t row = (int64_t)blockIdx.x * 256 + tid; row < V.F; row += (int64_t)gridDim.x * 256) {
        float hv[H];
        float out = bd;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const uint4 v = *reinterpret_cast<const uint4*>(h4 + row * H + 8 * c);
            const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const float2 f = unpack_bf16(w4[t]);
                hv[8 * c + 2 * t] = f.x;
                hv[8 * c + 2 * t + 1] = f.y;
            }
        }
#pragma unroll
        for (int q = 0; q < H; ++q) out = fmaf(hv[q], swd[q], out);
        const bool fixed = V.fixed[row] != 0;
        const double diff = fixed ? 0.0 : ((double)out - target[row]);
        acc_l += diff * diff;
        const float dout = (float)(2.0 * diff * inv_nt);
        acc_db += dout;
#pragma unroll
        for (int q = 0; q < H; ++q) acc_w[q] = fmaf(dout, hv[q], acc_w[q]);
        float* dh = V.dh + row * H;
#pragma unroll
        for (int c = 0; c < H / 4; ++c)
            *reinterpret_cast<float4*>(dh + 4 * c) =
                make_float4(dout * swd[4 * c], dout * swd[4 * c + 1], dout * swd[4 * c + 2], dout * swd[4 * c + 3]);
    }
    // block reduction of (dwd[64], dbd, loss) into partials[block][66]
#pragma unroll
    for (int q = 0; q < H; ++q) {
        float v = acc_w[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][q] = v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        acc_db += __shfl_down_sync(0xffffffffu, acc_db, o);
        acc_l += __shfl_down_sync(0xffffffffu, acc_l, o);
    }
    if (lane == 0) { red[warp][H] = acc_db; red[warp][H + 1] = acc_l; }
    __syncthreads();
    if (tid < H + 2) {
        double s = 0;
        for (int w = 0; w < 256 / 32; ++w) s += red[w][tid];
        V.dec_partials[(int64_t)blockIdx.x * (H + 2) + tid] = s;
    }
}

// ---- backward: dX = dZ W^T ------------------------------------------------------

// A = dZ (128 x 64) with dZ = dH * (Z > 0), B = W_in (128 x 64: row k = input k).
// dH of layer l + 1 is the stored partial dH (the residual and self paths)
// plus, below the top layer, the transpose of the neighbour mean of layer
// l + 1: the sum over the neighbours E' of g_{l+1}(E') (the adjacency is
// symmetric), gathered here while staging instead of in a pass of its own.
// Epilogue: dH_l = dH + dX[:, :64], g_l = dX[:, 64:] / deg (BF16, into the
// other of the two g buffers: layer l reads g[(l + 1) % 2], writes g[l % 2]).
//
// Global traffic is row-coalesced, as in the forward layer: thread
// (slot, c8) = (t / 8, t % 8) moves columns 4 c8 .. 4 c8 + 3 and
// 32 + 4 c8 .. 32 + 4 c8 + 3 of rows slot and slot + 64, so the eight lanes
// of a row cover 128 contiguous bytes of its FP32 dH row per load (64 of a
// BF16 row), and a warp instruction touches four rows -- for the neighbour
// gather too.  (A row per thread made every instruction touch 32 rows,
// which bound the kernel by L1 wavefronts at about a third of HBM.)  The
// thread keeps its 16 dH values in registers across the MMA.  The TMEM
// epilogue is row-per-thread ((r, qs) = (t % 128, t / 128); warp % 4 is the
// TMEM lane quarter), so it passes dX through shared memory: the FP32 half
// into sD, the scaled BF16 neighbour half into the A tile's space (the MMA
// has read it by then), both with 16-byte chunks XOR-swizzled by row % 8 so
// the row-per-thread stores and the row-coalesced loads are free of bank
// conflicts.
constexpr int kDxSmem = (TB + 2 * H) * H * 2 + TB * H * 4;  // A, B tiles (BF16) + FP32 dX staging

__device__ __forceinline__ int swz(int r, int chunk) { return chunk ^ (r & 7); }

__global__ void __launch_bounds__(NT, 2) k_mpnn_bwd_dx(const MpnnView V, int layer)
{
    extern __shared__ __align__(128) uint8_t smem[];
    uint8_t* sA = smem;                                                   // 128 x 64 BF16: dZ, then g
    uint8_t* sB = smem + TB * H * 2;                                      // 128 x 64 BF16: W_in
    float* sD = reinterpret_cast<float*>(smem + (TB + 2 * H) * H * 2);   // 128 x 64 FP32: dX[:, :64]
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int r = tid & (TB - 1), qs = tid >> 7;  // epilogue mapping
    const int c8 = tid & 7, slot = tid >> 3;      // row-coalesced mapping
    const int64_t F = V.F;
    const bool gather = layer < kMpnnLayers;
    const __nv_bfloat16* gin = V.gb[(layer + 1) & 1];
    __nv_bfloat16* gout = V.gb[layer & 1];
    const __nv_bfloat16* Wb = V.w_bwd[layer];  // [128][64]
    for (int idx = tid; idx < 2 * H * H / 8; idx += NT) {
        const int rr = idx / (H / 8), k0 = (idx % (H / 8)) * 8;
        st_tile(sB, rr, k0, H, *reinterpret_cast<const uint4*>(Wb + rr * H + k0));
    }
    if (warp == 0) {
        tc::tmem_alloc(&tbase, 2 * H);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(&mbar, 1);
    tile_done();
    const uint32_t tlane = tbase + ((uint32_t)(32 * (warp & 3)) << 16);
    TileSync ts{&mbar, 0};
    const int64_t ntiles = (F + TB - 1) / TB;
    const int col0 = 4 * c8, col1 = H / 2 + 4 * c8;  // the thread's two column quads
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        // ---- staging: dH (+ the neighbours' g), dZ = dH * (Z > 0)
        float dhv[2][8];
        int32_t nb[2][kMpnnMaxWidth];
#pragma unroll
        for (int ps = 0; ps < 2; ++ps) {
            const int64_t row = tile * TB + slot + 64 * ps;
#pragma unroll
            for (int q = 0; q < 8; ++q) dhv[ps][q] = 0.f;
#pragma unroll
            for (int k = 0; k < kMpnnMaxWidth; ++k) nb[ps][k] = -1;
            if (row < F) {
                const float4 a = *reinterpret_cast<const float4*>(V.dh + row * H + col0);
                const float4 b = *reinterpret_cast<const float4*>(V.dh + row * H + col1);
                dhv[ps][0] = a.x; dhv[ps][1] = a.y; dhv[ps][2] = a.z; dhv[ps][3] = a.w;
                dhv[ps][4] = b.x; dhv[ps][5] = b.y; dhv[ps][6] = b.z; dhv[ps][7] = b.w;
                if (gather)
#pragma unroll
                    for (int k = 0; k < kMpnnMaxWidth; ++k) {
                        const int32_t e = (k < V.W) ? __ldg(V.nbr + (int64_t)k * F + row) : (int32_t)row;
                        nb[ps][k] = (e == (int32_t)row) ? -1 : e;
                    }
            }
        }
        if (gather)
#pragma unroll
            for (int ps = 0; ps < 2; ++ps) {
                uint2 g[kMpnnMaxWidth][2];
#pragma unroll
                for (int k = 0; k < kMpnnMaxWidth; ++k) {
                    const __nv_bfloat16* src = gin + (int64_t)(nb[ps][k] >= 0 ? nb[ps][k] : 0) * H;
                    g[k][0] = nb[ps][k] >= 0 ? __ldg(reinterpret_cast<const uint2*>(src + col0)) : make_uint2(0, 0);
                    g[k][1] = nb[ps][k] >= 0 ? __ldg(reinterpret_cast<const uint2*>(src + col1)) : make_uint2(0, 0);
                }
#pragma unroll
                for (int k = 0; k < kMpnnMaxWidth; ++k)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const float2 lo = unpack_bf16(g[k][h].x), hi = unpack_bf16(g[k][h].y);
                        dhv[ps][4 * h] += lo.x;
                        dhv[ps][4 * h + 1] += lo.y;
                        dhv[ps][4 * h + 2] += hi.x;
                        dhv[ps][4 * h + 3] += hi.y;
                    }
            }
#pragma unroll
        for (int ps = 0; ps < 2; ++ps) {
            const int rl = slot + 64 * ps;
            const int64_t row = tile * TB + rl;
            uint2 out[2] = {make_uint2(0, 0), make_uint2(0, 0)};
            if (row < F) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int col = h ? col1 : col0;
                    const uint2 zz = *reinterpret_cast<const uint2*>(V.z[layer] + row * H + col);
                    const float2 z0 = unpack_bf16(zz.x), z1 = unpack_bf16(zz.y);
                    const float* d = dhv[ps] + 4 * h;
                    out[h] = make_uint2(pack_bf16(z0.x > 0 ? d[0] : 0.f, z0.y > 0 ? d[1] : 0.f),
                                        pack_bf16(z1.x > 0 ? d[2] : 0.f, z1.y > 0 ? d[3] : 0.f));
                    *reinterpret_cast<uint2*>(V.dz + row * H + col) = out[h];
                }
            }
            *reinterpret_cast<uint2*>(sA + tc::kmajor_offset(rl, col0, H)) = out[0];
            *reinterpret_cast<uint2*>(sA + tc::kmajor_offset(rl, col1, H)) = out[1];
        }
        if (!tile_mma<TB, 2 * H, H>(sA, sB, tbase, ts, false)) {
            if (tid == 0) atomicOr(V.err, 4);
            break;
        }
        // ---- epilogue, row-per-thread: dX into the staging tiles
        {
            const int64_t row = tile * TB + r;
            float acc[16];
            tc::tmem_ld_x16(tlane + 16 * qs, acc);
#pragma unroll
            for (int c = 0; c < 4; ++c)
                *reinterpret_cast<float4*>(sD + r * H + 4 * swz(r, 4 * qs + c)) =
                    make_float4(acc[4 * c], acc[4 * c + 1], acc[4 * c + 2], acc[4 * c + 3]);
            tc::tmem_ld_x16(tlane + H + 16 * qs, acc);
            const int d = row < F ? V.deg[row] : 0;
            const float inv = d > 0 ? 1.0f / (float)d : 0.f;
            uint32_t w[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) w[t] = pack_bf16(acc[2 * t] * inv, acc[2 * t + 1] * inv);
#pragma unroll
            for (int c = 0; c < 2; ++c)
                *reinterpret_cast<uint4*>(sA + r * (2 * H) + 16 * swz(r, 2 * qs + c)) =
                    make_uint4(w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]);
        }
        __syncthreads();
        // ---- row-coalesced writes: dH_l = dH + dX[:, :64], g_l
#pragma unroll
        for (int ps = 0; ps < 2; ++ps) {
            const int rl = slot + 64 * ps;
            const int64_t row = tile * TB + rl;
            if (row >= F) continue;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int col = h ? col1 : col0;
                const float4 x = *reinterpret_cast<const float4*>(sD + rl * H + 4 * swz(rl, col / 4));
                const float* d = dhv[ps] + 4 * h;
                *reinterpret_cast<float4*>(V.dh + row * H + col) = make_float4(d[0] + x.x, d[1] + x.y, d[2] + x.z, d[3] + x.w);
                const uint2 gv = *reinterpret_cast<const uint2*>(sA + rl * (2 * H) + 16 * swz(rl, col / 8) + 2 * (col & 7));
                *reinterpret_cast<uint2*>(gout + row * H + col) = gv;
            }
        }
        tile_done();
    }
    tile_done();
    if (warp == 0) tc::tmem_dealloc(tbase, 2 * H);
}

// Encoder: dz0 = dH_1 * (z0 > 0) in BF16, with dH_1 = the stored dH plus the
// neighbour sum of g_1 (as in k_mpnn_bwd_dx).  One thread per 8 columns of a face.
__global__ void __launch_bounds__(256) k_mpnn_dz0(const MpnnView V)
{
    const int64_t gid = (int64_t)blockIdx.x * 256 + threadIdx.x;
    const int64_t row = gid >> 3;
    const int col = (int)(gid & 7) * 8;
    if (row >= V.F) return;
    const __nv_bfloat16* gin = V.gb[1 & 1];  // written by layer 1
    float d[8];
    const float4 d0 = *reinterpret_cast<const float4*>(V.dh + row * H + col);
    const float4 d1 = *reinterpret_cast<const float4*>(V.dh + row * H + col + 4);
    d[0] = d0.x; d[1] = d0.y; d[2] = d0.z; d[3] = d0.w; d[4] = d1.x; d[5] = d1.y; d[6] = d1.z; d[7] = d1.w;
    uint4 g[kMpnnMaxWidth];
#pragma unroll
    for (int k = 0; k < kMpnnMaxWidth; ++k) {
        const int32_t e = (k < V.W) ? __ldg(V.nbr + (int64_t)k * V.F + row) : (int32_t)row;
        g[k] = e != (int32_t)row ? __ldg(reinterpret_cast<const uint4*>(gin + (int64_t)e * H + col)) : make_uint4(0, 0, 0, 0);
    }
#pragma unroll
    for (int k = 0; k < kMpnnMaxWidth; ++k) {
        const uint32_t w4[4] = {g[k].x, g[k].y, g[k].z, g[k].w};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const float2 f = unpack_bf16(w4[t]);
            d[2 * t] += f.x;
            d[2 * t + 1] += f.y;
        }
    }
    const uint4 zz = *reinterpret_cast<const uint4*>(V.z[0] + row * H + col);
    const uint32_t zw[4] = {zz.x, zz.y, zz.z, zz.w};
    uint32_t o[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const float2 z2 = unpack_bf16(zw[t]);
        o[t] = pack_bf16(z2.x > 0 ? d[2 * t] : 0.f, z2.y > 0 ? d[2 * t + 1] : 0.f);
    }
    *reinterpret_cast<uint4*>(V.dz + row * H + col) = make_uint4(o[0], o[1], o[2], o[3]);
}

// ---- backward: dW = X^T dZ (split over faces) -----------------------------------

// X = [h_l, a_l] (KF = 128) or x0 (KF = 16, zero-padded to 128 rows).  Each
// CTA accumulates dW over its tiles of 128 faces in TMEM (M = 128 features,
// N = 64 outputs, K = 128 faces), writes one FP32 partial (summed in a fixed
// order by k_mpnn_reduce_dw) and its share of db = the sum of dZ over faces.
// The MMA operands are K-major over the face index, the transpose of the
// face-major rows in global memory, so a tile is staged in two steps:
//  1. the CTA copies the tile's rows (X | dZ) with row-coalesced 16-byte
//     loads (eight lanes per 128-byte row) into a face-major shared tile;
//  2. each thread assembles 16-byte core-matrix rows (eight consecutive
//     faces of one feature) from it and stores them into the operand tiles:
//     a warp reads 32 consecutive features of one face per 2-byte load (no
//     bank conflicts) and each 8-lane phase of the 16-byte stores fills one
//     128-byte core matrix.
// (Loading with a row per thread and scattering 2-byte values into the
// operand tiles made every load touch 32 rows and every store conflict.)
template <int KF>
struct DwShape {
    static constexpr int XW = KF == 16 ? 16 : 2 * H;  // X columns of a staged face row
    static constexpr int ROW = XW + H + 8;             // staged row: X | dZ | 16 bytes of padding (bf16)
};
constexpr int kDwSmem = (TB + H) * TB * 2 + TB * DwShape<128>::ROW * 2;

template <int KF>
__global__ void __launch_bounds__(NT) k_mpnn_bwd_dw(const MpnnView V, int layer, float* partials)
{
    extern __shared__ __align__(128) uint8_t smem[];
    uint8_t* sA = smem;                // 128 features x 128 faces (K-major)
    uint8_t* sB = smem + TB * TB * 2;  // 64 outputs x 128 faces (K-major)
    uint8_t* sR = smem + (TB + H) * TB * 2;  // [128 faces][ROW] bf16, face-major
    constexpr int XW = DwShape<KF>::XW, ROW = DwShape<KF>::ROW;
    constexpr int XCH = XW / 8, RCH = XCH + H / 8;  // 16-byte chunks of X and of a staged row
    __shared__ uint64_t mbar;
    __shared__ uint32_t tbase;
    __shared__ float red[NT / 32][16];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int r = tid & (TB - 1), qs = tid >> 7;
    const int64_t F = V.F;
    if (KF < TB) {
        // rows KF..127 of the feature tile stay zero
        for (int idx = tid; idx < TB * TB / 8; idx += NT) {
            const int rr = idx / (TB / 8), k0 = (idx % (TB / 8)) * 8;
            st_tile(sA, rr, k0, TB, make_uint4(0, 0, 0, 0));
        }
    }
    if (warp == 0) {
        tc::tmem_alloc(&tbase, H);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(&mbar, 1);
    tile_done();
    TileSync ts{&mbar, 0};
    float dbs[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) dbs[q] = 0.f;
    const int64_t ntiles = (F + TB - 1) / TB;
    bool first = true;
    const __nv_bfloat16* hl = V.h[layer];
    const __nv_bfloat16* al = V.a[layer];
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        // 1. the tile's rows, row-coalesced, into the face-major staging tile
        for (int idx = tid; idx < TB * RCH; idx += NT) {
            const int f = idx / RCH, ch = idx - f * RCH;
            const int64_t row = tile * TB + f;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (row < F) {
                const __nv_bfloat16* src;
                if (ch >= XCH) src = V.dz + row * H + 8 * (ch - XCH);
                else if constexpr (KF == 16) src = V.x0 + row * 16 + 8 * ch;
                else src = ch < H / 8 ? hl + row * H + 8 * ch : al + row * H + 8 * (ch - H / 8);
                v = *reinterpret_cast<const uint4*>(src);
            }
            *reinterpret_cast<uint4*>(sR + (f * ROW + 8 * ch) * 2) = v;
        }
        __syncthreads();
        // 2. transpose into the K-major operand tiles: column c of the staged
        //    rows (X: feature c; dZ: output c - XW), faces 8 kg .. 8 kg + 7
        const uint16_t* sRh = reinterpret_cast<const uint16_t*>(sR);
        for (int idx = tid; idx < (XW + H) * (TB / 8); idx += NT) {
            const int kg = idx / (XW + H), c = idx - kg * (XW + H);
            uint32_t w[4];
#pragma unroll
            for (int j = 0; j < 4; ++j)
                w[j] = (uint32_t)sRh[(8 * kg + 2 * j) * ROW + c] | ((uint32_t)sRh[(8 * kg + 2 * j + 1) * ROW + c] << 16);
            const uint4 v = make_uint4(w[0], w[1], w[2], w[3]);
            if (c < XW) st_tile(sA, c, 8 * kg, TB, v);
            else st_tile(sB, c - XW, 8 * kg, TB, v);
        }
        // db: thread (r, qs) adds dZ[r][16 qs .. 16 qs + 15]
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const uint4 v = *reinterpret_cast<const uint4*>(sR + (r * ROW + XW + 16 * qs + 8 * c) * 2);
            const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const float2 f = unpack_bf16(w4[t]);
                dbs[8 * c + 2 * t] += f.x;
                dbs[8 * c + 2 * t + 1] += f.y;
            }
        }
        if (!tile_mma<TB, H, TB>(sA, sB, tbase, ts, !first)) {
            if (tid == 0) atomicOr(V.err, 4);
            break;
        }
        first = false;
        tile_done();
    }
    // partial dW: TMEM lane m = feature (row r of this thread), columns 16 qs ..
    float acc[16];
    if (first) {
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[q] = 0.f;
    }
    else
        tc::tmem_ld_x16(tbase + ((uint32_t)(32 * (warp & 3)) << 16) + 16 * qs, acc);
    float* P = partials + (int64_t)blockIdx.x * (TB * H + H);
#pragma unroll
    for (int c = 0; c < 4; ++c)
        *reinterpret_cast<float4*>(P + r * H + 16 * qs + 4 * c) =
            make_float4(acc[4 * c], acc[4 * c + 1], acc[4 * c + 2], acc[4 * c + 3]);
    // db partial: reduce over the 128 faces that share this thread's column slice
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        float v = dbs[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][q] = v;
    }
    tile_done();
    if (tid < H) {
        const int sq = tid / 16, j = tid % 16;
        float sum = 0;
        for (int w = 0; w < 4; ++w) sum += red[4 * sq + w][j];
        P[TB * H + tid] = sum;
    }
    if (warp == 0) tc::tmem_dealloc(tbase, H);
}

// Sums the per-CTA dW / db partials in a fixed order into the flat gradient.
__global__ void k_mpnn_reduce_dw(const float* partials, int nparts, int KF, float* gW, float* gb)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int total = KF * H + H;
    if (idx >= total) return;
    const int src = idx < KF * H ? idx : TB * H + (idx - KF * H);
    double s = 0;
    for (int p = 0; p < nparts; ++p) s += partials[(int64_t)p * (TB * H + H) + src];
    if (idx < KF * H) gW[idx] = (float)s;
    else gb[idx - KF * H] = (float)s;
}

__global__ void k_mpnn_reduce_dec(const double* partials, int nparts, float* gwd, float* gbd, double* loss,
                                  double inv_nt)
{
    const int idx = threadIdx.x;
    if (idx >= H + 2) return;
    double s = 0;
    for (int p = 0; p < nparts; ++p) s += partials[(int64_t)p * (H + 2) + idx];
    if (idx < H) gwd[idx] = (float)s;
    else if (idx == H) gbd[0] = (float)s;
    else *loss = s * inv_nt;  // mean over the training faces
}

// Adam on the FP32 master parameters, then the BF16 copies in both layouts.
__global__ void k_mpnn_adam(float* params, const float* grads, float* m1, float* m2, int n, float lr, float b1,
                            float b2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = grads[i];
    const float a = b1 * m1[i] + (1.f - b1) * g;
    const float b = b2 * m2[i] + (1.f - b2) * g * g;
    m1[i] = a;
    m2[i] = b;
    params[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

// w_fwd[n][k] = W[k][n] and w_bwd[k][n] = W[k][n] (BF16) for one layer.
__global__ void k_mpnn_publish(const float* W, int K, __nv_bfloat16* wf, __nv_bfloat16* wb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= K * H) return;
    const int k = i / H, n = i % H;
    const __nv_bfloat16 v = __float2bfloat16(W[i]);
    wf[n * K + k] = v;
    if (wb) wb[i] = v;
}

}  // namespace

// ---- launchers -----------------------------------------------------------------------

static int mpnn_grid(int64_t F)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t tiles = (F + TB - 1) / TB;
    const int64_t g = (int64_t)(sms > 0 ? sms : 152) * 4;
    return (int)(tiles < g ? (tiles > 0 ? tiles : 1) : g);
}

int mpnn_grid_size(int64_t F) { return mpnn_grid(F); }

// Dynamic shared memory limit of a kernel, with the carveout at its maximum
// so that the occupancy the registers allow is not cut by a small default
// shared-memory partition.
template <typename Kern>
static void set_smem(Kern k, int bytes)
{
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}

// Every tensor-core kernel requests at least this much shared memory, so at
// most 4 CTAs share an SM and their TMEM allocations (<= 128 columns each)
// never exceed the SM's 512 columns.
constexpr int kMinSmem = 56 * 1024;
static int smem_req(int need) { return need > kMinSmem ? need : kMinSmem; }

// Grid of a forward layer kernel: every CTA resident at once (the kernel
// loops over tiles), so no second wave waits for the first.
template <typename Kern>
static int resident_grid(Kern k, int smem, int64_t F)
{
    int dev = 0, sms = 0, regs_sm = 0, smem_sm = 0, thr_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
    cudaFuncAttributes fa{};
    int per_sm = 1;
    if (cudaFuncGetAttributes(&fa, k) == cudaSuccess && fa.numRegs > 0) {
        // registers are allocated per warp in units of 256
        const int regs_warp = ((fa.numRegs * 32 + 255) / 256) * 256;
        const int by_regs = regs_sm / (regs_warp * (NT / 32));
        const int by_smem = smem_sm / ((int)fa.sharedSizeBytes + smem + 1024);  // 1 KB reserved per CTA
        const int by_thr = thr_sm / NT;
        per_sm = by_regs < by_smem ? by_regs : by_smem;
        per_sm = per_sm < by_thr ? per_sm : by_thr;
    }
    if (per_sm < 1) per_sm = 1;
    if (per_sm > 4) per_sm = 4;  // TMEM: at most 4 CTAs x 128 columns per SM
    const int64_t tiles = (F + TB - 1) / TB;
    const int64_t g = (int64_t)(sms > 0 ? sms : 152) * per_sm;
    return (int)(tiles < g ? (tiles > 0 ? tiles : 1) : g);
}

// Shared memory of a forward layer: A and B tiles, the output staging tile
// and, in training, the pre-activation staging tile.
static int layer_smem(int kin, bool train)
{
    return smem_req((TB + H) * kin * 2 + (train ? 2 : 1) * TB * kOutStride);
}

template <bool TRAIN>
static void forward_layers(const MpnnView& V, cudaStream_t s)
{
    const int sm16 = layer_smem(16, TRAIN), sm128 = layer_smem(128, TRAIN);
    set_smem(k_mpnn_layer<16, TRAIN>, sm16);
    set_smem(k_mpnn_layer<128, TRAIN>, sm128);
    k_mpnn_layer<16, TRAIN><<<resident_grid(k_mpnn_layer<16, TRAIN>, sm16, V.F), NT, sm16, s>>>(V, 0);
    const int g = resident_grid(k_mpnn_layer<128, TRAIN>, sm128, V.F);
    for (int l = 1; l <= kMpnnLayers; ++l) k_mpnn_layer<128, TRAIN><<<g, NT, sm128, s>>>(V, l);
}

void mpnn_forward(const MpnnView& V, bool train, cudaStream_t s)
{
    if (train) forward_layers<true>(V, s);
    else forward_layers<false>(V, s);
}

void mpnn_infer_guess(const MpnnView& V, cudaStream_t s)
{
    const int sm16 = layer_smem(16, false), sm128 = layer_smem(128, false);
    set_smem(k_mpnn_layer<16, false>, sm16);
    set_smem(k_mpnn_layer<128, false>, sm128);
    set_smem(k_mpnn_layer<128, false, true>, sm128);
    k_mpnn_layer<16, false><<<resident_grid(k_mpnn_layer<16, false>, sm16, V.F), NT, sm16, s>>>(V, 0);
    const int g = resident_grid(k_mpnn_layer<128, false>, sm128, V.F);
    for (int l = 1; l < kMpnnLayers; ++l) k_mpnn_layer<128, false><<<g, NT, sm128, s>>>(V, l);
    k_mpnn_layer<128, false, true><<<resident_grid(k_mpnn_layer<128, false, true>, sm128, V.F), NT, sm128, s>>>(
        V, kMpnnLayers);
}

void mpnn_backward(const MpnnView& V, const double* target, double inv_nt, MpnnGrads& G, cudaStream_t s)
{
    const int gdec = mpnn_grid(V.F);
    k_mpnn_decode<<<gdec, 256, 0, s>>>(V, target, inv_nt);
    k_mpnn_reduce_dec<<<1, 128, 0, s>>>(V.dec_partials, gdec, G.g + G.off_wd, G.g + G.off_bd, G.loss, inv_nt);
    const int smdx = smem_req(kDxSmem);
    const int smdw = smem_req(kDwSmem);
    set_smem(k_mpnn_bwd_dx, smdx);
    set_smem(k_mpnn_bwd_dw<128>, smdw);
    set_smem(k_mpnn_bwd_dw<16>, smdw);
    // one resident wave each; the dW partials (one per CTA) fit the buffer
    // sized for mpnn_grid, which resident_grid never exceeds (<= 4 CTAs/SM)
    const int gdx = resident_grid(k_mpnn_bwd_dx, smdx, V.F);
    const int gdw = resident_grid(k_mpnn_bwd_dw<128>, smdw, V.F);
    const int gdw0 = resident_grid(k_mpnn_bwd_dw<16>, smdw, V.F);
    for (int l = kMpnnLayers; l >= 1; --l) {
        k_mpnn_bwd_dx<<<gdx, NT, smdx, s>>>(V, l);
        k_mpnn_bwd_dw<128><<<gdw, NT, smdw, s>>>(V, l, G.partials);
        k_mpnn_reduce_dw<<<(2 * H * H + H + 255) / 256, 256, 0, s>>>(G.partials, gdw, 2 * H, G.g + G.off_W[l],
                                                                      G.g + G.off_b[l]);
    }
    k_mpnn_dz0<<<(unsigned)((V.F * (H / 8) + 255) / 256), 256, 0, s>>>(V);
    k_mpnn_bwd_dw<16><<<gdw0, NT, smdw, s>>>(V, 0, G.partials);
    k_mpnn_reduce_dw<<<(16 * H + H + 255) / 256, 256, 0, s>>>(G.partials, gdw0, 16, G.g + G.off_W[0],
                                                              G.g + G.off_b[0]);
}

void mpnn_adam(float* params, const float* grads, float* m1, float* m2, int n, float lr, int t, cudaStream_t s)
{
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
    k_mpnn_adam<<<(n + 255) / 256, 256, 0, s>>>(params, grads, m1, m2, n, lr, b1, b2, 1e-8f, c1, c2);
}

void mpnn_publish(const float* W, int K, __nv_bfloat16* wf, __nv_bfloat16* wb, cudaStream_t s)
{
    k_mpnn_publish<<<(K * H + 255) / 256, 256, 0, s>>>(W, K, wf, wb);
}

int mpnn_partials_floats(int64_t F) { return mpnn_grid(F) * (TB * H + H); }

}  // namespace mhfem
