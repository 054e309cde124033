#pragma once
// Building blocks shared by the Krylov solvers (k_krylov.cu: BiCGStab, FP64
// and FP32; k_gmres.cu: restarted GMRES): launch shapes, deterministic
// block reductions with a last-block ticket, programmatic dependent launch,
// the unit-diagonal ELL row product and vector access helpers.
#include <mutex>
#include <unordered_map>
#include <utility>

#include "mhfem_internal.h"

namespace mhfem {

constexpr int KB = 256;

// SM count of a device (cached per device ordinal).
static int sm_count(int dev)
{
    static std::mutex mu;
    static std::unordered_map<int, int> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
    cache[dev] = sms;
    return sms;
}

// Grid of a grid-stride kernel on the current device: as many CTAs of KB
// threads as can be resident at once on every SM, at most 8 per SM (fixed per
// kernel and device, so reductions stay deterministic).
template <typename Kern>
static int occ_grid(Kern kernel)
{
    static std::mutex mu;
    static std::unordered_map<unsigned long long, int> cache;  // key: device ordinal, kernel address
    int dev = 0;
    cudaGetDevice(&dev);
    const int sms = sm_count(dev);
    std::lock_guard<std::mutex> lock(mu);
    const unsigned long long key = ((unsigned long long)(unsigned)dev << 48) ^ (unsigned long long)(uintptr_t)kernel;
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, KB, 0);
    const int g = sms * (nb > 0 ? (nb < 8 ? nb : 8) : 1);
    cache[key] = g;
    return g;
}

// Grid of a grid-stride kernel over `rows` rows: the resident wave
// (occ_grid), or fewer CTAs for a small system, so that every thread has at
// least kMinRowsPerThread rows.  A small system's kernels are bound by
// latency, and each reduction's last CTA then sums fewer partials (the
// 128^2 heat-equation system, 49,408 rows: 48 CTAs instead of 1,216).  The
// grid is fixed per kernel, device and row count, so reductions stay
// deterministic.
constexpr int kMinRowsPerThread = 4;

template <typename Kern>
static int row_grid(Kern kernel, int64_t rows)
{
    const int64_t per_cta = (int64_t)KB * kMinRowsPerThread;
    const int64_t need = (rows + per_cta - 1) / per_cta;
    const int64_t g = occ_grid(kernel);
    return (int)(need < 1 ? 1 : (need < g ? need : g));
}

// Launches an iteration kernel (at most one wave: row_grid CTAs) with
// programmatic stream serialization, so that its CTAs are scheduled while the
// preceding kernel of the iteration drains (the kernel itself waits for that
// kernel's results with griddepcontrol.wait).  Captured into a CUDA graph
// this becomes a programmatic dependency edge.
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kernel)(KArgs...), cudaStream_t s, int64_t grid_rows, Args&&... args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)row_grid(kernel, grid_rows));
    cfg.blockDim = dim3(KB);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Compile-time ELL widths (2f - 1) n - 1 of the common cases: triangles
// (4, 9), tetrahedra and rectangles (6, 13) with one or two components,
// cuboids with one (10); other widths (three components, two-component
// cuboids, meshes without interior faces) take the run-time loop.
#define MHFEM_WIDTH_DISPATCH(W, CALL)                                   \
    do {                                                                \
        switch (W) {                                                    \
            case 4: { constexpr int WW = 4; CALL; } break;              \
            case 6: { constexpr int WW = 6; CALL; } break;              \
            case 9: { constexpr int WW = 9; CALL; } break;              \
            case 10: { constexpr int WW = 10; CALL; } break;            \
            case 13: { constexpr int WW = 13; CALL; } break;            \
            default: { constexpr int WW = 0; CALL; } break;             \
        }                                                               \
    } while (0)
// restart threshold of |(rh, r)| relative to ||r|| ||rh|| (same as the oracle)
constexpr double kRestartEps = 1e-14;

// Per-block partial sums: up to kPartStride values per block.
constexpr int kPartStride = 8;

// FP64 sums: every thread parks its sums in shared memory and warp 0 adds
// them, each lane the KB/32 values of its column in order, then a shuffle
// tree; that is 12 FP64 additions per sum for the block, against 5 in each
// of the 8 warps plus 8 in thread 0 for a shuffle tree per warp.  The FP64
// pipe (about 2 operations per clock per SM on GB300) co-limits the FP64
// iteration kernels with HBM, and at one wave of CTAs over 3.2M rows those
// trees were about 12% of their FP64 operations.  FP32 sums keep the
// per-warp trees (their additions use the FP32 pipe).
template <typename T, int NV>
__device__ __forceinline__ void block_reduce_store(T (&acc)[NV], double* partials)
{
    static_assert(NV <= kPartStride, "too many partial sums");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if constexpr (sizeof(T) == 8) {
        __shared__ double col[NV][KB];
#pragma unroll
        for (int q = 0; q < NV; ++q) col[q][threadIdx.x] = acc[q];
        __syncthreads();
        if (warp == 0) {
#pragma unroll
            for (int q = 0; q < NV; ++q) {
                double v = col[q][lane];
#pragma unroll
                for (int w = 1; w < KB / 32; ++w) v += col[q][lane + 32 * w];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
                if (lane == 0) partials[(int64_t)blockIdx.x * kPartStride + q] = v;
            }
        }
    }
    else {
        __shared__ double sh[KB / 32][kPartStride];
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            T v = acc[q];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) sh[warp][q] = (double)v;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
#pragma unroll
            for (int q = 0; q < NV; ++q) {
                double s = 0;
                for (int w = 0; w < KB / 32; ++w) s += sh[w][q];
                partials[(int64_t)blockIdx.x * kPartStride + q] = s;
            }
        }
    }
}

// Returns true in the last block to finish; that block then sees every
// partial.  Thread 0 wrote this block's partial, so only thread 0 fences
// before taking its ticket (the other threads' stores need no ordering: the
// last block reads partials only).  The counter is reset for the next launch.
__device__ __forceinline__ bool ticket_last(uint32_t* counter)
{
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t prev = atomicAdd(counter, 1u);
        last = (prev == gridDim.x - 1);
        if (last) *counter = 0;
    }
    __syncthreads();
    return last;
}

// Deterministic sum of the partials by the last block (fixed order): every
// thread issues its (at most four per pass) partial loads together, the warp
// sums them with shuffles and warp 0 adds the eight warp sums in order.
template <int NV>
__device__ __forceinline__ void final_sums(const double* partials, double (&out)[NV])
{
    __shared__ double sh[KB / 32][kPartStride];
    double acc[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) acc[q] = 0;
    const int nb = (int)gridDim.x;
    for (int b0 = threadIdx.x; b0 < nb; b0 += 4 * KB) {
        double v[4][NV];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int b = b0 + j * KB;
#pragma unroll
            for (int q = 0; q < NV; ++q) v[j][q] = (b < nb) ? __ldcg(partials + (int64_t)b * kPartStride + q) : 0.0;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < NV; ++q) acc[q] += v[j][q];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double v = acc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[warp][q] = v;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double t = 0;
#pragma unroll
        for (int w = 0; w < KB / 32; ++w) t += sh[w][q];
        out[q] = t;
    }
}

// Programmatic dependent launch: the iteration kernels are launched with
// programmatic stream serialization, so the next kernel's CTAs are scheduled
// while this one drains.  pdl_wait() blocks until the preceding kernel has
// completed and its writes are visible (a no-op for an ordinary launch);
// every kernel calls it before its first global access and releases its
// dependent right after.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// y_r = x_r + sum_k vals[k][r] x[cols[k][r]] (unit diagonal).  With a
// compile-time width WW every column and value load of the row is issued
// before the gathers, so all of a row's memory accesses are in flight at once.
// The ELL words are streaming loads (evict-first, see ldv_stream below).
template <typename T, int WW>
__device__ __forceinline__ T spmv_row(const int32_t* __restrict__ cols, const T* __restrict__ vals, int W,
                                      int64_t rows, int64_t r, const T* __restrict__ x)
{
    if constexpr (WW > 0) {
        int32_t c[WW];
        T v[WW];
#pragma unroll
        for (int k = 0; k < WW; ++k) {
            c[k] = __ldcs(cols + (int64_t)k * rows + r);
            v[k] = __ldcs(vals + (int64_t)k * rows + r);
        }
        T xg[WW];
#pragma unroll
        for (int k = 0; k < WW; ++k) xg[k] = x[c[k]];
        T y = x[r];
#pragma unroll
        for (int k = 0; k < WW; ++k) y = fma(v[k], xg[k], y);
        return y;
    }
    else {
        T y = x[r];
        for (int k = 0; k < W; ++k) {
            const int64_t o = (int64_t)k * rows + r;
            y = fma(__ldcs(vals + o), x[__ldcs(cols + o)], y);
        }
        return y;
    }
}

__device__ __forceinline__ bool finite(double v) { return isfinite(v); }

// ---- vector access -------------------------------------------------------------
//
// The iteration kernels move V consecutive rows per thread and access (float4,
// double2: 16-byte loads and stores) so that enough bytes are in flight per SM
// to saturate HBM; the SpMVs of the FP32 solve also process RPT consecutive
// rows per thread, loading each ELL slot of the RPT rows as one 16-byte word.
// The host picks V and RPT from the pointers' alignment and the row count.

template <typename T, int V>
struct alignas(sizeof(T) * V) VecT {
    T v[V];
};

template <typename T, int V>
__device__ __forceinline__ VecT<T, V> ldv(const T* p, int64_t q)
{
    return *reinterpret_cast<const VecT<T, V>*>(p + q * V);
}

// The ELL matrix is read once per SpMV and is larger than L2: its words are
// loaded with the streaming (evict-first) policy, ld.global.cs, so that they
// do not evict the vectors the next kernels of the iteration read.  Measured
// on the 64^3 tetrahedral workload: FP64 iteration 197.3 -> 189.3 us, FP32
// inner iteration of the mixed form 108.9 -> 98.2 us (its seven FP32
// vectors then stay in L2).
template <typename T, int V>
__device__ __forceinline__ VecT<T, V> ldv_stream(const T* p, int64_t q)
{
    const T* a = p + q * V;
    VecT<T, V> r;
    if constexpr (sizeof(T) * V == 16) {
        const int4 w = __ldcs(reinterpret_cast<const int4*>(a));
        memcpy(&r, &w, 16);
    }
    else if constexpr (sizeof(T) * V == 8) {
        const int2 w = __ldcs(reinterpret_cast<const int2*>(a));
        memcpy(&r, &w, 8);
    }
    else {
        static_assert(sizeof(T) * V == 4, "4, 8 or 16 bytes");
        const int w = __ldcs(reinterpret_cast<const int*>(a));
        memcpy(&r, &w, 4);
    }
    return r;
}

template <typename T, int V>
__device__ __forceinline__ void stv(T* p, int64_t q, const VecT<T, V>& x)
{
    *reinterpret_cast<VecT<T, V>*>(p + q * V) = x;
}

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// ---- persistent small-system solves: bounded grid barriers, sums in CTA order,
// gathered SpMV rows (k_bicgstab_small, k_gmres_small) ---------------------------
//
// Every barrier wait is bounded: a CTA that polls kBarrierPolls times
// records the failure in *bar_err and returns, and the others then fail
// their next wait at once.

constexpr unsigned int kBarrierPolls = 1u << 22;  // seconds, far beyond any barrier of a working launch

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p)
{
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Arrive at the grid barrier whose cumulative arrival count is `target`
// (the count starts at 0 for a launch and grows by gridDim.x per barrier)
// and wait for every CTA.  False (in every thread of the CTA) when the wait
// gave up.
__device__ __forceinline__ bool grid_barrier(unsigned int* count, int* err, unsigned int target,
                                             unsigned int max_polls = kBarrierPolls)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int good = 1;
        __threadfence();
        // the last CTA to arrive sees the target in its own add and does not
        // poll: it is the one the others wait for in the next phase too
        const unsigned int seen = atomicAdd(count, 1u) + 1u;
        unsigned int polls = 0;
        while (seen < target && ld_acquire_u32(count) < target) {
            if (++polls > max_polls || *(volatile int*)err != 0) {
                good = 0;
                atomicExch(err, 1);
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// Sum of the per-CTA partials [cta][kPartStride] in CTA order, identical in
// every CTA (same loads, same order); the result is in out[] of every thread.
template <int NV>
__device__ __forceinline__ void grid_sums(const double* partials, double (&out)[NV])
{
    __shared__ double col[NV][KB];
    __shared__ double tot[NV];
    const int nb = (int)gridDim.x;
#pragma unroll
    for (int q = 0; q < NV; ++q)
        col[q][threadIdx.x] = threadIdx.x < nb ? __ldcg(partials + (int64_t)threadIdx.x * kPartStride + q) : 0.0;
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double v = col[q][lane];
#pragma unroll
            for (int w = 1; w < KB / 32; ++w) v += col[q][lane + 32 * w];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) tot[q] = v;
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) out[q] = tot[q];
}

// y = self + sum_k a_k g(c_k), where g(j) forms the gathered vector's value
// at row j (loaded past L1); same operation order as spmv_rows, so the
// products match the five-kernel path's.
template <int WW, typename G>
__device__ __forceinline__ double small_row(const int32_t* __restrict__ cols, const double* __restrict__ vals, int W,
                                            int64_t rows, int64_t q, double self, G&& g)
{
    double acc = self;
    if constexpr (WW > 0) {
        int32_t c[WW];
        double a[WW], xg[WW];
#pragma unroll
        for (int k = 0; k < WW; ++k) {
            c[k] = __ldg(cols + (int64_t)k * rows + q);
            a[k] = __ldg(vals + (int64_t)k * rows + q);
        }
#pragma unroll
        for (int k = 0; k < WW; ++k) xg[k] = g(c[k]);
#pragma unroll
        for (int k = 0; k < WW; ++k) acc = fma(a[k], xg[k], acc);
    }
    else
        for (int k = 0; k < W; ++k) {
            const int64_t o = (int64_t)k * rows + q;
            acc = fma(__ldg(vals + o), g(__ldg(cols + o)), acc);
        }
    return acc;
}

}  // namespace mhfem
