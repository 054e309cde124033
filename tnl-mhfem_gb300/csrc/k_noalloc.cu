// Allocation-free FP64 BiCGStab over a caller-owned system.
//
// Who needs it: applications whose device memory is owned by their own pool
// allocator -- a TNL application or a larger simulation framework that
// hands every buffer out of one pre-reserved arena -- cannot let a library
// call cudaMalloc or cudaFree behind their back: it would bypass their
// memory accounting, and allocating or freeing device memory synchronizes
// the device, which stalls their other streams.  They own the matrix, the
// right-hand side and the solution; this entry point borrows nothing else.
//
// The Krylov work vectors, the per-CTA partial sums and the device scalars
// live in one file-scope static device array of fixed size (about 17 MB).
// Every system it takes fits the persistent small-system solve (one
// cooperative launch per chunk of 256 iterations, the convergence test in
// every iteration), which mhfem_solve runs for the same sizes.
// Under CUDA's lazy module loading the array is committed on a device at the
// first call there (the cudaGetSymbolAddress below loads the module), not when
// the library is loaded, and it stays until the process exits; systems with
// more than MHFEM_NOALLOC_MAX_ROWS rows are rejected.
#include <chrono>
#include <mutex>

#include "handle.h"
#include "mhfem_internal.h"

namespace {

constexpr int64_t kMaxRows = MHFEM_NOALLOC_MAX_ROWS;   // even: the vectors below are spaced by an even count
constexpr int64_t kMaxGrid = 4096;                     // per-CTA partials (>= any Krylov grid here)
constexpr int64_t kVecDoubles = 8 * kMaxRows;          // r, rh, p, v, s, t and the second p, v buffers
constexpr int64_t kPartialDoubles = 8 * kMaxGrid;
constexpr int64_t kScalarDoubles = (sizeof(mhfem::KrylovScalars) + 7) / 8;
// 8 uint32: [0] reduction ticket, [2] grid-barrier count and [3] its failure
// flag (the small-system solve), [4] bad-column count
constexpr int64_t kCounterDoubles = 4;
constexpr int kBadColumns = 4;
constexpr int64_t kScratchDoubles = kVecDoubles + kPartialDoubles + kScalarDoubles + kCounterDoubles;

// The scratch.  Host code must not use this name as a device address: in host
// code it is a host-side stand-in.  Its device address comes from
// cudaGetSymbolAddress, once per device, below.
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_addr[kMaxDevices] = {};

// Device address of the scratch on the current device (set-up on first use).
cudaError_t scratch_address(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = static_cast<double*>(p);
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

// Counts the ELL column indices outside [0, rows) into *bad.  The solve's
// SpMVs gather x[col] without a bounds test, so the caller's columns are
// checked before any of them runs.
__global__ void __launch_bounds__(256) k_check_cols(const int32_t* __restrict__ cols, int64_t count, int64_t rows,
                                                    uint32_t* bad)
{
    int mine = 0;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < count; q += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = __ldg(cols + q);
        if (c < 0 || (int64_t)c >= rows) mine = 1;
    }
    const int n = __syncthreads_count(mine);
    if (threadIdx.x == 0 && n > 0) atomicAdd(bad, (uint32_t)n);
}

double elapsed_s(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" mhfem_status mhfem_bicgstab_noalloc(const int32_t* cols, const double* vals, int32_t width, int64_t rows,
                                               const double* rhs, double* x, double tol, int32_t max_iter,
                                               double timeout_s, int32_t* iterations, double* residual, void* stream)
{
    if (rows < 1 || rows > kMaxRows) return MHFEM_ERR_INVALID_ARGUMENT;  // beyond the scratch size
    if (width < 0 || !rhs || !x || (width > 0 && (!cols || !vals))) return MHFEM_ERR_INVALID_ARGUMENT;
    if (!(tol > 0) || max_iter < 1) return MHFEM_ERR_INVALID_ARGUMENT;
    const auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* base = nullptr;
    if (scratch_address(&base) != cudaSuccess) return MHFEM_ERR_CUDA;

    mhfem::EllMatrix A;
    A.rows = rows;
    A.width = width;
    A.cols = const_cast<int32_t*>(cols);
    A.vals = const_cast<double*>(vals);
    mhfem::KrylovWork W;
    W.rows = rows;
    W.grid = mhfem::krylov_grid();
    // vectors spaced by an even row count, so each starts on a 16-byte
    // boundary and the updates keep their 16-byte accesses for odd row counts
    const int64_t ld = (rows + 1) & ~int64_t(1);
    W.r = base;
    W.rh = base + ld;
    W.p = base + 2 * ld;
    W.v = base + 3 * ld;
    W.s = base + 4 * ld;
    W.t = base + 5 * ld;
    W.p2 = base + 6 * ld;
    W.v2 = base + 7 * ld;
    W.partials = base + kVecDoubles;
    W.sc = reinterpret_cast<mhfem::KrylovScalars*>(base + kVecDoubles + kPartialDoubles);
    W.counters = reinterpret_cast<uint32_t*>(base + kVecDoubles + kPartialDoubles + kScalarDoubles);
    if (W.grid > kMaxGrid) return MHFEM_ERR_UNSUPPORTED;

    // the ticket counter, the barrier words and the bad-column count must
    // start at zero; every other scratch word is written before it is read
    if (cudaMemsetAsync(W.counters, 0, kCounterDoubles * sizeof(double), s) != cudaSuccess) return MHFEM_ERR_CUDA;
    if (width > 0) {
        const int64_t count = (int64_t)width * rows;
        const unsigned grid = (unsigned)std::min<int64_t>((count + 255) / 256, 1024);
        k_check_cols<<<grid, 256, 0, s>>>(cols, count, rows, W.counters + kBadColumns);
        if (cudaGetLastError() != cudaSuccess) return MHFEM_ERR_CUDA;
        uint32_t bad = 0;
        if (cudaMemcpyAsync(&bad, W.counters + kBadColumns, sizeof(bad), cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return MHFEM_ERR_CUDA;
        if (cudaStreamSynchronize(s) != cudaSuccess) return MHFEM_ERR_CUDA;
        if (bad != 0) return MHFEM_ERR_INVALID_ARGUMENT;  // a column outside [0, rows): nothing else was queued
    }
    mhfem::krylov_init_fp64(A, rhs, x, W, tol, max_iter, s);
    if (cudaGetLastError() != cudaSuccess) return MHFEM_ERR_CUDA;
    bool small = rows <= mhfem::krylov_small_rows();  // always, at this size limit
    mhfem::KrylovScalars hs{};
    int32_t barrier_failed = 0;
    for (bool first = true;; first = false) {
        if (cudaMemcpyAsync(&hs, W.sc, sizeof(hs), cudaMemcpyDeviceToHost, s) != cudaSuccess) return MHFEM_ERR_CUDA;
        if (small && cudaMemcpyAsync(&barrier_failed, W.counters + 3, sizeof(barrier_failed), cudaMemcpyDeviceToHost,
                                     s) != cudaSuccess)
            return MHFEM_ERR_CUDA;
        if (cudaStreamSynchronize(s) != cudaSuccess) return MHFEM_ERR_CUDA;
        if (barrier_failed) return MHFEM_ERR_CUDA;  // a grid barrier wait ran out (the context stays usable)
        if (hs.done) break;
        // the stream has drained here, so the shared scratch is idle when the limit ends the call
        if (timeout_s > 0 && elapsed_s(t0) > timeout_s) {
            if (iterations) *iterations = hs.it;
            if (residual) *residual = hs.res;
            return MHFEM_ERR_TIMEOUT;
        }
        if (small) {
            const cudaError_t e = mhfem::krylov_small_fp64(A, x, W, 256, s);
            if (first && e == cudaErrorCooperativeLaunchTooLarge) {
                // the device cannot hold the grid at once (a partitioned or
                // shared GPU): nothing ran, the five-kernel iteration goes on
                cudaGetLastError();
                small = false;
            }
            else if (e != cudaSuccess)
                return MHFEM_ERR_CUDA;
        }
        if (!small) mhfem::krylov_iterate_fp64(A, x, W, 8, s);
        if (cudaGetLastError() != cudaSuccess) return MHFEM_ERR_CUDA;
    }
    if (iterations) *iterations = hs.it;
    if (residual) *residual = hs.res;
    switch (hs.status) {
        case mhfem::KS_CONVERGED: return MHFEM_OK;
        case mhfem::KS_MAXITER: return MHFEM_ERR_NOT_CONVERGED;
        case mhfem::KS_BREAKDOWN: return MHFEM_ERR_BREAKDOWN;
        default: return MHFEM_ERR_NOT_FINITE;
    }
}
