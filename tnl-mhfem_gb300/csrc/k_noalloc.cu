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
// live in one file-scope static device array of fixed size: every GPU that
// loads the library holds it (about 12.8 MB) until the process exits, and
// systems with more than MHFEM_NOALLOC_MAX_ROWS rows are rejected.
#include <mutex>

#include "handle.h"
#include "mhfem_internal.h"

namespace {

constexpr int64_t kMaxRows = MHFEM_NOALLOC_MAX_ROWS;
constexpr int64_t kMaxGrid = 4096;                     // per-CTA partials (>= any Krylov grid here)
constexpr int64_t kVecDoubles = 6 * kMaxRows;          // r, rh, p, v, s, t
constexpr int64_t kPartialDoubles = 8 * kMaxGrid;
constexpr int64_t kScalarDoubles = (sizeof(mhfem::KrylovScalars) + 7) / 8;
constexpr int64_t kCounterDoubles = 2;                 // ticket counters (uint32)
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

}  // namespace

extern "C" mhfem_status mhfem_bicgstab_noalloc(const int32_t* cols, const double* vals, int32_t width, int64_t rows,
                                               const double* rhs, double* x, double tol, int32_t max_iter,
                                               int32_t* iterations, double* residual, void* stream)
{
    if (rows < 1 || rows > kMaxRows) return MHFEM_ERR_INVALID_ARGUMENT;  // beyond the scratch size
    if (width < 0 || !rhs || !x || (width > 0 && (!cols || !vals))) return MHFEM_ERR_INVALID_ARGUMENT;
    if (!(tol > 0) || max_iter < 1) return MHFEM_ERR_INVALID_ARGUMENT;
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
    W.r = base;
    W.rh = base + rows;
    W.p = base + 2 * rows;
    W.v = base + 3 * rows;
    W.s = base + 4 * rows;
    W.t = base + 5 * rows;
    W.partials = base + kVecDoubles;
    W.sc = reinterpret_cast<mhfem::KrylovScalars*>(base + kVecDoubles + kPartialDoubles);
    W.counters = reinterpret_cast<uint32_t*>(base + kVecDoubles + kPartialDoubles + kScalarDoubles);
    if (W.grid > kMaxGrid) return MHFEM_ERR_UNSUPPORTED;

    // the ticket counters must start at zero; every other scratch word is written before it is read
    if (cudaMemsetAsync(W.counters, 0, kCounterDoubles * sizeof(double), s) != cudaSuccess) return MHFEM_ERR_CUDA;
    mhfem::krylov_init_fp64(A, rhs, x, W, tol, max_iter, s);
    mhfem::KrylovScalars hs{};
    for (;;) {
        if (cudaMemcpyAsync(&hs, W.sc, sizeof(hs), cudaMemcpyDeviceToHost, s) != cudaSuccess) return MHFEM_ERR_CUDA;
        if (cudaStreamSynchronize(s) != cudaSuccess) return MHFEM_ERR_CUDA;
        if (hs.done) break;
        mhfem::krylov_iterate_fp64(A, x, W, 8, s);
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
