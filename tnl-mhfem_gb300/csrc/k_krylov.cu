// BiCGStab on the unit-diagonal face system (sm_103a), FP64 and FP32.
//
// Replaces the TNL Krylov solve of Solver::solveLinearSystem
// (Solver.hpp:1230-1264; solver and preconditioner from configSetup.h:32-62).
// Every row of the assembled system has a unit diagonal (LinearSystem.h:196-201,
// BoundaryConditions.hpp:200-203, 367-377), so the "diagonal" (Jacobi)
// preconditioner is the identity and the SpMV is y = x + offdiag(A) x.
//
// Design for GB300:
//  - the SpMV reads the ELL off-diagonal part column-major (coalesced) and
//    fuses the following dot product(s); BLAS-1 updates fuse their dots;
//  - every reduction is deterministic: a fixed grid, one partial per block,
//    and the last block to finish (atomic ticket) sums the partials in a
//    fixed order and computes the next Krylov scalar on the device, so an
//    iteration needs no host round trip;
//  - every kernel returns at once when the device "done" flag is set, so the
//    host may launch (or replay as a CUDA graph) several iterations between
//    convergence checks;
//  - FP32 kernels accumulate per-thread sums in FP32 and block sums in FP64:
//    GB300 issues FP64 at 1/57 of the FP32 rate.
#include <mutex>
#include <unordered_map>

#include "mhfem_internal.h"

namespace mhfem {

static int g_grid = 0;

int krylov_grid()
{
    if (g_grid == 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        g_grid = (sms > 0 ? sms : 152) * 8;  // 8 x 256 threads = full occupancy
    }
    return g_grid;
}

constexpr int KB = 256;

// Grid of a grid-stride kernel: as many CTAs of KB threads as can be resident
// at once on every SM (fixed per kernel and device, so reductions stay
// deterministic).
template <typename Kern>
static int occ_grid(Kern kernel)
{
    static std::mutex mu;
    static std::unordered_map<const void*, int> cache;
    static int sms = 0;
    std::lock_guard<std::mutex> lock(mu);
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 152;
    }
    auto it = cache.find((const void*)kernel);
    if (it != cache.end()) return it->second;
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, KB, 0);
    const int g = sms * (nb > 0 ? (nb < 8 ? nb : 8) : 1);
    cache[(const void*)kernel] = g;
    return g;
}

// Compile-time ELL widths of the supported cell types: (2f - 1) n - 1 for
// triangles / tetrahedra with one or two components; other widths (meshes
// without interior faces) take the run-time loop.
#define MHFEM_WIDTH_DISPATCH(W, CALL)                                   \
    do {                                                                \
        switch (W) {                                                    \
            case 4: { constexpr int WW = 4; CALL; } break;              \
            case 6: { constexpr int WW = 6; CALL; } break;              \
            case 9: { constexpr int WW = 9; CALL; } break;              \
            case 13: { constexpr int WW = 13; CALL; } break;            \
            default: { constexpr int WW = 0; CALL; } break;             \
        }                                                               \
    } while (0)
// restart threshold of |(rh, r)| relative to ||r|| ||rh|| (same as the oracle)
constexpr double kRestartEps = 1e-14;

template <typename T, int NV>
__device__ __forceinline__ void block_reduce_store(T (&acc)[NV], double* partials)
{
    __shared__ double sh[KB / 32][4];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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
            partials[(int64_t)blockIdx.x * 4 + q] = s;
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

// Deterministic sum of the partials by the last block (fixed order).
template <int NV>
__device__ __forceinline__ void final_sums(const double* partials, double (&out)[NV])
{
    __shared__ double sh[KB][4];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = 0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += KB) s += __ldcg(partials + (int64_t)b * 4 + q);
        sh[threadIdx.x][q] = s;
    }
    __syncthreads();
    for (int w = KB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
#pragma unroll
            for (int q = 0; q < NV; ++q) sh[threadIdx.x][q] += sh[threadIdx.x + w][q];
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < NV; ++q) out[q] = sh[0][q];
}

// y_r = x_r + sum_k vals[k][r] x[cols[k][r]] (unit diagonal).  With a
// compile-time width WW every column and value load of the row is issued
// before the gathers, so all of a row's memory accesses are in flight at once.
template <typename T, int WW>
__device__ __forceinline__ T spmv_row(const int32_t* __restrict__ cols, const T* __restrict__ vals, int W,
                                      int64_t rows, int64_t r, const T* __restrict__ x)
{
    if constexpr (WW > 0) {
        int32_t c[WW];
        T v[WW];
#pragma unroll
        for (int k = 0; k < WW; ++k) {
            c[k] = __ldg(cols + (int64_t)k * rows + r);
            v[k] = __ldg(vals + (int64_t)k * rows + r);
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
            y = fma(__ldg(vals + o), x[__ldg(cols + o)], y);
        }
        return y;
    }
}

__device__ __forceinline__ bool finite(double v) { return isfinite(v); }

// r = b - A x ; rh = r ; p = r ; partials: r.r, b.b
template <typename T, int WW>
__global__ void __launch_bounds__(KB) k_init(const int32_t* cols, const T* vals, int W, int64_t rows,
                                             const T* b, const T* x, T* r, T* rh, T* p,
                                             KrylovScalars* sc, double* partials, uint32_t* counter)
{
    T acc[2] = {0, 0};
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
        const T rv = b[q] - spmv_row<T, WW>(cols, vals, W, rows, q, x);
        r[q] = rv; rh[q] = rv; p[q] = rv;
        acc[0] = fma(rv, rv, acc[0]);
        acc[1] = fma(b[q], b[q], acc[1]);
    }
    block_reduce_store<T, 2>(acc, partials);
    if (!ticket_last(counter)) return;
    double s[2];
    final_sums<2>(partials, s);
    if (threadIdx.x == 0) {
        double bn = sqrt(s[1]);
        if (bn == 0) bn = 1;
        sc->bnorm = bn;
        sc->rho = s[0];
        sc->rhnorm = sqrt(s[0]);
        sc->restart = 0;
        sc->res = sqrt(s[0]) / bn;
        sc->it = 0;
        sc->snorm = 0;
        sc->status = KS_RUNNING;
        sc->done = 0;
        if (!finite(sc->res)) { sc->status = KS_NOTFINITE; sc->done = 1; }
        else if (sc->res < sc->tol) { sc->status = KS_CONVERGED; sc->done = 1; }
    }
}

// v = A p ; alpha = rho / (rh . v)
template <typename T, int WW>
__global__ void __launch_bounds__(KB) k_spmv_dot(const int32_t* cols, const T* vals, int W, int64_t rows,
                                                 const T* p, const T* rh, T* v,
                                                 KrylovScalars* sc, double* partials, uint32_t* counter)
{
    if (*(volatile int32_t*)&sc->done) return;
    T acc[1] = {0};
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
        const T y = spmv_row<T, WW>(cols, vals, W, rows, q, p);
        v[q] = y;
        acc[0] = fma(rh[q], y, acc[0]);
    }
    block_reduce_store<T, 1>(acc, partials);
    if (!ticket_last(counter)) return;
    double s[1];
    final_sums<1>(partials, s);
    if (threadIdx.x == 0) {
        sc->rv = s[0];
        if (!finite(s[0])) { sc->status = KS_NOTFINITE; sc->done = 1; }
        else if (s[0] == 0) { sc->status = KS_BREAKDOWN; sc->done = 1; }
        else sc->alpha = sc->rho / s[0];
    }
}

// s = r - alpha v ; ||s||
template <typename T>
__global__ void __launch_bounds__(KB) k_update_s(int64_t rows, const T* r, const T* v, T* s,
                                                 KrylovScalars* sc, double* partials, uint32_t* counter)
{
    if (*(volatile int32_t*)&sc->done) return;
    const T alpha = (T)sc->alpha;
    T acc[1] = {0};
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
        const T sv = fma(-alpha, v[q], r[q]);
        s[q] = sv;
        acc[0] = fma(sv, sv, acc[0]);
    }
    block_reduce_store<T, 1>(acc, partials);
    if (!ticket_last(counter)) return;
    double sum[1];
    final_sums<1>(partials, sum);
    if (threadIdx.x == 0) sc->snorm = sqrt(sum[0]) / sc->bnorm;
}

// t = A s ; omega = (t.s)/(t.t)  (skipped when ||s|| already meets the tolerance)
template <typename T, int WW>
__global__ void __launch_bounds__(KB) k_spmv_dots2(const int32_t* cols, const T* vals, int W, int64_t rows,
                                                   const T* s, T* t,
                                                   KrylovScalars* sc, double* partials, uint32_t* counter)
{
    if (*(volatile int32_t*)&sc->done) return;
    if (sc->snorm < sc->tol) return;
    T acc[2] = {0, 0};
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
        const T y = spmv_row<T, WW>(cols, vals, W, rows, q, s);
        t[q] = y;
        acc[0] = fma(y, s[q], acc[0]);
        acc[1] = fma(y, y, acc[1]);
    }
    block_reduce_store<T, 2>(acc, partials);
    if (!ticket_last(counter)) return;
    double sum[2];
    final_sums<2>(partials, sum);
    if (threadIdx.x == 0) {
        sc->ts = sum[0];
        sc->tt = sum[1];
        if (!finite(sum[0]) || !finite(sum[1])) { sc->status = KS_NOTFINITE; sc->done = 1; }
        else if (sum[1] == 0) { sc->status = KS_BREAKDOWN; sc->done = 1; }
        else sc->omega = sum[0] / sum[1];
    }
}

// x += alpha p + omega s ; r = s - omega t ; rho_new = rh.r ; ||r|| ; beta
template <typename T>
__global__ void __launch_bounds__(KB) k_update_xr(int64_t rows, T* x, const T* p, const T* s, const T* t,
                                                  T* r, const T* rh,
                                                  KrylovScalars* sc, double* partials, uint32_t* counter)
{
    if (*(volatile int32_t*)&sc->done) return;
    const T alpha = (T)sc->alpha;
    if (sc->snorm < sc->tol) {
        // early exit on the half step: x += alpha p
        for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB)
            x[q] = fma(alpha, p[q], x[q]);
        if (!ticket_last(counter)) return;
        if (threadIdx.x == 0) {
            sc->res = sc->snorm;
            sc->it += 1;
            sc->status = KS_CONVERGED;
            sc->done = 1;
        }
        return;
    }
    const T omega = (T)sc->omega;
    T acc[2] = {0, 0};
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
        const T sv = s[q];
        x[q] = fma(omega, sv, fma(alpha, p[q], x[q]));
        const T rv = fma(-omega, t[q], sv);
        r[q] = rv;
        acc[0] = fma(rh[q], rv, acc[0]);
        acc[1] = fma(rv, rv, acc[1]);
    }
    block_reduce_store<T, 2>(acc, partials);
    if (!ticket_last(counter)) return;
    double sum[2];
    final_sums<2>(partials, sum);
    if (threadIdx.x == 0) {
        sc->it += 1;
        sc->rr = sum[1];
        sc->res = sqrt(sum[1]) / sc->bnorm;
        if (!finite(sc->res)) { sc->status = KS_NOTFINITE; sc->done = 1; }
        else if (sc->res < sc->tol) { sc->status = KS_CONVERGED; sc->done = 1; }
        else if (sc->it >= sc->max_iter) { sc->status = KS_MAXITER; sc->done = 1; }
        else if (sc->omega == 0 || sc->rho == 0) { sc->status = KS_BREAKDOWN; sc->done = 1; }
        else if (fabs(sum[0]) <= kRestartEps * sqrt(sum[1]) * sc->rhnorm) {
            // shadow residual (numerically) orthogonal to r: restart with rh = p = r
            sc->restart = 1;
            sc->beta = 0;
            sc->rho = sum[1];
            sc->rhnorm = sqrt(sum[1]);
        }
        else {
            sc->restart = 0;
            sc->beta = (sum[0] / sc->rho) * (sc->alpha / sc->omega);
            sc->rho = sum[0];
        }
    }
}

// p = r + beta (p - omega v); on a restart rh = p = r
template <typename T>
__global__ void __launch_bounds__(KB) k_update_p(int64_t rows, T* p, const T* r, const T* v, T* rh,
                                                 const KrylovScalars* sc)
{
    if (*(volatile const int32_t*)&sc->done) return;
    const T beta = (T)sc->beta, omega = (T)sc->omega;
    if (sc->restart) {
        for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
            const T rv = r[q];
            p[q] = rv;
            rh[q] = rv;
        }
        return;
    }
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB)
        p[q] = fma(beta, fma(-omega, v[q], p[q]), r[q]);
}

// ---- FP64 solve --------------------------------------------------------------

void krylov_init_fp64(const EllMatrix& A, const double* b, double* x, KrylovWork& W,
                      double tol, int max_iter, cudaStream_t s)
{
    KrylovScalars h{};
    h.tol = tol;
    h.max_iter = max_iter;
    cudaMemcpyAsync(W.sc, &h, sizeof(h), cudaMemcpyHostToDevice, s);
    MHFEM_WIDTH_DISPATCH(A.width, (k_init<double, WW><<<occ_grid(k_init<double, WW>), KB, 0, s>>>(A.cols, A.vals, A.width, A.rows, b, x,
                                              W.r, W.rh, W.p, W.sc, W.partials, W.counters)));
}

void krylov_iterate_fp64(const EllMatrix& A, double* x, KrylovWork& W, int iters, cudaStream_t s)
{
    for (int it = 0; it < iters; ++it) {
        MHFEM_WIDTH_DISPATCH(A.width, (k_spmv_dot<double, WW><<<occ_grid(k_spmv_dot<double, WW>), KB, 0, s>>>(A.cols, A.vals, A.width, A.rows,
                                                  W.p, W.rh, W.v, W.sc, W.partials, W.counters)));
        k_update_s<double><<<occ_grid(k_update_s<double>), KB, 0, s>>>(A.rows, W.r, W.v, W.s, W.sc, W.partials, W.counters);
        MHFEM_WIDTH_DISPATCH(A.width, (k_spmv_dots2<double, WW><<<occ_grid(k_spmv_dots2<double, WW>), KB, 0, s>>>(A.cols, A.vals, A.width,
                                                    A.rows, W.s, W.t, W.sc, W.partials, W.counters)));
        k_update_xr<double><<<occ_grid(k_update_xr<double>), KB, 0, s>>>(A.rows, x, W.p, W.s, W.t, W.r, W.rh, W.sc, W.partials,
                                                  W.counters);
        k_update_p<double><<<occ_grid(k_update_p<double>), KB, 0, s>>>(A.rows, W.p, W.r, W.v, W.rh, W.sc);
    }
}

// ---- residual of a candidate (learned gate) ------------------------------------

template <int WW>
__global__ void __launch_bounds__(KB) k_residual_norm(const int32_t* cols, const double* vals, int W,
                                                      int64_t rows, const double* b, const double* x,
                                                      KrylovScalars* sc, double* partials, uint32_t* counter)
{
    double acc[2] = {0, 0};
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
        const double rv = b[q] - spmv_row<double, WW>(cols, vals, W, rows, q, x);
        acc[0] = fma(rv, rv, acc[0]);
        acc[1] = fma(b[q], b[q], acc[1]);
    }
    block_reduce_store<double, 2>(acc, partials);
    if (!ticket_last(counter)) return;
    double s[2];
    final_sums<2>(partials, s);
    if (threadIdx.x == 0) {
        double bn = sqrt(s[1]);
        if (bn == 0) bn = 1;
        sc->bnorm = bn;
        sc->res = sqrt(s[0]) / bn;
    }
}

void residual_norm_fp64(const EllMatrix& A, const double* b, const double* x, KrylovWork& W, cudaStream_t s)
{
    MHFEM_WIDTH_DISPATCH(A.width, (k_residual_norm<WW><<<occ_grid(k_residual_norm<WW>), KB, 0, s>>>(A.cols, A.vals, A.width, A.rows, b, x,
                                                W.sc, W.partials, W.counters)));
}

// ---- mixed precision: FP64 outer residual, FP32 inner BiCGStab ------------------

// r = b - A x (FP64) and its norm; sc->res is the outer relative residual,
// sc->snorm carries ||r|| (the scale of the FP32 right-hand side).
template <int WW>
__global__ void __launch_bounds__(KB) k_outer_residual(const int32_t* cols, const double* vals, int W,
                                                       int64_t rows, const double* b, const double* x,
                                                       double* r, KrylovScalars* sc, double* partials,
                                                       uint32_t* counter)
{
    double acc[2] = {0, 0};
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
        const double rv = b[q] - spmv_row<double, WW>(cols, vals, W, rows, q, x);
        r[q] = rv;
        acc[0] = fma(rv, rv, acc[0]);
        acc[1] = fma(b[q], b[q], acc[1]);
    }
    block_reduce_store<double, 2>(acc, partials);
    if (!ticket_last(counter)) return;
    double s[2];
    final_sums<2>(partials, s);
    if (threadIdx.x == 0) {
        double bn = sqrt(s[1]);
        if (bn == 0) bn = 1;
        sc->bnorm = bn;
        sc->snorm = sqrt(s[0]);
        sc->res = sc->snorm / bn;
        sc->it += 1;  // refinement sweep counter
        sc->done = 0;
        if (!finite(sc->res)) { sc->status = KS_NOTFINITE; sc->done = 1; }
        else if (sc->res < sc->tol) { sc->status = KS_CONVERGED; sc->done = 1; }
        else if (sc->it > sc->max_iter) { sc->status = KS_MAXITER; sc->done = 1; }
    }
}

// r32 = r / ||r|| ; rh32 = p32 = r32 ; x32 = 0 ; inner scalars
__global__ void __launch_bounds__(KB) k_inner_init(int64_t rows, const double* r, float* r32, float* rh32,
                                                   float* p32, float* x32, const KrylovScalars* outer,
                                                   KrylovScalars* sc, double inner_tol, int adaptive, int max_iter,
                                                   double* partials, uint32_t* counter)
{
    const double scale = (outer->snorm > 0) ? 1.0 / outer->snorm : 0.0;
    float acc[1] = {0.f};
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
        const float v = (float)(r[q] * scale);
        r32[q] = v; rh32[q] = v; p32[q] = v; x32[q] = 0.f;
        acc[0] = fmaf(v, v, acc[0]);
    }
    block_reduce_store<float, 1>(acc, partials);
    if (!ticket_last(counter)) return;
    double s[1];
    final_sums<1>(partials, s);
    if (threadIdx.x == 0) {
        // The last sweeps only need to close the remaining gap to the outer
        // tolerance: with adaptivity on, the inner tolerance is relaxed to
        // 0.3 tol / res (never tighter than inner_tol).
        double itol = inner_tol;
        if (adaptive && outer->res > 0) itol = fmax(inner_tol, fmin(0.5, 0.3 * outer->tol / outer->res));
        sc->tol = itol;
        sc->max_iter = max_iter;
        sc->bnorm = sqrt(s[0]) > 0 ? sqrt(s[0]) : 1.0;
        sc->rho = s[0];
        sc->rhnorm = sqrt(s[0]);
        sc->restart = 0;
        sc->res = 1.0;
        sc->it = 0;
        sc->snorm = 1.0;
        sc->status = KS_RUNNING;
        sc->done = (outer->done || s[0] == 0) ? 1 : 0;
    }
}

// x += ||r|| * x32
__global__ void __launch_bounds__(KB) k_apply_correction(int64_t rows, double* x, const float* x32,
                                                         const KrylovScalars* outer)
{
    const double scale = outer->snorm;
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB)
        x[q] = fma(scale, (double)x32[q], x[q]);
}

void mixed_outer_residual(const EllMatrix& A, const double* b, const double* x, KrylovWork& W,
                          double tol, int max_sweeps, cudaStream_t s)
{
    (void)tol; (void)max_sweeps;
    MHFEM_WIDTH_DISPATCH(A.width, (k_outer_residual<WW><<<occ_grid(k_outer_residual<WW>), KB, 0, s>>>(A.cols, A.vals, A.width, A.rows, b,
                                                 x, W.r, W.sc, W.partials, W.counters)));
}

void mixed_inner_init(KrylovWork& W, double inner_tol, int adaptive, int max_iter, cudaStream_t s)
{
    k_inner_init<<<occ_grid(k_inner_init), KB, 0, s>>>(W.rows, W.r, W.r32, W.rh32, W.p32, W.x32, W.sc, W.sc32, inner_tol,
                                       adaptive, max_iter, W.partials, W.counters);
}

void krylov_iterate_fp32(const EllMatrix& A, KrylovWork& W, int iters, cudaStream_t s)
{
    for (int it = 0; it < iters; ++it) {
        MHFEM_WIDTH_DISPATCH(A.width, (k_spmv_dot<float, WW><<<occ_grid(k_spmv_dot<float, WW>), KB, 0, s>>>(A.cols, A.vals32, A.width, A.rows,
                                                 W.p32, W.rh32, W.v32, W.sc32, W.partials, W.counters)));
        k_update_s<float><<<occ_grid(k_update_s<float>), KB, 0, s>>>(A.rows, W.r32, W.v32, W.s32, W.sc32, W.partials, W.counters);
        MHFEM_WIDTH_DISPATCH(A.width, (k_spmv_dots2<float, WW><<<occ_grid(k_spmv_dots2<float, WW>), KB, 0, s>>>(A.cols, A.vals32, A.width,
                                                   A.rows, W.s32, W.t32, W.sc32, W.partials, W.counters)));
        k_update_xr<float><<<occ_grid(k_update_xr<float>), KB, 0, s>>>(A.rows, W.x32, W.p32, W.s32, W.t32, W.r32, W.rh32, W.sc32,
                                                 W.partials, W.counters);
        k_update_p<float><<<occ_grid(k_update_p<float>), KB, 0, s>>>(A.rows, W.p32, W.r32, W.v32, W.rh32, W.sc32);
    }
}

void krylov_spmv_dot_once(const EllMatrix& A, KrylovWork& W, bool fp32, cudaStream_t s)
{
    if (fp32)
        MHFEM_WIDTH_DISPATCH(A.width, (k_spmv_dot<float, WW><<<occ_grid(k_spmv_dot<float, WW>), KB, 0, s>>>(A.cols, A.vals32, A.width, A.rows,
                                                 W.p32, W.rh32, W.v32, W.sc32, W.partials, W.counters)));
    else
        MHFEM_WIDTH_DISPATCH(A.width, (k_spmv_dot<double, WW><<<occ_grid(k_spmv_dot<double, WW>), KB, 0, s>>>(A.cols, A.vals, A.width, A.rows,
                                                  W.p, W.rh, W.v, W.sc, W.partials, W.counters)));
}

void mixed_apply_correction(double* x, KrylovWork& W, cudaStream_t s)
{
    k_apply_correction<<<occ_grid(k_apply_correction), KB, 0, s>>>(W.rows, x, W.x32, W.sc);
}

}  // namespace mhfem
