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
#include <algorithm>
#include <initializer_list>
#include <type_traits>
#include <vector>

#include "fp_convert.h"
#include "krylov_common.cuh"

namespace mhfem {

// Partial-sum slots of the reductions: 8 CTAs of KB threads per SM of the
// current device (full occupancy; no iteration kernel launches more).
int krylov_grid()
{
    int dev = 0;
    cudaGetDevice(&dev);
    return 8 * sm_count(dev);
}

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
        sc->rr = s[0];
        sc->rhnorm = sqrt(s[0]);
        sc->restart = 0;
        sc->half = 0;
        sc->res = sqrt(s[0]) / bn;
        sc->it = 0;
        sc->snorm = 0;
        sc->status = KS_RUNNING;
        sc->done = 0;
        if (!finite(sc->res)) { sc->status = KS_NOTFINITE; sc->done = 1; }
        else if (sc->res < sc->tol) { sc->status = KS_CONVERGED; sc->done = 1; }
    }
}

// y_j = x_{r_j} + sum_k vals[k][r_j] x[cols[k][r_j]] for the RPT rows
// r_j = RPT q + j; self_j = x_{r_j}.  RPT > 1 needs rows % RPT == 0 and a
// compile-time width.
template <typename T, int WW, int RPT>
__device__ __forceinline__ void spmv_rows(const int32_t* __restrict__ cols, const T* __restrict__ vals, int W,
                                          int64_t rows, int64_t q, const T* __restrict__ x, T (&y)[RPT],
                                          T (&self)[RPT])
{
    if constexpr (WW > 0) {
        VecT<int32_t, RPT> c[WW];
        VecT<T, RPT> a[WW];
#pragma unroll
        for (int k = 0; k < WW; ++k) {
            c[k] = ldv_stream<int32_t, RPT>(cols + (int64_t)k * rows, q);
            a[k] = ldv_stream<T, RPT>(vals + (int64_t)k * rows, q);
        }
        T xg[WW][RPT];
#pragma unroll
        for (int k = 0; k < WW; ++k)
#pragma unroll
            for (int j = 0; j < RPT; ++j) xg[k][j] = x[c[k].v[j]];
        const VecT<T, RPT> xs = ldv<T, RPT>(x, q);
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            T acc = xs.v[j];
#pragma unroll
            for (int k = 0; k < WW; ++k) acc = fma(a[k].v[j], xg[k][j], acc);
            y[j] = acc;
            self[j] = xs.v[j];
        }
    }
    else {
        static_assert(RPT == 1, "the run-time width takes one row per thread");
        const T xs = x[q];
        T acc = xs;
        for (int k = 0; k < W; ++k) {
            const int64_t o = (int64_t)k * rows + q;
            acc = fma(__ldcs(vals + o), x[__ldcs(cols + o)], acc);
        }
        y[0] = acc;
        self[0] = xs;
    }
}

// Pipelined SpMV: a thread loads the ELL entries of its next group of rows
// (grid-stride sequence) before gathering for the current group, so the two
// memory round trips of a row (ELL entries, then the gathered x) overlap
// with the neighbouring group's.  It doubles the registers that hold ELL
// entries (40 -> 64 for the FP64 width-6 SpMVs: 4 instead of 6 CTAs per
// SM), and pays where latency, not the FP64 pipe, bounds the kernel
// (measured on GB300):
//  - FP64, width 10 (cuboids): 172.8 against 198.9 us per launch on 6.3M rows
//    (79% against 69% of HBM);
//  - FP64, width 6 (tetrahedra, 3.17M rows), once the block reductions left
//    the FP64 pipe (block_reduce_store): second SpMV 54.6 against 57.1 us,
//    the whole in-step iteration 172.7 against 179.4 us (the first SpMV
//    alone 53.4 against 53.0 us); before that change the plain loop was
//    faster (58.2 against 60.2 us).  With the first row's ELL words loaded
//    before the dependency wait (as in the plain loop): 52.3 and 53.0 us,
//    iteration 171.2 us;
//  - FP32, 4 rows per thread (the mixed form's inner solve, tetrahedra):
//    5.37 against 4.87 TB/s, mixed form 1.69x against 1.59x the FP64 form.
template <typename T>
constexpr bool spmv_pipelined(int WW, int RPT)
{
    return (sizeof(T) == 8 && RPT == 1 && (WW == 10 || WW == 6)) ||
           (sizeof(T) == 4 && RPT == 4 && (WW == 4 || WW == 6));
}

// RPT consecutive rows of the ELL matrix (one 16-byte word per slot when RPT > 1)
template <typename T, int WW, int RPT>
struct EllRows {
    VecT<int32_t, RPT> c[WW];
    VecT<T, RPT> a[WW];
};

template <typename T, int WW, int RPT>
__device__ __forceinline__ void ell_load(const int32_t* __restrict__ cols, const T* __restrict__ vals, int64_t rows,
                                         int64_t q, EllRows<T, WW, RPT>& e)
{
#pragma unroll
    for (int k = 0; k < WW; ++k) {
        e.c[k] = ldv_stream<int32_t, RPT>(cols + (int64_t)k * rows, q);
        e.a[k] = ldv_stream<T, RPT>(vals + (int64_t)k * rows, q);
    }
}

template <typename T, int WW, int RPT>
__device__ __forceinline__ void ell_apply(const EllRows<T, WW, RPT>& e, const T* __restrict__ x,
                                          const VecT<T, RPT>& self, T (&y)[RPT])
{
    T xg[WW][RPT];
#pragma unroll
    for (int k = 0; k < WW; ++k)
#pragma unroll
        for (int j = 0; j < RPT; ++j) xg[k][j] = x[e.c[k].v[j]];
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        T acc = self.v[j];
#pragma unroll
        for (int k = 0; k < WW; ++k) acc = fma(e.a[k].v[j], xg[k][j], acc);
        y[j] = acc;
    }
}

// The FP32 SpMVs' column indices as 24-bit offsets (EllMatrix::cols_lo,
// cols_hi): four rows per thread, so one slot is an 8-byte word of four low
// halves and a 4-byte word of four high bytes.  Three bytes per entry
// instead of four: the FP32 SpMV moves 7W + 12 instead of 8W + 12 bytes per
// row, and it is bound by HBM.  Measured on the tetrahedral workloads (mixed
// form, same iteration counts): the first FP32 SpMV 211 against 219 us at
// 128^3 (25.3M rows), the mixed step 746 against 766 ms (2.6%); at 64^3
// 27.4 against 29.7 us and 39.6 against 40.3 ms.
struct Cols24 {
    const uint16_t* lo = nullptr;
    const uint8_t* hi = nullptr;
};

template <int WW>
struct EllRows24 {
    uint2 lo[WW];
    uint32_t hi[WW];
    VecT<float, 4> a[WW];
};

template <int WW>
__device__ __forceinline__ void ell_load24(Cols24 pc, const float* __restrict__ vals, int64_t rows, int64_t q,
                                           EllRows24<WW>& e)
{
#pragma unroll
    for (int k = 0; k < WW; ++k) {
        e.lo[k] = __ldcs(reinterpret_cast<const uint2*>(pc.lo + (int64_t)k * rows) + q);
        e.hi[k] = __ldcs(reinterpret_cast<const unsigned int*>(pc.hi + (int64_t)k * rows) + q);
        e.a[k] = ldv_stream<float, 4>(vals + (int64_t)k * rows, q);
    }
}

// Rows 4q .. 4q + 3: column = row + (hi << 16 | lo) - 2^23.
template <int WW>
__device__ __forceinline__ void ell_apply24(const EllRows24<WW>& e, int64_t q, const float* __restrict__ x,
                                            const VecT<float, 4>& self, float (&y)[4])
{
    const int32_t r0 = (int32_t)(4 * q) - kCol24Bias;
    float xg[WW][4];
#pragma unroll
    for (int k = 0; k < WW; ++k) {
        const uint32_t l01 = e.lo[k].x, l23 = e.lo[k].y, h = e.hi[k];
        xg[k][0] = x[r0 + (int32_t)((l01 & 0xffffu) | ((h & 0xffu) << 16))];
        xg[k][1] = x[r0 + 1 + (int32_t)((l01 >> 16) | ((h & 0xff00u) << 8))];
        xg[k][2] = x[r0 + 2 + (int32_t)((l23 & 0xffffu) | (h & 0xff0000u))];
        xg[k][3] = x[r0 + 3 + (int32_t)((l23 >> 16) | ((h >> 8) & 0xff0000u))];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float acc = self.v[j];
#pragma unroll
        for (int k = 0; k < WW; ++k) acc = fmaf(e.a[k].v[j], xg[k][j], acc);
        y[j] = acc;
    }
}

// Grid-stride bounds: threads of the whole grid, this thread's first index.
#define MHFEM_GRID_STRIDE                                                  \
    const int64_t gstride = (int64_t)gridDim.x * KB;                       \
    const int64_t gtid = (int64_t)blockIdx.x * KB + threadIdx.x

// ---- iteration phases ------------------------------------------------------------
//
// Each phase is a grid-stride loop over rows plus, for the reductions, the
// scalar update that the last CTA applies.  The five iteration kernels below
// each run one phase.
//
// Loads before the dependency wait.  Every iteration kernel is launched
// with programmatic stream serialization and waits (griddepcontrol.wait)
// for the kernel before it, whose last CTA computes the scalar this kernel
// needs.  Its CTAs become resident while that kernel drains.  The FP64
// SpMVs load the ELL words of their first row (constant during a solve)
// before waiting, which overlaps one memory round trip with the previous
// kernel's tail (measured on the 64^3 workload: 56.0 -> 54.7 and 62.7 ->
// 60.2 us per launch).  The same early loads of the vectors written two or
// more kernels back slowed the three vector updates (10.0 -> 10.9, 37.0 ->
// 38.8, 15.1 -> 16.4 us), so those wait first.  Each phase takes `gate`,
// which waits, releases the next kernel and returns false when the solve is
// done; a phase calls it exactly once, before it touches the previous
// kernel's outputs or the scalars.

// v = A p ; acc = (rh, v).  The FP64 loops load the ELL words of their
// first row before gate(); the pipelined FP32 loop starts after it.
template <typename T, int WW, int RPT, bool PK = false, typename Gate>
__device__ __forceinline__ bool phase_spmv_dot(const int32_t* cols, const T* vals, int W, int64_t rows,
                                               const T* p, const T* rh, T* v, int64_t gtid, int64_t gstride,
                                               T (&acc)[1], Gate&& gate, Cols24 pc = {})
{
    const int64_t ng = rows / RPT;
    auto finish = [&](int64_t q, const T (&y)[RPT]) {
        VecT<T, RPT> yv;
#pragma unroll
        for (int j = 0; j < RPT; ++j) yv.v[j] = y[j];
        stv<T, RPT>(v, q, yv);
        const VecT<T, RPT> h = ldv<T, RPT>(rh, q);
#pragma unroll
        for (int j = 0; j < RPT; ++j) acc[0] = fma(h.v[j], y[j], acc[0]);
    };
    if constexpr (PK) {
        static_assert(sizeof(T) == 4 && RPT == 4 && WW > 0, "24-bit columns: FP32, 4 rows per thread");
        if (!gate()) return false;
        int64_t q = gtid;
        EllRows24<WW> cur;
        if (q < ng) ell_load24<WW>(pc, vals, rows, q, cur);
        for (; q < ng; q += gstride) {
            EllRows24<WW> nxt;
            const int64_t qn = q + gstride;
            if (qn < ng) ell_load24<WW>(pc, vals, rows, qn, nxt);
            T y[RPT];
            ell_apply24<WW>(cur, q, p, ldv<T, RPT>(p, q), y);
            finish(q, y);
            cur = nxt;
        }
    }
    else if constexpr (spmv_pipelined<T>(WW, RPT)) {
        int64_t q = gtid;
        EllRows<T, WW, RPT> cur;
        if constexpr (sizeof(T) == 8)
            if (q < ng) ell_load<T, WW, RPT>(cols, vals, rows, q, cur);
        if (!gate()) return false;
        if constexpr (sizeof(T) == 4)
            if (q < ng) ell_load<T, WW, RPT>(cols, vals, rows, q, cur);
        for (; q < ng; q += gstride) {
            EllRows<T, WW, RPT> nxt;
            const int64_t qn = q + gstride;
            if (qn < ng) ell_load<T, WW, RPT>(cols, vals, rows, qn, nxt);
            T y[RPT];
            ell_apply<T, WW, RPT>(cur, p, ldv<T, RPT>(p, q), y);
            finish(q, y);
            cur = nxt;
        }
    }
    else if constexpr (WW > 0 && RPT == 1) {
        EllRows<T, WW, 1> first;
        if (gtid < ng) ell_load<T, WW, 1>(cols, vals, rows, gtid, first);
        if (!gate()) return false;
        if (gtid < ng) {
            T y[1];
            ell_apply<T, WW, 1>(first, p, ldv<T, 1>(p, gtid), y);
            finish(gtid, y);
        }
        for (int64_t q = gtid + gstride; q < ng; q += gstride) {
            T y[1], self[1];
            spmv_rows<T, WW, 1>(cols, vals, W, rows, q, p, y, self);
            finish(q, y);
        }
    }
    else {
        if (!gate()) return false;
        for (int64_t q = gtid; q < ng; q += gstride) {
            T y[RPT], self[RPT];
            spmv_rows<T, WW, RPT>(cols, vals, W, rows, q, p, y, self);
            finish(q, y);
        }
    }
    return true;
}

// Streams the groups of V rows of a grid-stride loop through fn(q, in) with
// the K input vectors of the thread's next group loaded before the current
// group is processed, so each thread keeps two groups of loads in flight.
// The FP32 updates use it: at 4 bytes per element a group's loads are too
// few to cover the memory latency at the occupancy they run with (measured:
// 1.5% per inner iteration of the mixed form, 0.1136 -> 0.1119 ms on 3.17M
// rows; the FP64 updates are bound by the FP64 pipe and keep the plain loop).
template <typename T, int V, int K, typename Fn>
__device__ __forceinline__ void stream_groups(int64_t nv, const T* const (&in)[K], int64_t gtid, int64_t gstride,
                                              Fn&& fn)
{
    int64_t q = gtid;
    VecT<T, V> cur[K];
    if (q < nv)
#pragma unroll
        for (int k = 0; k < K; ++k) cur[k] = ldv<T, V>(in[k], q);
    for (; q < nv; q += gstride) {
        VecT<T, V> nxt[K];
        const int64_t qn = q + gstride;
        if (qn < nv)
#pragma unroll
            for (int k = 0; k < K; ++k) nxt[k] = ldv<T, V>(in[k], qn);
        fn(q, cur);
#pragma unroll
        for (int k = 0; k < K; ++k) cur[k] = nxt[k];
    }
}

// alpha = rho / (rh, v)
__device__ __forceinline__ void scalars_alpha(KrylovScalars* sc, const double (&s)[1])
{
    sc->rv = s[0];
    if (!finite(s[0])) { sc->status = KS_NOTFINITE; sc->done = 1; }
    else if (s[0] == 0) { sc->status = KS_BREAKDOWN; sc->done = 1; }
    else sc->alpha = sc->rho / s[0];
}

// s = r - alpha v
template <typename T, int V>
__device__ __forceinline__ void phase_update_s(int64_t rows, const T* r, const T* v, T* s, T alpha, int64_t gtid,
                                               int64_t gstride)
{
    const int64_t nv = rows / V;
    if constexpr (sizeof(T) == 4) {
        const T* const in[2] = {r, v};
        stream_groups<T, V, 2>(nv, in, gtid, gstride, [&](int64_t q, const VecT<T, V>(&g)[2]) {
            VecT<T, V> ss;
#pragma unroll
            for (int j = 0; j < V; ++j) ss.v[j] = fma(-alpha, g[1].v[j], g[0].v[j]);
            stv<T, V>(s, q, ss);
        });
    }
    else
        for (int64_t q = gtid; q < nv; q += gstride) {
            const VecT<T, V> rr = ldv<T, V>(r, q), vv = ldv<T, V>(v, q);
            VecT<T, V> ss;
#pragma unroll
            for (int j = 0; j < V; ++j) ss.v[j] = fma(-alpha, vv.v[j], rr.v[j]);
            stv<T, V>(s, q, ss);
        }
    for (int64_t q = nv * V + gtid; q < rows; q += gstride) s[q] = fma(-alpha, v[q], r[q]);
}

// t = A s ; acc = (t, s), (t, t) and, on a check iteration, (s, s).  The
// FP64 loops load the ELL words of their first row before gate().
template <typename T, int WW, int RPT, bool CHECK, bool PK = false, typename Gate>
__device__ __forceinline__ bool phase_spmv_dots2(const int32_t* cols, const T* vals, int W, int64_t rows,
                                                 const T* s, T* t, int64_t gtid, int64_t gstride,
                                                 T (&acc)[CHECK ? 3 : 2], Gate&& gate, Cols24 pc = {})
{
    const int64_t ng = rows / RPT;
    auto finish = [&](int64_t q, const T (&y)[RPT], const T (&sv)[RPT]) {
        VecT<T, RPT> yv;
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            yv.v[j] = y[j];
            acc[0] = fma(y[j], sv[j], acc[0]);
            acc[1] = fma(y[j], y[j], acc[1]);
            if constexpr (CHECK) acc[2] = fma(sv[j], sv[j], acc[2]);
        }
        stv<T, RPT>(t, q, yv);
    };
    if constexpr (PK) {
        static_assert(sizeof(T) == 4 && RPT == 4 && WW > 0, "24-bit columns: FP32, 4 rows per thread");
        if (!gate()) return false;
        int64_t q = gtid;
        EllRows24<WW> cur;
        if (q < ng) ell_load24<WW>(pc, vals, rows, q, cur);
        for (; q < ng; q += gstride) {
            EllRows24<WW> nxt;
            const int64_t qn = q + gstride;
            if (qn < ng) ell_load24<WW>(pc, vals, rows, qn, nxt);
            const VecT<T, RPT> svv = ldv<T, RPT>(s, q);
            T y[RPT], sv[RPT];
            ell_apply24<WW>(cur, q, s, svv, y);
#pragma unroll
            for (int j = 0; j < RPT; ++j) sv[j] = svv.v[j];
            finish(q, y, sv);
            cur = nxt;
        }
    }
    else if constexpr (spmv_pipelined<T>(WW, RPT)) {
        int64_t q = gtid;
        EllRows<T, WW, RPT> cur;
        if constexpr (sizeof(T) == 8)
            if (q < ng) ell_load<T, WW, RPT>(cols, vals, rows, q, cur);
        if (!gate()) return false;
        if constexpr (sizeof(T) == 4)
            if (q < ng) ell_load<T, WW, RPT>(cols, vals, rows, q, cur);
        for (; q < ng; q += gstride) {
            EllRows<T, WW, RPT> nxt;
            const int64_t qn = q + gstride;
            if (qn < ng) ell_load<T, WW, RPT>(cols, vals, rows, qn, nxt);
            const VecT<T, RPT> svv = ldv<T, RPT>(s, q);
            T y[RPT], sv[RPT];
            ell_apply<T, WW, RPT>(cur, s, svv, y);
#pragma unroll
            for (int j = 0; j < RPT; ++j) sv[j] = svv.v[j];
            finish(q, y, sv);
            cur = nxt;
        }
    }
    else if constexpr (WW > 0 && RPT == 1) {
        EllRows<T, WW, 1> first;
        if (gtid < ng) ell_load<T, WW, 1>(cols, vals, rows, gtid, first);
        if (!gate()) return false;
        if (gtid < ng) {
            const VecT<T, 1> svv = ldv<T, 1>(s, gtid);
            T y[1], sv[1] = {svv.v[0]};
            ell_apply<T, WW, 1>(first, s, svv, y);
            finish(gtid, y, sv);
        }
        for (int64_t q = gtid + gstride; q < ng; q += gstride) {
            T y[1], sv[1];
            spmv_rows<T, WW, 1>(cols, vals, W, rows, q, s, y, sv);
            finish(q, y, sv);
        }
    }
    else {
        if (!gate()) return false;
        for (int64_t q = gtid; q < ng; q += gstride) {
            T y[RPT], sv[RPT];
            spmv_rows<T, WW, RPT>(cols, vals, W, rows, q, s, y, sv);
            finish(q, y, sv);
        }
    }
    return true;
}

// check iteration: ||s|| and the half-step test; omega = (t, s) / (t, t)
template <bool CHECK>
__device__ __forceinline__ void scalars_omega(KrylovScalars* sc, const double (&sum)[CHECK ? 3 : 2])
{
    if constexpr (CHECK) {
        sc->snorm = sqrt(sum[2]) / sc->bnorm;
        sc->half = (sc->snorm < sc->tol) ? 1 : 0;
        if (sc->half) return;
    }
    else
        sc->half = 0;
    sc->ts = sum[0];
    sc->tt = sum[1];
    if (!finite(sum[0]) || !finite(sum[1])) { sc->status = KS_NOTFINITE; sc->done = 1; }
    else if (sum[1] == 0) {
        if constexpr (CHECK) { sc->status = KS_BREAKDOWN; sc->done = 1; }  // ||s|| >= tol, yet A s = 0
        else {
            // A s = 0 on an iteration that does not form ||s||: the matrix is
            // nonsingular, so s = 0 and x + alpha p solves the system -- the
            // half step, which the reference's loop takes on its ||s|| test
            // (a system whose every row is its unit diagonal gets here on
            // the first iteration)
            sc->snorm = 0;
            sc->half = 1;
        }
    }
    else sc->omega = sum[0] / sum[1];
}

// half step: x += alpha p
template <typename T, int V>
__device__ __forceinline__ void phase_half(int64_t rows, T* x, const T* p, T alpha, int64_t gtid, int64_t gstride)
{
    const int64_t nv = rows / V;
    for (int64_t q = gtid; q < nv; q += gstride) {
        VecT<T, V> xx = ldv<T, V>(x, q);
        const VecT<T, V> pp = ldv<T, V>(p, q);
#pragma unroll
        for (int j = 0; j < V; ++j) xx.v[j] = fma(alpha, pp.v[j], xx.v[j]);
        stv<T, V>(x, q, xx);
    }
    for (int64_t q = nv * V + gtid; q < rows; q += gstride) x[q] = fma(alpha, p[q], x[q]);
}

__device__ __forceinline__ void scalars_half(KrylovScalars* sc)
{
    sc->res = sc->snorm;
    sc->it += 1;
    sc->status = KS_CONVERGED;
    sc->done = 1;
}

// x += alpha p + omega s ; r = s - omega t ; acc = (rh, r) and, on a check iteration, (r, r)
template <typename T, int V, bool CHECK>
__device__ __forceinline__ void phase_update_xr(int64_t rows, T* x, const T* p, const T* s, const T* t, T* r,
                                                const T* rh, T alpha, T omega, int64_t gtid, int64_t gstride,
                                                T (&acc)[CHECK ? 2 : 1])
{
    const int64_t nv = rows / V;
    auto apply = [&](int64_t q, VecT<T, V> xx, const VecT<T, V>& pp, const VecT<T, V>& ss, const VecT<T, V>& tt,
                     const VecT<T, V>& hh) {
        VecT<T, V> rr;
#pragma unroll
        for (int j = 0; j < V; ++j) {
            xx.v[j] = fma(omega, ss.v[j], fma(alpha, pp.v[j], xx.v[j]));
            rr.v[j] = fma(-omega, tt.v[j], ss.v[j]);
            acc[0] = fma(hh.v[j], rr.v[j], acc[0]);
            if constexpr (CHECK) acc[1] = fma(rr.v[j], rr.v[j], acc[1]);
        }
        stv<T, V>(x, q, xx);
        stv<T, V>(r, q, rr);
    };
    if constexpr (sizeof(T) == 4) {
        const T* const in[5] = {x, p, s, t, rh};
        stream_groups<T, V, 5>(nv, in, gtid, gstride,
                               [&](int64_t q, const VecT<T, V>(&g)[5]) { apply(q, g[0], g[1], g[2], g[3], g[4]); });
    }
    else
        for (int64_t q = gtid; q < nv; q += gstride)
            apply(q, ldv<T, V>(x, q), ldv<T, V>(p, q), ldv<T, V>(s, q), ldv<T, V>(t, q), ldv<T, V>(rh, q));
    for (int64_t q = nv * V + gtid; q < rows; q += gstride) {
        const T sv = s[q];
        x[q] = fma(omega, sv, fma(alpha, p[q], x[q]));
        const T rv = fma(-omega, t[q], sv);
        r[q] = rv;
        acc[0] = fma(rh[q], rv, acc[0]);
        if constexpr (CHECK) acc[1] = fma(rv, rv, acc[1]);
    }
}

// iteration count, convergence, restart test, beta
// The residual norm (the convergence test) is formed on check iterations
// only, the last of each group the host replays between its checks: the
// other iterations skip the (r, r) and (s, s) products, two of the about 24
// FP64 operations per row of an iteration.  Convergence is then detected at
// the end of such a group, up to check_every - 1 iterations later.  The
// restart test compares (rh, r) with the last known ||r||; on a restart,
// update_p forms (r, r) for the new rho.
template <bool CHECK>
__device__ __forceinline__ void scalars_beta(KrylovScalars* sc, const double (&sum)[CHECK ? 2 : 1])
{
    sc->it += 1;
    if constexpr (CHECK) {
        sc->rr = sum[1];
        sc->res = sqrt(sum[1]) / sc->bnorm;
        if (!finite(sc->res)) { sc->status = KS_NOTFINITE; sc->done = 1; return; }
        if (sc->res < sc->tol) { sc->status = KS_CONVERGED; sc->done = 1; return; }
    }
    else if (!finite(sum[0])) { sc->status = KS_NOTFINITE; sc->done = 1; return; }
    if (sc->it >= sc->max_iter) { sc->status = KS_MAXITER; sc->done = 1; }
    else if (sc->omega == 0 || sc->rho == 0) { sc->status = KS_BREAKDOWN; sc->done = 1; }
    else if (fabs(sum[0]) <= kRestartEps * sqrt(sc->rr) * sc->rhnorm) {
        // shadow residual (numerically) orthogonal to r: restart with rh = p = r
        // (rho = (r, r) and ||rh|| come from update_p's restart pass)
        sc->restart = 1;
        sc->beta = 0;
    }
    else {
        sc->restart = 0;
        sc->beta = (sum[0] / sc->rho) * (sc->alpha / sc->omega);
        sc->rho = sum[0];
    }
}

// p = r + beta (p - omega v); on a restart rh = p = r and acc = (r, r)
template <typename T, int V>
__device__ __forceinline__ void phase_update_p(int64_t rows, T* p, const T* r, const T* v, T* rh, T beta, T omega,
                                               bool restart, int64_t gtid, int64_t gstride, T (&acc)[1])
{
    const int64_t nv = rows / V;
    if (restart) {
        for (int64_t q = gtid; q < nv; q += gstride) {
            const VecT<T, V> rr = ldv<T, V>(r, q);
            stv<T, V>(p, q, rr);
            stv<T, V>(rh, q, rr);
#pragma unroll
            for (int j = 0; j < V; ++j) acc[0] = fma(rr.v[j], rr.v[j], acc[0]);
        }
        for (int64_t q = nv * V + gtid; q < rows; q += gstride) {
            const T rv = r[q];
            p[q] = rv;
            rh[q] = rv;
            acc[0] = fma(rv, rv, acc[0]);
        }
        return;
    }
    if constexpr (sizeof(T) == 4) {
        const T* const in[3] = {p, r, v};
        stream_groups<T, V, 3>(nv, in, gtid, gstride, [&](int64_t q, const VecT<T, V>(&g)[3]) {
            VecT<T, V> pp;
#pragma unroll
            for (int j = 0; j < V; ++j) pp.v[j] = fma(beta, fma(-omega, g[2].v[j], g[0].v[j]), g[1].v[j]);
            stv<T, V>(p, q, pp);
        });
    }
    else
        for (int64_t q = gtid; q < nv; q += gstride) {
            VecT<T, V> pp = ldv<T, V>(p, q);
            const VecT<T, V> rr = ldv<T, V>(r, q), vv = ldv<T, V>(v, q);
#pragma unroll
            for (int j = 0; j < V; ++j) pp.v[j] = fma(beta, fma(-omega, vv.v[j], pp.v[j]), rr.v[j]);
            stv<T, V>(p, q, pp);
        }
    for (int64_t q = nv * V + gtid; q < rows; q += gstride) p[q] = fma(beta, fma(-omega, v[q], p[q]), r[q]);
}

// ---- one kernel per phase ----------------------------------------------------------

// Waits for the preceding kernel, lets the next one launch, and tells whether
// the solve is still running (the "done" flag that preceding kernel may set).
#define MHFEM_GATE(sc) [&]() { pdl_wait(); pdl_release(); return *(volatile const int32_t*)&(sc)->done == 0; }

template <typename T, int WW, int RPT>
__global__ void __launch_bounds__(KB) k_spmv_dot(const int32_t* cols, const T* vals, int W, int64_t rows,
                                                 const T* p, const T* rh, T* v,
                                                 KrylovScalars* sc, double* partials, uint32_t* counter)
{
    MHFEM_GRID_STRIDE;
    T acc[1] = {0};
    if (!phase_spmv_dot<T, WW, RPT>(cols, vals, W, rows, p, rh, v, gtid, gstride, acc, MHFEM_GATE(sc))) return;
    block_reduce_store<T, 1>(acc, partials);
    if (!ticket_last(counter)) return;
    double s[1];
    final_sums<1>(partials, s);
    if (threadIdx.x == 0) scalars_alpha(sc, s);
}

// The FP32 SpMV over 24-bit column offsets (the mixed form's inner solve).
template <int WW>
__global__ void __launch_bounds__(KB) k_spmv_dot24(Cols24 pc, const float* vals, int64_t rows, const float* p,
                                                   const float* rh, float* v, KrylovScalars* sc, double* partials,
                                                   uint32_t* counter)
{
    MHFEM_GRID_STRIDE;
    float acc[1] = {0};
    if (!phase_spmv_dot<float, WW, 4, true>(nullptr, vals, WW, rows, p, rh, v, gtid, gstride, acc, MHFEM_GATE(sc), pc))
        return;
    block_reduce_store<float, 1>(acc, partials);
    if (!ticket_last(counter)) return;
    double s[1];
    final_sums<1>(partials, s);
    if (threadIdx.x == 0) scalars_alpha(sc, s);
}

template <typename T, int V>
__global__ void __launch_bounds__(KB) k_update_s(int64_t rows, const T* r, const T* v, T* s, const KrylovScalars* sc)
{
    pdl_wait();
    pdl_release();
    if (*(volatile const int32_t*)&sc->done) return;
    MHFEM_GRID_STRIDE;
    phase_update_s<T, V>(rows, r, v, s, (T)sc->alpha, gtid, gstride);
}

// On a check iteration the half-step decision (||s|| < tol) is taken here,
// after the SpMV: the same decision as testing ||s|| before it; t is then
// unused.
template <typename T, int WW, int RPT, bool CHECK>
__global__ void __launch_bounds__(KB) k_spmv_dots2(const int32_t* cols, const T* vals, int W, int64_t rows,
                                                   const T* s, T* t,
                                                   KrylovScalars* sc, double* partials, uint32_t* counter)
{
    constexpr int NS = CHECK ? 3 : 2;
    MHFEM_GRID_STRIDE;
    T acc[NS] = {};
    if (!phase_spmv_dots2<T, WW, RPT, CHECK>(cols, vals, W, rows, s, t, gtid, gstride, acc, MHFEM_GATE(sc))) return;
    block_reduce_store<T, NS>(acc, partials);
    if (!ticket_last(counter)) return;
    double sum[NS];
    final_sums<NS>(partials, sum);
    if (threadIdx.x == 0) scalars_omega<CHECK>(sc, sum);
}

template <int WW, bool CHECK>
__global__ void __launch_bounds__(KB) k_spmv_dots2_24(Cols24 pc, const float* vals, int64_t rows, const float* s,
                                                      float* t, KrylovScalars* sc, double* partials, uint32_t* counter)
{
    constexpr int NS = CHECK ? 3 : 2;
    MHFEM_GRID_STRIDE;
    float acc[NS] = {};
    if (!phase_spmv_dots2<float, WW, 4, CHECK, true>(nullptr, vals, WW, rows, s, t, gtid, gstride, acc,
                                                     MHFEM_GATE(sc), pc))
        return;
    block_reduce_store<float, NS>(acc, partials);
    if (!ticket_last(counter)) return;
    double sum[NS];
    final_sums<NS>(partials, sum);
    if (threadIdx.x == 0) scalars_omega<CHECK>(sc, sum);
}

template <typename T, int V, bool CHECK>
__global__ void __launch_bounds__(KB) k_update_xr(int64_t rows, T* x, const T* p, const T* s, const T* t,
                                                  T* r, const T* rh,
                                                  KrylovScalars* sc, double* partials, uint32_t* counter)
{
    pdl_wait();
    pdl_release();
    if (*(volatile int32_t*)&sc->done) return;
    MHFEM_GRID_STRIDE;
    const T alpha = (T)sc->alpha;
    if (sc->half) {
        phase_half<T, V>(rows, x, p, alpha, gtid, gstride);
        if (!ticket_last(counter)) return;
        if (threadIdx.x == 0) scalars_half(sc);
        return;
    }
    constexpr int NS = CHECK ? 2 : 1;
    T acc[NS] = {};
    phase_update_xr<T, V, CHECK>(rows, x, p, s, t, r, rh, alpha, (T)sc->omega, gtid, gstride, acc);
    block_reduce_store<T, NS>(acc, partials);
    if (!ticket_last(counter)) return;
    double sum[NS];
    final_sums<NS>(partials, sum);
    if (threadIdx.x == 0) scalars_beta<CHECK>(sc, sum);
}

template <typename T, int V>
__global__ void __launch_bounds__(KB) k_update_p(int64_t rows, T* p, const T* r, const T* v, T* rh,
                                                 KrylovScalars* sc, double* partials, uint32_t* counter)
{
    pdl_wait();
    pdl_release();
    if (*(volatile const int32_t*)&sc->done) return;
    MHFEM_GRID_STRIDE;
    const bool restart = sc->restart != 0;  // the same in every block
    T acc[1] = {0};
    phase_update_p<T, V>(rows, p, r, v, rh, (T)sc->beta, (T)sc->omega, restart, gtid, gstride, acc);
    if (!restart) return;
    // the new shadow residual rh = r: rho = (rh, r) = (r, r)
    block_reduce_store<T, 1>(acc, partials);
    if (!ticket_last(counter)) return;
    double sum[1];
    final_sums<1>(partials, sum);
    if (threadIdx.x == 0) {
        sc->rho = sum[0];
        sc->rr = sum[0];
        sc->rhnorm = sqrt(sum[0]);
    }
}

// ---- small systems: one persistent launch per chunk of iterations ----------------
//
// A system of a few ten thousand rows (the 128^2 heat-equation workload:
// 49,408 rows, about 2 MB of matrix and vectors, all L2-resident) leaves the
// five-kernel iteration bound by launch and drain latency: about 30 us per
// iteration for a few microseconds of memory traffic.  Here one cooperative
// launch (every CTA resident) runs a chunk of iterations:
//  - an iteration is three phases separated by grid barriers (below:
//    k_bicgstab_small), the p and s updates being formed where they are
//    gathered; measured on the 128^2 system: 24.7 us per iteration against
//    26.8 us with five phases and 30.6 us for the five-kernel iteration;
//  - each reduction's per-CTA partials are summed by every CTA itself, in
//    the same fixed order, so every CTA holds the same scalars (in shared
//    memory) with no last-block step, and the result is deterministic;
//  - the convergence test runs every iteration, as in the reference's loop
//    (the five-kernel path tests every check_every iterations);
//  - a thread owns the same rows in every phase, so its own rows need no
//    synchronization; values of other CTAs' rows (the SpMV gathers, the
//    partials) are loaded past L1 (ld.global.cg), which is not coherent
//    between SMs; the matrix, constant during the solve, stays in L1.
// Every barrier wait is bounded: a CTA that polls kBarrierPolls times
// records the failure in *bar_err and returns, and the others then fail
// their next wait at once.

// Check of the bounded barrier: every CTA but `skip` (none if negative)
// arrives once and reports 1 (passed) or 0 (gave up); CTA `skip` never
// arrives and reports -1, so the others' waits run out after max_polls.
__global__ void __launch_bounds__(KB) k_grid_barrier_check(unsigned int* count, int* err, int skip,
                                                           unsigned int max_polls, int* result)
{
    if ((int)blockIdx.x == skip) {
        if (threadIdx.x == 0) result[blockIdx.x] = -1;
        return;
    }
    const bool ok = grid_barrier(count, err, gridDim.x, max_polls);
    if (threadIdx.x == 0) result[blockIdx.x] = ok ? 1 : 0;
}


// The ELL words of one row held in registers for a whole launch (the
// matrix does not change during a solve).
template <int WW>
struct SmallEll {
    int32_t c[WW > 0 ? WW : 1];
    double a[WW > 0 ? WW : 1];
};

template <int WW>
__device__ __forceinline__ void small_load(const int32_t* __restrict__ cols, const double* __restrict__ vals,
                                           int64_t rows, int64_t q, SmallEll<WW>& e)
{
#pragma unroll
    for (int k = 0; k < WW; ++k) {
        e.c[k] = __ldg(cols + (int64_t)k * rows + q);
        e.a[k] = __ldg(vals + (int64_t)k * rows + q);
    }
}

template <int WW, typename G>
__device__ __forceinline__ double small_apply(const SmallEll<WW>& e, double self, G&& g)
{
    double xg[WW > 0 ? WW : 1];
#pragma unroll
    for (int k = 0; k < WW; ++k) xg[k] = g(e.c[k]);
    double acc = self;
#pragma unroll
    for (int k = 0; k < WW; ++k) acc = fma(e.a[k], xg[k], acc);
    return acc;
}

// Rows per thread whose ELL words stay in registers for the launch: two for
// the compile-time widths up to 6, one for the wider ones, none for the
// run-time width.
constexpr int small_rows_in_registers(int WW) { return WW == 0 ? 0 : (WW <= 6 ? 2 : 1); }

// Three phases and three grid barriers per iteration: the p update of the
// previous iteration and the s update are formed where they are needed,
// for the own rows and again for each gathered neighbour (the same
// operations, so the same values), instead of in phases of their own.  p
// and v therefore alternate between two buffers: the neighbours' old p and
// v stay readable while the new ones are written.
//  1. p = r + beta (p' - omega v') (on a restart and in the first
//     iteration p = rh = r), v = A p, (rh, v) -> alpha;
//  2. s = r - alpha v, t = A s, (t, s), (t, t), (s, s) -> the half-step
//     test and omega;
//  3. x += alpha p + omega s, r = s - omega t, (rh, r), (r, r) -> the
//     convergence test, the restart test and beta.
template <int WW>
__global__ void __launch_bounds__(KB) k_bicgstab_small(const int32_t* __restrict__ cols,
                                                       const double* __restrict__ vals, int W, int64_t rows,
                                                       double* x, double* r, double* rh, double* p0, double* p1,
                                                       double* v0, double* v1, double* s, double* t,
                                                       KrylovScalars* sc, double* partials, unsigned int* bar,
                                                       int* bar_err, int max_its)
{
    __shared__ KrylovScalars S;
    if (threadIdx.x == 0) S = *sc;
    __syncthreads();
    if (S.done) return;
    MHFEM_GRID_STRIDE;
    const unsigned int nb = gridDim.x;
    unsigned int target = 0;
    double* pa = partials;
    double* pc = partials + (int64_t)nb * kPartStride;
    double* pd = partials + 2 * (int64_t)nb * kPartStride;
    // The ELL words of the thread's first RK rows, loaded once: both SpMVs of
    // every iteration then start with the gathers, one L2 round trip instead
    // of two behind each grid barrier.
    constexpr int RK = small_rows_in_registers(WW);
    SmallEll<WW> er[RK > 0 ? RK : 1];
#pragma unroll
    for (int j = 0; j < RK; ++j) {
        const int64_t q = gtid + (int64_t)j * gstride;
        if (q < rows) small_load<WW>(cols, vals, rows, q, er[j]);
    }
    // For the widths up to 6, the own-row values of those rows that the
    // third phase needs (p, rh, s, t, x) stay in registers from the phase
    // that forms or loads them, so the third phase reaches its reduction
    // without a memory round trip; s and t of these rows are then never
    // stored.  (For the wider rows the extra registers cost more than the
    // round trip: 36.1 against 35.2 us per iteration on the 128^2
    // two-component system, width 9.)
    constexpr int R3 = WW <= 6 ? RK : 0;
    double preg[R3 > 0 ? R3 : 1], hreg[R3 > 0 ? R3 : 1], sreg[R3 > 0 ? R3 : 1], treg[R3 > 0 ? R3 : 1],
        xreg[R3 > 0 ? R3 : 1];
    // y = A x over the thread's rows with x given by xval (own row and
    // gathered neighbours); the register rows first, all their loads ahead of
    // their stores, then any further rows from the matrix in memory.
    // finish(j, q, x_q, y_q) gets the register slot j, or -1.
    auto spmv_rows = [&](auto&& xval, auto&& finish) {
        double xr[RK > 0 ? RK : 1], yr[RK > 0 ? RK : 1];
#pragma unroll
        for (int j = 0; j < RK; ++j) {
            const int64_t q = gtid + (int64_t)j * gstride;
            if (q < rows) {
                xr[j] = xval(q);
                yr[j] = small_apply<WW>(er[j], xr[j], xval);
            }
        }
#pragma unroll
        for (int j = 0; j < RK; ++j) {
            const int64_t q = gtid + (int64_t)j * gstride;
            if (q < rows) finish(j, q, xr[j], yr[j]);
        }
        for (int64_t q = gtid + (int64_t)RK * gstride; q < rows; q += gstride) {
            const double xq = xval(q);
            finish(-1, q, xq, small_row<WW>(cols, vals, W, rows, q, xq, xval));
        }
    };
    for (int k = 0; k < max_its; ++k) {
        const int cur = S.it & 1;
        const double* P = cur ? p1 : p0;
        double* Pn = cur ? p0 : p1;
        const double* V = cur ? v1 : v0;
        double* Vn = cur ? v0 : v1;
        // 1. p, v = A p, (rh, v) -> alpha
        {
            const bool fresh = S.restart || S.it == 0;
            const double beta = S.beta, omega = S.omega;
            auto pval = [&](int64_t j) {
                const double rj = __ldcg(r + j);
                return fresh ? rj : fma(beta, fma(-omega, __ldcg(V + j), __ldcg(P + j)), rj);
            };
            double acc[1] = {0};
            spmv_rows(pval, [&](int j, int64_t q, double pq, double y) {
                Pn[q] = pq;
                Vn[q] = y;
                double hq;
                if (fresh) { hq = __ldcg(r + q); rh[q] = hq; }
                else hq = rh[q];
                acc[0] = fma(hq, y, acc[0]);
                if (j >= 0 && j < R3) { preg[j] = pq; hreg[j] = hq; }
            });
            block_reduce_store<double, 1>(acc, pa);
            if (!grid_barrier(bar, bar_err, target += nb)) return;
            double sum[1];
            grid_sums<1>(pa, sum);
            if (threadIdx.x == 0) scalars_alpha(&S, sum);
            __syncthreads();
            if (S.done) break;
        }
        const double alpha = S.alpha;
        // 2. s = r - alpha v, t = A s, (t, s), (t, t), (s, s) -> half step, omega
        {
            auto sval = [&](int64_t j) { return fma(-alpha, __ldcg(Vn + j), __ldcg(r + j)); };
            double acc[3] = {0, 0, 0};
            spmv_rows(sval, [&](int j, int64_t q, double sv, double y) {
                if (j >= 0 && j < R3) {
                    sreg[j] = sv;
                    treg[j] = y;
                    xreg[j] = x[q];  // own row, written only by this thread
                }
                else {
                    s[q] = sv;
                    t[q] = y;
                }
                acc[0] = fma(y, sv, acc[0]);
                acc[1] = fma(y, y, acc[1]);
                acc[2] = fma(sv, sv, acc[2]);
            });
            block_reduce_store<double, 3>(acc, pc);
            if (!grid_barrier(bar, bar_err, target += nb)) return;
            double sum[3];
            grid_sums<3>(pc, sum);
            if (threadIdx.x == 0) scalars_omega<true>(&S, sum);
            __syncthreads();
        }
        if (S.half) {
            for (int64_t q = gtid; q < rows; q += gstride) x[q] = fma(alpha, Pn[q], x[q]);
            if (threadIdx.x == 0) scalars_half(&S);
            __syncthreads();
            break;
        }
        if (S.done) break;
        // 3. x, r, (rh, r), (r, r) -> convergence, restart, beta
        {
            const double omega = S.omega;
            double acc[2] = {0, 0};
#pragma unroll
            for (int j = 0; j < R3; ++j) {
                const int64_t q = gtid + (int64_t)j * gstride;
                if (q < rows) {
                    const double sv = sreg[j];
                    x[q] = fma(omega, sv, fma(alpha, preg[j], xreg[j]));
                    const double rv = fma(-omega, treg[j], sv);
                    r[q] = rv;
                    acc[0] = fma(hreg[j], rv, acc[0]);
                    acc[1] = fma(rv, rv, acc[1]);
                }
            }
            for (int64_t q = gtid + (int64_t)R3 * gstride; q < rows; q += gstride) {
                const double sv = s[q];
                x[q] = fma(omega, sv, fma(alpha, Pn[q], x[q]));
                const double rv = fma(-omega, t[q], sv);
                r[q] = rv;
                acc[0] = fma(rh[q], rv, acc[0]);
                acc[1] = fma(rv, rv, acc[1]);
            }
            block_reduce_store<double, 2>(acc, pd);
            if (!grid_barrier(bar, bar_err, target += nb)) return;
            double sum[2];
            grid_sums<2>(pd, sum);
            if (threadIdx.x == 0) {
                scalars_beta<true>(&S, sum);
                if (!S.done && S.restart) {  // rh = r (formed in phase 1): rho = (r, r)
                    S.rho = S.rr;
                    S.rhnorm = sqrt(S.rr);
                }
            }
            __syncthreads();
            if (S.done) break;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *sc = S;
}

// ---- launch shapes ---------------------------------------------------------------


// Vector width of the streaming updates: 16-byte accesses when every vector
// of the solve starts on a 16-byte boundary (the tail rows go one by one).
template <typename T>
static bool vec_ok(std::initializer_list<const void*> ptrs)
{
    for (const void* p : ptrs)
        if (!aligned16(p)) return false;
    return true;
}

// Rows per thread of the SpMV: 4 (FP32) when the ELL slots and the vectors
// are 16-byte aligned (rows % 4 == 0) and the width is a compile-time one of
// at most 6 entries (so the 4 rows' loads stay in registers).
static bool spmv4_ok(const EllMatrix& A, std::initializer_list<const void*> ptrs)
{
    if (A.rows % 4 != 0 || (A.width != 4 && A.width != 6)) return false;
    for (const void* p : ptrs)
        if (!aligned16(p)) return false;
    return aligned16(A.cols) && aligned16(A.vals32);
}

// Rows per thread of an SpMV instance: RPT for the widths 4 and 6, else 1.
constexpr int spmv_rpt(int WW, int RPT) { return (WW == 4 || WW == 6) ? RPT : 1; }

// One BiCGStab iteration: five kernels, each a single wave.  Streaming
// updates with V rows per thread, SpMVs with RPT rows per thread.
template <typename T, int V, int RPT>
static void iterate(const EllMatrix& A, const T* vals, T* x, T* r, T* rh, T* p, T* v, T* s, T* t,
                    KrylovScalars* sc, KrylovWork& W, int iters, cudaStream_t st)
{
    const int32_t* cols = A.cols;
    const Cols24 pc{A.cols_lo, A.cols_hi};
    // 24-bit column offsets: FP32, 4 rows per thread, widths 4 and 6
    const bool pk = sizeof(T) == 4 && RPT == 4 && A.cols_lo && A.cols_hi && (A.width == 4 || A.width == 6);
    auto spmv1 = [&]() {
        if constexpr (sizeof(T) == 4 && RPT == 4)
            if (pk) {
                if (A.width == 4) launch_pdl(k_spmv_dot24<4>, st, A.rows, pc, vals, A.rows, (const T*)p, (const T*)rh, v, sc,
                                             W.partials, W.counters);
                else launch_pdl(k_spmv_dot24<6>, st, A.rows, pc, vals, A.rows, (const T*)p, (const T*)rh, v, sc,
                                W.partials, W.counters);
                return;
            }
        MHFEM_WIDTH_DISPATCH(A.width, launch_pdl(k_spmv_dot<T, WW, spmv_rpt(WW, RPT)>, st, A.rows, cols, vals, A.width,
                                                 A.rows, (const T*)p, (const T*)rh, v, sc, W.partials, W.counters));
    };
    auto spmv2 = [&](auto ctag) {
        constexpr bool C = decltype(ctag)::value;
        if constexpr (sizeof(T) == 4 && RPT == 4)
            if (pk) {
                if (A.width == 4) launch_pdl(k_spmv_dots2_24<4, C>, st, A.rows, pc, vals, A.rows, (const T*)s, t, sc,
                                             W.partials, W.counters);
                else launch_pdl(k_spmv_dots2_24<6, C>, st, A.rows, pc, vals, A.rows, (const T*)s, t, sc, W.partials,
                                W.counters);
                return;
            }
        MHFEM_WIDTH_DISPATCH(A.width, launch_pdl(k_spmv_dots2<T, WW, spmv_rpt(WW, RPT), C>, st, A.rows, cols, vals,
                                                 A.width, A.rows, (const T*)s, t, sc, W.partials, W.counters));
    };
    for (int it = 0; it < iters; ++it) {
        const bool check = (it == iters - 1);  // the last iteration before the host's check
        spmv1();
        launch_pdl(k_update_s<T, V>, st, A.rows, A.rows, (const T*)r, (const T*)v, s, (const KrylovScalars*)sc);
        if (check) {
            spmv2(std::true_type{});
            launch_pdl(k_update_xr<T, V, true>, st, A.rows, A.rows, x, (const T*)p, (const T*)s, (const T*)t, r,
                       (const T*)rh, sc, W.partials, W.counters);
        }
        else {
            spmv2(std::false_type{});
            launch_pdl(k_update_xr<T, V, false>, st, A.rows, A.rows, x, (const T*)p, (const T*)s, (const T*)t, r,
                       (const T*)rh, sc, W.partials, W.counters);
        }
        launch_pdl(k_update_p<T, V>, st, A.rows, A.rows, p, (const T*)r, (const T*)v, rh, sc, W.partials, W.counters);
    }
}

// ---- FP64 solve --------------------------------------------------------------

void krylov_init_fp64(const EllMatrix& A, const double* b, double* x, KrylovWork& W,
                      double tol, int max_iter, cudaStream_t s)
{
    KrylovScalars h{};
    h.tol = tol;
    h.max_iter = max_iter;
    cudaMemcpyAsync(W.sc, &h, sizeof(h), cudaMemcpyHostToDevice, s);
    MHFEM_WIDTH_DISPATCH(A.width, (k_init<double, WW><<<row_grid(k_init<double, WW>, A.rows), KB, 0, s>>>(A.cols, A.vals, A.width, A.rows, b, x,
                                              W.r, W.rh, W.p, W.sc, W.partials, W.counters)));
}

// The FP64 SpMV keeps one row per thread (pipelined for the widths 6 and
// 10): it is bound by the FP64 pipe as much as by HBM.  Two rows per thread
// with 16-byte ELL loads (plain loop) measured 175.2 us per iteration on the
// 64^3 workload, against 171.2 us for the pipelined single row.
void krylov_iterate_fp64(const EllMatrix& A, double* x, KrylovWork& W, int iters, cudaStream_t s)
{
    if (vec_ok<double>({x, W.r, W.rh, W.p, W.v, W.s, W.t}))
        iterate<double, 2, 1>(A, A.vals, x, W.r, W.rh, W.p, W.v, W.s, W.t, W.sc, W, iters, s);
    else
        iterate<double, 1, 1>(A, A.vals, x, W.r, W.rh, W.p, W.v, W.s, W.t, W.sc, W, iters, s);
}

// ---- learned form: one pass for the guess inputs --------------------------------

// r_base = b - A base for the extrapolated base (formed beforehand), and the
// norms the guess needs, in one pass over the matrix: A Zn and A base are
// formed row by row, so the ELL arrays are read once.  Sums: r_base^2,
// (b - A Zn)^2, b^2 over all rows; Zn^2, (Zn - Zn1)^2 and the count over the
// free rows.  The last block writes out[0] = rms(Zn) and out[1] = rms(Zn -
// Zn1) over the free rows, out[2] = ||r_base||, out[3] = ||b - A Zn|| / ||b||
// (the warm start's relative residual), out[4] = ||b||, out[9] = ||r_base|| /
// ||b||, out[10] = the network's output scale for this step (the last
// measured base error out[8] once there is one, else out[1]), and the rms
// over the free rows of the second and third time differences of the
// traces (out[11], out[12]; 0 until the history reaches them).
template <int WW>
__global__ void __launch_bounds__(KB) k_learned_prep(const int32_t* __restrict__ cols,
                                                     const double* __restrict__ vals, int W, int64_t rows,
                                                     const double* __restrict__ b, const double* __restrict__ Zn,
                                                     const double* __restrict__ Zn1, const double* __restrict__ Zn2,
                                                     const double* __restrict__ Zn3, int hist,
                                                     const double* __restrict__ base,
                                                     const uint8_t* __restrict__ fixed, double* __restrict__ rbase,
                                                     double* out, double* partials, uint32_t* counter)
{
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
        const double z = Zn[q], bq = b[q];
        double yz = z, yb = base[q];
        if constexpr (WW > 0) {
            int32_t c[WW];
            double v[WW];
#pragma unroll
            for (int k = 0; k < WW; ++k) {
                c[k] = __ldcs(cols + (int64_t)k * rows + q);
                v[k] = __ldcs(vals + (int64_t)k * rows + q);
            }
#pragma unroll
            for (int k = 0; k < WW; ++k) {
                yz = fma(v[k], Zn[c[k]], yz);
                yb = fma(v[k], base[c[k]], yb);
            }
        }
        else {
            for (int k = 0; k < W; ++k) {
                const int64_t o = (int64_t)k * rows + q;
                const double v = __ldcs(vals + o);
                const int32_t c = __ldcs(cols + o);
                yz = fma(v, Zn[c], yz);
                yb = fma(v, base[c], yb);
            }
        }
        const double rb = bq - yb, rw = bq - yz;
        rbase[q] = rb;
        acc[0] = fma(rb, rb, acc[0]);
        acc[1] = fma(rw, rw, acc[1]);
        acc[2] = fma(bq, bq, acc[2]);
        if (!fixed[q]) {
            const double z1 = Zn1[q];
            const double d = z - z1;
            acc[3] = fma(z, z, acc[3]);
            acc[4] = fma(d, d, acc[4]);
            acc[5] += 1.0;
            if (hist >= 2) {
                const double z2 = Zn2[q];
                const double d2 = fma(-2.0, z1, z + z2);
                acc[6] = fma(d2, d2, acc[6]);
                if (hist >= 3) {
                    const double d3 = (z - Zn3[q]) + 3.0 * (z2 - z1);
                    acc[7] = fma(d3, d3, acc[7]);
                }
            }
        }
    }
    block_reduce_store<double, 8>(acc, partials);
    if (!ticket_last(counter)) return;
    double s[8];
    final_sums<8>(partials, s);
    if (threadIdx.x == 0) {
        const double n = s[5] > 0 ? s[5] : 1.0;
        const double bn = s[2] > 0 ? sqrt(s[2]) : 1.0;
        out[0] = sqrt(s[3] / n);
        out[1] = sqrt(s[4] / n);
        out[2] = sqrt(s[0]);
        out[3] = sqrt(s[1]) / bn;
        out[4] = bn;
        out[9] = sqrt(s[0]) / bn;
        out[10] = out[8] > 0 ? out[8] : out[1];
        out[11] = sqrt(s[6] / n);
        out[12] = sqrt(s[7] / n);
    }
}

void learned_prep_fp64(const EllMatrix& A, const double* b, const double* Zn, const double* Zn1, const double* Zn2,
                       const double* Zn3, int hist, const double* base, const uint8_t* fixed, double* rbase,
                       double* out, KrylovWork& W, cudaStream_t s)
{
    MHFEM_WIDTH_DISPATCH(A.width, (k_learned_prep<WW><<<row_grid(k_learned_prep<WW>, A.rows), KB, 0, s>>>(
                                      A.cols, A.vals, A.width, A.rows, b, Zn, Zn1, Zn2, Zn3, hist, base, fixed,
                                      rbase, out, W.partials, W.counters)));
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
    MHFEM_WIDTH_DISPATCH(A.width, (k_residual_norm<WW><<<row_grid(k_residual_norm<WW>, A.rows), KB, 0, s>>>(A.cols, A.vals, A.width, A.rows, b, x,
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
        const float v = f64_to_f32_rn(r[q] * scale);
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
        sc->rr = s[0];
        sc->rhnorm = sqrt(s[0]);
        sc->restart = 0;
        sc->half = 0;
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
        x[q] = fma(scale, f32_to_f64(x32[q]), x[q]);
}

void mixed_outer_residual(const EllMatrix& A, const double* b, const double* x, KrylovWork& W,
                          double tol, int max_sweeps, cudaStream_t s)
{
    (void)tol; (void)max_sweeps;
    MHFEM_WIDTH_DISPATCH(A.width, (k_outer_residual<WW><<<row_grid(k_outer_residual<WW>, A.rows), KB, 0, s>>>(A.cols, A.vals, A.width, A.rows, b,
                                                 x, W.r, W.sc, W.partials, W.counters)));
}

void mixed_inner_init(KrylovWork& W, double inner_tol, int adaptive, int max_iter, cudaStream_t s)
{
    k_inner_init<<<row_grid(k_inner_init, W.rows), KB, 0, s>>>(W.rows, W.r, W.r32, W.rh32, W.p32, W.x32, W.sc, W.sc32, inner_tol,
                                       adaptive, max_iter, W.partials, W.counters);
}

void krylov_iterate_fp32(const EllMatrix& A, KrylovWork& W, int iters, cudaStream_t s)
{
    const bool v4 = vec_ok<float>({W.x32, W.r32, W.rh32, W.p32, W.v32, W.s32, W.t32});
    if (v4 && spmv4_ok(A, {W.p32, W.rh32, W.v32, W.s32, W.t32}))
        iterate<float, 4, 4>(A, A.vals32, W.x32, W.r32, W.rh32, W.p32, W.v32, W.s32, W.t32, W.sc32, W, iters, s);
    else if (v4)
        iterate<float, 4, 1>(A, A.vals32, W.x32, W.r32, W.rh32, W.p32, W.v32, W.s32, W.t32, W.sc32, W, iters, s);
    else
        iterate<float, 1, 1>(A, A.vals32, W.x32, W.r32, W.rh32, W.p32, W.v32, W.s32, W.t32, W.sc32, W, iters, s);
}

void krylov_spmv_dot_once(const EllMatrix& A, KrylovWork& W, bool fp32, cudaStream_t s)
{
    if (fp32) {
        const Cols24 pc{A.cols_lo, A.cols_hi};
        if (spmv4_ok(A, {W.p32, W.rh32, W.v32}) && A.cols_lo && A.cols_hi) {
            if (A.width == 4) launch_pdl(k_spmv_dot24<4>, s, A.rows, pc, (const float*)A.vals32, A.rows, (const float*)W.p32,
                                         (const float*)W.rh32, W.v32, W.sc32, W.partials, W.counters);
            else launch_pdl(k_spmv_dot24<6>, s, A.rows, pc, (const float*)A.vals32, A.rows, (const float*)W.p32,
                            (const float*)W.rh32, W.v32, W.sc32, W.partials, W.counters);
        }
        else if (spmv4_ok(A, {W.p32, W.rh32, W.v32}))
            MHFEM_WIDTH_DISPATCH(A.width, launch_pdl(k_spmv_dot<float, WW, spmv_rpt(WW, 4)>, s, A.rows,
                                                     (const int32_t*)A.cols, (const float*)A.vals32, A.width, A.rows,
                                                     (const float*)W.p32, (const float*)W.rh32, W.v32, W.sc32,
                                                     W.partials, W.counters));
        else
            MHFEM_WIDTH_DISPATCH(A.width, launch_pdl(k_spmv_dot<float, WW, 1>, s, A.rows, (const int32_t*)A.cols,
                                                     (const float*)A.vals32, A.width, A.rows, (const float*)W.p32,
                                                     (const float*)W.rh32, W.v32, W.sc32, W.partials, W.counters));
    }
    else
        MHFEM_WIDTH_DISPATCH(A.width, launch_pdl(k_spmv_dot<double, WW, 1>, s, A.rows, (const int32_t*)A.cols,
                                                 (const double*)A.vals, A.width, A.rows, (const double*)W.p,
                                                 (const double*)W.rh, W.v, W.sc, W.partials, W.counters));
}

// One launch of one FP64 iteration kernel on the current Krylov vectors
// (timing): 0 the SpMV + (rh, v), 1 the second SpMV + (t, s), (t, t), 2 the
// s update, 3 the x / r update (with W.v standing in for x, so the solution
// is left alone), 4 the p update.
void krylov_fp64_kernel_once(const EllMatrix& A, KrylovWork& W, int which, cudaStream_t s)
{
    const int32_t* cols = A.cols;
    const bool v2 = vec_ok<double>({W.r, W.rh, W.p, W.v, W.s, W.t});
    auto run = [&](auto vtag) {
        constexpr int V = decltype(vtag)::value;
        switch (which) {
            case 0:
                MHFEM_WIDTH_DISPATCH(A.width, launch_pdl(k_spmv_dot<double, WW, 1>, s, A.rows, cols, (const double*)A.vals,
                                                         A.width, A.rows, (const double*)W.p, (const double*)W.rh,
                                                         W.v, W.sc, W.partials, W.counters));
                break;
            case 1:
                MHFEM_WIDTH_DISPATCH(A.width, launch_pdl(k_spmv_dots2<double, WW, 1, false>, s, A.rows, cols,
                                                         (const double*)A.vals, A.width, A.rows, (const double*)W.s,
                                                         W.t, W.sc, W.partials, W.counters));
                break;
            case 2:
                launch_pdl(k_update_s<double, V>, s, A.rows, A.rows, (const double*)W.r, (const double*)W.v, W.s,
                           (const KrylovScalars*)W.sc);
                break;
            case 3:
                launch_pdl(k_update_xr<double, V, false>, s, A.rows, A.rows, W.v, (const double*)W.p, (const double*)W.s,
                           (const double*)W.t, W.r, (const double*)W.rh, W.sc, W.partials, W.counters);
                break;
            default:
                launch_pdl(k_update_p<double, V>, s, A.rows, A.rows, W.p, (const double*)W.r, (const double*)W.v, W.rh, W.sc,
                           W.partials, W.counters);
                break;
        }
    };
    if (v2) run(std::integral_constant<int, 2>{});
    else run(std::integral_constant<int, 1>{});
}


// ---- small systems: host side ----------------------------------------------------

// Rows up to which the FP64 solve takes the persistent path, and rows per
// thread it aims at (more CTAs spread the memory traffic over more SMs, but
// every CTA adds an arrival to each grid barrier).
constexpr int64_t kSmallSystemRows = (int64_t)1 << 18;
constexpr int kSmallRowsPerThread = 2;

int64_t krylov_small_rows() { return kSmallSystemRows; }

cudaError_t krylov_small_fp64(const EllMatrix& A, double* x, KrylovWork& W, int iters, cudaStream_t s)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int sms = sm_count(dev);
    int nb = 0;
    MHFEM_WIDTH_DISPATCH(A.width, e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_bicgstab_small<WW>, KB, 0));
    if (e != cudaSuccess) return e;
    if (nb < 1) return cudaErrorCooperativeLaunchTooLarge;
    const int64_t want = (A.rows + (int64_t)KB * kSmallRowsPerThread - 1) / ((int64_t)KB * kSmallRowsPerThread);
    // every CTA resident (a cooperative launch), at most one per SM, and few
    // enough that the three reductions' partials fit the per-CTA buffer
    int grid = (int)std::min<int64_t>(std::min<int64_t>(want, (int64_t)sms), (int64_t)nb * sms);
    grid = std::max(1, std::min(grid, W.grid / 3));
    unsigned int* bar = W.counters + 2;
    int* bar_err = reinterpret_cast<int*>(W.counters + 3);
    e = cudaMemsetAsync(bar, 0, 2 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    const int32_t* cols = A.cols;
    const double* vals = A.vals;
    int W_ = A.width;
    int64_t rows = A.rows;
    double *r = W.r, *rh = W.rh, *p0 = W.p, *p1 = W.p2, *v0 = W.v, *v1 = W.v2, *sv = W.s, *t = W.t;
    if (!p1 || !v1) return cudaErrorInvalidValue;
    KrylovScalars* sc = W.sc;
    double* partials = W.partials;
    int its = iters;
    void* args[] = {(void*)&cols, (void*)&vals, (void*)&W_, (void*)&rows, (void*)&x, (void*)&r, (void*)&rh,
                    (void*)&p0, (void*)&p1, (void*)&v0, (void*)&v1, (void*)&sv, (void*)&t, (void*)&sc,
                    (void*)&partials, (void*)&bar, (void*)&bar_err, (void*)&its};
    MHFEM_WIDTH_DISPATCH(A.width, e = cudaLaunchCooperativeKernel((const void*)k_bicgstab_small<WW>, dim3(grid), dim3(KB),
                                                                 args, 0, s));
    return e;
}

cudaError_t grid_barrier_check(int ctas, int skip, unsigned int max_polls, int* passed, int* gave_up, int* flag)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_grid_barrier_check, KB, 0);
    if (e != cudaSuccess) return e;
    if (ctas < 1 || ctas > nb * sm_count(dev)) return cudaErrorInvalidValue;
    unsigned int* buf = nullptr;  // [0] arrival count, [1] failure flag, [2 ..] per-CTA results
    e = cudaMalloc(&buf, sizeof(unsigned int) * (2 + (size_t)ctas));
    if (e != cudaSuccess) return e;
    std::vector<int> res((size_t)ctas + 2, 0);
    e = cudaMemset(buf, 0, sizeof(unsigned int) * (2 + (size_t)ctas));
    if (e == cudaSuccess) {
        unsigned int* count = buf;
        int* err = reinterpret_cast<int*>(buf + 1);
        int* result = reinterpret_cast<int*>(buf + 2);
        void* args[] = {(void*)&count, (void*)&err, (void*)&skip, (void*)&max_polls, (void*)&result};
        e = cudaLaunchCooperativeKernel((const void*)k_grid_barrier_check, dim3(ctas), dim3(KB), args, 0, 0);
        if (e == cudaSuccess) e = cudaMemcpy(res.data(), buf, sizeof(int) * (2 + (size_t)ctas), cudaMemcpyDeviceToHost);
    }
    cudaFree(buf);
    if (e != cudaSuccess) return e;
    *passed = 0;
    *gave_up = 0;
    for (int b = 0; b < ctas; ++b) {
        *passed += res[2 + b] == 1;
        *gave_up += res[2 + b] == 0;
    }
    *flag = res[1];
    return cudaSuccess;
}

void mixed_apply_correction(double* x, KrylovWork& W, cudaStream_t s)
{
    k_apply_correction<<<row_grid(k_apply_correction, W.rows), KB, 0, s>>>(W.rows, x, W.x32, W.sc);
}

}  // namespace mhfem
