// Restarted GMRES on the unit-diagonal face system (sm_103a), FP64.
//
// The reference's own example configuration selects it
// (examples/HeatEquation/config.ini: linear-solver = gmres, gmres-variant =
// CGS, gmres-restarting-max = 30) through the solver factory of
// Solver::setup (Solver.hpp:192-204; configSetup.h:32-62).  TNL's
// implementation is not in the reference tree; this restates the published
// algorithm (Saad and Schultz, "GMRES: a generalized minimal residual
// algorithm for solving nonsymmetric linear systems", 1986): Arnoldi with
// classical Gram-Schmidt (optionally one reorthogonalization pass), Givens
// rotations of the Hessenberg matrix, the least-squares solution at the end
// of a cycle and restarts from the true residual.  The restart length is
// gmres-restarting-max, or, with gmres-restarting-min and the steps set,
// varies between the two from cycle to cycle (gmres_restart.h: Baker,
// Jessup and Kolev's rule, applied by the host between cycles, or by the
// device inside the persistent small-system solve; the device reads the
// cycle length from its state in every iteration).
//
// Design for GB300:
//  - the basis is stored unnormalized (v_i = inv_i u_i), so no pass only
//    scales a vector: an Arnoldi iteration is two kernels (four with the
//    reorthogonalization):
//      k_gm_arnoldi: z = A u_j (unit-diagonal SpMV) stored as u_{j+1}, with
//                    the j+1 dot products (z, u_i) in the same pass;
//      k_gm_orth:    u_{j+1} -= sum_i c_i u_i and ||u_{j+1}||^2;
//    the last block of k_gm_orth rotates the new Hessenberg column on the
//    device and decides whether the cycle ends, so an iteration needs no
//    host round trip;
//  - reductions are deterministic (fixed grid, one partial per block, the
//    last block sums them in a fixed order);
//  - every iteration kernel returns at once when the cycle has ended or the
//    solve is done, so the host replays a CUDA graph of several iterations
//    between checks;
//  - systems of at most 2^18 rows run k_gmres_small instead: a persistent
//    cooperative launch per chunk of iterations, restarts included (below).
#include <algorithm>
#include <initializer_list>

#include "gmres_restart.h"
#include "krylov_common.cuh"

namespace mhfem {

constexpr int kGmDots = kGmresMaxM + 1;
static_assert(kGmDots <= kGmStride && kGmDots <= KB, "GMRES dot products per block");

// r = b - A x -> u_0 and the restart scalars; first: also ||b|| and it = 0.
// The true residual decides convergence (the rotated estimate only ends a
// cycle early).
template <int WW>
__global__ void __launch_bounds__(KB) k_gm_init(const int32_t* cols, const double* vals, int W, int64_t rows,
                                                const double* b, const double* x, double* U, GmresState* st,
                                                int first, double* partials, uint32_t* counter)
{
    double acc[2] = {0, 0};
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
        const double bq = b[q];
        const double r = bq - spmv_row<double, WW>(cols, vals, W, rows, q, x);
        U[q] = r;
        acc[0] = fma(r, r, acc[0]);
        acc[1] = fma(bq, bq, acc[1]);
    }
    block_reduce_store<double, 2>(acc, partials);
    if (!ticket_last(counter)) return;
    double s[2];
    final_sums<2>(partials, s);
    if (threadIdx.x == 0) {
        GmresCtl& c = st->ctl;
        if (first) {
            double bn = sqrt(s[1]);
            if (bn == 0) bn = 1;
            c.bnorm = bn;
            c.it = 0;
            c.status = KS_RUNNING;
            c.done = 0;
        }
        const double beta = sqrt(s[0]);
        c.res = beta / c.bnorm;
        st->g[0] = beta;
        st->inv[0] = beta > 0 ? 1.0 / beta : 0.0;
        st->j = 0;
        c.cycle_end = 0;
        if (!finite(c.res)) { c.status = KS_NOTFINITE; c.done = 1; }
        else if (c.res < st->tol) { c.status = KS_CONVERGED; c.done = 1; }
        else if (c.it >= st->max_iter) { c.status = KS_MAXITER; c.done = 1; }
    }
}

// The dot products are taken in chunks of kGmChunk basis vectors: a pass
// over the rows per chunk with kGmChunk accumulators per thread (re-reading
// the row's z, 8 bytes, per chunk), which keeps registers low and the
// per-row work exact.
constexpr int kGmChunk = 8;

// Block sums of the per-thread dot products of one chunk into
// partials[block][c0 .. c0 + n - 1]: warp shuffles, then thread k adds value
// k over the warps in order.
__device__ __forceinline__ void gm_block_dots(const double (&acc)[kGmChunk], int c0, int n, double* partials)
{
    __shared__ double sh[KB / 32][kGmChunk];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < kGmChunk; ++k) {
        double v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < n) {
        double s = 0;
        for (int w = 0; w < KB / 32; ++w) s += sh[w][threadIdx.x];
        partials[(int64_t)blockIdx.x * kGmStride + c0 + threadIdx.x] = s;
    }
    __syncthreads();  // sh is reused by the next chunk
}

// The last block sums value i (i <= j) over the blocks in a fixed order:
// warp w takes i = w, w + 8, ...; its lanes stride over the blocks.
__device__ __forceinline__ void gm_final_dots(const double* partials, int j, double* out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nb = (int)gridDim.x;
    for (int i = warp; i <= j; i += KB / 32) {
        double s = 0;
        for (int b = lane; b < nb; b += 32) s += __ldcg(partials + (int64_t)b * kGmStride + i);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) out[i] = s;
    }
    __syncthreads();
}

// SPMV: z = A u_j -> u_{j+1}, d_i = (z, u_i); else (the reorthogonalization
// pass) d_i = (u_{j+1}, u_i).  The last block turns d into the Hessenberg
// entries h_ij = (A v_j, v_i) = inv_j inv_i d_i (added to them on the second
// pass) and the multipliers c_i = inv_i^2 d_i of the orthogonalization.
template <int WW, bool SPMV>
__global__ void __launch_bounds__(KB) k_gm_arnoldi(const int32_t* cols, const double* vals, int W, int64_t rows,
                                                   double* U, GmresState* st, double* partials, uint32_t* counter)
{
    pdl_wait();
    if (st->ctl.done || st->ctl.cycle_end) {
        pdl_release();
        return;
    }
    const int j = st->j;
    const double* uj = U + (int64_t)j * rows;
    double* un = U + (int64_t)(j + 1) * rows;
    for (int c0 = 0; c0 <= j; c0 += kGmChunk) {
        const int n = (j + 1 - c0 < kGmChunk) ? j + 1 - c0 : kGmChunk;
        double acc[kGmChunk];
#pragma unroll
        for (int k = 0; k < kGmChunk; ++k) acc[k] = 0;
        for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
            double z;
            if (SPMV && c0 == 0) {  // the first chunk forms z = A u_j; later chunks re-read it
                z = spmv_row<double, WW>(cols, vals, W, rows, q, uj);
                un[q] = z;
            }
            else
                z = un[q];
            if (n == kGmChunk) {
#pragma unroll
                for (int k = 0; k < kGmChunk; ++k) acc[k] = fma(z, U[(int64_t)(c0 + k) * rows + q], acc[k]);
            }
            else
                for (int k = 0; k < n; ++k) acc[k] = fma(z, U[(int64_t)(c0 + k) * rows + q], acc[k]);
        }
        gm_block_dots(acc, c0, n, partials);
    }
    pdl_release();
    if (!ticket_last(counter)) return;
    __shared__ double d[kGmDots];
    gm_final_dots(partials, j, d);
    if (threadIdx.x == 0) {
        const double invj = st->inv[j];
        for (int i = 0; i <= j; ++i) {
            const double invi = st->inv[i];
            const double h = invj * invi * d[i];
            if constexpr (SPMV) st->H[i][j] = h;
            else st->H[i][j] += h;
            st->c[i] = invi * invi * d[i];
        }
    }
}

// u_{j+1} -= sum_i c_i u_i.  FINAL: ||u_{j+1}||, h_{j+1,j} = inv_j ||u_{j+1}||,
// the earlier Givens rotations applied to column j and a new one that zeroes
// h_{j+1,j}, the rotated right-hand side g and the residual estimate
// |g_{j+1}| / ||b||; the cycle ends on that estimate, after m columns, on a
// breakdown (u_{j+1} = 0: the solution lies in the current space) or at the
// iteration cap.
template <bool FINAL>
__global__ void __launch_bounds__(KB) k_gm_orth(int64_t rows, double* U, GmresState* st, double* partials,
                                                uint32_t* counter)
{
    pdl_wait();
    if (st->ctl.done || st->ctl.cycle_end) {
        pdl_release();
        return;
    }
    const int j = st->j;
    __shared__ double c[kGmDots];
    if (threadIdx.x <= j) c[threadIdx.x] = st->c[threadIdx.x];
    __syncthreads();
    double* un = U + (int64_t)(j + 1) * rows;
    double acc[1] = {0};
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
        double t = un[q];
#pragma unroll 4
        for (int i = 0; i <= j; ++i) t = fma(-c[i], U[(int64_t)i * rows + q], t);
        un[q] = t;
        if constexpr (FINAL) acc[0] = fma(t, t, acc[0]);
    }
    pdl_release();
    if constexpr (FINAL) {
        block_reduce_store<double, 1>(acc, partials);
        if (!ticket_last(counter)) return;
        double s[1];
        final_sums<1>(partials, s);
        if (threadIdx.x == 0) {
            GmresCtl& C = st->ctl;
            const double nrm = sqrt(s[0]);
            const double hn = st->inv[j] * nrm;  // h_{j+1,j}
            for (int k = 0; k < j; ++k) {
                const double a = st->H[k][j], b = st->H[k + 1][j];
                st->H[k][j] = st->cs[k] * a + st->sn[k] * b;
                st->H[k + 1][j] = -st->sn[k] * a + st->cs[k] * b;
            }
            const double a = st->H[j][j];
            const double den = sqrt(a * a + hn * hn);
            const double cs = den > 0 ? a / den : 1.0, sn = den > 0 ? hn / den : 0.0;
            st->cs[j] = cs;
            st->sn[j] = sn;
            st->H[j][j] = den;
            st->g[j + 1] = -sn * st->g[j];
            st->g[j] = cs * st->g[j];
            st->inv[j + 1] = nrm > 0 ? 1.0 / nrm : 0.0;
            const double res = fabs(st->g[j + 1]) / C.bnorm;
            C.res = res;
            C.it += 1;
            st->j = j + 1;
            if (!finite(res) || !finite(den)) { C.status = KS_NOTFINITE; C.done = 1; }
            else if (res < st->tol || j + 1 >= st->m || nrm == 0 || C.it >= st->max_iter) C.cycle_end = 1;
        }
    }
}

// End of a cycle: back substitution R y = g over the k = j columns, then the
// multipliers of x += sum_i y_i v_i = sum_i (y_i inv_i) u_i.
__global__ void k_gm_solve(GmresState* st)
{
    if (threadIdx.x != 0 || st->ctl.done) return;
    const int k = st->j;
    double y[kGmresMaxM];
    for (int i = k - 1; i >= 0; --i) {
        double s = st->g[i];
        for (int l = i + 1; l < k; ++l) s -= st->H[i][l] * y[l];
        y[i] = s / st->H[i][i];
    }
    for (int i = 0; i < kGmDots; ++i) st->c[i] = (i < k) ? y[i] * st->inv[i] : 0.0;
}

__global__ void __launch_bounds__(KB) k_gm_update_x(int64_t rows, const double* U, double* x, const GmresState* st)
{
    if (st->ctl.done) return;
    const int k = st->j;
    __shared__ double c[kGmDots];
    if (threadIdx.x < kGmDots) c[threadIdx.x] = st->c[threadIdx.x];
    __syncthreads();
    for (int64_t q = (int64_t)blockIdx.x * KB + threadIdx.x; q < rows; q += (int64_t)gridDim.x * KB) {
        double t = x[q];
#pragma unroll 4
        for (int i = 0; i < k; ++i) t = fma(c[i], U[(int64_t)i * rows + q], t);
        x[q] = t;
    }
}

// ---- small systems: one persistent launch per chunk of iterations ----------------
//
// On a system of a few ten thousand rows the two kernels of an Arnoldi
// iteration are bound by launch, drain and last-block latency (53 us per
// iteration on the 128^2 heat-equation system).  Here one cooperative
// launch runs up to `max_its` iterations, restarts included:
//  A. z = A u_j -> u_{j+1} and the dot products (z, u_i), i <= j, in chunks
//     of kGmChunk basis vectors (with the reorthogonalization, A2: u_{j+1}
//     -= sum c_i u_i and the dot products again, into a second partials
//     region);
//  B. u_{j+1} -= sum c_i u_i and ||u_{j+1}||^2;
//  then, at the end of a cycle: x += sum_i y_i inv_i u_i, a barrier (the
//  residual gathers other CTAs' x), r = b - A x -> u_0 and ||r||^2, and the
//  next cycle's length by the adaptive rule (gmres_restart.h).
// Every CTA sums the partials in CTA order and keeps its own copy of the
// solve state (Hessenberg column rotations, least-squares solve) in shared
// memory, applying the same operations to the same values, so all copies
// stay identical and the result is deterministic.  Barrier waits are
// bounded as in k_bicgstab_small.
template <int WW, bool REORTH>
__global__ void __launch_bounds__(KB) k_gmres_small(const int32_t* __restrict__ cols,
                                                    const double* __restrict__ vals, int W, int64_t rows,
                                                    const double* __restrict__ b, double* x, double* U,
                                                    GmresState* st, double* pdots, double* pnorm,
                                                    unsigned int* bar, int* bar_err, int max_its)
{
    __shared__ GmresState S;
    __shared__ double d[kGmDots];
    {
        // the state, copied word by word
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(st);
        unsigned long long* dst = reinterpret_cast<unsigned long long*>(&S);
        for (int k = threadIdx.x; k < (int)(sizeof(GmresState) / 8); k += KB) dst[k] = src[k];
    }
    __syncthreads();
    if (S.ctl.done) return;
    const int64_t gstride = (int64_t)gridDim.x * KB;
    const int64_t gtid = (int64_t)blockIdx.x * KB + threadIdx.x;
    const unsigned int nb = gridDim.x;
    unsigned int target = 0;
    double* pd0 = pdots;
    double* pd1 = pdots + (int64_t)nb * kGmStride;
    // the dot products (w, u_i), i <= j, of the own rows into partials pd
    // (w = u_{j+1}, formed first as A u_j when SPMV)
    auto dots = [&](int j, bool spmv, double* pd) {
        const double* uj = U + (int64_t)j * rows;
        double* un = U + (int64_t)(j + 1) * rows;
        for (int c0 = 0; c0 <= j; c0 += kGmChunk) {
            const int n = (j + 1 - c0 < kGmChunk) ? j + 1 - c0 : kGmChunk;
            double acc[kGmChunk];
#pragma unroll
            for (int k = 0; k < kGmChunk; ++k) acc[k] = 0;
            for (int64_t q = gtid; q < rows; q += gstride) {
                double z;
                if (spmv && c0 == 0) {
                    z = small_row<WW>(cols, vals, W, rows, q, uj[q], [&](int64_t c) { return __ldcg(uj + c); });
                    un[q] = z;
                }
                else
                    z = un[q];
                if (n == kGmChunk) {
#pragma unroll
                    for (int k = 0; k < kGmChunk; ++k) acc[k] = fma(z, U[(int64_t)(c0 + k) * rows + q], acc[k]);
                }
                else
                    for (int k = 0; k < n; ++k) acc[k] = fma(z, U[(int64_t)(c0 + k) * rows + q], acc[k]);
            }
            gm_block_dots(acc, c0, n, pd);
        }
    };
    // u_{j+1} -= sum_{i <= j} c_i u_i over the own rows; returns sum t^2 when NORM
    auto orth = [&](int j, bool norm) {
        double* un = U + (int64_t)(j + 1) * rows;
        double acc = 0;
        for (int64_t q = gtid; q < rows; q += gstride) {
            double t = un[q];
#pragma unroll 4
            for (int i = 0; i <= j; ++i) t = fma(-S.c[i], U[(int64_t)i * rows + q], t);
            un[q] = t;
            if (norm) acc = fma(t, t, acc);
        }
        return acc;
    };
    for (int it = 0; it < max_its; ++it) {
        const int j = S.j;
        // A. z = A u_j, h_ij, c_i
        dots(j, true, pd0);
        if (!grid_barrier(bar, bar_err, target += nb)) return;
        gm_final_dots(pd0, j, d);
        if (threadIdx.x == 0) {
            const double invj = S.inv[j];
            for (int i = 0; i <= j; ++i) {
                const double invi = S.inv[i];
                S.H[i][j] = invj * invi * d[i];
                S.c[i] = invi * invi * d[i];
            }
        }
        __syncthreads();
        if constexpr (REORTH) {
            // A2. u_{j+1} -= sum c_i u_i, then the dot products again
            orth(j, false);
            dots(j, false, pd1);
            if (!grid_barrier(bar, bar_err, target += nb)) return;
            gm_final_dots(pd1, j, d);
            if (threadIdx.x == 0) {
                const double invj = S.inv[j];
                for (int i = 0; i <= j; ++i) {
                    const double invi = S.inv[i];
                    S.H[i][j] += invj * invi * d[i];
                    S.c[i] = invi * invi * d[i];
                }
            }
            __syncthreads();
        }
        // B. u_{j+1} -= sum c_i u_i, ||u_{j+1}||, the rotations, the cycle's end
        {
            double acc[1] = {orth(j, true)};
            block_reduce_store<double, 1>(acc, pnorm);
            if (!grid_barrier(bar, bar_err, target += nb)) return;
            double sum[1];
            grid_sums<1>(pnorm, sum);
            if (threadIdx.x == 0) {
                GmresCtl& C = S.ctl;
                const double nrm = sqrt(sum[0]);
                const double hn = S.inv[j] * nrm;  // h_{j+1,j}
                for (int k = 0; k < j; ++k) {
                    const double a = S.H[k][j], bb = S.H[k + 1][j];
                    S.H[k][j] = S.cs[k] * a + S.sn[k] * bb;
                    S.H[k + 1][j] = -S.sn[k] * a + S.cs[k] * bb;
                }
                const double a = S.H[j][j];
                const double den = sqrt(a * a + hn * hn);
                const double cs = den > 0 ? a / den : 1.0, sn = den > 0 ? hn / den : 0.0;
                S.cs[j] = cs;
                S.sn[j] = sn;
                S.H[j][j] = den;
                S.g[j + 1] = -sn * S.g[j];
                S.g[j] = cs * S.g[j];
                S.inv[j + 1] = nrm > 0 ? 1.0 / nrm : 0.0;
                const double res = fabs(S.g[j + 1]) / C.bnorm;
                C.res = res;
                C.it += 1;
                S.j = j + 1;
                if (!finite(res) || !finite(den)) { C.status = KS_NOTFINITE; C.done = 1; }
                else if (res < S.tol || j + 1 >= S.m || nrm == 0 || C.it >= S.max_iter) C.cycle_end = 1;
            }
            __syncthreads();
        }
        if (S.ctl.done) break;
        if (!S.ctl.cycle_end) continue;
        // the end of the cycle: y from R y = g, x += sum_i y_i inv_i u_i
        if (threadIdx.x == 0) {
            const int k = S.j;
            double y[kGmresMaxM];
            for (int i = k - 1; i >= 0; --i) {
                double sacc = S.g[i];
                for (int l = i + 1; l < k; ++l) sacc -= S.H[i][l] * y[l];
                y[i] = sacc / S.H[i][i];
            }
            for (int i = 0; i < kGmDots; ++i) S.c[i] = (i < k) ? y[i] * S.inv[i] : 0.0;
        }
        __syncthreads();
        {
            const int k = S.j;
            for (int64_t q = gtid; q < rows; q += gstride) {
                double t = x[q];
#pragma unroll 4
                for (int i = 0; i < k; ++i) t = fma(S.c[i], U[(int64_t)i * rows + q], t);
                x[q] = t;
            }
        }
        if (!grid_barrier(bar, bar_err, target += nb)) return;
        // the restart: r = b - A x -> u_0, the true residual, the next length
        {
            double acc[1] = {0};
            for (int64_t q = gtid; q < rows; q += gstride) {
                const double r = b[q] - small_row<WW>(cols, vals, W, rows, q, x[q], [&](int64_t c) { return __ldcg(x + c); });
                U[q] = r;
                acc[0] = fma(r, r, acc[0]);
            }
            block_reduce_store<double, 1>(acc, pnorm);
            if (!grid_barrier(bar, bar_err, target += nb)) return;
            double sum[1];
            grid_sums<1>(pnorm, sum);
            if (threadIdx.x == 0) {
                GmresCtl& C = S.ctl;
                const double beta = sqrt(sum[0]);
                C.res = beta / C.bnorm;
                S.g[0] = beta;
                S.inv[0] = beta > 0 ? 1.0 / beta : 0.0;
                S.j = 0;
                C.cycle_end = 0;
                if (!finite(C.res)) { C.status = KS_NOTFINITE; C.done = 1; }
                else if (C.res < S.tol) { C.status = KS_CONVERGED; C.done = 1; }
                else if (C.it >= S.max_iter) { C.status = KS_MAXITER; C.done = 1; }
                else {
                    const RestartRule R{S.m_min, S.m_max, S.step_min, S.step_max};
                    S.m = next_restart_with(S.m, S.res_prev > 0 ? C.res / S.res_prev : 0.0, R, S.max_cr, S.min_cr);
                }
                S.res_prev = C.res;
            }
            __syncthreads();
            if (S.ctl.done) break;
        }
    }
    if (blockIdx.x == 0) {
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&S);
        unsigned long long* dst = reinterpret_cast<unsigned long long*>(st);
        for (int k = threadIdx.x; k < (int)(sizeof(GmresState) / 8); k += KB) dst[k] = src[k];
    }
}

// ---- launchers --------------------------------------------------------------

void gmres_init(const EllMatrix& A, const double* b, const double* x, GmresWork& G, KrylovWork& W, bool first,
                cudaStream_t s)
{
    MHFEM_WIDTH_DISPATCH(A.width, (k_gm_init<WW><<<row_grid(k_gm_init<WW>, A.rows), KB, 0, s>>>(
                                      A.cols, A.vals, A.width, A.rows, b, x, G.U, G.st, first ? 1 : 0, W.partials,
                                      W.counters)));
}

void gmres_iterate(const EllMatrix& A, GmresWork& G, KrylovWork& W, int iters, bool reorth, cudaStream_t s)
{
    for (int it = 0; it < iters; ++it) {
        MHFEM_WIDTH_DISPATCH(A.width, launch_pdl(k_gm_arnoldi<WW, true>, s, A.rows, (const int32_t*)A.cols,
                                                 (const double*)A.vals, A.width, A.rows, G.U, G.st, G.partials,
                                                 W.counters));
        if (reorth) {
            launch_pdl(k_gm_orth<false>, s, A.rows, A.rows, G.U, G.st, W.partials, W.counters);
            launch_pdl(k_gm_arnoldi<0, false>, s, A.rows, (const int32_t*)A.cols, (const double*)A.vals, A.width, A.rows,
                       G.U, G.st, G.partials, W.counters);
        }
        launch_pdl(k_gm_orth<true>, s, A.rows, A.rows, G.U, G.st, W.partials, W.counters);
    }
}

void gmres_update(double* x, GmresWork& G, int64_t rows, cudaStream_t s)
{
    k_gm_solve<<<1, 32, 0, s>>>(G.st);
    k_gm_update_x<<<row_grid(k_gm_update_x, rows), KB, 0, s>>>(rows, G.U, x, G.st);
}

cudaError_t gmres_small(const EllMatrix& A, const double* b, double* x, GmresWork& G, KrylovWork& W, bool reorth,
                        int iters, cudaStream_t s)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const int sms = sm_count(dev);
    int nb = 0;
    auto occ = [&](auto kern) { return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, KB, 0); };
    if (reorth) MHFEM_WIDTH_DISPATCH(A.width, e = occ(k_gmres_small<WW, true>));
    else MHFEM_WIDTH_DISPATCH(A.width, e = occ(k_gmres_small<WW, false>));
    if (e != cudaSuccess) return e;
    if (nb < 1) return cudaErrorCooperativeLaunchTooLarge;
    // about two rows per thread, every CTA resident, at most one per SM, and
    // at most as many CTAs as the partials regions hold
    const int64_t want = (A.rows + 2 * (int64_t)KB - 1) / (2 * (int64_t)KB);
    int grid = (int)std::min<int64_t>(std::min<int64_t>(want, (int64_t)sms), (int64_t)nb * sms);
    grid = std::max(1, std::min(grid, std::min(krylov_grid() / 2, W.grid)));
    unsigned int* bar = W.counters + 2;
    int* bar_err = reinterpret_cast<int*>(W.counters + 3);
    e = cudaMemsetAsync(bar, 0, 2 * sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    const int32_t* cols = A.cols;
    const double* vals = A.vals;
    int W_ = A.width;
    int64_t rows = A.rows;
    double* U = G.U;
    GmresState* st = G.st;
    double* pdots = G.partials;
    double* pnorm = W.partials;
    int its = iters;
    void* args[] = {(void*)&cols, (void*)&vals, (void*)&W_, (void*)&rows, (void*)&b, (void*)&x, (void*)&U,
                    (void*)&st, (void*)&pdots, (void*)&pnorm, (void*)&bar, (void*)&bar_err, (void*)&its};
    if (reorth)
        MHFEM_WIDTH_DISPATCH(A.width, e = cudaLaunchCooperativeKernel((const void*)k_gmres_small<WW, true>, dim3(grid),
                                                                     dim3(KB), args, 0, s));
    else
        MHFEM_WIDTH_DISPATCH(A.width, e = cudaLaunchCooperativeKernel((const void*)k_gmres_small<WW, false>, dim3(grid),
                                                                     dim3(KB), args, 0, s));
    return e;
}

}  // namespace mhfem
