// Internal declarations shared by the host orchestration and the kernels.
#pragma once

#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mhfem.h"

namespace mhfem {

// A coefficient: a uniform value (stride 0) or a full array.
struct Coef {
    const double* p = nullptr;
    int full = 0;
};

// Krylov scalars kept on the device; written by the last block of each
// reduction kernel so an iteration never round-trips to the host.
struct KrylovScalars {
    double rho, alpha, omega, beta;
    double bnorm, res, snorm;
    double rv, ts, tt, rr, rhnorm;
    int32_t it, done, status, max_iter;
    int32_t restart, half;  // half: the iteration ends on the half step (||s|| < tol)
    double tol;
};

// Krylov status codes written to KrylovScalars::status.
enum : int32_t { KS_RUNNING = 0, KS_CONVERGED = 1, KS_MAXITER = 2, KS_BREAKDOWN = 3, KS_NOTFINITE = 4 };

#ifdef __CUDACC__
// 1 / d in FP64 for the row scaling of the assembly and the LU pivots of the
// cell kernel.  GB300 issues FP64 at 1/57 of the FP32 rate and both kernels
// are bound by their FP64 pipe, where an IEEE FP64 division costs about as
// much as the rest of a face row.  One third-order step from an FP32
// reciprocal estimate r0: with u = 1 - d r0, 1/d = r0 / (1 - u) = r0 (1 + u
// + u^2 + ...), truncated after u^2 (Halley's iteration for f(r) = 1/r - d,
// cubic convergence): r = r0 + r0 (u + u^2).  The estimate's relative error
// is below 2^-22, so the truncation error is below 2^-66, under FP64
// rounding: the result is within an ulp of the correctly rounded quotient
// (the GPU parity tests bound the local quantities and the assembled values
// at 1e-12 relative against the oracle's IEEE division).  The FP32 operand
// and the FP32 estimate move between the two IEEE formats by integer bit
// operations (sign, rebiased exponent, truncated mantissa), so the FP64
// pipe only sees three fused multiply-adds.  Magnitudes outside
// [2^-100, 2^100] (and 0, inf, NaN) take the IEEE division.
static __device__ __noinline__ double recip_ieee(double d) { return 1.0 / d; }

__device__ __forceinline__ double recip_newton(double d)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const int e = (int)((b >> 52) & 0x7ff);
    if (e < 1023 - 100 || e > 1023 + 100) return recip_ieee(d);
    const unsigned fb = ((unsigned)(b >> 32) & 0x80000000u) | ((unsigned)(e - 1023 + 127) << 23) |
                        (unsigned)((b >> 29) & 0x7fffffu);
    const unsigned rb = __float_as_uint(__frcp_rn(__uint_as_float(fb)));
    const unsigned long long r64 = ((unsigned long long)(rb & 0x80000000u) << 32) |
                                   ((unsigned long long)(((rb >> 23) & 0xffu) - 127u + 1023u) << 52) |
                                   ((unsigned long long)(rb & 0x7fffffu) << 29);
    const double r = __longlong_as_double((long long)r64);
    const double u = fma(-d, r, 1.0);
    return fma(r, fma(u, u, u), r);
}

// d > 0 (including +inf; false for zero, negatives and NaN) as an integer
// test on the bit pattern, which keeps the compare off the FP64 pipe.
__device__ __forceinline__ bool positive_bits(double d)
{
    const long long b = __double_as_longlong(d);
    return b > 0 && b <= 0x7ff0000000000000LL;
}
#endif

// Device-side view of a problem, passed by value to kernels.
struct DevProblem {
    int dim, cell, nf, n, S, lumping, advection, mobility_upwind;  // cell: 0 simplices, 1 boxes
    int64_t V, C, F, rows;
    const double* coords;        // [V][dim]
    const int32_t* cell_verts;   // SoA [v][C]
    const int32_t* cell_faces;   // SoA [e][C]
    const uint8_t* cell_bmask;   // bit e set: local face e lies on the boundary
    const int2* face_cells;      // [F] (K0, K1), K1 = -1 on the boundary
    const uint8_t* face_local;   // [F][2] local index of the face in K0, K1
    const double* face_measure;  // [F]
    Coef N, u, m, D, w, a, r, f, m_upw_in, m_bnd, psi;
    double src_amp, src_omega, src_time;  // time-modulated source
    const uint8_t* bc_tags;      // (i*F + E)
    const double* bc_values;
    const double* bc_dirichlet;
    double* Z_iF;                // (E, i)
    double* Z_iK;                // (i, K)
    double* v_iKe;               // (i, e, K)
    double* m_upw;               // (E, i) when computed
    double* Z_upw;               // (E, j, i)
    double* b;                   // (i, j, s, K)
    double* R_ijKe;              // (i, j, e, K)
    double* R_iK;                // (i, K)
    double* rec;                 // per (K, e) assembly record, stride rec_stride doubles
    int rec_stride;
    int use_m_upw_array;         // m_upw read from an (E,i) array (computed or model input)
    const double* m_upw_read;    // the array read when use_m_upw_array
    int explicit_adv_active;     // explicit upwind with a or u not identically zero
    int32_t* err_flags;          // device error word (bit 0: non-positive diagonal, bit 1: non-finite)
};

// ELL storage of the off-diagonal part of the unit-diagonal face system.
struct EllMatrix {
    int64_t rows = 0;
    int width = 0;               // off-diagonal entries per row (max)
    int32_t* cols = nullptr;     // [width][rows]
    double* vals = nullptr;      // [width][rows]
    float* vals32 = nullptr;     // [width][rows] (mixed form)
    // The FP32 SpMVs' column indices as 24-bit offsets from the row (mixed
    // form, when every |col - row| < 2^23): col - row + 2^23 split into the
    // low 16 bits and the high 8 bits, each [width][rows].  Three bytes per
    // entry instead of four; null when not built.
    uint16_t* cols_lo = nullptr;
    uint8_t* cols_hi = nullptr;
};
constexpr int32_t kCol24Bias = 1 << 23;

// Per-row assembly map: which ELL slot each (side, local face) goes to.
struct AssemblyMap {
    void* qmap = nullptr;        // per face: 4 bits per (side, local face): merged position q;
                                 // uint32 words up to 4 faces per cell, uint64 for cuboids
    uint8_t* qdiag = nullptr;    // per face: merged position of the face itself
};

// Launchers (k_local.cu)
// Each launcher returns the number of kernels it launched.
int launch_face_average(const DevProblem& P, cudaStream_t s);
int launch_upwind(const DevProblem& P, cudaStream_t s);
int launch_cell_local(const DevProblem& P, double tau, cudaStream_t s);
// b alone (before a model's vector-coefficient hook; the cell kernel writes the same b again)
int launch_update_b(const DevProblem& P, cudaStream_t s);
int launch_reconstruct(const DevProblem& P, cudaStream_t s);

// Launchers (k_assemble.cu)
int launch_assemble(const DevProblem& P, const AssemblyMap& M, EllMatrix& A, double* rhs,
                    int write32, cudaStream_t s);

// Krylov (k_krylov.cu)
struct KrylovWork {
    int64_t rows = 0;
    int grid = 0, block = 256;
    double *r = nullptr, *rh = nullptr, *p = nullptr, *v = nullptr, *s = nullptr, *t = nullptr;
    double *p2 = nullptr, *v2 = nullptr;  // second p and v buffers of the small-system solve
    float *r32 = nullptr, *rh32 = nullptr, *p32 = nullptr, *v32 = nullptr, *s32 = nullptr,
          *t32 = nullptr, *x32 = nullptr;
    double* partials = nullptr;      // [grid][8]
    uint32_t* counters = nullptr;    // last-block counters
    KrylovScalars* sc = nullptr;     // device scalars (FP64 solve / outer)
    KrylovScalars* sc32 = nullptr;   // device scalars (inner FP32 solve)
    KrylovScalars* host_sc = nullptr;// pinned mirror
};

void krylov_init_fp64(const EllMatrix& A, const double* b, double* x, KrylovWork& W,
                      double tol, int max_iter, cudaStream_t s);

// ---- restarted GMRES (k_gmres.cu) ---------------------------------------------

constexpr int kGmresMaxM = 32;  // longest restart cycle
constexpr int kGmStride = 40;   // partial sums per block of the Arnoldi dot products (>= kGmresMaxM + 1)

// The part of the GMRES state the host polls (one small copy per check).
struct GmresCtl {
    int32_t it, done, status, cycle_end;
    double res;    // ||b - A x|| / ||b|| at the last restart, or the rotated estimate inside a cycle
    double bnorm;
};

// Device state of one GMRES solve.  The basis is stored unnormalized:
// v_i = inv[i] * u_i.  H holds the Hessenberg columns of the cycle, rotated
// in place into the triangular factor; g is the rotated right-hand side.
struct GmresState {
    GmresCtl ctl;
    double tol;
    int32_t m, j, max_iter, pad;
    double inv[kGmresMaxM + 1];
    double c[kGmresMaxM + 1];  // multipliers of u_i in the current orthogonalization / x update
    double H[kGmresMaxM + 1][kGmresMaxM];
    double cs[kGmresMaxM], sn[kGmresMaxM];
    double g[kGmresMaxM + 1];
    // restarts inside the persistent small-system solve: the true relative
    // residual at the last restart, and the adaptive restart rule
    // (gmres_restart.h) with its two thresholds
    double res_prev;
    double max_cr, min_cr;
    int32_t m_min, m_max, step_min, step_max;
};

struct GmresWork {
    int m = 0;
    double* U = nullptr;          // [m + 1][rows] basis
    double* partials = nullptr;   // [grid][kGmStride]
    GmresState* st = nullptr;     // device
    GmresCtl* host = nullptr;     // pinned mirror of st->ctl
    int32_t* host_m = nullptr;    // pinned: the next cycle's restart length (adaptive restarting)
};

// r = b - A x into u_0 and the restart scalars; first: also ||b|| and it = 0
void gmres_init(const EllMatrix& A, const double* b, const double* x, GmresWork& G, KrylovWork& W,
                bool first, cudaStream_t s);
// `iters` Arnoldi iterations (each returns at once after the cycle ended)
void gmres_iterate(const EllMatrix& A, GmresWork& G, KrylovWork& W, int iters, bool reorth, cudaStream_t s);
// end of a cycle: solve the triangular system and update x
void gmres_update(double* x, GmresWork& G, int64_t rows, cudaStream_t s);
// Small systems (at most krylov_small_rows() rows): up to `iters` Arnoldi
// iterations, restarts included, in one cooperative launch (bounded grid
// barriers; W.counters + 2 and + 3 are its barrier count and failure flag).
cudaError_t gmres_small(const EllMatrix& A, const double* b, double* x, GmresWork& G, KrylovWork& W, bool reorth,
                        int iters, cudaStream_t s);
void krylov_iterate_fp64(const EllMatrix& A, double* x, KrylovWork& W, int iters, cudaStream_t s);
// Small systems (rows <= krylov_small_rows()): up to `iters` FP64 BiCGStab
// iterations in one cooperative launch on a solve set up by krylov_init_fp64
// (p and v alternate between W.p / W.p2 and W.v / W.v2); the two words at
// W.counters + 2 are the grid barrier's arrival count and its failure flag
// (non-zero after a barrier wait gave up).
int64_t krylov_small_rows();
cudaError_t krylov_small_fp64(const EllMatrix& A, double* x, KrylovWork& W, int iters, cudaStream_t s);
// One cooperative launch of `ctas` CTAs through the small-system solve's
// bounded grid barrier, CTA `skip` (none if negative) never arriving; counts
// the CTAs that passed and that gave up, and returns the failure flag.
cudaError_t grid_barrier_check(int ctas, int skip, unsigned int max_polls, int* passed, int* gave_up, int* flag);

// mixed: outer residual r = b - A x (FP64) -> sc; scale into r32; inner FP32 solve; x += scale*e
void mixed_outer_residual(const EllMatrix& A, const double* b, const double* x, KrylovWork& W,
                          double tol, int max_sweeps, cudaStream_t s);
void mixed_inner_init(KrylovWork& W, double inner_tol, int adaptive, int max_iter, cudaStream_t s);
void krylov_iterate_fp32(const EllMatrix& A, KrylovWork& W, int iters, cudaStream_t s);
void mixed_apply_correction(double* x, KrylovWork& W, cudaStream_t s);

// Residual of a candidate x: ||b - A x|| / ||b|| into W.sc->res (used by the learned gate)
void residual_norm_fp64(const EllMatrix& A, const double* b, const double* x, KrylovWork& W,
                        cudaStream_t s);

int krylov_grid();

// Learned form, one pass before the network, on the extrapolated base formed
// beforehand: rbase = b - A base, out[0..4] = rms(Zn), rms(Zn - Zn1) (free
// rows), ||rbase||, ||b - A Zn|| / ||b||, ||b||; out[9] = ||rbase|| / ||b||,
// out[10] = the network's output scale (out[8] when set, else out[1]);
// out[11], out[12] = rms of the second and third time differences (free
// rows) when hist (the traces before Zn) reaches 2 and 3.
void learned_prep_fp64(const EllMatrix& A, const double* b, const double* Zn, const double* Zn1, const double* Zn2,
                       const double* Zn3, int hist, const double* base, const uint8_t* fixed, double* rbase,
                       double* out, KrylovWork& W, cudaStream_t s);

// One launch of the SpMV + dot kernel on the current Krylov vectors (timing).
void krylov_spmv_dot_once(const EllMatrix& A, KrylovWork& W, bool fp32, cudaStream_t s);
// One launch of FP64 iteration kernel `which` (0 SpMV + dot, 1 second SpMV + dots,
// 2 s update, 3 x / r update on W.v instead of x, 4 p update) (timing).
void krylov_fp64_kernel_once(const EllMatrix& A, KrylovWork& W, int which, cudaStream_t s);

}  // namespace mhfem
