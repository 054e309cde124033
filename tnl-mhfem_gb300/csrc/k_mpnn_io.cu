// Inputs and outputs of the learned warm-start network: the 16 BF16 input
// features of every face, the extrapolated base, the training target and
// the gate that picks the solve's initial guess (the per-step scales and
// the residuals come from learned_prep_fp64).
//
// Features of face E (x0[E][c]):
//   0  Zn / sz                 current trace (the previous step's solution)
//   1  (Zn - Zn1) / sd         last increment
//   2  rhs / sz                right-hand side of the current system
//   3  log D, mean of the adjacent cells (static)
//   4  source f, mean of the adjacent cells, at the current time
//   5-7 |n_x|, |n_y|, |n_z|   unit normal, sign-free (static)
//   8  face measure / mean face measure (static)
//   9  boundary flag, 10 Dirichlet flag, 11 constant 1 (static)
//   12 r / rms(r), r = b - A base the residual of the extrapolated base
//   13 (Zn - 2 Zn1 + Zn2) / s2, 14 (Zn - 3 Zn1 + 3 Zn2 - Zn3) / s3: the second
//      and third time differences (zero until the history reaches them)
//   15 zero
// The base is the polynomial extrapolation of the last traces in time (order
// 1 to 3: 2 Zn - Zn1, 3 Zn - 3 Zn1 + Zn2, 4 Zn - 6 Zn1 + 4 Zn2 - Zn3), and the
// network predicts (Z_new - base) / c, with c the root mean square of the
// previous step's base error (Z_new - base over the free rows).
//
// Device scalars (scal[]): 0 rms(Zn), 1 sd = rms(Zn - Zn1), 2 ||b - A base||,
// 3 ||b - A Zn|| / ||b||, 4 ||b||, 5 the network guess's relative residual,
// 6 the gate's choice (0 warm start, 1 network guess, 2 base), 8 the last
// measured base error c, 9 ||b - A base|| / ||b||, 10 the scale used this
// step (c, or sd until c is known), 11 and 12 the rms of the second and third
// time differences.
#include <cuda_bf16.h>

#include "krylov_common.cuh"
#include "mpnn.h"

namespace mhfem {

namespace {

// The scales come from the device (learned_prep_fp64's output), once per block.
__global__ void __launch_bounds__(256) k_features(int64_t F, MpnnInputs in, __nv_bfloat16* x0)
{
    __shared__ double rsz, rsd, rs2, rs3;
    __shared__ float rscale;
    if (threadIdx.x == 0) {
        const double sz = in.scal[0], sd = in.scal[1], rn = in.scal[2], s2 = in.scal[11], s3 = in.scal[12];
        rsz = sz > 0 ? 1.0 / sz : 0.0;
        rsd = sd > 0 ? 1.0 / sd : 0.0;
        rs2 = (in.hist >= 2 && s2 > 0) ? 1.0 / s2 : 0.0;
        rs3 = (in.hist >= 3 && s3 > 0) ? 1.0 / s3 : 0.0;
        rscale = rn > 0 ? (float)(sqrt((double)F) / rn) : 0.f;
    }
    __syncthreads();
    const int64_t E = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (E >= F) return;
    float v[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) v[c] = in.stat[E * 16 + c];
    const double z = in.Zn[E];
    v[0] = (float)(z * rsz);
    v[1] = (float)((z - in.Zn1[E]) * rsd);
    v[2] = (float)(in.rhs[E] * rsz);
    v[4] = (float)((in.f_base[E] + in.src_scale * in.f_psi[E]) * in.f_norm);
    v[12] = (float)in.rbase[E] * rscale;
    if (in.hist >= 2) {
        const double z1 = in.Zn1[E], z2 = in.Zn2[E];
        v[13] = (float)(fma(-2.0, z1, z + z2) * rs2);
        if (in.hist >= 3) v[14] = (float)(((z - in.Zn3[E]) + 3.0 * (z2 - z1)) * rs3);
    }
    uint32_t w[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const __nv_bfloat162 p = __floats2bfloat162_rn(v[2 * c], v[2 * c + 1]);
        w[c] = *reinterpret_cast<const uint32_t*>(&p);
    }
    uint4* dst = reinterpret_cast<uint4*>(x0 + E * 16);
    dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
    dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
}

// base = polynomial extrapolation of the last traces; the Dirichlet rows take
// their prescribed value (their row of the system is the identity)
__global__ void __launch_bounds__(256) k_extrapolate(int64_t F, int order, const double* Z0, const double* Z1,
                                                     const double* Z2, const double* Z3, const uint8_t* fixed,
                                                     const double* rhs, double* base)
{
    const int64_t E = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (E >= F) return;
    double v;
    if (fixed[E]) v = rhs[E];
    else if (order >= 3) v = fma(4.0, Z0[E], fma(-6.0, Z1[E], fma(4.0, Z2[E], -Z3[E])));
    else if (order == 2) v = fma(3.0, Z0[E] - Z1[E], Z2[E]);
    else if (order == 1) v = fma(2.0, Z0[E], -Z1[E]);
    else v = Z0[E];
    base[E] = v;
}

// y = (Znew - base) / scal[10] (training target, when y != nullptr) and the
// base's error c = rms(Znew - base) over the free rows into scal[8] for the
// next step: per-block partial sums, summed in a fixed order by the last block.
__global__ void __launch_bounds__(KB) k_target(int64_t F, const double* Znew, const double* base, const uint8_t* fixed,
                                               double* scal, double* y, double* partials, uint32_t* counter)
{
    const double c = scal[10];
    const double rc = c > 0 ? 1.0 / c : 0.0;
    double acc[2] = {0, 0};
    for (int64_t E = (int64_t)blockIdx.x * KB + threadIdx.x; E < F; E += (int64_t)gridDim.x * KB) {
        const double d = Znew[E] - base[E];
        if (y) y[E] = d * rc;
        if (!fixed[E]) {
            acc[0] = fma(d, d, acc[0]);
            acc[1] += 1.0;
        }
    }
    block_reduce_store<double, 2>(acc, partials);
    if (!ticket_last(counter)) return;
    double sum[2];
    final_sums<2>(partials, sum);
    if (threadIdx.x == 0 && sum[1] > 0) scal[8] = sqrt(sum[0] / sum[1]);
}

// The learned gate, decided on the device so that no host round trip sits
// between the guess and the solve: of the warm start (scal[3]), the
// extrapolated base (scal[9]) and the network's guess (*rguess, when it ran)
// the one with the lowest relative FP64 residual becomes the initial guess.
__global__ void __launch_bounds__(256) k_gate(int64_t F, const double* guess, const double* base, double* Z,
                                              const double* rguess, double* scal)
{
    const double rw = scal[3], rb = scal[9];
    const double rg = guess ? *rguess : INFINITY;
    int choice = 0;
    double best = rw;
    if (isfinite(rb) && rb < best) { choice = 2; best = rb; }
    if (isfinite(rg) && rg < best) { choice = 1; best = rg; }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        scal[5] = guess ? rg : -1.0;
        scal[6] = (double)choice;
    }
    if (choice == 0) return;
    const double* src = choice == 1 ? guess : base;
    for (int64_t q = (int64_t)blockIdx.x * 256 + threadIdx.x; q < F; q += (int64_t)gridDim.x * 256) Z[q] = src[q];
}

__global__ void k_from_host(int64_t n, const float* xf, __nv_bfloat16* x0)
{
    const int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (i < n) x0[i] = __float2bfloat16(xf[i]);
}

__global__ void __launch_bounds__(256) k_out(MpnnView V, float* out)
{
    const int64_t E = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (E >= V.F) return;
    const __nv_bfloat16* h4 = V.h[kMpnnLayers + 1] + E * kMpnnHidden;
    float s = V.bd[0];
    for (int q = 0; q < kMpnnHidden; ++q) s = fmaf(__bfloat162float(h4[q]), V.wd[q], s);
    out[E] = s;
}

}  // namespace

static unsigned nb(int64_t n) { return (unsigned)((n + 255) / 256); }

void mpnn_features(int64_t F, const MpnnInputs& in, __nv_bfloat16* x0, cudaStream_t s)
{
    k_features<<<nb(F), 256, 0, s>>>(F, in, x0);
}

void mpnn_extrapolate(int64_t F, int order, const double* Z0, const double* Z1, const double* Z2, const double* Z3,
                      const uint8_t* fixed, const double* rhs, double* base, cudaStream_t s)
{
    k_extrapolate<<<nb(F), 256, 0, s>>>(F, order, Z0, Z1, Z2, Z3, fixed, rhs, base);
}

void mpnn_target(int64_t F, const double* Znew, const double* base, const uint8_t* fixed, double* scal, double* y,
                 double* partials, uint32_t* counter, cudaStream_t s)
{
    k_target<<<row_grid(k_target, F), KB, 0, s>>>(F, Znew, base, fixed, scal, y, partials, counter);
}

void mpnn_gate(int64_t F, const double* guess, const double* base, double* Z, const double* rguess, double* scal,
               cudaStream_t s)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t cap = (int64_t)(sms > 0 ? sms : 152) * 8;
    const int64_t g = (int64_t)nb(F) < cap ? (int64_t)nb(F) : cap;
    k_gate<<<(unsigned)(g > 0 ? g : 1), 256, 0, s>>>(F, guess, base, Z, rguess, scal);
}

void mpnn_features_from_host(int64_t F, const float* xf, __nv_bfloat16* x0, cudaStream_t s)
{
    k_from_host<<<nb(F * 16), 256, 0, s>>>(F * 16, xf, x0);
}

void mpnn_out(const MpnnView& V, float* out, cudaStream_t s) { k_out<<<nb(V.F), 256, 0, s>>>(V, out); }

}  // namespace mhfem
