// Inputs and outputs of the learned warm-start network: the 16 BF16 input
// features of every face, the training target and the gate that accepts or
// rejects the guess (the per-step scales, the extrapolated base and its
// residual come from learned_prep_fp64).
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
//   12 r / rms(r), r = b - A (2 Zn - Zn1) the residual of the extrapolated guess
//   13-15 zero
// The network predicts (Z_new - (2 Zn - Zn1)) / sd.
#include <cuda_bf16.h>

#include "mhfem_internal.h"
#include "mpnn.h"

namespace mhfem {

namespace {

// The scales come from the device (learned_prep_fp64's output), once per block.
__global__ void __launch_bounds__(256) k_features(int64_t F, MpnnInputs in, __nv_bfloat16* x0)
{
    __shared__ double rsz, rsd;
    __shared__ float rscale;
    if (threadIdx.x == 0) {
        const double sz = in.scal[0], sd = in.scal[1], rn = in.scal[2];
        rsz = sz > 0 ? 1.0 / sz : 0.0;
        rsd = sd > 0 ? 1.0 / sd : 0.0;
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

__global__ void k_target(int64_t F, const double* Znew, const double* base, const double* scal, double* y)
{
    const double sd = scal[1];
    const double rsd = sd > 0 ? 1.0 / sd : 0.0;
    const int64_t E = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (E < F) y[E] = (Znew[E] - base[E]) * rsd;
}

// The learned gate, decided on the device so that no host round trip sits
// between the guess and the solve.
__global__ void __launch_bounds__(256) k_gate(int64_t F, const double* guess, double* Z, const double* rguess,
                                              double* scal)
{
    const double rg = *rguess, rw = scal[3];
    const bool use = isfinite(rg) && rg < rw;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        scal[5] = rg;
        scal[6] = use ? 1.0 : 0.0;
    }
    if (!use) return;
    for (int64_t q = (int64_t)blockIdx.x * 256 + threadIdx.x; q < F; q += (int64_t)gridDim.x * 256) Z[q] = guess[q];
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

void mpnn_target(int64_t F, const double* Znew, const double* base, const double* scal, double* y, cudaStream_t s)
{
    k_target<<<nb(F), 256, 0, s>>>(F, Znew, base, scal, y);
}

void mpnn_gate(int64_t F, const double* guess, double* Z, const double* rguess, double* scal, cudaStream_t s)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t cap = (int64_t)(sms > 0 ? sms : 152) * 8;
    const int64_t g = (int64_t)nb(F) < cap ? (int64_t)nb(F) : cap;
    k_gate<<<(unsigned)(g > 0 ? g : 1), 256, 0, s>>>(F, guess, Z, rguess, scal);
}

void mpnn_features_from_host(int64_t F, const float* xf, __nv_bfloat16* x0, cudaStream_t s)
{
    k_from_host<<<nb(F * 16), 256, 0, s>>>(F * 16, xf, x0);
}

void mpnn_out(const MpnnView& V, float* out, cudaStream_t s) { k_out<<<nb(V.F), 256, 0, s>>>(V, out); }

}  // namespace mhfem
