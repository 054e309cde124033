// Inputs and outputs of the learned warm-start network: per-step scales,
// the 16 BF16 input features of every face, the extrapolated base guess and
// the training target.
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

// sz = rms(Zn), sd = rms(Zn - Zn1) over the free rows.  Grid-stride over a
// fixed grid; the last block to finish sums the per-block partials with all
// its threads, in a fixed order.
__global__ void __launch_bounds__(256) k_scales(int64_t F, const double* Zn, const double* Zn1, const uint8_t* fixed,
                                                double* partials, double* scal, uint32_t* counter)
{
    double s0 = 0, s1 = 0, c = 0;
    for (int64_t q = (int64_t)blockIdx.x * 256 + threadIdx.x; q < F; q += (int64_t)gridDim.x * 256) {
        if (fixed[q]) continue;
        const double z = Zn[q], d = z - Zn1[q];
        s0 = fma(z, z, s0);
        s1 = fma(d, d, s1);
        c += 1;
    }
    __shared__ double red[3][256 / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_down_sync(0xffffffffu, s0, o);
        s1 += __shfl_down_sync(0xffffffffu, s1, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if (lane == 0) { red[0][warp] = s0; red[1][warp] = s1; red[2][warp] = c; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0, n = 0;
        for (int w = 0; w < 256 / 32; ++w) { a += red[0][w]; b += red[1][w]; n += red[2][w]; }
        partials[blockIdx.x * 3 + 0] = a;
        partials[blockIdx.x * 3 + 1] = b;
        partials[blockIdx.x * 3 + 2] = n;
        __threadfence();
        const uint32_t prev = atomicAdd(counter, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    double A = 0, B = 0, N = 0;
    for (unsigned p = threadIdx.x; p < gridDim.x; p += 256) {
        A += __ldcg(partials + 3 * p);
        B += __ldcg(partials + 3 * p + 1);
        N += __ldcg(partials + 3 * p + 2);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        A += __shfl_down_sync(0xffffffffu, A, o);
        B += __shfl_down_sync(0xffffffffu, B, o);
        N += __shfl_down_sync(0xffffffffu, N, o);
    }
    __syncthreads();
    if (lane == 0) { red[0][warp] = A; red[1][warp] = B; red[2][warp] = N; }
    __syncthreads();
    if (threadIdx.x == 0) {
        A = B = N = 0;
        for (int w = 0; w < 256 / 32; ++w) { A += red[0][w]; B += red[1][w]; N += red[2][w]; }
        N = N > 0 ? N : 1;
        scal[0] = sqrt(A / N);
        scal[1] = sqrt(B / N);
        *counter = 0;
    }
}

__global__ void __launch_bounds__(256) k_features(int64_t F, MpnnInputs in, double rsz, double rsd,
                                                  __nv_bfloat16* x0)
{
    // scale of the residual channel, once per block (FP64 division and square
    // root are scarce on this part)
    __shared__ float rscale;
    if (threadIdx.x == 0) {
        const double rn = in.rnorm->snorm;
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

__global__ void k_base(int64_t F, const double* Zn, const double* Zn1, double* base)
{
    const int64_t E = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (E < F) base[E] = 2.0 * Zn[E] - Zn1[E];
}

__global__ void k_target(int64_t F, const double* Znew, const double* base, double rsd, double* y)
{
    const int64_t E = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (E < F) y[E] = (Znew[E] - base[E]) * rsd;
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

void mpnn_scales(int64_t F, const MpnnInputs& in, const uint8_t* fixed, double* partials, double* scal,
                 cudaStream_t s)
{
    // partials: [kScalesMaxGrid*3] doubles followed by one uint32 ticket
    // counter (zero-initialized); 8 CTAs per SM
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = (sms > 0 ? sms : 152) * 8;
    if (grid > kScalesMaxGrid) grid = kScalesMaxGrid;
    if ((int64_t)grid * 256 > F) grid = (int)((F + 255) / 256) > 0 ? (int)((F + 255) / 256) : 1;
    uint32_t* counter = reinterpret_cast<uint32_t*>(partials + kScalesMaxGrid * 3);
    k_scales<<<grid, 256, 0, s>>>(F, in.Zn, in.Zn1, fixed, partials, scal, counter);
}

void mpnn_features(int64_t F, const MpnnInputs& in, double sz, double sd, __nv_bfloat16* x0, cudaStream_t s)
{
    k_features<<<nb(F), 256, 0, s>>>(F, in, sz > 0 ? 1.0 / sz : 0.0, sd > 0 ? 1.0 / sd : 0.0, x0);
}

void mpnn_base(int64_t F, const double* Zn, const double* Zn1, double* base, cudaStream_t s)
{
    k_base<<<nb(F), 256, 0, s>>>(F, Zn, Zn1, base);
}

void mpnn_target(int64_t F, const double* Znew, const double* base, double sd, double* y, cudaStream_t s)
{
    k_target<<<nb(F), 256, 0, s>>>(F, Znew, base, sd > 0 ? 1.0 / sd : 0.0, y);
}

void mpnn_features_from_host(int64_t F, const float* xf, __nv_bfloat16* x0, cudaStream_t s)
{
    k_from_host<<<nb(F * 16), 256, 0, s>>>(F * 16, xf, x0);
}

void mpnn_out(const MpnnView& V, float* out, cudaStream_t s) { k_out<<<nb(V.F), 256, 0, s>>>(V, out); }

}  // namespace mhfem
