// Device views and launchers of the learned warm-start network (k_mpnn.cu).
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mhfem_internal.h"

namespace mhfem {

constexpr int kMpnnHidden = 64;
constexpr int kMpnnFeatures = 16;
constexpr int kMpnnLayers = 3;
// Largest neighbour count the network kernels take (triangles: 4, tetrahedra: 6
// for one equation).
constexpr int kMpnnMaxWidth = 6;
// FP32 master parameters: W0 [16][64], b0, W1..W3 [128][64], b1..b3, wd [64], bd
constexpr int kMpnnParams = kMpnnFeatures * kMpnnHidden + kMpnnHidden
                          + kMpnnLayers * (2 * kMpnnHidden * kMpnnHidden + kMpnnHidden) + kMpnnHidden + 1;

struct MpnnView {
    int64_t F = 0;
    int W = 0;
    const int32_t* nbr = nullptr;     // [W][F], padding = own index
    const uint8_t* deg = nullptr;     // [F]
    const uint8_t* fixed = nullptr;   // [F] Dirichlet rows (excluded from the loss, guess = rhs)
    __nv_bfloat16* x0 = nullptr;      // [F][16]
    __nv_bfloat16* h[kMpnnLayers + 2] = {};  // h[1..4] [F][64]
    __nv_bfloat16* a[kMpnnLayers + 1] = {};  // a[1..3] [F][64] (training)
    __nv_bfloat16* z[kMpnnLayers + 1] = {};  // z[0..3] [F][64] (training)
    __nv_bfloat16* dz = nullptr;      // [F][64]
    float* dh = nullptr;              // [F][64]
    __nv_bfloat16* gb[2] = {};        // [F][64] each: neighbour-mean gradients, layer l writes gb[l % 2]
    const __nv_bfloat16* w_fwd[kMpnnLayers + 1] = {};  // [64][K_l]
    const __nv_bfloat16* w_bwd[kMpnnLayers + 1] = {};  // [K_l][64]
    const float* bias[kMpnnLayers + 1] = {};           // [64]
    const float* wd = nullptr;        // [64]
    const float* bd = nullptr;        // [1]
    double* dec_partials = nullptr;   // [grid][66]
    int32_t* err = nullptr;
    // inference: the decoder fused into the last layer writes
    // guess = base + sd (h4 . wd + bd) on free rows, the Dirichlet value on fixed rows
    const double* dec_base = nullptr;
    const double* dec_rhs = nullptr;
    const double* dec_scal = nullptr;  // device scalars; the output scale c at [10]
    double* dec_guess = nullptr;
};

struct MpnnGrads {
    float* g = nullptr;               // flat, same layout as the master parameters
    int off_W[kMpnnLayers + 1] = {}, off_b[kMpnnLayers + 1] = {}, off_wd = 0, off_bd = 0;
    float* partials = nullptr;        // [grid][128*64 + 64]
    double* loss = nullptr;
};

// All layers; every hidden state is written (training, and the forward of
// the C ABI's parity entry point).
void mpnn_forward(const MpnnView& V, bool train, cudaStream_t s);
// Inference: layers 0..2, then the last layer with the decoder fused into its
// epilogue (V.dec_* set); h4 is not stored.
void mpnn_infer_guess(const MpnnView& V, cudaStream_t s);
void mpnn_backward(const MpnnView& V, const double* target, double inv_nt, MpnnGrads& G, cudaStream_t s);
void mpnn_adam(float* params, const float* grads, float* m1, float* m2, int n, float lr, int t, cudaStream_t s);
void mpnn_publish(const float* W, int K, __nv_bfloat16* wf, __nv_bfloat16* wb, cudaStream_t s);
int mpnn_partials_floats(int64_t F);
int mpnn_grid_size(int64_t F);

// feature / target helpers (k_mpnn_io.cu)
struct MpnnInputs {
    const double* Zn;        // current face traces (warm start)
    const double* Zn1;       // previous step's traces
    const double* Zn2;       // the traces two and three steps back (read when hist reaches 2, 3)
    const double* Zn3;
    int hist;                // traces available before Zn (0..3)
    const double* rhs;       // scaled right-hand side of the current system
    const float* stat;       // [F][16] static features (channels 3, 5..11 filled)
    const float* f_base;     // [F] face average of the source
    const float* f_psi;      // [F] face average of the source shape psi
    double src_scale;        // amplitude * sin(2 pi t / T)
    double f_norm;           // scale of the source channel
    const double* rbase;     // residual b - A base of the extrapolated base
    const double* scal;      // device scalars (k_mpnn_io.cu): rms(Zn), rms(Zn - Zn1), ||rbase||, ...
};
void mpnn_features(int64_t F, const MpnnInputs& in, __nv_bfloat16* x0, cudaStream_t s);
// base = polynomial extrapolation of order `order` (0..3) of Z0 (newest) .. Z3;
// rhs on the Dirichlet rows
void mpnn_extrapolate(int64_t F, int order, const double* Z0, const double* Z1, const double* Z2, const double* Z3,
                      const uint8_t* fixed, const double* rhs, double* base, cudaStream_t s);
// training target y = (Znew - base) / scal[10] (y may be null) and scal[8] =
// rms(Znew - base) over the free rows; partials / counter: reduction scratch
void mpnn_target(int64_t F, const double* Znew, const double* base, const uint8_t* fixed, double* scal, double* y,
                 double* partials, uint32_t* counter, cudaStream_t s);
// the gate: Z = the candidate with the lowest finite relative residual among
// the warm start Z (scal[3]), base (scal[9]) and guess (*rguess; guess may be
// null); scal[5] = *rguess, scal[6] = the choice (0 warm, 1 guess, 2 base)
void mpnn_gate(int64_t F, const double* guess, const double* base, double* Z, const double* rguess, double* scal,
               cudaStream_t s);
void mpnn_features_from_host(int64_t F, const float* xf, __nv_bfloat16* x0, cudaStream_t s);
void mpnn_out(const MpnnView& V, float* out, cudaStream_t s);

}  // namespace mhfem
