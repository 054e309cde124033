// The solver handle shared by the C ABI (capi.cpp) and the learned form
// (learned.cpp).
#pragma once

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "mhfem_internal.h"
#include "topology.h"

namespace mhfem {
struct LearnedState;
}

constexpr int NCOEF = 11;

struct DevCoef {
    double* p = nullptr;
    int64_t count = 0;  // 1 = uniform
};

struct mhfem_solver_s {
    mhfem_desc desc{};
    int dim = 0, cell = 0, nf = 0, nv = 0, n = 0, S = 0;  // nv: vertices per cell
    std::string err;
    cudaStream_t stream = nullptr;
    int sms = 0;

    mhfem::HostTopology topo;
    mhfem::HostPattern pat;
    bool has_mesh = false, has_bc = false, has_state = false;
    bool pattern_ready = false;
    std::vector<uint8_t> h_tags;

    // device topology
    double* coords = nullptr;
    int32_t* cell_verts = nullptr;   // SoA
    int32_t* cell_faces = nullptr;   // SoA
    uint8_t* cell_bmask = nullptr;
    int2* face_cells = nullptr;
    uint8_t* face_local = nullptr;
    double* face_measure = nullptr;

    DevCoef coef[NCOEF];
    bool coef_nonzero[NCOEF] = {};
    double src_amp = 0, src_period = 1;

    uint8_t* tags = nullptr;
    double* bvalues = nullptr;
    double* bdirichlet = nullptr;

    double *Z_iF = nullptr, *Z_iK = nullptr, *v_iKe = nullptr, *m_upw = nullptr, *Z_upw = nullptr;
    double *b = nullptr, *R_ijKe = nullptr, *R_iK = nullptr, *rec = nullptr;
    int rec_stride = 0;

    mhfem::EllMatrix A;
    mhfem::AssemblyMap amap;
    double* rhs = nullptr;
    int32_t* err_flags = nullptr;
    int32_t* host_err = nullptr;
    mhfem::KrylovWork W;
    mhfem::GmresWork G;

    mhfem_solver_opts opts{};
    // the matrix keeps an FP32 copy and the FP32 Krylov vectors exist: the
    // mixed form, or the learned form with its mixed solve
    bool fp32_copy = false;
    int64_t total_iters = 0, total_steps = 0, launches = 0;
    double cur_t = 0, cur_tau = 0;

    cudaGraphExec_t g64 = nullptr, g32 = nullptr, ggm = nullptr;  // ggm: GMRES iterations
    int g64_iters = 0, g32_iters = 0;

    cudaEvent_t ev[7] = {};  // phase boundaries 0..4; 5, 6: the learned guess
    struct Hook {
        mhfem_hook fn = nullptr;
        void* user = nullptr;
    } hooks[3];              // MHFEM_HOOK_PRE_ITERATE, MHFEM_HOOK_POST_ITERATE, MHFEM_HOOK_VECTOR_COEFFICIENTS
    bool guess_timed = false;
    std::vector<void*> allocs;

    // host copies: the coordinates and (learned form) D, f, psi build the
    // learned form's static features; a and u give the advection zero test
    std::vector<double> h_coords;
    std::vector<double> h_coef[NCOEF];
    mhfem::LearnedState* learned = nullptr;
};


namespace mhfem {

inline mhfem_status fail(mhfem_t h, mhfem_status code, const char* fmt, ...)
{
    if (h) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        h->err = buf;
    }
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(h, e_ == cudaErrorMemoryAllocation ? MHFEM_ERR_OUT_OF_MEMORY : MHFEM_ERR_CUDA, \
                        "%s failed: %s", #call, cudaGetErrorString(e_));                          \
    } while (0)

template <typename T>
inline cudaError_t dalloc(mhfem_t h, T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
    if (e == cudaSuccess) h->allocs.push_back((void*)*p);
    return e;
}

template <typename T>
inline void dfree(mhfem_t h, T*& p)
{
    if (!p) return;
    auto it = std::find(h->allocs.begin(), h->allocs.end(), (void*)p);
    if (it != h->allocs.end()) h->allocs.erase(it);
    cudaFree((void*)p);
    p = nullptr;
}

// FP64 BiCGStab from the current Z_iF (capi.cpp).
mhfem_status run_fp64(mhfem_t h, double tol, int max_iter, int* iters, double* res);
// Mixed-precision refinement from the current Z_iF (capi.cpp); needs fp32_copy.
mhfem_status run_mixed(mhfem_t h, int* iters, int* sweeps, double* res);
// Learned form (learned.cpp): the gate, the solve (FP64 or mixed) and online training.
mhfem_status learned_solve(mhfem_t h, int* iters, int* sweeps, double* res, mhfem_step_stats* stats);
void learned_release(mhfem_t h);
// Marks the network state stale (the pattern changed); the parameters are kept.
void learned_invalidate(mhfem_t h);
// Forgets the trace history (the state was set from outside: a restart).
void learned_reset_history(mhfem_t h);

}  // namespace mhfem
