// C ABI and host orchestration of one MHFEM solver instance (one GPU,
// one CUDA stream).  Mirrors TNL::MHFEM::Solver (Solver.h:28-210) and the
// time-step sequence of MHFEM::solve (control.h:64-102).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gmres_restart.h"
#include "mhfem_internal.h"
#include "topology.h"

using namespace mhfem;

#include "handle.h"

namespace {

int64_t coef_size(mhfem_t h, int which)
{
    const int64_t n = h->n, nf = h->nf, C = h->topo.C, F = h->topo.F;
    switch (which) {
        case MHFEM_COEF_N: case MHFEM_COEF_D: case MHFEM_COEF_R: return n * n * C;
        case MHFEM_COEF_U: case MHFEM_COEF_A: return n * n * nf * C;
        case MHFEM_COEF_M: case MHFEM_COEF_F: return n * C;
        case MHFEM_COEF_W: return n * nf * C;
        case MHFEM_COEF_M_UPW: return F * n;
        case MHFEM_COEF_M_BND: return n * F;
        case MHFEM_COEF_PSI: return C;
    }
    return -1;
}

bool is_device_pointer(const void* p)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // a plain host pointer on older drivers: clear the error
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Copies a coefficient (host or device source) into its device array and
// keeps a host copy (the learned form's static features, the zero test of
// the explicit advection switch).
mhfem_status set_coef_device(mhfem_t h, int which, const double* data, int64_t count)
{
    if (h->coef[which].count != count || !h->coef[which].p) {
        dfree(h, h->coef[which].p);
        CK(dalloc(h, &h->coef[which].p, (size_t)count));
    }
    const bool dev = is_device_pointer(data);
    CK(cudaMemcpyAsync(h->coef[which].p, data, sizeof(double) * count,
                       dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
    h->coef[which].count = count;
    // A host copy is kept only where the host reads the values: the zero
    // test of the advection coefficients (it selects the advection terms of
    // the kernels) and the learned form's static features (D, f, psi).  A
    // per-step upload of a full field (the source f of a time-varying
    // model) then costs its transfer and no host-side copy.
    const bool flag = which == MHFEM_COEF_A || which == MHFEM_COEF_U;
    const bool shadow = flag || (h->desc.form == MHFEM_FORM_LEARNED &&
                                 (which == MHFEM_COEF_D || which == MHFEM_COEF_F || which == MHFEM_COEF_PSI));
    if (shadow) {
        h->h_coef[which].resize(count);
        if (dev)
            CK(cudaMemcpyAsync(h->h_coef[which].data(), data, sizeof(double) * count, cudaMemcpyDeviceToHost,
                               h->stream));
        else
            std::copy(data, data + count, h->h_coef[which].begin());
    }
    else
        std::vector<double>().swap(h->h_coef[which]);
    CK(cudaStreamSynchronize(h->stream));  // the caller may reuse its buffer on return
    if (flag) {
        bool nz = false;
        for (int64_t q = 0; q < count && !nz; ++q) nz = (h->h_coef[which][q] != 0.0);
        h->coef_nonzero[which] = nz;
    }
    return MHFEM_OK;
}

// The device array behind an MHFEM_ARRAY_* identifier and its size.
mhfem_status array_ptr(mhfem_t h, int32_t which, double** p, int64_t* size)
{
    const int64_t n = h->n, nf = h->nf, C = h->topo.C, F = h->topo.F;
    switch (which) {
        case MHFEM_ARRAY_B: *p = h->b; *size = n * n * h->S * C; break;
        case MHFEM_ARRAY_R_IJKE: *p = h->R_ijKe; *size = n * n * nf * C; break;
        case MHFEM_ARRAY_R_IK: *p = h->R_iK; *size = n * C; break;
        case MHFEM_ARRAY_M_UPW: *p = h->m_upw; *size = n * F; break;
        case MHFEM_ARRAY_Z_UPW: *p = h->Z_upw; *size = n * n * F; break;
        case MHFEM_ARRAY_V: *p = h->v_iKe; *size = n * nf * C; break;
        case MHFEM_ARRAY_RHS: *p = h->rhs; *size = n * F; break;
        case MHFEM_ARRAY_Z_IF: *p = h->Z_iF; *size = n * F; break;
        case MHFEM_ARRAY_Z_IK: *p = h->Z_iK; *size = n * C; break;
        default: return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "unknown array %d", which);
    }
    if (!*p) return fail(h, MHFEM_ERR_STATE, "array %d is not allocated in this configuration", which);
    return MHFEM_OK;
}

mhfem_status run_hook(mhfem_t h, int point, double t, double tau)
{
    const auto& k = h->hooks[point];
    if (!k.fn) return MHFEM_OK;
    k.fn(k.user, t, tau, (void*)h->stream);
    cudaSetDevice(h->desc.device);
    CK(cudaGetLastError());
    return MHFEM_OK;
}

Coef as_coef(const DevCoef& c) { return Coef{c.p, c.count > 1 ? 1 : 0}; }

void invalidate_graphs(mhfem_t h)
{
    if (h->g64) cudaGraphExecDestroy(h->g64);
    if (h->g32) cudaGraphExecDestroy(h->g32);
    if (h->ggm) cudaGraphExecDestroy(h->ggm);
    h->g64 = h->g32 = h->ggm = nullptr;
    h->g64_iters = h->g32_iters = 0;
}

DevProblem make_problem(mhfem_t h)
{
    DevProblem P{};
    P.dim = h->dim; P.cell = h->cell; P.nf = h->nf; P.n = h->n; P.S = h->S;
    P.lumping = h->desc.mass_lumping;
    P.advection = h->desc.advection;
    P.mobility_upwind = h->desc.mobility_upwind;
    P.V = h->topo.V; P.C = h->topo.C; P.F = h->topo.F; P.rows = h->topo.F * h->n;
    P.coords = h->coords;
    P.cell_verts = h->cell_verts;
    P.cell_faces = h->cell_faces;
    P.cell_bmask = h->cell_bmask;
    P.face_cells = h->face_cells;
    P.face_local = h->face_local;
    P.face_measure = h->face_measure;
    P.N = as_coef(h->coef[MHFEM_COEF_N]);
    P.u = as_coef(h->coef[MHFEM_COEF_U]);
    P.m = as_coef(h->coef[MHFEM_COEF_M]);
    P.D = as_coef(h->coef[MHFEM_COEF_D]);
    P.w = as_coef(h->coef[MHFEM_COEF_W]);
    P.a = as_coef(h->coef[MHFEM_COEF_A]);
    P.r = as_coef(h->coef[MHFEM_COEF_R]);
    P.f = as_coef(h->coef[MHFEM_COEF_F]);
    P.m_upw_in = as_coef(h->coef[MHFEM_COEF_M_UPW]);
    P.m_bnd = as_coef(h->coef[MHFEM_COEF_M_BND]);
    P.psi = (h->src_amp != 0 && h->coef[MHFEM_COEF_PSI].p) ? as_coef(h->coef[MHFEM_COEF_PSI]) : Coef{};
    P.src_amp = h->src_amp;
    P.src_omega = 2.0 * M_PI / h->src_period;
    P.src_time = h->cur_t;
    P.bc_tags = h->tags;
    P.bc_values = h->bvalues;
    P.bc_dirichlet = h->bdirichlet;
    P.Z_iF = h->Z_iF; P.Z_iK = h->Z_iK; P.v_iKe = h->v_iKe;
    P.m_upw = h->m_upw; P.Z_upw = h->Z_upw;
    P.b = h->b; P.R_ijKe = h->R_ijKe; P.R_iK = h->R_iK;
    P.rec = h->rec; P.rec_stride = h->rec_stride;
    if (h->desc.mobility_upwind) { P.use_m_upw_array = 1; P.m_upw_read = h->m_upw; }
    else if (h->coef[MHFEM_COEF_M_UPW].count > 1) { P.use_m_upw_array = 1; P.m_upw_read = h->coef[MHFEM_COEF_M_UPW].p; }
    else { P.use_m_upw_array = 0; P.m_upw_read = nullptr; }
    P.explicit_adv_active = (h->desc.advection == MHFEM_EXPLICIT_UPWIND) &&
                            (h->coef_nonzero[MHFEM_COEF_A] || h->coef_nonzero[MHFEM_COEF_U]);
    P.err_flags = h->err_flags;
    return P;
}

mhfem_status require_ready(mhfem_t h)
{
    if (!h) return MHFEM_ERR_INVALID_ARGUMENT;
    if (!h->has_mesh) return fail(h, MHFEM_ERR_STATE, "mhfem_set_mesh has not been called");
    return MHFEM_OK;
}

mhfem_status ensure_pattern(mhfem_t h);

}  // namespace

extern "C" {

void mhfem_default_solver_opts(mhfem_solver_opts* o)
{
    if (!o) return;
    o->tol = 1e-10;
    o->max_iter = 10000;
    o->inner_tol = 1e-4;
    o->max_sweeps = 50;
    o->check_every = 8;
    o->timeout_s = 0;
    o->inner_adaptive = 1;
    o->linear_solver = MHFEM_SOLVER_BICGSTAB;
    o->gmres_restart = 30;
    o->gmres_variant = MHFEM_GMRES_CGS;
    o->gmres_restart_min = 0;
    o->gmres_restart_step_min = 0;
    o->gmres_restart_step_max = 0;
}

mhfem_status mhfem_create(const mhfem_desc* desc, mhfem_t* out)
{
    if (!desc || !out) return MHFEM_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (desc->dim != 2 && desc->dim != 3) return MHFEM_ERR_INVALID_ARGUMENT;
    if (desc->n_eq < 1 || desc->n_eq > 3) return MHFEM_ERR_UNSUPPORTED;
    if (desc->advection < 0 || desc->advection > 2) return MHFEM_ERR_INVALID_ARGUMENT;
    if (desc->form < 0 || desc->form > 2) return MHFEM_ERR_INVALID_ARGUMENT;
    if (desc->cell != MHFEM_CELL_SIMPLEX && desc->cell != MHFEM_CELL_BOX) return MHFEM_ERR_INVALID_ARGUMENT;
    if (desc->cell == MHFEM_CELL_BOX && desc->form == MHFEM_FORM_LEARNED) return MHFEM_ERR_UNSUPPORTED;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MHFEM_ERR_NO_DEVICE;
    if (desc->device < 0 || desc->device >= ndev) return MHFEM_ERR_NO_DEVICE;
    if (cudaSetDevice(desc->device) != cudaSuccess) return MHFEM_ERR_NO_DEVICE;
    mhfem_t h = new mhfem_solver_s();
    h->desc = *desc;
    h->dim = desc->dim;
    h->cell = desc->cell;
    h->n = desc->n_eq;
    if (desc->cell == MHFEM_CELL_BOX) {
        // MassMatrix<Quadrangle / Hexahedron>::size: one value per face orientation
        h->nf = 2 * desc->dim;
        h->nv = 1 << desc->dim;
        h->S = desc->dim;
    }
    else {
        // MassMatrix<Triangle / Tetrahedron>::size: packed upper triangle + row sums
        h->nf = desc->dim + 1;
        h->nv = desc->dim + 1;
        h->S = (desc->dim == 2) ? 9 : 14;
    }
    mhfem_default_solver_opts(&h->opts);
    h->fp32_copy = (desc->form == MHFEM_FORM_MIXED);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return MHFEM_ERR_CUDA;
    }
    bool ok = true;
    for (auto& e : h->ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    ok = ok && cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, desc->device) == cudaSuccess;
    ok = ok && cudaMallocHost((void**)&h->W.host_sc, sizeof(KrylovScalars) * 2) == cudaSuccess;
    ok = ok && cudaMallocHost((void**)&h->host_err, sizeof(int32_t)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        mhfem_destroy(h);  // releases whatever was created
        return MHFEM_ERR_CUDA;
    }
    *out = h;
    return MHFEM_OK;
}

mhfem_status mhfem_destroy(mhfem_t h)
{
    if (!h) return MHFEM_ERR_INVALID_ARGUMENT;
    cudaSetDevice(h->desc.device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    invalidate_graphs(h);
    learned_release(h);
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
    if (h->W.host_sc) cudaFreeHost(h->W.host_sc);
    if (h->G.host) cudaFreeHost(h->G.host);
    if (h->G.host_m) cudaFreeHost(h->G.host_m);
    if (h->host_err) cudaFreeHost(h->host_err);
    for (auto& e : h->ev)
        if (e) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return MHFEM_OK;
}

const char* mhfem_last_error(mhfem_t h)
{
    if (!h) return "invalid handle";
    return h->err.c_str();
}

mhfem_status mhfem_set_mesh(mhfem_t h, int64_t V, const double* coords, int64_t C, const int32_t* cell_verts)
{
    if (!h || !coords || !cell_verts || V <= 0 || C <= 0) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "invalid mesh arguments");
    cudaSetDevice(h->desc.device);
    std::string msg = build_topology(h->dim, h->cell, V, coords, C, cell_verts, h->topo);
    if (!msg.empty()) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "%s", msg.c_str());
    const int nf = h->nf, nv = h->nv, n = h->n;
    const int64_t F = h->topo.F;
    // release everything that depends on the mesh; the handle has no mesh
    // until the new one is complete (a failed allocation leaves it unusable,
    // not pointing at freed arrays)
    h->has_mesh = false;
    invalidate_graphs(h);
    learned_release(h);
    for (void* p : h->allocs) cudaFree(p);
    h->allocs.clear();
    h->coords = nullptr; h->cell_verts = h->cell_faces = nullptr; h->cell_bmask = nullptr;
    h->face_cells = nullptr; h->face_local = nullptr; h->face_measure = nullptr;
    for (auto& c : h->coef) c = DevCoef();
    h->tags = nullptr; h->bvalues = h->bdirichlet = nullptr;
    h->Z_iF = h->Z_iK = h->v_iKe = h->m_upw = h->Z_upw = h->b = h->R_ijKe = h->R_iK = h->rec = nullptr;
    h->A = EllMatrix(); h->amap = AssemblyMap(); h->rhs = nullptr; h->err_flags = nullptr;
    KrylovScalars* keep = h->W.host_sc;
    h->W = KrylovWork();
    h->W.host_sc = keep;
    GmresCtl* keep_gm = h->G.host;
    h->G = GmresWork();
    h->G.host = keep_gm;
    h->pattern_ready = false;
    h->has_bc = h->has_state = false;

    h->h_coords.assign(coords, coords + V * h->dim);
    // topology on the device, SoA with the cell index innermost
    std::vector<int32_t> soa((size_t)C * std::max(nf, nv));
    CK(dalloc(h, &h->coords, (size_t)V * h->dim));
    CK(cudaMemcpy(h->coords, coords, sizeof(double) * V * h->dim, cudaMemcpyHostToDevice));
    for (int64_t K = 0; K < C; ++K)
        for (int v = 0; v < nv; ++v) soa[(size_t)v * C + K] = cell_verts[K * nv + v];
    CK(dalloc(h, &h->cell_verts, (size_t)C * nv));
    CK(cudaMemcpy(h->cell_verts, soa.data(), sizeof(int32_t) * C * nv, cudaMemcpyHostToDevice));
    for (int64_t K = 0; K < C; ++K)
        for (int e = 0; e < nf; ++e) soa[(size_t)e * C + K] = h->topo.cell_faces[K * nf + e];
    CK(dalloc(h, &h->cell_faces, (size_t)C * nf));
    CK(cudaMemcpy(h->cell_faces, soa.data(), sizeof(int32_t) * C * nf, cudaMemcpyHostToDevice));
    CK(dalloc(h, &h->cell_bmask, (size_t)C));
    CK(cudaMemcpy(h->cell_bmask, h->topo.cell_bmask.data(), C, cudaMemcpyHostToDevice));
    CK(dalloc(h, &h->face_cells, (size_t)F));
    CK(cudaMemcpy(h->face_cells, h->topo.face_cells.data(), sizeof(int2) * F, cudaMemcpyHostToDevice));
    CK(dalloc(h, &h->face_local, (size_t)2 * F));
    CK(cudaMemcpy(h->face_local, h->topo.face_local.data(), 2 * F, cudaMemcpyHostToDevice));
    CK(dalloc(h, &h->face_measure, (size_t)F));
    CK(cudaMemcpy(h->face_measure, h->topo.face_measure.data(), sizeof(double) * F, cudaMemcpyHostToDevice));

    // scheme arrays (BaseModel::allocate, BaseModel.h:168-195)
    CK(dalloc(h, &h->Z_iF, (size_t)n * F));
    CK(dalloc(h, &h->Z_iK, (size_t)n * C));
    CK(dalloc(h, &h->b, (size_t)n * n * h->S * C));
    CK(dalloc(h, &h->R_ijKe, (size_t)n * n * nf * C));
    CK(dalloc(h, &h->R_iK, (size_t)n * C));
    if (h->desc.mobility_upwind) {
        CK(dalloc(h, &h->m_upw, (size_t)n * F));
        CK(dalloc(h, &h->v_iKe, (size_t)n * nf * C));
        CK(cudaMemset(h->v_iKe, 0, sizeof(double) * n * nf * C));
    }
    if (h->desc.advection == MHFEM_EXPLICIT_UPWIND) {
        CK(dalloc(h, &h->Z_upw, (size_t)n * n * F));
        CK(cudaMemset(h->Z_upw, 0, sizeof(double) * n * n * F));
    }
    h->rec_stride = ((n * nf + 1) + 1) & ~1;
    CK(dalloc(h, &h->rec, (size_t)C * nf * n * h->rec_stride));
    CK(dalloc(h, &h->err_flags, 1));
    CK(cudaMemset(h->err_flags, 0, sizeof(int32_t)));
    CK(cudaMemset(h->Z_iK, 0, sizeof(double) * n * C));
    CK(cudaMemset(h->Z_iF, 0, sizeof(double) * n * F));

    // default coefficients: the heat-equation model (HeatEquationModel.h:114-133)
    h->has_mesh = true;
    const double one = 1.0, zero = 0.0;
    mhfem_status st;
    const int ones[] = {MHFEM_COEF_N, MHFEM_COEF_M, MHFEM_COEF_D, MHFEM_COEF_M_UPW, MHFEM_COEF_M_BND};
    const int zeros[] = {MHFEM_COEF_U, MHFEM_COEF_W, MHFEM_COEF_A, MHFEM_COEF_R, MHFEM_COEF_F};
    for (int w : ones)
        if ((st = set_coef_device(h, w, &one, 1)) != MHFEM_OK) { h->has_mesh = false; return st; }
    for (int w : zeros)
        if ((st = set_coef_device(h, w, &zero, 1)) != MHFEM_OK) { h->has_mesh = false; return st; }
    // default boundary conditions: zero Dirichlet everywhere (Solver.hpp:282-293)
    std::vector<uint8_t> t0((size_t)n * F, MHFEM_BC_FIXED_VALUE);
    std::vector<double> v0((size_t)n * F, 0.0);
    if ((st = mhfem_set_bc(h, t0.data(), v0.data(), v0.data())) != MHFEM_OK) { h->has_mesh = false; return st; }
    h->has_bc = false;  // defaults only
    return MHFEM_OK;
}

mhfem_status mhfem_get_sizes(mhfem_t h, int64_t* V, int64_t* C, int64_t* F, int64_t* rows, int64_t* nnz)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if (V) *V = h->topo.V;
    if (C) *C = h->topo.C;
    if (F) *F = h->topo.F;
    if (rows) *rows = h->topo.F * h->n;
    if (nnz) {
        if ((st = ensure_pattern(h)) != MHFEM_OK) return st;
        *nnz = h->pat.nnz;
    }
    return MHFEM_OK;
}

mhfem_status mhfem_get_topology(mhfem_t h, int32_t* face_verts, int32_t* face_cells, int32_t* cell_faces)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if (face_verts) std::memcpy(face_verts, h->topo.face_verts.data(), sizeof(int32_t) * h->topo.face_verts.size());
    if (face_cells) std::memcpy(face_cells, h->topo.face_cells.data(), sizeof(int32_t) * h->topo.face_cells.size());
    if (cell_faces) std::memcpy(cell_faces, h->topo.cell_faces.data(), sizeof(int32_t) * h->topo.cell_faces.size());
    return MHFEM_OK;
}

mhfem_status mhfem_set_coeff(mhfem_t h, int32_t which, const double* data, int64_t count)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if (which < 0 || which >= NCOEF || !data) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "invalid coefficient id %d", which);
    const int64_t full = coef_size(h, which);
    if (count != 1 && count != full)
        return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "coefficient %d: expected 1 or %lld values, got %lld", which,
                    (long long)full, (long long)count);
    if (which == MHFEM_COEF_PSI && count != full)
        return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "psi must be a full per-cell array");
    cudaSetDevice(h->desc.device);
    return set_coef_device(h, which, data, count);
}

mhfem_status mhfem_set_source_modulation(mhfem_t h, double amplitude, double period)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if (!(period > 0)) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "period must be positive");
    if (amplitude != 0 && !h->coef[MHFEM_COEF_PSI].p)
        return fail(h, MHFEM_ERR_STATE, "set MHFEM_COEF_PSI before enabling the source modulation");
    h->src_amp = amplitude;
    h->src_period = period;
    return MHFEM_OK;
}

mhfem_status mhfem_set_bc(mhfem_t h, const uint8_t* tags, const double* values, const double* dirichlet)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if (!tags || !values || !dirichlet) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "null boundary arrays");
    const int64_t count = h->topo.F * h->n;
    for (int64_t q = 0; q < count; ++q)
        if (tags[q] > 3) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "unknown boundary condition tag %d at %lld", tags[q], (long long)q);
    cudaSetDevice(h->desc.device);
    if (!h->tags) {
        CK(dalloc(h, &h->tags, (size_t)count));
        CK(dalloc(h, &h->bvalues, (size_t)count));
        CK(dalloc(h, &h->bdirichlet, (size_t)count));
    }
    const bool same = h->h_tags.size() == (size_t)count && std::memcmp(h->h_tags.data(), tags, count) == 0;
    h->h_tags.assign(tags, tags + count);
    CK(cudaMemcpy(h->tags, tags, count, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->bvalues, values, sizeof(double) * count, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->bdirichlet, dirichlet, sizeof(double) * count, cudaMemcpyHostToDevice));
    if (!same) h->pattern_ready = false;
    h->has_bc = true;
    return MHFEM_OK;
}

mhfem_status mhfem_set_initial_condition(mhfem_t h, const double* Z_iK)
{
    return mhfem_set_state(h, Z_iK, nullptr);
}

mhfem_status mhfem_set_state(mhfem_t h, const double* Z_iK, const double* Z_iF)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if (!Z_iK) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "Z_iK is null");
    cudaSetDevice(h->desc.device);
    CK(cudaMemcpyAsync(h->Z_iK, Z_iK, sizeof(double) * h->n * h->topo.C, cudaMemcpyHostToDevice, h->stream));
    if (Z_iF) {
        CK(cudaMemcpyAsync(h->Z_iF, Z_iF, sizeof(double) * h->n * h->topo.F, cudaMemcpyHostToDevice, h->stream));
    }
    else {
        DevProblem P = make_problem(h);
        h->launches += launch_face_average(P, h->stream);
        CK(cudaGetLastError());
    }
    if (h->v_iKe) CK(cudaMemsetAsync(h->v_iKe, 0, sizeof(double) * h->n * h->nf * h->topo.C, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    learned_reset_history(h);  // the learned form's extrapolation restarts from this state
    h->has_state = true;
    return MHFEM_OK;
}

mhfem_status mhfem_set_solver(mhfem_t h, const mhfem_solver_opts* o)
{
    if (!h || !o) return MHFEM_ERR_INVALID_ARGUMENT;
    if (!(o->tol > 0) || o->max_iter < 1 || o->check_every < 1 || !(o->inner_tol > 0) || o->max_sweeps < 1)
        return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "invalid solver options");
    if (o->linear_solver != MHFEM_SOLVER_BICGSTAB && o->linear_solver != MHFEM_SOLVER_GMRES)
        return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "unknown linear solver %d", o->linear_solver);
    if (o->gmres_restart < 1 || o->gmres_restart > kGmresMaxM)
        return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "gmres restart must be 1 to %d", kGmresMaxM);
    if (o->gmres_variant != MHFEM_GMRES_CGS && o->gmres_variant != MHFEM_GMRES_CGSR)
        return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "unknown gmres variant %d", o->gmres_variant);
    if (o->gmres_restart_min < 0 || o->gmres_restart_min > o->gmres_restart || o->gmres_restart_step_min < 0 ||
        o->gmres_restart_step_max < 0)
        return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "gmres restart range %d..%d, steps %d..%d", o->gmres_restart_min,
                    o->gmres_restart, o->gmres_restart_step_min, o->gmres_restart_step_max);
    const bool regraph = (o->check_every != h->opts.check_every) || (o->gmres_restart != h->opts.gmres_restart) ||
                         (o->gmres_variant != h->opts.gmres_variant);
    h->opts = *o;
    if (regraph) invalidate_graphs(h);
    return MHFEM_OK;
}

}  // extern "C"

namespace {

mhfem_status ensure_pattern(mhfem_t h)
{
    if (h->pattern_ready) return MHFEM_OK;
    cudaSetDevice(h->desc.device);
    invalidate_graphs(h);
    learned_invalidate(h);  // the face graph follows the pattern
    const int n = h->n;
    const int64_t F = h->topo.F, rows = F * n;
    build_pattern(h->topo, n, h->h_tags.data(), h->pat);
    for (int64_t r = 0; r < rows; ++r)
        if (h->pat.row_len[r] <= 0)  // Solver.hpp:467-474
            return fail(h, MHFEM_ERR_STATE, "invalid row length at row %lld", (long long)r);
    dfree(h, h->A.cols);
    dfree(h, h->A.vals);
    dfree(h, h->A.vals32);
    dfree(h, h->A.cols_lo);
    dfree(h, h->A.cols_hi);
    dfree(h, h->amap.qmap);
    dfree(h, h->amap.qdiag);
    dfree(h, h->rhs);
    const int W = h->pat.W;
    h->A.rows = rows;
    h->A.width = W;
    CK(dalloc(h, &h->A.cols, (size_t)W * rows));
    if (W > 0)  // width 0: every row is its unit diagonal (all faces Dirichlet)
        CK(cudaMemcpy(h->A.cols, h->pat.ell_cols.data(), sizeof(int32_t) * W * rows, cudaMemcpyHostToDevice));
    CK(dalloc(h, &h->A.vals, (size_t)W * rows));
    CK(cudaMemset(h->A.vals, 0, sizeof(double) * W * rows));
    if (h->fp32_copy) {
        CK(dalloc(h, &h->A.vals32, (size_t)W * rows));
        CK(cudaMemset(h->A.vals32, 0, sizeof(float) * W * rows));
        // 24-bit column offsets for the FP32 SpMVs (the widths with an
        // FP32 4-rows-per-thread kernel), if every offset fits
        std::vector<uint16_t> lo;
        std::vector<uint8_t> hi;
        bool fits = (W == 4 || W == 6) && rows % 4 == 0;
        if (fits) {
            lo.resize((size_t)W * rows);
            hi.resize((size_t)W * rows);
            for (int64_t q = 0; q < (int64_t)W * rows && fits; ++q) {
                const int64_t d = (int64_t)h->pat.ell_cols[q] - q % rows + kCol24Bias;
                if (d < 0 || d >= (int64_t)1 << 24) fits = false;
                lo[q] = (uint16_t)(d & 0xffff);
                hi[q] = (uint8_t)(d >> 16);
            }
        }
        if (fits) {
            CK(dalloc(h, &h->A.cols_lo, (size_t)W * rows));
            CK(dalloc(h, &h->A.cols_hi, (size_t)W * rows));
            CK(cudaMemcpy(h->A.cols_lo, lo.data(), sizeof(uint16_t) * W * rows, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(h->A.cols_hi, hi.data(), W * rows, cudaMemcpyHostToDevice));
        }
    }
    if (h->nf > 4) {  // 12 positions of 4 bits: one 64-bit word per face
        uint64_t* q = nullptr;
        CK(dalloc(h, &q, (size_t)F));
        h->amap.qmap = q;
        CK(cudaMemcpy(q, h->pat.qmap.data(), sizeof(uint64_t) * F, cudaMemcpyHostToDevice));
    }
    else {
        const std::vector<uint32_t> q32(h->pat.qmap.begin(), h->pat.qmap.end());
        uint32_t* q = nullptr;
        CK(dalloc(h, &q, (size_t)F));
        h->amap.qmap = q;
        CK(cudaMemcpy(q, q32.data(), sizeof(uint32_t) * F, cudaMemcpyHostToDevice));
    }
    CK(dalloc(h, &h->amap.qdiag, (size_t)F));
    CK(cudaMemcpy(h->amap.qdiag, h->pat.qdiag.data(), F, cudaMemcpyHostToDevice));
    CK(dalloc(h, &h->rhs, (size_t)rows));
    CK(cudaMemset(h->rhs, 0, sizeof(double) * rows));

    // Krylov workspace (7 vectors as in Solver::estimateMemoryDemands, Solver.hpp:1424-1425)
    KrylovWork& Wk = h->W;
    dfree(h, Wk.r); dfree(h, Wk.rh); dfree(h, Wk.p); dfree(h, Wk.v); dfree(h, Wk.s); dfree(h, Wk.t);
    dfree(h, Wk.p2); dfree(h, Wk.v2);
    dfree(h, Wk.r32); dfree(h, Wk.rh32); dfree(h, Wk.p32); dfree(h, Wk.v32); dfree(h, Wk.s32); dfree(h, Wk.t32);
    dfree(h, Wk.x32); dfree(h, Wk.partials); dfree(h, Wk.counters); dfree(h, Wk.sc); dfree(h, Wk.sc32);
    Wk.rows = rows;
    Wk.grid = krylov_grid();
    CK(dalloc(h, &Wk.r, (size_t)rows)); CK(dalloc(h, &Wk.rh, (size_t)rows)); CK(dalloc(h, &Wk.p, (size_t)rows));
    CK(dalloc(h, &Wk.v, (size_t)rows)); CK(dalloc(h, &Wk.s, (size_t)rows)); CK(dalloc(h, &Wk.t, (size_t)rows));
    if (rows <= krylov_small_rows()) { CK(dalloc(h, &Wk.p2, (size_t)rows)); CK(dalloc(h, &Wk.v2, (size_t)rows)); }
    if (h->fp32_copy) {
        CK(dalloc(h, &Wk.r32, (size_t)rows)); CK(dalloc(h, &Wk.rh32, (size_t)rows)); CK(dalloc(h, &Wk.p32, (size_t)rows));
        CK(dalloc(h, &Wk.v32, (size_t)rows)); CK(dalloc(h, &Wk.s32, (size_t)rows)); CK(dalloc(h, &Wk.t32, (size_t)rows));
        CK(dalloc(h, &Wk.x32, (size_t)rows));
    }
    CK(dalloc(h, &Wk.partials, (size_t)Wk.grid * 8));  // 8 partial sums per block at most
    CK(dalloc(h, &Wk.counters, (size_t)4));
    CK(cudaMemset(Wk.counters, 0, sizeof(uint32_t) * 4));
    CK(dalloc(h, &Wk.sc, (size_t)1));
    CK(dalloc(h, &Wk.sc32, (size_t)1));
    CK(cudaMemset(Wk.sc, 0, sizeof(KrylovScalars)));
    CK(cudaMemset(Wk.sc32, 0, sizeof(KrylovScalars)));
    // the GMRES basis follows the row count: reallocated at the next GMRES solve
    dfree(h, h->G.U);
    dfree(h, h->G.partials);
    dfree(h, h->G.st);
    h->G.m = 0;
    h->pattern_ready = true;
    return MHFEM_OK;
}

// Captures `iters` Krylov iterations plus the read-back of the device
// scalars as one CUDA graph (replayed between host convergence checks).
mhfem_status build_graph(mhfem_t h, bool fp32, int iters)
{
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    if (fp32) {
        krylov_iterate_fp32(h->A, h->W, iters, h->stream);
        cudaMemcpyAsync(h->W.host_sc + 1, h->W.sc32, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, h->stream);
    }
    else {
        krylov_iterate_fp64(h->A, h->Z_iF, h->W, iters, h->stream);
        cudaMemcpyAsync(h->W.host_sc, h->W.sc, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, h->stream);
    }
    CK(cudaStreamEndCapture(h->stream, &g));
    cudaGraphExec_t ex = nullptr;
    cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(h, MHFEM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    if (fp32) { h->g32 = ex; h->g32_iters = iters; }
    else { h->g64 = ex; h->g64_iters = iters; }
    return MHFEM_OK;
}

mhfem_status status_from_krylov(mhfem_t h, const KrylovScalars& s, const char* what)
{
    switch (s.status) {
        case KS_CONVERGED: return MHFEM_OK;
        case KS_MAXITER:
            return fail(h, MHFEM_ERR_NOT_CONVERGED,
                        "MHFEM error: the linear system solver did not converge (%d iterations, %s, residual %.3e)",
                        s.it, what, s.res);
        case KS_BREAKDOWN: return fail(h, MHFEM_ERR_BREAKDOWN, "%s: BiCGStab breakdown after %d iterations", what, s.it);
        case KS_NOTFINITE: return fail(h, MHFEM_ERR_NOT_FINITE, "%s: non-finite value after %d iterations", what, s.it);
    }
    return fail(h, MHFEM_ERR_STATE, "%s: unexpected Krylov status %d", what, s.status);
}

double elapsed_s(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

mhfem_status status_from_gmres(mhfem_t h, const GmresCtl& c)
{
    switch (c.status) {
        case KS_CONVERGED: return MHFEM_OK;
        case KS_MAXITER:
            return fail(h, MHFEM_ERR_NOT_CONVERGED,
                        "MHFEM error: the linear system solver did not converge (%d iterations, GMRES, residual %.3e)",
                        c.it, c.res);
        case KS_NOTFINITE: return fail(h, MHFEM_ERR_NOT_FINITE, "GMRES: non-finite value after %d iterations", c.it);
    }
    return fail(h, MHFEM_ERR_STATE, "GMRES: unexpected status %d", c.status);
}

// Restarted GMRES from the current Z_iF: CUDA graphs of check_every Arnoldi
// iterations between host checks; at the end of each cycle the host runs the
// small solve, the update of x and the restart from the true residual.
mhfem_status run_gmres(mhfem_t h, double tol, int max_iter, int* iters, double* res)
{
    const auto t0 = std::chrono::steady_clock::now();
    const int m = h->opts.gmres_restart;
    const int64_t rows = h->A.rows;
    GmresWork& G = h->G;
    if (G.m != m || !G.U) {
        dfree(h, G.U);
        dfree(h, G.partials);
        dfree(h, G.st);
        if (h->ggm) { cudaGraphExecDestroy(h->ggm); h->ggm = nullptr; }
        CK(dalloc(h, &G.U, (size_t)(m + 1) * rows));
        CK(dalloc(h, &G.partials, (size_t)krylov_grid() * kGmStride));
        CK(dalloc(h, &G.st, (size_t)1));
        G.m = m;
    }
    if (!G.host) CK(cudaMallocHost((void**)&G.host, sizeof(GmresCtl)));
    if (!G.host_m) CK(cudaMallocHost((void**)&G.host_m, sizeof(int32_t)));
    // adaptive restart length (gmres_restart.h): the first cycle runs m
    const RestartRule rule{h->opts.gmres_restart_min, m, h->opts.gmres_restart_step_min,
                           h->opts.gmres_restart_step_max};
    const bool adaptive = restart_adaptive(rule);
    int m_cur = m;
    GmresState init{};
    init.tol = tol;
    init.m = m;
    init.max_iter = max_iter;
    init.m_min = rule.m_min;
    init.m_max = rule.m_max;
    init.step_min = rule.step_min;
    init.step_max = rule.step_max;
    init.max_cr = restart_max_cr();
    init.min_cr = restart_min_cr();
    CK(cudaMemcpyAsync(G.st, &init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    gmres_init(h->A, h->rhs, h->Z_iF, G, h->W, true, h->stream);
    h->launches += 1;
    CK(cudaMemcpyAsync(G.host, &G.st->ctl, sizeof(GmresCtl), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    double res_prev = G.host->res;
    const bool reorth = h->opts.gmres_variant == MHFEM_GMRES_CGSR;
    if (rows <= krylov_small_rows() && !G.host->done) {
        // small system: chunks of iterations, restarts included, in one
        // persistent launch each (k_gmres_small), one host round trip per
        // chunk; the device applies the restart rule
        CK(cudaMemcpyAsync(&G.st->res_prev, &res_prev, sizeof(double), cudaMemcpyHostToDevice, h->stream));
        constexpr int kChunk = 256;
        bool small = true;
        for (bool first = true;; first = false) {
            const cudaError_t e = gmres_small(h->A, h->rhs, h->Z_iF, G, h->W, reorth, kChunk, h->stream);
            if (first && e == cudaErrorCooperativeLaunchTooLarge) {
                // the device cannot hold the grid at once: nothing ran, the
                // graph of iterations below goes on from the same state
                cudaGetLastError();
                small = false;
                break;
            }
            CK(e);
            h->launches += 1;
            CK(cudaMemcpyAsync(G.host, &G.st->ctl, sizeof(GmresCtl), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaMemcpyAsync(h->host_err, h->W.counters + 3, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            if (*h->host_err) return fail(h, MHFEM_ERR_CUDA, "GMRES (small system): a grid barrier wait gave up");
            if (G.host->done) break;
            if (h->opts.timeout_s > 0 && elapsed_s(t0) > h->opts.timeout_s)
                return fail(h, MHFEM_ERR_TIMEOUT, "Krylov solve exceeded %.1f s", h->opts.timeout_s);
        }
        if (small) {
            *iters = G.host->it;
            *res = G.host->res;
            return status_from_gmres(h, *G.host);
        }
    }
    if (!h->ggm) {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        gmres_iterate(h->A, G, h->W, h->opts.check_every, reorth, h->stream);
        cudaMemcpyAsync(G.host, &G.st->ctl, sizeof(GmresCtl), cudaMemcpyDeviceToHost, h->stream);
        CK(cudaStreamEndCapture(h->stream, &g));
        const cudaError_t e = cudaGraphInstantiate(&h->ggm, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(h, MHFEM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    }
    while (!G.host->done) {
        const bool restarted = G.host->cycle_end != 0;
        if (restarted) {
            gmres_update(h->Z_iF, G, rows, h->stream);
            gmres_init(h->A, h->rhs, h->Z_iF, G, h->W, false, h->stream);
            h->launches += 3;
            CK(cudaMemcpyAsync(G.host, &G.st->ctl, sizeof(GmresCtl), cudaMemcpyDeviceToHost, h->stream));
        }
        else {
            CK(cudaGraphLaunch(h->ggm, h->stream));
            h->launches += (reorth ? 4 : 2) * h->opts.check_every;
        }
        CK(cudaStreamSynchronize(h->stream));
        if (restarted && adaptive && !G.host->done) {
            // the next cycle's length from the ratio of the true residuals at
            // the last two restarts; the device reads st->m in every iteration
            const int next = next_restart(m_cur, res_prev > 0 ? G.host->res / res_prev : 0.0, rule);
            res_prev = G.host->res;
            if (next != m_cur) {
                m_cur = next;
                *G.host_m = next;
                CK(cudaMemcpyAsync(&G.st->m, G.host_m, sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
            }
        }
        if (h->opts.timeout_s > 0 && elapsed_s(t0) > h->opts.timeout_s)
            return fail(h, MHFEM_ERR_TIMEOUT, "Krylov solve exceeded %.1f s", h->opts.timeout_s);
    }
    *iters = G.host->it;
    *res = G.host->res;
    return status_from_gmres(h, *G.host);
}

}  // namespace

// Runs FP64 BiCGStab from the current Z_iF until the device flag says done.
mhfem_status mhfem::run_fp64(mhfem_t h, double tol, int max_iter, int* iters, double* res)
{
    if (h->opts.linear_solver == MHFEM_SOLVER_GMRES) return run_gmres(h, tol, max_iter, iters, res);
    const auto t0 = std::chrono::steady_clock::now();
    krylov_init_fp64(h->A, h->rhs, h->Z_iF, h->W, tol, max_iter, h->stream);
    bool small = h->A.rows <= krylov_small_rows() && h->W.p2 && h->W.v2;
    if (small) {
        // small system: chunks of iterations in one persistent launch each
        // (k_bicgstab_small), one host round trip per chunk
        constexpr int kChunk = 256;
        h->launches += 1;
        for (bool first = true;; first = false) {
            const cudaError_t e = krylov_small_fp64(h->A, h->Z_iF, h->W, kChunk, h->stream);
            if (first && e == cudaErrorCooperativeLaunchTooLarge) {
                // the device cannot hold the grid at once (a partitioned or
                // shared GPU): nothing ran, so the five-kernel iteration
                // below starts from the same initial state
                cudaGetLastError();
                small = false;
                break;
            }
            CK(e);
            h->launches += 1;
            CK(cudaMemcpyAsync(h->W.host_sc, h->W.sc, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaMemcpyAsync(h->host_err, h->W.counters + 3, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            if (*h->host_err)
                return fail(h, MHFEM_ERR_CUDA, "FP64 BiCGStab (small system): a grid barrier wait gave up");
            if (h->W.host_sc->done) break;
            if (h->opts.timeout_s > 0 && elapsed_s(t0) > h->opts.timeout_s)
                return fail(h, MHFEM_ERR_TIMEOUT, "Krylov solve exceeded %.1f s", h->opts.timeout_s);
        }
        if (small) {
            *iters = h->W.host_sc->it;
            *res = h->W.host_sc->res;
            return status_from_krylov(h, *h->W.host_sc, "FP64 BiCGStab");
        }
    }
    CK(cudaMemcpyAsync(h->W.host_sc, h->W.sc, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    if (!h->g64) {
        mhfem_status st = build_graph(h, false, h->opts.check_every);
        if (st) return st;
    }
    h->launches += 1;
    while (!h->W.host_sc->done) {
        CK(cudaGraphLaunch(h->g64, h->stream));
        h->launches += 5 * h->g64_iters;
        CK(cudaStreamSynchronize(h->stream));
        if (h->opts.timeout_s > 0 && elapsed_s(t0) > h->opts.timeout_s)
            return fail(h, MHFEM_ERR_TIMEOUT, "Krylov solve exceeded %.1f s", h->opts.timeout_s);
    }
    *iters = h->W.host_sc->it;
    *res = h->W.host_sc->res;
    return status_from_krylov(h, *h->W.host_sc, "FP64 BiCGStab");
}

// FP32 inner BiCGStab on the FP32 copy of the matrix, FP64 outer residuals
// and corrections, until the FP64 residual meets the tolerance.
mhfem_status mhfem::run_mixed(mhfem_t h, int* iters, int* sweeps, double* res)
{
    const auto t0 = std::chrono::steady_clock::now();
    KrylovScalars init{};
    init.tol = h->opts.tol;
    init.max_iter = h->opts.max_sweeps;
    CK(cudaMemcpyAsync(h->W.sc, &init, sizeof(init), cudaMemcpyHostToDevice, h->stream));
    if (!h->g32) {
        mhfem_status st = build_graph(h, true, h->opts.check_every);
        if (st) return st;
    }
    int total_inner = 0;
    for (;;) {
        mixed_outer_residual(h->A, h->rhs, h->Z_iF, h->W, h->opts.tol, h->opts.max_sweeps, h->stream);
        h->launches += 2;
        CK(cudaMemcpyAsync(h->W.host_sc, h->W.sc, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, h->stream));
        mixed_inner_init(h->W, h->opts.inner_tol, h->opts.inner_adaptive, h->opts.max_iter, h->stream);
        CK(cudaMemcpyAsync(h->W.host_sc + 1, h->W.sc32, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        CK(cudaGetLastError());
        const KrylovScalars outer = h->W.host_sc[0];
        if (outer.done) {
            *iters = total_inner;
            *sweeps = outer.it - 1;
            *res = outer.res;
            return status_from_krylov(h, outer, "mixed-precision refinement");
        }
        while (!h->W.host_sc[1].done) {
            CK(cudaGraphLaunch(h->g32, h->stream));
            h->launches += 5 * h->g32_iters;
            CK(cudaStreamSynchronize(h->stream));
            if (h->opts.timeout_s > 0 && elapsed_s(t0) > h->opts.timeout_s)
                return fail(h, MHFEM_ERR_TIMEOUT, "mixed solve exceeded %.1f s", h->opts.timeout_s);
        }
        const KrylovScalars inner = h->W.host_sc[1];
        total_inner += inner.it;
        if (inner.status == KS_NOTFINITE)
            return fail(h, MHFEM_ERR_NOT_FINITE, "FP32 inner solve produced a non-finite value");
        if (inner.status == KS_BREAKDOWN && inner.it == 0)  // no correction: the next sweep would repeat it
            return fail(h, MHFEM_ERR_BREAKDOWN, "mixed-precision refinement: FP32 BiCGStab breakdown in its first iteration");
        mixed_apply_correction(h->Z_iF, h->W, h->stream);
        h->launches += 1;
    }
}

extern "C" {

mhfem_status mhfem_setup_linear_system(mhfem_t h)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    h->pattern_ready = false;
    return ensure_pattern(h);
}

mhfem_status mhfem_pre_iterate(mhfem_t h, double t, double tau)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if (!(tau > 0)) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "time step must be positive");
    cudaSetDevice(h->desc.device);
    if ((st = ensure_pattern(h)) != MHFEM_OK) return st;
    h->cur_t = t;
    h->cur_tau = tau;
    if ((st = run_hook(h, MHFEM_HOOK_PRE_ITERATE, t, tau)) != MHFEM_OK) return st;
    DevProblem P = make_problem(h);
    cudaEventRecord(h->ev[0], h->stream);
    if (h->hooks[MHFEM_HOOK_VECTOR_COEFFICIENTS].fn) {
        // Solver.hpp:627-652: this step's b first, then the model's
        // updateVectorCoefficients (its RT0 projections of u, w, a read b),
        // then upwinding and the rest of the cell work.  Without the hook the
        // fused cell kernel forms b and everything after it in one pass.
        h->launches += launch_update_b(P, h->stream);
        CK(cudaGetLastError());
        if ((st = run_hook(h, MHFEM_HOOK_VECTOR_COEFFICIENTS, t, tau)) != MHFEM_OK) return st;
        P = make_problem(h);  // the hook may have asked for a or u (explicit advection terms on)
    }
    h->launches += launch_upwind(P, h->stream);
    h->launches += launch_cell_local(P, tau, h->stream);
    cudaEventRecord(h->ev[1], h->stream);
    CK(cudaGetLastError());
    return MHFEM_OK;
}

mhfem_status mhfem_assemble(mhfem_t h, double t, double tau)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    (void)t; (void)tau;  // stationary boundary values (BoundaryModels/Stationary.h)
    if (!h->pattern_ready) return fail(h, MHFEM_ERR_STATE, "mhfem_pre_iterate must run before mhfem_assemble");
    cudaSetDevice(h->desc.device);
    DevProblem P = make_problem(h);
    h->launches += launch_assemble(P, h->amap, h->A, h->rhs, h->fp32_copy, h->stream);
    cudaEventRecord(h->ev[2], h->stream);
    CK(cudaGetLastError());
    return MHFEM_OK;
}

mhfem_status mhfem_solve(mhfem_t h, mhfem_step_stats* stats)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if (!h->pattern_ready) return fail(h, MHFEM_ERR_STATE, "the linear system is not assembled");
    cudaSetDevice(h->desc.device);
    // assembly error word (non-positive or non-finite diagonal)
    CK(cudaMemcpyAsync(h->host_err, h->err_flags, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (*h->host_err) {
        cudaMemsetAsync(h->err_flags, 0, sizeof(int32_t), h->stream);
        return fail(h, MHFEM_ERR_NONPOSITIVE_DIAGONAL, "the diagonal matrix element is not positive");
    }
    int iters = 0, sweeps = 1;
    double res = 0;
    h->guess_timed = false;
    if (stats) {
        stats->guess_used = 0;
        stats->guess_residual = -1;
        stats->warm_residual = -1;
        stats->ms_guess = 0;
        stats->base_residual = -1;
        stats->guess_source = 0;
    }
    if (h->desc.form == MHFEM_FORM_MIXED) st = run_mixed(h, &iters, &sweeps, &res);
    else if (h->desc.form == MHFEM_FORM_LEARNED) st = learned_solve(h, &iters, &sweeps, &res, stats);
    else st = run_fp64(h, h->opts.tol, h->opts.max_iter, &iters, &res);
    cudaEventRecord(h->ev[3], h->stream);
    h->total_iters += iters;
    if (stats) {
        stats->iterations = iters;
        stats->sweeps = sweeps;
        stats->residual = res;
    }
    return st;
}

mhfem_status mhfem_post_iterate(mhfem_t h, double t, double tau)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    cudaSetDevice(h->desc.device);
    DevProblem P = make_problem(h);
    h->launches += launch_reconstruct(P, h->stream);
    cudaEventRecord(h->ev[4], h->stream);
    CK(cudaGetLastError());
    return run_hook(h, MHFEM_HOOK_POST_ITERATE, t, tau);
}

mhfem_status mhfem_set_hook(mhfem_t h, int32_t point, mhfem_hook fn, void* user)
{
    if (!h) return MHFEM_ERR_INVALID_ARGUMENT;
    if (point != MHFEM_HOOK_PRE_ITERATE && point != MHFEM_HOOK_POST_ITERATE && point != MHFEM_HOOK_VECTOR_COEFFICIENTS)
        return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "unknown hook point %d", point);
    h->hooks[point].fn = fn;
    h->hooks[point].user = user;
    return MHFEM_OK;
}

mhfem_status mhfem_coeff_device(mhfem_t h, int32_t which, double** data, int64_t* count)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if (which < 0 || which >= NCOEF || !data) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "invalid coefficient id %d", which);
    if (!h->coef[which].p) return fail(h, MHFEM_ERR_STATE, "coefficient %d has no storage", which);
    *data = h->coef[which].p;
    if (count) *count = h->coef[which].count;
    if (which == MHFEM_COEF_A || which == MHFEM_COEF_U) h->coef_nonzero[which] = true;
    return MHFEM_OK;
}

mhfem_status mhfem_array_device(mhfem_t h, int32_t which, double** data, int64_t* count)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if (!data) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "null output");
    int64_t size = 0;
    if ((st = array_ptr(h, which, data, &size)) != MHFEM_OK) return st;
    if (count) *count = size;
    return MHFEM_OK;
}

mhfem_status mhfem_step(mhfem_t h, double t, double tau, mhfem_step_stats* stats)
{
    mhfem_status st;
    if ((st = mhfem_pre_iterate(h, t, tau)) != MHFEM_OK) return st;
    if ((st = mhfem_assemble(h, t, tau)) != MHFEM_OK) return st;
    if ((st = mhfem_solve(h, stats)) != MHFEM_OK) return st;
    if ((st = mhfem_post_iterate(h, t, tau)) != MHFEM_OK) return st;
    h->total_steps += 1;
    if (stats) {
        CK(cudaEventSynchronize(h->ev[4]));
        float a = 0, b = 0, c = 0, d = 0;
        cudaEventElapsedTime(&a, h->ev[0], h->ev[1]);
        cudaEventElapsedTime(&b, h->ev[1], h->ev[2]);
        cudaEventElapsedTime(&c, h->ev[2], h->ev[3]);
        cudaEventElapsedTime(&d, h->ev[3], h->ev[4]);
        stats->ms_pre = a; stats->ms_assemble = b; stats->ms_solve = c; stats->ms_post = d;
        float g = 0;
        if (h->guess_timed) cudaEventElapsedTime(&g, h->ev[5], h->ev[6]);
        stats->ms_guess = g;
    }
    return MHFEM_OK;
}

mhfem_status mhfem_get_state(mhfem_t h, double* Z_iF, double* Z_iK)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    cudaSetDevice(h->desc.device);
    if (Z_iF) CK(cudaMemcpyAsync(Z_iF, h->Z_iF, sizeof(double) * h->n * h->topo.F, cudaMemcpyDeviceToHost, h->stream));
    if (Z_iK) CK(cudaMemcpyAsync(Z_iK, h->Z_iK, sizeof(double) * h->n * h->topo.C, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return MHFEM_OK;
}

mhfem_status mhfem_get_array(mhfem_t h, int32_t which, double* out, int64_t count)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    double* src = nullptr;
    int64_t size = 0;
    if ((st = array_ptr(h, which, &src, &size)) != MHFEM_OK) return st;
    if (!out || count != size) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "array %d has %lld values", which, (long long)size);
    cudaSetDevice(h->desc.device);
    CK(cudaMemcpyAsync(out, src, sizeof(double) * size, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return MHFEM_OK;
}

mhfem_status mhfem_get_system(mhfem_t h, int64_t* rowptr, int32_t* cols, double* vals, double* rhs)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if ((st = ensure_pattern(h)) != MHFEM_OK) return st;
    cudaSetDevice(h->desc.device);
    const int64_t rows = h->pat.rows;
    const int W = h->pat.W;
    std::vector<double> ev((size_t)W * rows);
    if (W > 0)
        CK(cudaMemcpyAsync(ev.data(), h->A.vals, sizeof(double) * W * rows, cudaMemcpyDeviceToHost, h->stream));
    if (rhs) CK(cudaMemcpyAsync(rhs, h->rhs, sizeof(double) * rows, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    int64_t pos = 0;
    for (int64_t r = 0; r < rows; ++r) {
        if (rowptr) rowptr[r] = pos;
        const int len = h->pat.row_len[r];
        int k = 0;
        bool diag_done = false;
        for (int q = 0; q < len; ++q) {
            int32_t c;
            double v;
            const bool take_diag = !diag_done && (k >= len - 1 || h->pat.ell_cols[(size_t)k * rows + r] > r);
            if (take_diag) { c = (int32_t)r; v = 1.0; diag_done = true; }
            else { c = h->pat.ell_cols[(size_t)k * rows + r]; v = ev[(size_t)k * rows + r]; ++k; }
            if (cols) cols[pos] = c;
            if (vals) vals[pos] = v;
            ++pos;
        }
    }
    if (rowptr) rowptr[rows] = pos;
    return MHFEM_OK;
}

mhfem_status mhfem_get_system32(mhfem_t h, float* vals32)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if (!vals32) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "null output");
    if ((st = ensure_pattern(h)) != MHFEM_OK) return st;
    if (!h->fp32_copy || !h->A.vals32)
        return fail(h, MHFEM_ERR_STATE, "no FP32 copy of the matrix (mixed form or the learned form's mixed solve)");
    cudaSetDevice(h->desc.device);
    const int64_t rows = h->pat.rows;
    const int W = h->pat.W;
    std::vector<float> ev((size_t)W * rows);
    if (W > 0)
        CK(cudaMemcpyAsync(ev.data(), h->A.vals32, sizeof(float) * W * rows, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    int64_t pos = 0;
    for (int64_t r = 0; r < rows; ++r) {
        const int len = h->pat.row_len[r];
        int k = 0;
        bool diag_done = false;
        for (int q = 0; q < len; ++q) {
            const bool take_diag = !diag_done && (k >= len - 1 || h->pat.ell_cols[(size_t)k * rows + r] > r);
            if (take_diag) { vals32[pos++] = 1.0f; diag_done = true; }
            else vals32[pos++] = ev[(size_t)(k++) * rows + r];
        }
    }
    return MHFEM_OK;
}

mhfem_status mhfem_get_totals(mhfem_t h, int64_t* iterations, int64_t* time_steps, int64_t* kernel_launches)
{
    if (!h) return MHFEM_ERR_INVALID_ARGUMENT;
    if (iterations) *iterations = h->total_iters;
    if (time_steps) *time_steps = h->total_steps;
    if (kernel_launches) *kernel_launches = h->launches;
    return MHFEM_OK;
}

mhfem_status mhfem_get_stream(mhfem_t h, void** stream)
{
    if (!h || !stream) return MHFEM_ERR_INVALID_ARGUMENT;
    *stream = (void*)h->stream;
    return MHFEM_OK;
}

mhfem_status mhfem_check_grid_barrier(int32_t device, int32_t ctas, int32_t skip_cta, int32_t max_polls,
                                      int32_t* ctas_passed, int32_t* ctas_gave_up, int32_t* failure_flag)
{
    if (!ctas_passed || !ctas_gave_up || !failure_flag || ctas < 1 || max_polls < 1)
        return MHFEM_ERR_INVALID_ARGUMENT;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return MHFEM_ERR_NO_DEVICE;
    if (device < 0 || device >= n) return MHFEM_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return MHFEM_ERR_CUDA;
    int passed = 0, gave_up = 0, flag = 0;
    const cudaError_t e = grid_barrier_check(ctas, skip_cta, (unsigned int)max_polls, &passed, &gave_up, &flag);
    if (e == cudaErrorInvalidValue) return MHFEM_ERR_INVALID_ARGUMENT;
    if (e != cudaSuccess) return MHFEM_ERR_CUDA;
    *ctas_passed = passed;
    *ctas_gave_up = gave_up;
    *failure_flag = flag;
    return MHFEM_OK;
}

mhfem_status mhfem_time_kernel(mhfem_t h, int32_t kernel, int32_t reps, double* ms, double* bytes, double* flops)
{
    mhfem_status st = require_ready(h);
    if (st) return st;
    if (reps < 1) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "reps must be positive");
    if ((st = ensure_pattern(h)) != MHFEM_OK) return st;
    cudaSetDevice(h->desc.device);
    const double n = h->n, nf = h->nf, S = h->S, C = (double)h->topo.C, F = (double)h->topo.F;
    const double R = F * n, W = h->A.width, V = (double)h->topo.V, d = h->dim;
    const double rec = nf * n * (n * nf + 1) * C * 8;  // assembly records (one per cell side)
    DevProblem P = make_problem(h);
    double B = 0, FL = 0;
    // algorithmic bytes: each array once at its size; FLOPs: FP64 (FP32 for the SpMV32) operations
    switch (kernel) {
        case MHFEM_KERNEL_CELL_LOCAL:
            // a box cell reads two of its vertices (the lowest and the opposite corner)
            B = 4 * (h->cell ? 2 : h->nv) * C + 8 * d * V + (h->coef[MHFEM_COEF_D].count > 1 ? 8 * n * n * C : 0)
              + 8 * n * C + 4 * nf * C + C + 8 * n * n * S * C + 8 * n * n * nf * C + 8 * n * C + rec;
            FL = C * (h->cell ? 4.0 * nf * nf : (nf == 4 ? 420.0 : 220.0)) * n * n;
            break;
        case MHFEM_KERNEL_ASSEMBLE:
            B = 8 * F + 2 * F + (nf > 4 ? 8 : 4) * F + F + rec + 8 * W * R + 8 * R
              + (h->fp32_copy ? 4 * W * R : 0);
            FL = R * (W + 3);
            break;
        case MHFEM_KERNEL_SPMV_FP64: B = R * (12 * W + 24); FL = 2 * R * (W + 1); break;
        // the other FP64 BiCGStab iteration kernels: ELL words, s, t (second SpMV);
        // r, v, s (s update); x, p, s, t, rh read and x, r written; p, r, v, p
        case MHFEM_KERNEL_SPMV2_FP64: B = R * (12 * W + 16); FL = 2 * R * (W + 2); break;
        case MHFEM_KERNEL_UPDATE_S_FP64: B = R * 24; FL = 2 * R; break;
        case MHFEM_KERNEL_UPDATE_XR_FP64: B = R * 56; FL = 8 * R; break;
        case MHFEM_KERNEL_UPDATE_P_FP64: B = R * 32; FL = 4 * R; break;
        case MHFEM_KERNEL_SPMV_FP32:
            if (!h->fp32_copy) return fail(h, MHFEM_ERR_STATE, "FP32 SpMV needs the FP32 matrix (mixed form or mixed learned solve)");
            B = R * ((h->A.cols_lo ? 7 : 8) * W + 12); FL = 2 * R * (W + 1); break;
        case MHFEM_KERNEL_RECONSTRUCT:
            B = 4 * nf * C + 8 * n * F + 8 * n * n * nf * C + 8 * n * C + 8 * n * C;
            FL = 2 * C * n * (n * nf + 1);
            break;
        default: return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "unknown kernel %d", kernel);
    }
    const int fp64_iter = kernel == MHFEM_KERNEL_SPMV_FP64 ? 0 : kernel == MHFEM_KERNEL_SPMV2_FP64 ? 1
                        : kernel == MHFEM_KERNEL_UPDATE_S_FP64 ? 2 : kernel == MHFEM_KERNEL_UPDATE_XR_FP64 ? 3
                        : kernel == MHFEM_KERNEL_UPDATE_P_FP64 ? 4 : -1;
    if (fp64_iter >= 0 || kernel == MHFEM_KERNEL_SPMV_FP32) {
        // Make the Krylov kernels run: scalars that keep every launch going
        // (not done, no half step, no restart, finite non-zero alpha, omega,
        // beta, no iteration cap).  The FP64 vectors start as copies of the
        // current face traces, so the reductions see finite non-zero values.
        // The Krylov vectors are scratch between solves (the next solve
        // initializes them); Z_iF is only read.
        KrylovScalars z{};
        z.rho = 1.0;
        z.alpha = z.omega = z.beta = 0.5;
        z.bnorm = z.rr = z.rhnorm = 1.0;
        z.max_iter = 0x7fffffff;
        if (fp64_iter >= 0) {
            const size_t bytes = sizeof(double) * (size_t)R;
            for (double* v : {h->W.r, h->W.rh, h->W.p, h->W.v, h->W.s, h->W.t})
                CK(cudaMemcpyAsync(v, h->Z_iF, bytes, cudaMemcpyDeviceToDevice, h->stream));
        }
        CK(cudaMemcpyAsync(kernel == MHFEM_KERNEL_SPMV_FP32 ? h->W.sc32 : h->W.sc, &z, sizeof(z),
                           cudaMemcpyHostToDevice, h->stream));
    }
    auto launch = [&]() {
        switch (kernel) {
            case MHFEM_KERNEL_CELL_LOCAL: launch_cell_local(P, h->cur_tau > 0 ? h->cur_tau : 1.0, h->stream); break;
            case MHFEM_KERNEL_ASSEMBLE:
                launch_assemble(P, h->amap, h->A, h->rhs, h->fp32_copy, h->stream); break;
            case MHFEM_KERNEL_SPMV_FP64: case MHFEM_KERNEL_SPMV2_FP64: case MHFEM_KERNEL_UPDATE_S_FP64:
            case MHFEM_KERNEL_UPDATE_XR_FP64: case MHFEM_KERNEL_UPDATE_P_FP64:
                krylov_fp64_kernel_once(h->A, h->W, fp64_iter, h->stream); break;
            case MHFEM_KERNEL_SPMV_FP32: krylov_spmv_dot_once(h->A, h->W, true, h->stream); break;
            case MHFEM_KERNEL_RECONSTRUCT: launch_reconstruct(P, h->stream); break;
        }
    };
    launch();  // warm-up
    CK(cudaEventRecord(h->ev[0], h->stream));
    for (int r = 0; r < reps; ++r) launch();
    CK(cudaEventRecord(h->ev[1], h->stream));
    CK(cudaEventSynchronize(h->ev[1]));
    CK(cudaGetLastError());
    float total = 0;
    CK(cudaEventElapsedTime(&total, h->ev[0], h->ev[1]));
    h->launches += reps + 1;
    if (ms) *ms = total / reps;
    if (bytes) *bytes = B;
    if (flops) *flops = FL;
    return MHFEM_OK;
}

}  // extern "C"
