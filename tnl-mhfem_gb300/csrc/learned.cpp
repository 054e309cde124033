// Learned warm-start form: host orchestration of the message-passing network
// (k_mpnn.cu) around the unchanged FP64 BiCGStab solve.
//
// Per time step (after the assembly):
//   1. Zn = the previous step's traces (the default warm start); the last
//      four traces are kept;
//   2. base = the polynomial extrapolation in time of the last traces (order
//      1 to 3, as far as the history reaches);
//   3. once the network is trained: guess = base + c * net(features), c the
//      size of the base's error in the previous step;
//   4. of the warm start, the base and the guess, the one with the lowest
//      relative residual ||b - A x|| / ||b|| starts the solve (a network that
//      keeps losing this comparison is run only every few steps);
//   5. the FP64 BiCGStab runs to the same tolerance as the plain form, so the
//      initial guess can only change the iteration count;
//   6. during the first `train_steps` steps the network is trained online
//      (Adam) on the solution the method just produced.
#include <cmath>
#include <cstring>
#include <vector>

#include "handle.h"
#include "mpnn.h"

namespace mhfem {

struct LearnedState {
    bool ready = false;
    int64_t F = 0;
    int64_t free_rows = 0;
    uint8_t* deg = nullptr;
    uint8_t* fixed = nullptr;
    float* stat = nullptr;
    float* f_base = nullptr;
    float* f_psi = nullptr;
    double f_norm = 1.0;
    __nv_bfloat16* x0 = nullptr;
    __nv_bfloat16* h[kMpnnLayers + 2] = {};
    __nv_bfloat16* a[kMpnnLayers + 1] = {};
    __nv_bfloat16* z[kMpnnLayers + 1] = {};
    __nv_bfloat16* dz = nullptr;
    float* dh = nullptr;
    __nv_bfloat16* gb[2] = {};
    float* params = nullptr;
    float* grads = nullptr;
    float* m1 = nullptr;
    float* m2 = nullptr;
    __nv_bfloat16* w_fwd[kMpnnLayers + 1] = {};
    __nv_bfloat16* w_bwd[kMpnnLayers + 1] = {};
    double* dec_partials = nullptr;
    float* dw_partials = nullptr;
    double* loss = nullptr;
    double* scal = nullptr;  // [16] device scalars, laid out in k_mpnn_io.cu
    double* Zs[4] = {};      // the last traces, a ring: Zs[cur] is this step's Zn
    int cur = 0;
    double* base = nullptr;
    double* guess = nullptr;
    double* target = nullptr;
    float* out = nullptr;
    double* host = nullptr;  // pinned: scales, residuals, loss
    int32_t* err = nullptr;
    int hist = 0;
    int net_losses = 0;   // consecutive steps whose network guess lost the gate
    int trained_steps = 0;
    int adam_t = 0;
    bool params_set = false;
    bool params_loaded = false;  // given by mhfem_learned_set_params: usable before any training
    // options
    int mixed_solve = 0;  // solve from the guess with the mixed-precision refinement
    int train_steps = 200;
    int train_iters = 2;
    float lr = 1e-3f;
    double lr_final = 1.0;  // fraction of lr at the last training step (cosine decay)
    int use_during_training = 0;
    int order = 3;        // extrapolation order of the base
    uint64_t seed = 1234;
    double last_loss = -1;
    std::vector<void*> allocs;
};

namespace {

constexpr int H = kMpnnHidden;
// After kNetBackoff consecutive steps in which the network's guess lost the
// gate (the extrapolated base or the warm start was closer), the network is
// run only every kNetRetry-th step until it wins again: its inference costs
// about as much as ten FP64 iterations on the 64^3 workload.
constexpr int kNetBackoff = 4;
constexpr int kNetRetry = 16;

int off_W(int l) { return l == 0 ? 0 : kMpnnFeatures * H + H + (l - 1) * (2 * H * H + H); }
int off_b(int l) { return off_W(l) + (l == 0 ? kMpnnFeatures : 2 * H) * H; }
int off_wd() { return off_W(kMpnnLayers + 1); }
int off_bd() { return off_wd() + H; }

template <typename T>
cudaError_t lalloc(LearnedState* L, T** p, size_t n)
{
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * n);
    if (e == cudaSuccess) L->allocs.push_back((void*)*p);
    return e;
}

#define LCK(call)                                                                                   \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return fail(h, e_ == cudaErrorMemoryAllocation ? MHFEM_ERR_OUT_OF_MEMORY : MHFEM_ERR_CUDA, \
                        "%s failed: %s", #call, cudaGetErrorString(e_));                            \
    } while (0)

// splitmix64 + Box-Muller: deterministic initial weights
struct Rng {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() { return std::sqrt(-2.0 * std::log(uniform())) * std::cos(6.283185307179586 * uniform()); }
};

void init_params_host(std::vector<float>& p, uint64_t seed)
{
    Rng r{seed};
    p.assign(kMpnnParams, 0.f);
    for (int i = 0; i < kMpnnFeatures * H; ++i) p[off_W(0) + i] = (float)(r.normal() * std::sqrt(2.0 / kMpnnFeatures));
    for (int l = 1; l <= kMpnnLayers; ++l)
        for (int i = 0; i < 2 * H * H; ++i) p[off_W(l) + i] = (float)(r.normal() * std::sqrt(1.0 / (2 * H)));
    for (int i = 0; i < H; ++i) p[off_wd() + i] = (float)(r.normal() * 0.01);
}

MpnnView make_view(mhfem_t h)
{
    LearnedState* L = h->learned;
    MpnnView V;
    V.F = L->F;
    V.W = h->A.width;
    V.nbr = h->A.cols;
    V.deg = L->deg;
    V.fixed = L->fixed;
    V.x0 = L->x0;
    for (int l = 0; l < kMpnnLayers + 2; ++l) V.h[l] = L->h[l];
    for (int l = 0; l < kMpnnLayers + 1; ++l) {
        V.a[l] = L->a[l];
        V.z[l] = L->z[l];
        V.w_fwd[l] = L->w_fwd[l];
        V.w_bwd[l] = L->w_bwd[l];
        V.bias[l] = L->params + off_b(l);
    }
    V.dz = L->dz;
    V.dh = L->dh;
    V.gb[0] = L->gb[0];
    V.gb[1] = L->gb[1];
    V.wd = L->params + off_wd();
    V.bd = L->params + off_bd();
    V.dec_partials = L->dec_partials;
    V.err = L->err;
    return V;
}

MpnnGrads make_grads(mhfem_t h)
{
    LearnedState* L = h->learned;
    MpnnGrads G;
    G.g = L->grads;
    for (int l = 0; l <= kMpnnLayers; ++l) {
        G.off_W[l] = off_W(l);
        G.off_b[l] = off_b(l);
    }
    G.off_wd = off_wd();
    G.off_bd = off_bd();
    G.partials = L->dw_partials;
    G.loss = L->loss;
    return G;
}

void publish(mhfem_t h)
{
    LearnedState* L = h->learned;
    for (int l = 0; l <= kMpnnLayers; ++l)
        mpnn_publish(L->params + off_W(l), l == 0 ? kMpnnFeatures : 2 * H, L->w_fwd[l], l == 0 ? nullptr : L->w_bwd[l],
                     h->stream);
}

double coef_at(mhfem_t h, int which, int64_t idx, double dflt)
{
    const auto& c = h->h_coef[which];
    if (c.empty()) return dflt;
    return c.size() == 1 ? c[0] : c[idx];
}

}  // namespace

void learned_invalidate(mhfem_t h)
{
    if (h->learned) h->learned->ready = false;
}

void learned_reset_history(mhfem_t h)
{
    if (h->learned) {
        h->learned->hist = 0;
        h->learned->net_losses = 0;
    }
}

void learned_release(mhfem_t h)
{
    if (!h->learned) return;
    for (void* p : h->learned->allocs) cudaFree(p);
    if (h->learned->host) cudaFreeHost(h->learned->host);
    delete h->learned;
    h->learned = nullptr;
}

// Allocates the network state for the current pattern and builds the static features.
static mhfem_status learned_prepare(mhfem_t h)
{
    if (!h->learned) h->learned = new LearnedState();
    LearnedState* L = h->learned;
    if (L->ready && L->F == h->topo.F) return MHFEM_OK;
    if (h->n != 1) return fail(h, MHFEM_ERR_UNSUPPORTED, "the learned form supports one equation (n = 1)");
    if (h->pat.W > kMpnnMaxWidth)
        return fail(h, MHFEM_ERR_UNSUPPORTED, "the learned form takes at most %d neighbours per face", kMpnnMaxWidth);
    const int64_t F = h->topo.F, C = h->topo.C;
    const int nf = h->nf, dim = h->dim;
    // keep options and parameters across re-preparation
    const bool had_params = L->params_set;
    std::vector<float> keep;
    if (had_params && L->params) {
        keep.resize(kMpnnParams);
        cudaMemcpy(keep.data(), L->params, sizeof(float) * kMpnnParams, cudaMemcpyDeviceToHost);
    }
    for (void* p : L->allocs) cudaFree(p);
    L->allocs.clear();
    L->F = F;

    // graph: degree (non-padding ELL entries) and Dirichlet rows
    std::vector<uint8_t> deg(F, 0), fixed(F, 0);
    const int W = h->pat.W;
    for (int64_t E = 0; E < F; ++E) {
        int d = 0;
        for (int k = 0; k < W; ++k)
            if (h->pat.ell_cols[(size_t)k * F + E] != (int32_t)E) ++d;
        deg[E] = (uint8_t)d;
        fixed[E] = (h->topo.face_cells[2 * E + 1] < 0 && h->h_tags[E] == MHFEM_BC_FIXED_VALUE) ? 1 : 0;
    }
    int64_t nfree = 0;
    for (int64_t E = 0; E < F; ++E) nfree += fixed[E] ? 0 : 1;
    L->free_rows = nfree;

    // static features
    std::vector<float> stat((size_t)F * 16, 0.f), fb(F, 0.f), fp(F, 0.f);
    double mean_area = 0;
    for (int64_t E = 0; E < F; ++E) mean_area += h->topo.face_measure[E];
    mean_area = F > 0 ? mean_area / F : 1.0;
    std::vector<double> logD(F, 0.0);
    double lmean = 0, lsq = 0;
    double fmax = 0;
    for (int64_t E = 0; E < F; ++E) {
        const int32_t K0 = h->topo.face_cells[2 * E], K1 = h->topo.face_cells[2 * E + 1];
        double ld = std::log(std::max(coef_at(h, MHFEM_COEF_D, K0, 1.0), 1e-300));
        double f0 = coef_at(h, MHFEM_COEF_F, K0, 0.0), p0 = coef_at(h, MHFEM_COEF_PSI, K0, 0.0);
        if (K1 >= 0) {
            ld = 0.5 * (ld + std::log(std::max(coef_at(h, MHFEM_COEF_D, K1, 1.0), 1e-300)));
            f0 = 0.5 * (f0 + coef_at(h, MHFEM_COEF_F, K1, 0.0));
            p0 = 0.5 * (p0 + coef_at(h, MHFEM_COEF_PSI, K1, 0.0));
        }
        logD[E] = ld;
        lmean += ld;
        lsq += ld * ld;
        fb[E] = (float)f0;
        fp[E] = (float)p0;
        fmax = std::max(fmax, std::fabs(f0) + std::fabs(h->src_amp * p0));
    }
    lmean /= std::max<int64_t>(F, 1);
    const double lsd = std::sqrt(std::max(lsq / std::max<int64_t>(F, 1) - lmean * lmean, 0.0));
    L->f_norm = fmax > 0 ? 1.0 / fmax : 0.0;
    for (int64_t E = 0; E < F; ++E) {
        float* s = &stat[(size_t)E * 16];
        s[3] = (float)(lsd > 0 ? (logD[E] - lmean) / lsd : 0.0);
        // unit normal, sign-free
        const int32_t* fv = &h->topo.face_verts[(size_t)E * dim];
        double n[3] = {0, 0, 0};
        const double* X0 = &h->h_coords[(size_t)fv[0] * dim];
        const double* X1 = &h->h_coords[(size_t)fv[1] * dim];
        if (dim == 2) {
            n[0] = X1[1] - X0[1];
            n[1] = -(X1[0] - X0[0]);
        }
        else {
            const double* X2 = &h->h_coords[(size_t)fv[2] * dim];
            const double a[3] = {X1[0] - X0[0], X1[1] - X0[1], X1[2] - X0[2]};
            const double b[3] = {X2[0] - X0[0], X2[1] - X0[1], X2[2] - X0[2]};
            n[0] = a[1] * b[2] - a[2] * b[1];
            n[1] = a[2] * b[0] - a[0] * b[2];
            n[2] = a[0] * b[1] - a[1] * b[0];
        }
        const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int d = 0; d < 3; ++d) s[5 + d] = (float)(nn > 0 ? std::fabs(n[d]) / nn : 0.0);
        s[8] = (float)(h->topo.face_measure[E] / mean_area);
        s[9] = h->topo.face_cells[2 * E + 1] < 0 ? 1.f : 0.f;
        s[10] = fixed[E] ? 1.f : 0.f;
        s[11] = 1.f;
    }
    (void)C;
    (void)nf;

    LCK(lalloc(L, &L->deg, F));
    LCK(cudaMemcpy(L->deg, deg.data(), F, cudaMemcpyHostToDevice));
    LCK(lalloc(L, &L->fixed, F));
    LCK(cudaMemcpy(L->fixed, fixed.data(), F, cudaMemcpyHostToDevice));
    LCK(lalloc(L, &L->stat, (size_t)F * 16));
    LCK(cudaMemcpy(L->stat, stat.data(), sizeof(float) * F * 16, cudaMemcpyHostToDevice));
    LCK(lalloc(L, &L->f_base, F));
    LCK(cudaMemcpy(L->f_base, fb.data(), sizeof(float) * F, cudaMemcpyHostToDevice));
    LCK(lalloc(L, &L->f_psi, F));
    LCK(cudaMemcpy(L->f_psi, fp.data(), sizeof(float) * F, cudaMemcpyHostToDevice));
    LCK(lalloc(L, &L->x0, (size_t)F * 16));
    for (int l = 1; l <= kMpnnLayers + 1; ++l) LCK(lalloc(L, &L->h[l], (size_t)F * H));
    for (int l = 1; l <= kMpnnLayers; ++l) LCK(lalloc(L, &L->a[l], (size_t)F * H));
    for (int l = 0; l <= kMpnnLayers; ++l) LCK(lalloc(L, &L->z[l], (size_t)F * H));
    LCK(lalloc(L, &L->dz, (size_t)F * H));
    LCK(lalloc(L, &L->dh, (size_t)F * H));
    for (auto& g : L->gb) LCK(lalloc(L, &g, (size_t)F * H));
    LCK(lalloc(L, &L->params, kMpnnParams));
    LCK(lalloc(L, &L->grads, kMpnnParams));
    LCK(lalloc(L, &L->m1, kMpnnParams));
    LCK(lalloc(L, &L->m2, kMpnnParams));
    LCK(cudaMemset(L->m1, 0, sizeof(float) * kMpnnParams));
    LCK(cudaMemset(L->m2, 0, sizeof(float) * kMpnnParams));
    for (int l = 0; l <= kMpnnLayers; ++l) {
        const int K = l == 0 ? kMpnnFeatures : 2 * H;
        LCK(lalloc(L, &L->w_fwd[l], (size_t)K * H));
        LCK(lalloc(L, &L->w_bwd[l], (size_t)K * H));
    }
    LCK(lalloc(L, &L->dec_partials, (size_t)mpnn_grid_size(F) * (H + 2)));
    LCK(lalloc(L, &L->dw_partials, (size_t)mpnn_partials_floats(F)));
    LCK(lalloc(L, &L->loss, 1));
    LCK(lalloc(L, &L->scal, 16));
    LCK(cudaMemset(L->scal, 0, sizeof(double) * 16));
    for (auto& z : L->Zs) LCK(lalloc(L, &z, F));
    L->cur = 0;
    LCK(lalloc(L, &L->base, F));
    LCK(lalloc(L, &L->guess, F));
    LCK(lalloc(L, &L->target, F));
    LCK(lalloc(L, &L->out, F));
    LCK(lalloc(L, &L->err, 1));
    LCK(cudaMemset(L->err, 0, sizeof(int32_t)));
    if (!L->host) LCK(cudaMallocHost((void**)&L->host, sizeof(double) * 16));
    std::vector<float> p0;
    if (had_params && !keep.empty()) p0 = keep;
    else init_params_host(p0, L->seed);
    LCK(cudaMemcpy(L->params, p0.data(), sizeof(float) * kMpnnParams, cudaMemcpyHostToDevice));
    L->params_set = true;
    publish(h);
    LCK(cudaStreamSynchronize(h->stream));
    L->hist = 0;
    L->ready = true;
    return MHFEM_OK;
}

static mhfem_status check_err(mhfem_t h)
{
    LearnedState* L = h->learned;
    int32_t e = 0;
    LCK(cudaMemcpyAsync(&L->host[7], L->err, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    LCK(cudaStreamSynchronize(h->stream));
    std::memcpy(&e, &L->host[7], sizeof(int32_t));
    if (e) return fail(h, MHFEM_ERR_CUDA, "tensor-core kernel reported error flags 0x%x (mbarrier wait timed out)", e);
    return MHFEM_OK;
}

static mhfem_status train_once(mhfem_t h, int iters)
{
    LearnedState* L = h->learned;
    MpnnView V = make_view(h);
    MpnnGrads G = make_grads(h);
    const double inv_nt = L->free_rows > 0 ? 1.0 / (double)L->free_rows : 0.0;
    // cosine decay from lr to lr * lr_final over the training steps
    const double prog = L->train_steps > 1 ? (double)L->trained_steps / (double)(L->train_steps - 1) : 1.0;
    const float lr = (float)(L->lr * (L->lr_final + (1.0 - L->lr_final) * 0.5 * (1.0 + std::cos(M_PI * std::fmin(prog, 1.0)))));
    for (int it = 0; it < iters; ++it) {
        mpnn_forward(V, true, h->stream);
        mpnn_backward(V, L->target, inv_nt, G, h->stream);
        L->adam_t += 1;
        mpnn_adam(L->params, L->grads, L->m1, L->m2, kMpnnParams, lr, L->adam_t, h->stream);
        publish(h);
        h->launches += 4 + 2 + 3 * kMpnnLayers + 3 + 1 + 4;
    }
    LCK(cudaMemcpyAsync(&L->host[4], L->loss, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    LCK(cudaGetLastError());
    return MHFEM_OK;
}

mhfem_status learned_solve(mhfem_t h, int* iters, int* sweeps, double* res, mhfem_step_stats* stats)
{
    mhfem_status st = learned_prepare(h);
    if (st) return st;
    LearnedState* L = h->learned;
    const int64_t F = L->F;
    cudaStream_t s = h->stream;
    double* Zn = L->Zs[L->cur];
    const double* Zprev[3] = {L->Zs[(L->cur + 3) & 3], L->Zs[(L->cur + 2) & 3], L->Zs[(L->cur + 1) & 3]};
    LCK(cudaMemcpyAsync(Zn, h->Z_iF, sizeof(double) * F, cudaMemcpyDeviceToDevice, s));
    const bool have_hist = L->hist >= 1;
    const bool training = L->trained_steps < L->train_steps;
    const bool backed_off = L->net_losses >= kNetBackoff && (L->hist % kNetRetry) != 0;
    const bool infer = have_hist && (!training || L->use_during_training) && (L->trained_steps > 0 || L->params_loaded) &&
                       !backed_off;
    MpnnInputs in{};
    in.Zn = Zn;
    in.Zn1 = Zprev[0];
    in.Zn2 = Zprev[1];
    in.Zn3 = Zprev[2];
    in.hist = std::min(L->hist, 3);
    in.rhs = h->rhs;
    in.stat = L->stat;
    in.f_base = L->f_base;
    in.f_psi = L->f_psi;
    in.src_scale = h->src_amp * std::sin(2.0 * M_PI * h->cur_t / h->src_period);
    in.f_norm = L->f_norm;
    in.rbase = h->W.r;  // the Krylov r vector is idle until the solve
    in.scal = L->scal;
    if (have_hist) {
        cudaEventRecord(h->ev[5], s);
        h->guess_timed = true;
    }
    // The base, its residual and the gate run without a host round trip:
    // the scales stay on the device and the gate decides there.  Training
    // reads the scales (the features divide by them), outside the timed use
    // phase.
    bool have_features = false;
    if (have_hist) {
        const int order = std::min(L->order, L->hist);
        mpnn_extrapolate(F, order, Zn, Zprev[0], Zprev[1], Zprev[2], L->fixed, h->rhs, L->base, s);
        learned_prep_fp64(h->A, h->rhs, Zn, Zprev[0], Zprev[1], Zprev[2], std::min(L->hist, 3), L->base, L->fixed,
                          h->W.r, L->scal, h->W, s);
        h->launches += 2;
        if (training || infer) {
            if (training) {
                LCK(cudaMemcpyAsync(L->host, L->scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
                LCK(cudaStreamSynchronize(s));
                have_features = L->host[0] > 0 && L->host[1] > 0;
            }
            else
                have_features = true;  // zero scales make the features zero; the gate rejects a useless guess
            if (have_features) {
                mpnn_features(F, in, L->x0, s);
                h->launches += 1;
            }
        }
    }
    const bool guessed = infer && have_features;
    if (guessed) {
        MpnnView V = make_view(h);
        V.dec_base = L->base;
        V.dec_rhs = h->rhs;
        V.dec_scal = L->scal;
        V.dec_guess = L->guess;
        mpnn_infer_guess(V, s);
        residual_norm_fp64(h->A, h->rhs, L->guess, h->W, s);
        h->launches += (kMpnnLayers + 1) + 1;
    }
    if (have_hist) {
        mpnn_gate(F, guessed ? L->guess : nullptr, L->base, h->Z_iF, &h->W.sc->res, L->scal, s);
        h->launches += 1;
    }
    if (h->guess_timed) cudaEventRecord(h->ev[6], s);
    st = L->mixed_solve ? run_mixed(h, iters, sweeps, res) : run_fp64(h, h->opts.tol, h->opts.max_iter, iters, res);
    if (st) return st;
    int source = 0;
    double r_warm = -1, r_guess = -1, r_base = -1;
    if (have_hist) {
        LCK(cudaMemcpyAsync(L->host, L->scal, 11 * sizeof(double), cudaMemcpyDeviceToHost, s));
        if ((st = check_err(h)) != MHFEM_OK) return st;  // synchronizes the stream
        r_warm = L->host[3];
        r_guess = guessed ? L->host[5] : -1;
        r_base = L->host[9];
        source = (int)L->host[6];
        if (guessed) L->net_losses = (source == 1) ? 0 : L->net_losses + 1;
        // the base's error in this step (and, while training, the target scaled by this step's c)
        const bool train_now = training && have_features;
        mpnn_target(F, h->Z_iF, L->base, L->fixed, L->scal, train_now ? L->target : nullptr, h->W.partials,
                    h->W.counters, s);
        h->launches += 1;
        if (train_now) {
            if ((st = train_once(h, L->train_iters)) != MHFEM_OK) return st;
            LCK(cudaStreamSynchronize(s));
            if ((st = check_err(h)) != MHFEM_OK) return st;
            L->last_loss = L->host[4];
            L->trained_steps += 1;
        }
    }
    L->cur = (L->cur + 1) & 3;  // this step's Zn becomes Zn1
    L->hist += 1;
    if (stats) {
        stats->guess_used = source == 1 ? 1 : 0;
        stats->guess_residual = r_guess;
        stats->warm_residual = r_warm;
        stats->base_residual = r_base;
        stats->guess_source = source;
    }
    return MHFEM_OK;
}

}  // namespace mhfem

using namespace mhfem;

namespace {

mhfem_status ready_for_learning(mhfem_t h)
{
    if (!h) return MHFEM_ERR_INVALID_ARGUMENT;
    if (!h->has_mesh) return fail(h, MHFEM_ERR_STATE, "mhfem_set_mesh has not been called");
    if (!h->pattern_ready) {
        mhfem_status st = mhfem_setup_linear_system(h);
        if (st) return st;
    }
    return learned_prepare(h);
}

}  // namespace

extern "C" {

mhfem_status mhfem_learned_set_options(mhfem_t h, const mhfem_learned_opts* o)
{
    if (!h || !o) return MHFEM_ERR_INVALID_ARGUMENT;
    if (o->train_steps < 0 || o->train_iters < 1 || !(o->learning_rate > 0) || !(o->lr_final > 0) ||
        o->lr_final > 1 || o->extrapolation_order < 0 || o->extrapolation_order > 3)
        return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "invalid learned-form options");
    if (!h->learned) h->learned = new LearnedState();
    LearnedState* L = h->learned;
    L->train_steps = o->train_steps;
    L->train_iters = o->train_iters;
    L->lr = (float)o->learning_rate;
    L->lr_final = o->lr_final;
    L->use_during_training = o->use_during_training;
    L->order = o->extrapolation_order;
    L->mixed_solve = o->mixed_solve ? 1 : 0;
    if (h->desc.form == MHFEM_FORM_LEARNED && (L->mixed_solve != 0) != h->fp32_copy) {
        // the FP32 matrix copy and work vectors follow; the pattern is rebuilt at the next step
        h->fp32_copy = L->mixed_solve != 0;
        h->pattern_ready = false;
    }
    if (o->seed != 0 && o->seed != L->seed) {
        L->seed = o->seed;
        L->params_set = false;
        L->ready = false;
    }
    return MHFEM_OK;
}

mhfem_status mhfem_learned_get_params(mhfem_t h, float* params, int64_t count)
{
    mhfem_status st = ready_for_learning(h);
    if (st) return st;
    if (!params || count != kMpnnParams)
        return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "the network has %d parameters", kMpnnParams);
    LCK(cudaMemcpyAsync(params, h->learned->params, sizeof(float) * kMpnnParams, cudaMemcpyDeviceToHost, h->stream));
    LCK(cudaStreamSynchronize(h->stream));
    return MHFEM_OK;
}

mhfem_status mhfem_learned_set_params(mhfem_t h, const float* params, int64_t count)
{
    mhfem_status st = ready_for_learning(h);
    if (st) return st;
    if (!params || count != kMpnnParams)
        return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "the network has %d parameters", kMpnnParams);
    LearnedState* L = h->learned;
    LCK(cudaMemcpyAsync(L->params, params, sizeof(float) * kMpnnParams, cudaMemcpyHostToDevice, h->stream));
    LCK(cudaMemsetAsync(L->m1, 0, sizeof(float) * kMpnnParams, h->stream));
    LCK(cudaMemsetAsync(L->m2, 0, sizeof(float) * kMpnnParams, h->stream));
    L->adam_t = 0;
    publish(h);
    LCK(cudaStreamSynchronize(h->stream));
    L->params_set = true;
    L->params_loaded = true;
    L->net_losses = 0;
    return MHFEM_OK;
}

mhfem_status mhfem_learned_forward(mhfem_t h, const float* features, float* out)
{
    mhfem_status st = ready_for_learning(h);
    if (st) return st;
    if (!features || !out) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "null buffers");
    LearnedState* L = h->learned;
    const int64_t F = L->F;
    float* dfeat = nullptr;
    LCK(cudaMalloc((void**)&dfeat, sizeof(float) * F * 16));
    cudaMemcpyAsync(dfeat, features, sizeof(float) * F * 16, cudaMemcpyHostToDevice, h->stream);
    mpnn_features_from_host(F, dfeat, L->x0, h->stream);
    MpnnView V = make_view(h);
    mpnn_forward(V, false, h->stream);
    mpnn_out(V, L->out, h->stream);
    cudaMemcpyAsync(out, L->out, sizeof(float) * F, cudaMemcpyDeviceToHost, h->stream);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    cudaFree(dfeat);
    if (e != cudaSuccess) return fail(h, MHFEM_ERR_CUDA, "learned forward: %s", cudaGetErrorString(e));
    return check_err(h);
}

mhfem_status mhfem_learned_gradients(mhfem_t h, const float* features, const double* target, float* grads,
                                     double* loss)
{
    mhfem_status st = ready_for_learning(h);
    if (st) return st;
    if (!features || !target || !grads) return fail(h, MHFEM_ERR_INVALID_ARGUMENT, "null buffers");
    LearnedState* L = h->learned;
    const int64_t F = L->F;
    float* dfeat = nullptr;
    LCK(cudaMalloc((void**)&dfeat, sizeof(float) * F * 16));
    cudaMemcpyAsync(dfeat, features, sizeof(float) * F * 16, cudaMemcpyHostToDevice, h->stream);
    cudaMemcpyAsync(L->target, target, sizeof(double) * F, cudaMemcpyHostToDevice, h->stream);
    mpnn_features_from_host(F, dfeat, L->x0, h->stream);
    MpnnView V = make_view(h);
    MpnnGrads G = make_grads(h);
    mpnn_forward(V, true, h->stream);
    const double inv_nt = L->free_rows > 0 ? 1.0 / (double)L->free_rows : 0.0;
    mpnn_backward(V, L->target, inv_nt, G, h->stream);
    cudaMemcpyAsync(grads, L->grads, sizeof(float) * kMpnnParams, cudaMemcpyDeviceToHost, h->stream);
    cudaMemcpyAsync(&L->host[5], L->loss, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    cudaFree(dfeat);
    if (e != cudaSuccess) return fail(h, MHFEM_ERR_CUDA, "learned gradients: %s", cudaGetErrorString(e));
    if (loss) *loss = L->host[5];
    return check_err(h);
}

mhfem_status mhfem_learned_status(mhfem_t h, int32_t* trained_steps, double* last_loss, int32_t* num_params)
{
    if (!h) return MHFEM_ERR_INVALID_ARGUMENT;
    if (trained_steps) *trained_steps = h->learned ? h->learned->trained_steps : 0;
    if (last_loss) *last_loss = h->learned ? h->learned->last_loss : -1;
    if (num_params) *num_params = kMpnnParams;
    return MHFEM_OK;
}

}  // extern "C"
