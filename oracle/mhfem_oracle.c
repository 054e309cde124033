/*
 * CPU oracle for the MHFEM per-time-step path (test infrastructure only).
 *
 * A plain C11 + OpenMP restatement of the reference algorithm, written from
 * the reference sources function by function (citations below are paths in
 * the TNL-MHFEM project).  Only tests/, the smoke check and the CPU-baseline
 * leg of bench.py use it.  Parity is UNPINNED: the reference has no tests or
 * golden vectors and cannot be built here (TNL is absent); the oracle is
 * pinned to mathematical known answers in tests/ instead.
 *
 * Third-party algorithms the reference takes from TNL @ 40f62622 (not
 * present) are restated from their published definitions:
 *   - LU_sequential_factorize / LU_sequential_solve_inplace: Doolittle LU
 *     without pivoting, unit lower triangle, forward then back substitution;
 *   - getEntityMeasure: |det| / d! of the simplex edge vectors (length,
 *     area, volume);
 *   - mesh face numbering: first appearance over cells and local faces;
 *   - Solvers::Linear::BICGStab with the Diagonal preconditioner: van der
 *     Vorst's BiCGStab; every row is scaled to a unit diagonal by the
 *     assembly, so the diagonal preconditioner is the identity.
 */
#include "mhfem_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXN 4   /* max equations supported by the oracle */
#define MAXF 6   /* max faces per cell (cuboid) */

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static inline double cget(orc_coef c, int64_t idx) { return c.full ? c.p[idx] : c.p[0]; }

/* ---- coefficient accessors in the reference CUDA layouts ---- */
#define IDX_ijK(p, i, j, K)      (((int64_t)(i) * (p)->n + (j)) * (p)->C + (K))
#define IDX_ijeK(p, i, j, e, K)  ((((int64_t)(i) * (p)->n + (j)) * (p)->nf + (e)) * (p)->C + (K))
#define IDX_iK(p, i, K)          ((int64_t)(i) * (p)->C + (K))
#define IDX_ieK(p, i, e, K)      (((int64_t)(i) * (p)->nf + (e)) * (p)->C + (K))
#define IDX_ijsK(p, i, j, s, K)  ((((int64_t)(i) * (p)->n + (j)) * (p)->S + (s)) * (p)->C + (K))
#define IDX_Fi(p, FF, i)         ((int64_t)(FF) * (p)->n + (i))
#define IDX_Eji(p, E, j, i)      (((int64_t)(E) * (p)->n + (j)) * (p)->n + (i))
#define IDX_iF(p, i, FF)         ((int64_t)(i) * (p)->F + (FF))

static inline double m_upw_get(const orc_problem* p, int i, int64_t E)
{
    if (p->mobility_upwind || p->m_upw_full) return p->m_upw[IDX_Fi(p, E, i)];
    return p->m_upw[0];
}

/* ------------------------------------------------------------------ */
/* Topology (TNL mesh initializer semantics, restated; mesh_helpers.h:49-265) */

typedef struct { int32_t v[4]; int64_t slot; } face_seed;

static int seed_cmp(const void* A, const void* B)
{
    const face_seed* a = (const face_seed*)A;
    const face_seed* b = (const face_seed*)B;
    for (int k = 0; k < 3; ++k) {
        if (a->v[k] < b->v[k]) return -1;
        if (a->v[k] > b->v[k]) return 1;
    }
    return (a->slot < b->slot) ? -1 : (a->slot > b->slot);
}

static int i64_cmp(const void* A, const void* B)
{
    const int64_t a = *(const int64_t*)A, b = *(const int64_t*)B;
    return (a < b) ? -1 : (a > b);
}

/* local vertices of the faces of a box cell (see the header) */
static const int kRectFaces[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
static const int kCuboidFaces[6][4] = {{0, 1, 2, 3}, {0, 1, 5, 4}, {1, 2, 6, 5},
                                       {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};

int64_t orc_build_faces(int dim, int64_t C, const int32_t* cell_verts,
                        int32_t* cell_faces, int32_t* face_cells, int32_t* face_verts)
{
    return orc_build_faces_ct(dim, 0, C, cell_verts, cell_faces, face_cells, face_verts);
}

int64_t orc_build_faces_ct(int dim, int cell, int64_t C, const int32_t* cell_verts,
                           int32_t* cell_faces, int32_t* face_cells, int32_t* face_verts)
{
    const int nf = cell ? 2 * dim : dim + 1;
    const int nv = cell ? (1 << dim) : dim + 1;
    const int fv = cell ? (1 << (dim - 1)) : dim;
    const int64_t total = C * nf;
    face_seed* seeds = (face_seed*)malloc(sizeof(face_seed) * (size_t)total);
    for (int64_t K = 0; K < C; ++K)
        for (int e = 0; e < nf; ++e) {
            face_seed s;
            int c = 0;
            if (!cell) {
                for (int v = 0; v < nv; ++v)
                    if (v != e) s.v[c++] = cell_verts[K * nv + v];
            }
            else
                for (int v = 0; v < fv; ++v)
                    s.v[c++] = cell_verts[K * nv + (dim == 2 ? kRectFaces[e][v] : kCuboidFaces[e][v])];
            for (; c < 4; ++c) s.v[c] = -1;
            /* sort the fv vertex ids (insertion sort) */
            for (int x = 1; x < fv; ++x)
                for (int y = x; y > 0 && s.v[y - 1] > s.v[y]; --y) {
                    int32_t tmp = s.v[y]; s.v[y] = s.v[y - 1]; s.v[y - 1] = tmp;
                }
            s.slot = K * nf + e;
            seeds[K * nf + e] = s;
        }
    qsort(seeds, (size_t)total, sizeof(face_seed), seed_cmp);
    /* group equal seeds; the group's first slot (smallest) defines the order */
    int64_t* firsts = (int64_t*)malloc(sizeof(int64_t) * (size_t)total);
    int64_t nfaces = 0;
    for (int64_t k = 0; k < total; ++k) {
        if (k == 0 || memcmp(seeds[k].v, seeds[k - 1].v, sizeof(seeds[k].v)) != 0)
            firsts[nfaces++] = seeds[k].slot;
    }
    qsort(firsts, (size_t)nfaces, sizeof(int64_t), i64_cmp);
    /* slot -> face id for the first slots; walk groups again */
    int32_t* first_id = (int32_t*)malloc(sizeof(int32_t) * (size_t)total);
    for (int64_t k = 0; k < total; ++k) first_id[k] = -1;
    for (int64_t E = 0; E < nfaces; ++E) first_id[firsts[E]] = (int32_t)E;
    for (int64_t E = 0; E < nfaces; ++E) { face_cells[2 * E] = -1; face_cells[2 * E + 1] = -1; }
    int64_t g0 = 0;
    for (int64_t k = 0; k <= total; ++k) {
        if (k == total || (k > g0 && memcmp(seeds[k].v, seeds[g0].v, sizeof(seeds[k].v)) != 0)) {
            const int32_t E = first_id[seeds[g0].slot];
            int nc = 0;
            for (int64_t q = g0; q < k; ++q) {
                const int64_t slot = seeds[q].slot;
                cell_faces[slot] = E;
                if (nc < 2) face_cells[2 * E + nc] = (int32_t)(slot / nf);
                ++nc;
            }
            for (int d = 0; d < fv; ++d) face_verts[(int64_t)E * fv + d] = seeds[g0].v[d];
            g0 = k;
        }
    }
    free(first_id);
    free(firsts);
    free(seeds);
    return nfaces;
}

/* ------------------------------------------------------------------ */
/* Geometry (TNL getEntityMeasure, restated) */

static void vsub(const double* a, const double* b, double* out, int dim)
{
    for (int d = 0; d < dim; ++d) out[d] = a[d] - b[d];
}

static double vdot(const double* a, const double* b, int dim)
{
    double s = 0;
    for (int d = 0; d < dim; ++d) s += a[d] * b[d];
    return s;
}

static double simplex_measure(const double* const* P, int k, int dim)
{
    /* measure of the k-simplex P[0..k] embedded in dim dimensions */
    double e1[3], e2[3], e3[3];
    if (k == 1) { vsub(P[1], P[0], e1, dim); return sqrt(vdot(e1, e1, dim)); }
    if (k == 2) {
        vsub(P[1], P[0], e1, dim); vsub(P[2], P[0], e2, dim);
        if (dim == 2) return 0.5 * fabs(e1[0] * e2[1] - e1[1] * e2[0]);
        const double cx = e1[1] * e2[2] - e1[2] * e2[1];
        const double cy = e1[2] * e2[0] - e1[0] * e2[2];
        const double cz = e1[0] * e2[1] - e1[1] * e2[0];
        return 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
    }
    vsub(P[1], P[0], e1, dim); vsub(P[2], P[0], e2, dim); vsub(P[3], P[0], e3, dim);
    const double det = e1[0] * (e2[1] * e3[2] - e2[2] * e3[1])
                     - e1[1] * (e2[0] * e3[2] - e2[2] * e3[0])
                     + e1[2] * (e2[0] * e3[1] - e2[1] * e3[0]);
    return fabs(det) / 6.0;
}

/* side lengths h_x, h_y (, h_z) of a box cell: the lowest corner v0 to the
 * opposite corner (v2 of a rectangle, v6 of a cuboid), MassMatrix.h:178-184,
 * 346-353 */
static void box_sides(const orc_problem* p, int64_t K, double* h)
{
    const double* v0 = p->coords + (int64_t)p->cell_verts[K * p->nv] * p->dim;
    const double* vd = p->coords + (int64_t)p->cell_verts[K * p->nv + (p->dim == 2 ? 2 : 6)] * p->dim;
    for (int d = 0; d < p->dim; ++d) h[d] = vd[d] - v0[d];
}

double orc_cell_measure(const orc_problem* p, int64_t K)
{
    if (p->cell) {
        double h[3];
        box_sides(p, K, h);
        double m = 1;
        for (int d = 0; d < p->dim; ++d) m *= h[d];
        return fabs(m);
    }
    const double* P[4];
    for (int v = 0; v < p->nv; ++v) P[v] = p->coords + (int64_t)p->cell_verts[K * p->nv + v] * p->dim;
    return simplex_measure(P, p->dim, p->dim);
}

double orc_face_measure(const orc_problem* p, int64_t E, const int32_t* face_verts)
{
    if (p->cell && p->dim == 3) {
        /* an axis-aligned rectangle: the product of its two nonzero extents */
        double lo[3], hi[3];
        for (int d = 0; d < 3; ++d) { lo[d] = 1e300; hi[d] = -1e300; }
        for (int v = 0; v < 4; ++v) {
            const double* X = p->coords + (int64_t)face_verts[E * 4 + v] * 3;
            for (int d = 0; d < 3; ++d) { lo[d] = fmin(lo[d], X[d]); hi[d] = fmax(hi[d], X[d]); }
        }
        double ext[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
        int dmin = 0;
        for (int d = 1; d < 3; ++d) if (ext[d] < ext[dmin]) dmin = d;
        double m = 1;
        for (int d = 0; d < 3; ++d) if (d != dmin) m *= ext[d];
        return m;
    }
    const double* P[3];
    for (int v = 0; v < p->fv; ++v) P[v] = p->coords + (int64_t)face_verts[E * p->fv + v] * p->dim;
    return simplex_measure(P, p->fv - 1, p->dim);
}

/* ------------------------------------------------------------------ */
/* Dense LU without pivoting (restated TNL LU_sequential_factorize/solve) */

static void lu_factorize(double* A, int N)
{
    /* Doolittle: A = L U, L unit lower triangular, stored in place */
    for (int k = 0; k < N; ++k) {
        for (int j = k; j < N; ++j) {
            double s = A[k * N + j];
            for (int q = 0; q < k; ++q) s -= A[k * N + q] * A[q * N + j];
            A[k * N + j] = s;
        }
        for (int i = k + 1; i < N; ++i) {
            double s = A[i * N + k];
            for (int q = 0; q < k; ++q) s -= A[i * N + q] * A[q * N + k];
            A[i * N + k] = s / A[k * N + k];
        }
    }
}

static void lu_solve(const double* A, int N, double* x)
{
    for (int i = 1; i < N; ++i) {
        double s = x[i];
        for (int q = 0; q < i; ++q) s -= A[i * N + q] * x[q];
        x[i] = s;
    }
    for (int i = N - 1; i >= 0; --i) {
        double s = x[i];
        for (int q = i + 1; q < N; ++q) s -= A[i * N + q] * x[q];
        x[i] = s / A[i * N + i];
    }
}

/* ------------------------------------------------------------------ */
/* Local RT0 mass matrix (MassMatrix.h:511-1050) */

static void mass_matrix_local(const orc_problem* p, int64_t K, double* M /* nf x nf */)
{
    const int dim = p->dim;
    const double* X[4];
    for (int v = 0; v < p->nv; ++v) X[v] = p->coords + (int64_t)p->cell_verts[K * p->nv + v] * dim;
    const double meas = orc_cell_measure(p, K);
    if (dim == 2 && !p->lumping) {
        /* MassMatrix.h:538-569 */
        double P0[3], P1[3];
        vsub(X[0], X[2], P0, dim); vsub(X[1], X[2], P1, dim);
        const double P00 = vdot(P0, P0, dim), P01 = vdot(P0, P1, dim), P11 = vdot(P1, P1, dim);
        const double den = 24 * meas;
        M[0 * 3 + 0] = (3 * P00 + P11 - 3 * P01) / den;
        M[1 * 3 + 1] = (P00 + 3 * P11 - 3 * P01) / den;
        M[2 * 3 + 2] = (P00 + P11 + P01) / den;
        M[0 * 3 + 1] = (3 * P01 - P00 - P11) / den;
        M[0 * 3 + 2] = (P11 - P00 - P01) / den;
        M[1 * 3 + 2] = (P00 - P11 - P01) / den;
    }
    else if (dim == 2) {
        /* MassMatrix.h:661-692 */
        double P01[3], P02[3], P12[3];
        vsub(X[0], X[1], P01, dim); vsub(X[0], X[2], P02, dim); vsub(X[1], X[2], P12, dim);
        const double a = vdot(P01, P01, dim), b = vdot(P02, P02, dim), c = vdot(P12, P12, dim);
        const double ab = vdot(P01, P02, dim), ac = vdot(P01, P12, dim), bc = vdot(P02, P12, dim);
        const double den = 12 * meas;
        M[0 * 3 + 0] = (a + b) / den;
        M[1 * 3 + 1] = (a + c) / den;
        M[2 * 3 + 2] = (b + c) / den;
        M[0 * 3 + 1] = (bc) / den;
        M[0 * 3 + 2] = (-ac) / den;
        M[1 * 3 + 2] = (ab) / den;
    }
    else if (!p->lumping) {
        /* MassMatrix.h:787-825 */
        double P0[3], P1[3], P2[3];
        vsub(X[0], X[3], P0, dim); vsub(X[1], X[3], P1, dim); vsub(X[2], X[3], P2, dim);
        const double P00 = vdot(P0, P0, dim), P11 = vdot(P1, P1, dim), P22 = vdot(P2, P2, dim);
        const double P01 = vdot(P0, P1, dim), P02 = vdot(P0, P2, dim), P12 = vdot(P1, P2, dim);
        const double den = 180 * meas;
        M[0 * 4 + 0] = (12 * P00 + 2 * P11 + 2 * P22 - 8 * P01 - 8 * P02 + 2 * P12) / den;
        M[1 * 4 + 1] = (2 * P00 + 12 * P11 + 2 * P22 - 8 * P01 + 2 * P02 - 8 * P12) / den;
        M[2 * 4 + 2] = (2 * P00 + 2 * P11 + 12 * P22 + 2 * P01 - 8 * P02 - 8 * P12) / den;
        M[3 * 4 + 3] = 2 * (P00 + P11 + P22 + P01 + P02 + P12) / den;
        M[0 * 4 + 1] = (-3 * P00 - 3 * P11 + 2 * P22 + 12 * P01 - 3 * P02 - 3 * P12) / den;
        M[0 * 4 + 2] = (-3 * P00 + 2 * P11 - 3 * P22 - 3 * P01 + 12 * P02 - 3 * P12) / den;
        M[1 * 4 + 2] = (2 * P00 - 3 * P11 - 3 * P22 - 3 * P01 - 3 * P02 + 12 * P12) / den;
        M[0 * 4 + 3] = (-3 * P00 + 2 * P11 + 2 * P22 - 3 * P01 - 3 * P02 + 2 * P12) / den;
        M[1 * 4 + 3] = (2 * P00 - 3 * P11 + 2 * P22 - 3 * P01 + 2 * P02 - 3 * P12) / den;
        M[2 * 4 + 3] = (2 * P00 + 2 * P11 - 3 * P22 + 2 * P01 - 3 * P02 - 3 * P12) / den;
    }
    else {
        /* MassMatrix.h:932-962 */
        double P01[3], P02[3], P03[3], P12[3], P13[3], P23[3];
        vsub(X[0], X[1], P01, dim); vsub(X[0], X[2], P02, dim); vsub(X[0], X[3], P03, dim);
        vsub(X[1], X[2], P12, dim); vsub(X[1], X[3], P13, dim); vsub(X[2], X[3], P23, dim);
        const double den = 36 * meas;
        M[0 * 4 + 0] = (vdot(P01, P01, 3) + vdot(P02, P02, 3) + vdot(P03, P03, 3)) / den;
        M[1 * 4 + 1] = (vdot(P01, P01, 3) + vdot(P12, P12, 3) + vdot(P13, P13, 3)) / den;
        M[2 * 4 + 2] = (vdot(P02, P02, 3) + vdot(P12, P12, 3) + vdot(P23, P23, 3)) / den;
        M[3 * 4 + 3] = (vdot(P03, P03, 3) + vdot(P13, P13, 3) + vdot(P23, P23, 3)) / den;
        M[0 * 4 + 1] = (vdot(P02, P12, 3) + vdot(P03, P13, 3)) / den;
        M[0 * 4 + 2] = (-vdot(P01, P12, 3) + vdot(P03, P23, 3)) / den;
        M[0 * 4 + 3] = (-vdot(P01, P13, 3) - vdot(P02, P23, 3)) / den;
        M[1 * 4 + 2] = (vdot(P01, P02, 3) + vdot(P13, P23, 3)) / den;
        M[1 * 4 + 3] = (vdot(P01, P03, 3) - vdot(P12, P23, 3)) / den;
        M[2 * 4 + 3] = (vdot(P02, P03, 3) + vdot(P12, P13, 3)) / den;
    }
    const int nf = p->nf;
    for (int i = 0; i < nf; ++i)
        for (int j = 0; j < i; ++j) M[i * nf + j] = M[j * nf + i];
}

/* orientation class of local face e of a box cell, the storage slot s of
 * its value: rectangle e % 2 (horizontal 0, 2 -> 0; vertical 1, 3 -> 1),
 * cuboid n_x (2, 4) -> 0, n_y (1, 3) -> 1, n_z (0, 5) -> 2
 * (MassMatrix.h:216-227, 392-403) */
static inline int box_class(int dim, int e)
{
    if (dim == 2) return e % 2;
    return (e == 2 || e == 4) ? 0 : (e == 1 || e == 3) ? 1 : 2;
}

void orc_update_b(orc_problem* p)
{
    const int nf = p->nf, n = p->n, S = p->S;
    if (p->cell) {
        /* MassMatrix::update for rectangles (MassMatrix.h:171-186, 249-264) and
         * cuboids (340-362, 424-446): the same values with and without lumping */
#pragma omp parallel for schedule(static)
        for (int64_t K = 0; K < p->C; ++K) {
            double h[3];
            box_sides(p, K, h);
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) {
                    const double D = cget(p->D, IDX_ijK(p, i, j, K));
                    if (p->dim == 2) {
                        p->b[IDX_ijsK(p, i, j, 0, K)] = 2 * D * h[0] / h[1];
                        p->b[IDX_ijsK(p, i, j, 1, K)] = 2 * D * h[1] / h[0];
                    }
                    else {
                        p->b[IDX_ijsK(p, i, j, 0, K)] = 2 * D * h[1] * h[2] / h[0];
                        p->b[IDX_ijsK(p, i, j, 1, K)] = 2 * D * h[0] * h[2] / h[1];
                        p->b[IDX_ijsK(p, i, j, 2, K)] = 2 * D * h[0] * h[1] / h[2];
                    }
                }
        }
        return;
    }
#pragma omp parallel for schedule(static)
    for (int64_t K = 0; K < p->C; ++K) {
        double M[MAXF * MAXF];
        mass_matrix_local(p, K, M);
        lu_factorize(M, nf);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                const double D = cget(p->D, IDX_ijK(p, i, j, K));
                /* packed upper triangle, column by column (MassMatrix.h:571-592) */
                for (int col = 0; col < nf; ++col) {
                    double v[MAXF] = {0, 0, 0, 0, 0, 0};
                    v[col] = 1.0;
                    lu_solve(M, nf, v);
                    for (int row = 0; row <= col; ++row)
                        p->b[IDX_ijsK(p, i, j, col * (col + 1) / 2 + row, K)] = v[row] * D;
                }
                /* row sums (MassMatrix.h:594-597) */
                for (int e = 0; e < nf; ++e) {
                    double s = 0;
                    for (int f = 0; f < nf; ++f) {
                        const int lo = e < f ? e : f, hi = e < f ? f : e;
                        s += p->b[IDX_ijsK(p, i, j, lo + hi * (hi + 1) / 2, K)];
                    }
                    p->b[IDX_ijsK(p, i, j, S - nf + e, K)] = s;
                }
            }
    }
}

/* MassMatrix::b_ijKef / b_ijKe: simplices MassMatrix.h:600-631; boxes
 * 188-227 (rectangle, lumped: diagonal), 268-319 (rectangle: 2s on the
 * diagonal, s between the two faces of one orientation, row sum 3s),
 * 364-403 and 448-507 (cuboid, the same with three orientations) */
static inline double b_ef(const orc_problem* p, int i, int j, int64_t K, int e, int f)
{
    if (p->cell) {
        const int ce = box_class(p->dim, e), cf = box_class(p->dim, f);
        if (p->lumping) return e == f ? p->b[IDX_ijsK(p, i, j, ce, K)] : 0.0;
        if (ce != cf) return 0.0;
        const double s = p->b[IDX_ijsK(p, i, j, ce, K)];
        return e == f ? 2 * s : s;
    }
    if (e > f) { int t = e; e = f; f = t; }
    return p->b[IDX_ijsK(p, i, j, e + f * (f + 1) / 2, K)];
}

static inline double b_e(const orc_problem* p, int i, int j, int64_t K, int e)
{
    if (p->cell) {
        const double s = p->b[IDX_ijsK(p, i, j, box_class(p->dim, e), K)];
        return p->lumping ? s : 3 * s;
    }
    return p->b[IDX_ijsK(p, i, j, p->S - p->nf + e, K)];
}

static inline int local_index(const int32_t* faces, int nf, int32_t E)
{
    for (int e = 0; e < nf; ++e)
        if (faces[e] == E) return e;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Initial face average (Solver.hpp:319-339) */

void orc_face_average(orc_problem* p)
{
#pragma omp parallel for schedule(static)
    for (int64_t E = 0; E < p->F; ++E)
        for (int i = 0; i < p->n; ++i) {
            const int32_t K0 = p->face_cells[2 * E], K1 = p->face_cells[2 * E + 1];
            if (K1 < 0) p->Z_iF[IDX_Fi(p, E, i)] = p->Z_iK[IDX_iK(p, i, K0)];
            else p->Z_iF[IDX_Fi(p, E, i)] = 0.5 * (p->Z_iK[IDX_iK(p, i, K0)] + p->Z_iK[IDX_iK(p, i, K1)]);
        }
    if (p->v_iKe) memset(p->v_iKe, 0, sizeof(double) * (size_t)(p->n * p->nf * p->C));
}

/* ------------------------------------------------------------------ */
/* Upwinding (Solver.hpp:663-769) */

void orc_upwind(orc_problem* p, double t, double tau)
{
    (void)t; (void)tau;
    const int n = p->n, nf = p->nf;
    if (p->mobility_upwind) {
#pragma omp parallel for schedule(static)
        for (int64_t E = 0; E < p->F; ++E)
            for (int i = 0; i < n; ++i) {
                const int32_t K1 = p->face_cells[2 * E], K2 = p->face_cells[2 * E + 1];
                const int e1 = local_index(p->cell_faces + (int64_t)K1 * nf, nf, (int32_t)E);
                double m;
                if (K2 < 0) {
                    int inflow = 0;
                    for (int j = 0; j < n; ++j)
                        if (p->v_iKe[IDX_ieK(p, j, e1, K1)] < 0) { inflow = 1; break; }
                    if (inflow) m = cget(p->m_bnd, IDX_iF(p, i, E));
                    else m = cget(p->m, IDX_iK(p, i, K1));
                }
                else {
                    const int e2 = local_index(p->cell_faces + (int64_t)K2 * nf, nf, (int32_t)E);
                    const double vel = p->v_iKe[IDX_ieK(p, i, e1, K1)] - p->v_iKe[IDX_ieK(p, i, e2, K2)];
                    if (vel == 0) m = 0.5 * (cget(p->m, IDX_iK(p, i, K1)) + cget(p->m, IDX_iK(p, i, K2)));
                    else if (vel > 0) m = cget(p->m, IDX_iK(p, i, K1));
                    else m = cget(p->m, IDX_iK(p, i, K2));
                }
                p->m_upw[IDX_Fi(p, E, i)] = m;
            }
    }
    if (p->advection == 0) {
#pragma omp parallel for schedule(static)
        for (int64_t E = 0; E < p->F; ++E)
            for (int j = 0; j < n; ++j)
                for (int i = 0; i < n; ++i) {
                    const int32_t K1 = p->face_cells[2 * E], K2 = p->face_cells[2 * E + 1];
                    const int e1 = local_index(p->cell_faces + (int64_t)K1 * nf, nf, (int32_t)E);
                    const double apu = cget(p->a, IDX_ijeK(p, i, j, e1, K1)) + cget(p->u, IDX_ijeK(p, i, j, e1, K1));
                    double z;
                    if (apu > 0.0) z = p->Z_iK[IDX_iK(p, j, K1)];
                    else if (apu == 0.0) z = 0;
                    else if (K2 >= 0) z = p->Z_iK[IDX_iK(p, j, K2)];
                    else z = p->Z_iF[IDX_Fi(p, E, j)];
                    p->Z_upw[IDX_Eji(p, E, j, i)] = z;
                }
    }
}

/* ------------------------------------------------------------------ */
/* R_ijKe, R_iK (SecondaryCoefficients.h:50-127; Solver.hpp:793-815) */

void orc_update_R(orc_problem* p, double tau)
{
    const int n = p->n, nf = p->nf;
#pragma omp parallel for schedule(static)
    for (int64_t K = 0; K < p->C; ++K) {
        const int32_t* faces = p->cell_faces + K * nf;
        const double measK = orc_cell_measure(p, K);
        for (int i = 0; i < n; ++i) {
            for (int j = 0; j < n; ++j)
                for (int e = 0; e < nf; ++e) {
                    double R = 0;
                    for (int f = 0; f < nf; ++f)
                        R += m_upw_get(p, i, faces[f]) * b_ef(p, i, j, K, f, e);
                    if (p->advection == 1) {
                        const double vel = cget(p->a, IDX_ijeK(p, i, j, e, K)) + cget(p->u, IDX_ijeK(p, i, j, e, K));
                        if (vel < 0) R -= 2 * vel;
                    }
                    if (p->advection == 2) {
                        const double vel = cget(p->a, IDX_ijeK(p, i, j, e, K)) + cget(p->u, IDX_ijeK(p, i, j, e, K));
                        R -= vel;
                    }
                    p->R_ijKe[IDX_ijeK(p, i, j, e, K)] = R;
                }
            double R = 0;
            for (int j = 0; j < n; ++j) R += cget(p->N, IDX_ijK(p, i, j, K)) * p->Z_iK[IDX_iK(p, j, K)];
            R *= measK / tau;
            R += measK * cget(p->f, IDX_iK(p, i, K));
            for (int e = 0; e < nf; ++e)
                R -= m_upw_get(p, i, faces[e]) * cget(p->w, IDX_ieK(p, i, e, K));
            if (p->advection == 0) {
                double aux = 0;
                for (int j = 0; j < n; ++j)
                    for (int e = 0; e < nf; ++e)
                        aux += (cget(p->a, IDX_ijeK(p, i, j, e, K)) + cget(p->u, IDX_ijeK(p, i, j, e, K)))
                               * p->Z_upw[IDX_Eji(p, faces[e], j, i)];
                R -= aux;
            }
            p->R_iK[IDX_iK(p, i, K)] = R;
        }
    }
}

/* Q_ijK, dummy equation for singular rows, LU, Q^{-1} R (Solver.hpp:817-871;
 * SecondaryCoefficients.h:129-159) */
void orc_update_Q(orc_problem* p, double tau)
{
    const int n = p->n, nf = p->nf;
#pragma omp parallel for schedule(static)
    for (int64_t K = 0; K < p->C; ++K) {
        const int32_t* faces = p->cell_faces + K * nf;
        const double measK = orc_cell_measure(p, K);
        double Q[MAXN * MAXN];
        for (int i = 0; i < n; ++i) {
            int singular = 1;
            for (int j = 0; j < n; ++j) {
                double q = 0;
                for (int e = 0; e < nf; ++e) {
                    q += m_upw_get(p, i, faces[e]) * b_e(p, i, j, K, e) - cget(p->u, IDX_ijeK(p, i, j, e, K));
                    if (p->advection == 1) {
                        const double vel = cget(p->a, IDX_ijeK(p, i, j, e, K)) + cget(p->u, IDX_ijeK(p, i, j, e, K));
                        if (vel >= 0) q += vel;
                        else q -= vel;
                    }
                }
                q += measK / tau * cget(p->N, IDX_ijK(p, i, j, K)) + measK * cget(p->r, IDX_ijK(p, i, j, K));
                Q[i * n + j] = q;
                if (q != 0.0) singular = 0;
            }
            if (singular) {
                Q[i * n + i] = 1.0;
                p->R_iK[IDX_iK(p, i, K)] += p->Z_iK[IDX_iK(p, i, K)];
            }
        }
        lu_factorize(Q, n);
        double rhs[MAXN];
        for (int i = 0; i < n; ++i) rhs[i] = p->R_iK[IDX_iK(p, i, K)];
        lu_solve(Q, n, rhs);
        for (int i = 0; i < n; ++i) p->R_iK[IDX_iK(p, i, K)] = rhs[i];
        for (int j = 0; j < n; ++j)
            for (int e = 0; e < nf; ++e) {
                for (int i = 0; i < n; ++i) rhs[i] = p->R_ijKe[IDX_ijeK(p, i, j, e, K)];
                lu_solve(Q, n, rhs);
                for (int i = 0; i < n; ++i) p->R_ijKe[IDX_ijeK(p, i, j, e, K)] = rhs[i];
            }
    }
}

/* ------------------------------------------------------------------ */
/* Local Schur entries and RHS terms (SecondaryCoefficients.h:187-349) */

static double A_no_adv(const orc_problem* p, int i, int j, int64_t K, int e, int f)
{
    double SQinvR = 0;
    for (int x = 0; x < p->n; ++x) SQinvR += b_e(p, i, x, K, e) * p->R_ijKe[IDX_ijeK(p, x, j, f, K)];
    return b_ef(p, i, j, K, e, f) - SQinvR;
}

static double A_adv(const orc_problem* p, int i, int j, int64_t K, int32_t E, int e, int32_t F, int f)
{
    const double m = m_upw_get(p, i, E);
    double SQinvR = 0;
    for (int x = 0; x < p->n; ++x) {
        double S = m * b_e(p, i, x, K, e);
        if (p->advection == 1) {
            const double vel = cget(p->a, IDX_ijeK(p, i, x, e, K)) + cget(p->u, IDX_ijeK(p, i, x, e, K));
            if (vel >= 0) S += vel;
            else S -= vel;
        }
        SQinvR += S * p->R_ijKe[IDX_ijeK(p, x, j, f, K)];
    }
    double T = m * b_ef(p, i, j, K, e, f);
    if (p->advection == 1 && E == F) {
        const double vel = cget(p->a, IDX_ijeK(p, i, j, e, K)) + cget(p->u, IDX_ijeK(p, i, j, e, K));
        if (vel < 0) T -= 2 * vel;
    }
    if (p->advection == 2 && E == F) {
        const double vel = cget(p->a, IDX_ijeK(p, i, j, e, K)) + cget(p->u, IDX_ijeK(p, i, j, e, K));
        T -= vel;
    }
    return T - SQinvR;
}

static double A_interior(const orc_problem* p, int i, int j, int64_t K, int32_t E, int e, int32_t F, int f)
{
    if (p->advection == 0) return A_no_adv(p, i, j, K, e, f);
    return A_adv(p, i, j, K, E, e, F, f);
}

static double RHS_no_adv(const orc_problem* p, int i, int64_t K, int e)
{
    double value = cget(p->w, IDX_ieK(p, i, e, K));
    for (int j = 0; j < p->n; ++j) value += b_e(p, i, j, K, e) * p->R_iK[IDX_iK(p, j, K)];
    return value;
}

static double RHS_adv(const orc_problem* p, int i, int64_t K, int32_t E, int e)
{
    const double m = m_upw_get(p, i, E);
    double value = m * cget(p->w, IDX_ieK(p, i, e, K));
    for (int j = 0; j < p->n; ++j) {
        double S = m * b_e(p, i, j, K, e);
        const double vel = cget(p->a, IDX_ijeK(p, i, j, e, K)) + cget(p->u, IDX_ijeK(p, i, j, e, K));
        if (p->advection == 1) {
            if (vel >= 0) S += vel;
            else S -= vel;
        }
        value += S * p->R_iK[IDX_iK(p, j, K)];
        if (p->advection == 0) value += p->Z_upw[IDX_Eji(p, E, j, i)] * vel;
    }
    return value;
}

static double RHS_interior(const orc_problem* p, int i, int64_t K, int32_t E, int e)
{
    if (p->advection == 0) return RHS_no_adv(p, i, K, e);
    return RHS_adv(p, i, K, E, e);
}

/* boundary coefficient sets (BoundaryConditions.hpp:11-130) */
static double A_bc(const orc_problem* p, int tag, int i, int j, int64_t K, int32_t E, int e, int32_t F, int f)
{
    if (tag == 1) return A_adv(p, i, j, K, E, e, F, f);
    if (tag == 3) return A_no_adv(p, i, j, K, e, f);
    /* AdvectiveOutflow (tag 2) */
    const double vel = cget(p->a, IDX_ijeK(p, i, i, e, K)) + cget(p->u, IDX_ijeK(p, i, i, e, K));
    if (vel >= 0) return A_no_adv(p, i, j, K, e, f);
    if (i == j && E == F) return 1;
    return 0;
}

static double RHS_bc(const orc_problem* p, int tag, int i, int64_t K, int32_t E, int e)
{
    if (tag == 1) return RHS_adv(p, i, K, E, e);
    if (tag == 3) return RHS_no_adv(p, i, K, e);
    const double vel = cget(p->a, IDX_ijeK(p, i, i, e, K)) + cget(p->u, IDX_ijeK(p, i, i, e, K));
    if (vel >= 0) return RHS_no_adv(p, i, K, e);
    return p->Z_iK[IDX_iK(p, i, K)];
}

/* ------------------------------------------------------------------ */
/* Row lengths (LinearSystem.h:26-34; BoundaryConditions.hpp:283-299) */

void orc_row_lengths(const orc_problem* p, int32_t* rowlen)
{
    const int n = p->n, nf = p->nf;
#pragma omp parallel for schedule(static)
    for (int64_t E = 0; E < p->F; ++E)
        for (int i = 0; i < n; ++i) {
            int32_t len;
            if (p->face_cells[2 * E + 1] < 0) {
                const int tag = p->bc_tags[IDX_iF(p, i, E)];
                len = (tag == 0) ? 1 : nf * n;
            }
            else len = (2 * nf - 1) * n;
            rowlen[E * n + i] = len;
        }
}

static void sort_local(const int32_t* faces, int nf, int* perm)
{
    /* bubble sort of local indices by global face index (LinearSystem.h:121-136) */
    for (int j = 0; j < nf; ++j) perm[j] = j;
    for (int k1 = nf - 1; k1 > 0; --k1)
        for (int k2 = 0; k2 < k1; ++k2)
            if (!(faces[perm[k2]] < faces[perm[k2 + 1]])) {
                int t = perm[k2]; perm[k2] = perm[k2 + 1]; perm[k2 + 1] = t;
            }
}

/* Assembly of the face-trace system (Solver.hpp:934-958; LinearSystem.h:66-256;
 * RightHandSide.h:18-45; BoundaryConditions.hpp:132-222, 335-508) */
int orc_assemble(const orc_problem* p, const int32_t* face_verts, double t, double tau,
                 const int64_t* rowptr, int32_t* cols, double* vals, double* rhs)
{
    (void)t; (void)tau;
    const int n = p->n, nf = p->nf;
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(|:bad)
    for (int64_t E = 0; E < p->F; ++E)
        for (int i = 0; i < n; ++i) {
            const int64_t row = E * n + i;
            int64_t pos = rowptr[row];
            const int32_t K0 = p->face_cells[2 * E], K1 = p->face_cells[2 * E + 1];
            if (K1 < 0) {
                const int tag = p->bc_tags[IDX_iF(p, i, E)];
                if (tag == 0) {
                    cols[pos] = (int32_t)row;
                    vals[pos] = 1.0;
                    rhs[row] = p->bc_dirichlet[IDX_iF(p, i, E)];
                    continue;
                }
                const int32_t* faces = p->cell_faces + (int64_t)K0 * nf;
                const int e = local_index(faces, nf, (int32_t)E);
                int perm[MAXF];
                sort_local(faces, nf, perm);
                const double diag = A_bc(p, tag, i, i, K0, (int32_t)E, e, (int32_t)E, e);
                if (!(diag > 0)) bad = 1;
                for (int g = 0; g < nf; ++g) {
                    const int f = perm[g];
                    for (int j = 0; j < n; ++j) {
                        cols[pos] = faces[f] * n + j;
                        if (j == i && faces[f] == E) vals[pos] = 1.0;
                        else vals[pos] = A_bc(p, tag, i, j, K0, (int32_t)E, e, faces[f], f) / diag;
                        ++pos;
                    }
                }
                /* Neumann value times the face measure; zero diffusive flux for outflow */
                double bval = 0;
                if (tag != 2)
                    bval = -p->bc_values[IDX_iF(p, i, E)] * orc_face_measure(p, E, face_verts);
                bval += RHS_bc(p, tag, i, K0, (int32_t)E, e);
                rhs[row] = bval / diag;
                continue;
            }
            /* interior row */
            const int32_t* fK0 = p->cell_faces + (int64_t)K0 * nf;
            const int32_t* fK1 = p->cell_faces + (int64_t)K1 * nf;
            int p0[MAXF], p1[MAXF];
            sort_local(fK0, nf, p0);
            sort_local(fK1, nf, p1);
            const int e0 = local_index(fK0, nf, (int32_t)E);
            const int e1 = local_index(fK1, nf, (int32_t)E);
            const double diag = A_interior(p, i, i, K0, (int32_t)E, e0, (int32_t)E, e0)
                              + A_interior(p, i, i, K1, (int32_t)E, e1, (int32_t)E, e1);
            if (!(diag > 0)) bad = 1;
            int g0 = 0, g1 = 0;
            while (g0 < nf && g1 < nf) {
                const int f0 = p0[g0], f1 = p1[g1];
                if (fK0[f0] < fK1[f1]) {
                    for (int j = 0; j < n; ++j) {
                        cols[pos] = fK0[f0] * n + j;
                        vals[pos] = A_interior(p, i, j, K0, (int32_t)E, e0, fK0[f0], f0) / diag;
                        ++pos;
                    }
                    ++g0;
                }
                else if (fK0[f0] == fK1[f1]) {
                    for (int j = 0; j < n; ++j) {
                        cols[pos] = fK0[f0] * n + j;
                        if (j == i) vals[pos] = 1.0;
                        else vals[pos] = (A_interior(p, i, j, K0, (int32_t)E, e0, fK0[f0], f0)
                                        + A_interior(p, i, j, K1, (int32_t)E, e1, fK1[f1], f1)) / diag;
                        ++pos;
                    }
                    ++g0; ++g1;
                }
                else {
                    for (int j = 0; j < n; ++j) {
                        cols[pos] = fK1[f1] * n + j;
                        vals[pos] = A_interior(p, i, j, K1, (int32_t)E, e1, fK1[f1], f1) / diag;
                        ++pos;
                    }
                    ++g1;
                }
            }
            while (g0 < nf) {
                const int f0 = p0[g0];
                for (int j = 0; j < n; ++j) {
                    cols[pos] = fK0[f0] * n + j;
                    vals[pos] = A_interior(p, i, j, K0, (int32_t)E, e0, fK0[f0], f0) / diag;
                    ++pos;
                }
                ++g0;
            }
            while (g1 < nf) {
                const int f1 = p1[g1];
                for (int j = 0; j < n; ++j) {
                    cols[pos] = fK1[f1] * n + j;
                    vals[pos] = A_interior(p, i, j, K1, (int32_t)E, e1, fK1[f1], f1) / diag;
                    ++pos;
                }
                ++g1;
            }
            rhs[row] = (RHS_interior(p, i, K0, (int32_t)E, e0) + RHS_interior(p, i, K1, (int32_t)E, e1)) / diag;
        }
    return bad ? 1 : 0;
}

/* ------------------------------------------------------------------ */
/* BiCGStab (van der Vorst), identity preconditioner.  When the shadow
 * residual becomes (numerically) orthogonal to the residual, the iteration
 * restarts from the current residual. */
#define BICG_RESTART_EPS 1e-14

static void spmv(int64_t rows, const int64_t* rowptr, const int32_t* cols, const double* vals,
                 const double* x, double* y)
{
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < rows; ++r) {
        double s = 0;
        for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) s += vals[k] * x[cols[k]];
        y[r] = s;
    }
}

static double dot(int64_t rows, const double* a, const double* b)
{
    double s = 0;
#pragma omp parallel for schedule(static) reduction(+:s)
    for (int64_t r = 0; r < rows; ++r) s += a[r] * b[r];
    return s;
}

int orc_bicgstab(int64_t rows, const int64_t* rowptr, const int32_t* cols, const double* vals,
                 const double* rhs, double* x, double tol, int max_iter,
                 int* iters, double* residual)
{
    double* r = (double*)malloc(sizeof(double) * (size_t)rows * 6);
    double* rh = r + rows;
    double* pv = rh + rows;
    double* v = pv + rows;
    double* s = v + rows;
    double* tv = s + rows;
    int status = 1, it = 0;
    double bnorm = sqrt(dot(rows, rhs, rhs));
    if (bnorm == 0) bnorm = 1;
    spmv(rows, rowptr, cols, vals, x, v);
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < rows; ++q) { r[q] = rhs[q] - v[q]; rh[q] = r[q]; pv[q] = r[q]; }
    double rho = dot(rows, rh, r);
    double res = sqrt(rho) / bnorm;
    double rhnorm = sqrt(rho);
    if (res < tol) { status = 0; goto done; }
    for (it = 1; it <= max_iter; ++it) {
        spmv(rows, rowptr, cols, vals, pv, v);
        const double rv = dot(rows, rh, v);
        if (rv == 0) { status = 2; break; }
        const double alpha = rho / rv;
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < rows; ++q) s[q] = r[q] - alpha * v[q];
        const double snorm = sqrt(dot(rows, s, s)) / bnorm;
        if (snorm < tol) {
#pragma omp parallel for schedule(static)
            for (int64_t q = 0; q < rows; ++q) x[q] += alpha * pv[q];
            res = snorm;
            status = 0;
            break;
        }
        spmv(rows, rowptr, cols, vals, s, tv);
        const double ts = dot(rows, tv, s), tt = dot(rows, tv, tv);
        if (tt == 0) { status = 2; break; }
        const double omega = ts / tt;
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < rows; ++q) {
            x[q] += alpha * pv[q] + omega * s[q];
            r[q] = s[q] - omega * tv[q];
        }
        const double rr = dot(rows, r, r);
        res = sqrt(rr) / bnorm;
        if (res < tol) { status = 0; break; }
        if (it >= max_iter) break;
        const double rho_new = dot(rows, rh, r);
        if (omega == 0) { status = 2; break; }
        if (fabs(rho_new) <= BICG_RESTART_EPS * sqrt(rr) * rhnorm) {
            /* loss of bi-orthogonality (e.g. a residual supported on rows
             * orthogonal to the shadow residual): restart with r^ = p = r */
#pragma omp parallel for schedule(static)
            for (int64_t q = 0; q < rows; ++q) { rh[q] = r[q]; pv[q] = r[q]; }
            rho = rr;
            rhnorm = sqrt(rr);
            continue;
        }
        const double beta = (rho_new / rho) * (alpha / omega);
        rho = rho_new;
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < rows; ++q) pv[q] = r[q] + beta * (pv[q] - omega * v[q]);
    }
    if (it > max_iter) it = max_iter;
done:
    *iters = it;
    *residual = res;
    free(r);
    return status;
}

/* ------------------------------------------------------------------ */
/* Reconstruction (Solver.hpp:1283-1313; SecondaryCoefficients.h:16-48, 161-185) */

void orc_reconstruct(orc_problem* p)
{
    const int n = p->n, nf = p->nf;
#pragma omp parallel for schedule(static)
    for (int64_t K = 0; K < p->C; ++K) {
        const int32_t* faces = p->cell_faces + K * nf;
        for (int i = 0; i < n; ++i) {
            double Z = 0;
            for (int f = 0; f < nf; ++f)
                for (int j = 0; j < n; ++j)
                    Z += p->R_ijKe[IDX_ijeK(p, i, j, f, K)] * p->Z_iF[IDX_Fi(p, faces[f], j)];
            Z += p->R_iK[IDX_iK(p, i, K)];
            p->Z_iK[IDX_iK(p, i, K)] = Z;
        }
    }
}

void orc_velocities(orc_problem* p)
{
    const int n = p->n, nf = p->nf;
#pragma omp parallel for schedule(static)
    for (int64_t K = 0; K < p->C; ++K) {
        const int32_t* faces = p->cell_faces + K * nf;
        for (int i = 0; i < n; ++i)
            for (int e = 0; e < nf; ++e) {
                double sum_K = 0, sum_E = 0;
                for (int j = 0; j < n; ++j) {
                    const double b = b_e(p, i, j, K, e);
                    sum_K += b * p->Z_iK[IDX_iK(p, j, K)];
                    for (int f = 0; f < nf; ++f)
                        sum_E += b_ef(p, i, j, K, e, f) * p->Z_iF[IDX_Fi(p, faces[f], j)];
                }
                p->v_iKe[IDX_ieK(p, i, e, K)] = sum_K - sum_E + cget(p->w, IDX_ieK(p, i, e, K));
            }
    }
}

/* ------------------------------------------------------------------ */

int orc_step(orc_problem* p, const int32_t* face_verts, double t, double tau,
             const int64_t* rowptr, int32_t* cols, double* vals, double* rhs,
             double tol, int max_iter, int* iters, double* residual)
{
    /* preIterate (Solver.hpp:596-892) */
    orc_update_b(p);
    orc_upwind(p, t, tau);
    orc_update_R(p, tau);
    orc_update_Q(p, tau);
    /* assembleLinearSystem with the BC time t + tau (Solver.hpp:899-962) */
    if (orc_assemble(p, face_verts, t + tau, tau, rowptr, cols, vals, rhs) != 0) return 3;
    /* solveLinearSystem: warm start from the previous Z_iF (Solver.hpp:1247-1255) */
    const int64_t rows = p->F * p->n;
    const int st = orc_bicgstab(rows, rowptr, cols, vals, rhs, p->Z_iF, tol, max_iter, iters, residual);
    if (st != 0) return st;
    /* postIterate (Solver.hpp:1268-1324) */
    orc_reconstruct(p);
    if (p->mobility_upwind) orc_velocities(p);
    return 0;
}
