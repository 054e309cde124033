// Host-side topology builder and face-system pattern (setup, not per step).
#include "topology.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace mhfem {

namespace {

double simplex_measure(const double* const* P, int k, int dim)
{
    double e1[3] = {0, 0, 0}, e2[3] = {0, 0, 0}, e3[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) e1[d] = P[1][d] - P[0][d];
    if (k == 1) return std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    for (int d = 0; d < dim; ++d) e2[d] = P[2][d] - P[0][d];
    if (k == 2) {
        if (dim == 2) return 0.5 * std::fabs(e1[0] * e2[1] - e1[1] * e2[0]);
        const double cx = e1[1] * e2[2] - e1[2] * e2[1];
        const double cy = e1[2] * e2[0] - e1[0] * e2[2];
        const double cz = e1[0] * e2[1] - e1[1] * e2[0];
        return 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
    }
    for (int d = 0; d < dim; ++d) e3[d] = P[3][d] - P[0][d];
    const double det = e1[0] * (e2[1] * e3[2] - e2[2] * e3[1]) - e1[1] * (e2[0] * e3[2] - e2[2] * e3[0])
                     + e1[2] * (e2[0] * e3[1] - e2[1] * e3[0]);
    return std::fabs(det) / 6.0;
}

// local vertices of the faces of a rectangle / cuboid (TNL Quadrangle and
// Hexahedron subentity topologies)
const int kRectFaces[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
const int kCuboidFaces[6][4] = {{0, 1, 2, 3}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};

// an axis-parallel rectangle in 3D given by its four corners: the product of
// its two nonzero extents
double box_face_measure(const double* const* P)
{
    double lo[3], hi[3];
    for (int d = 0; d < 3; ++d) lo[d] = hi[d] = P[0][d];
    for (int v = 1; v < 4; ++v)
        for (int d = 0; d < 3; ++d) {
            lo[d] = std::min(lo[d], P[v][d]);
            hi[d] = std::max(hi[d], P[v][d]);
        }
    const double ext[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    int dmin = 0;
    for (int d = 1; d < 3; ++d)
        if (ext[d] < ext[dmin]) dmin = d;
    double m = 1;
    for (int d = 0; d < 3; ++d)
        if (d != dmin) m *= ext[d];
    return m;
}

struct Key {
    int32_t b, c, d;
    int32_t slot;
};

}  // namespace

std::string build_topology(int dim, int cell, int64_t V, const double* coords, int64_t C,
                           const int32_t* cell_verts, HostTopology& T)
{
    if (dim != 2 && dim != 3) return "dim must be 2 or 3";
    if (cell != 0 && cell != 1) return "cell type must be 0 (simplices) or 1 (boxes)";
    const int nf = cell ? 2 * dim : dim + 1;
    const int nv = cell ? (1 << dim) : dim + 1;
    const int fv = cell ? (1 << (dim - 1)) : dim;
    const int64_t N = C * nf;
    if (N >= (int64_t)INT32_MAX) return "mesh too large for int32 face slots";
    for (int64_t q = 0; q < C * nv; ++q)
        if (cell_verts[q] < 0 || cell_verts[q] >= V) return "cell vertex index out of range";

    T = HostTopology();
    T.dim = dim;
    T.cell = cell;
    T.nf = nf;
    T.nv = nv;
    T.fv = fv;
    T.V = V;
    T.C = C;

    // 1. sorted vertex tuple of every (cell, local face) slot; bucket by its smallest vertex
    std::vector<int32_t> fa(N), fb(N), fc(N), fd(N);
#pragma omp parallel for schedule(static)
    for (int64_t K = 0; K < C; ++K)
        for (int e = 0; e < nf; ++e) {
            int32_t v[4] = {-1, -1, -1, -1};
            if (!cell) {
                int c = 0;
                for (int q = 0; q < nv; ++q)
                    if (q != e) v[c++] = cell_verts[K * nv + q];
            }
            else
                for (int q = 0; q < fv; ++q) v[q] = cell_verts[K * nv + (dim == 2 ? kRectFaces[e][q] : kCuboidFaces[e][q])];
            for (int x = 1; x < fv; ++x)
                for (int y = x; y > 0 && v[y - 1] > v[y]; --y) std::swap(v[y - 1], v[y]);
            const int64_t s = K * nf + e;
            fa[s] = v[0];
            fb[s] = v[1];
            fc[s] = v[2];
            fd[s] = v[3];
            for (int x = 1; x < fv; ++x)
                if (v[x] == v[x - 1]) fa[s] = -2;  // degenerate cell
        }
    for (int64_t s = 0; s < N; ++s)
        if (fa[s] == -2) return "degenerate cell (repeated vertex)";
    if (cell) {
        // The closed-form box mass matrix takes the side lengths from v0 to
        // v2 / v6 and the orientation of face e from the vertex order, so
        // a box must be axis-aligned with its vertices in that order:
        // vertex q sits at v0 + (bit 0 of q^(q>>1)) hx ex + (bit 1 of q) hy ey
        // + (bit 2 of q) hz ez, all h > 0.
        int64_t bad_cell = -1;
#pragma omp parallel for schedule(static) reduction(max : bad_cell)
        for (int64_t K = 0; K < C; ++K) {
            const double* x0 = coords + (int64_t)cell_verts[K * nv] * dim;
            const double* xo = coords + (int64_t)cell_verts[K * nv + nv - 2] * dim;  // v2 / v6
            double h[3] = {0, 0, 0}, ext = 0;
            for (int d = 0; d < dim; ++d) {
                h[d] = xo[d] - x0[d];
                ext = std::max(ext, std::fabs(h[d]));
            }
            bool ok = true;
            for (int d = 0; d < dim; ++d) ok = ok && h[d] > 0;
            for (int q = 0; q < nv && ok; ++q) {
                const int bits[3] = {(q ^ (q >> 1)) & 1, (q >> 1) & 1, (q >> 2) & 1};
                const double* xq = coords + (int64_t)cell_verts[K * nv + q] * dim;
                for (int d = 0; d < dim; ++d)
                    if (std::fabs(xq[d] - x0[d] - bits[d] * h[d]) > 1e-12 * ext) ok = false;
            }
            if (!ok) bad_cell = std::max(bad_cell, K);
        }
        if (bad_cell >= 0)
            return "box cell " + std::to_string(bad_cell) +
                   " is not axis-aligned with its vertices counterclockwise from the lowest corner "
                   "(bottom face before the top face)";
    }

    std::vector<int64_t> start(V + 1, 0);
    for (int64_t s = 0; s < N; ++s) start[fa[s] + 1]++;
    for (int64_t v = 0; v < V; ++v) start[v + 1] += start[v];
    std::vector<Key> keys(N);
    {
        std::vector<int64_t> pos(start.begin(), start.end() - 1);
        for (int64_t s = 0; s < N; ++s) keys[pos[fa[s]]++] = Key{fb[s], fc[s], fd[s], (int32_t)s};
    }

    // 2. group equal faces inside each bucket; rep = smallest slot of the group
    std::vector<int32_t> rep(N);
    int bad = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : bad)
    for (int64_t v = 0; v < V; ++v) {
        Key* k0 = keys.data() + start[v];
        Key* k1 = keys.data() + start[v + 1];
        std::sort(k0, k1, [](const Key& x, const Key& y) {
            if (x.b != y.b) return x.b < y.b;
            if (x.c != y.c) return x.c < y.c;
            if (x.d != y.d) return x.d < y.d;
            return x.slot < y.slot;
        });
        for (Key* g = k0; g < k1;) {
            Key* h = g + 1;
            while (h < k1 && h->b == g->b && h->c == g->c && h->d == g->d) ++h;
            if (h - g > 2) bad = 1;  // non-manifold: a face shared by more than two cells
            for (Key* q = g; q < h; ++q) rep[q->slot] = g->slot;
            g = h;
        }
    }
    if (bad) return "non-manifold mesh: a face is shared by more than two cells";

    // 3. face ids in order of first appearance
    std::vector<int32_t> id_of_rep(N, -1);
    int64_t F = 0;
    for (int64_t s = 0; s < N; ++s)
        if (rep[s] == s) id_of_rep[s] = (int32_t)F++;
    T.F = F;
    T.cell_faces.resize(N);
    T.face_cells.assign(2 * F, -1);
    T.face_local.assign(2 * F, 0);
    T.face_verts.resize(F * fv);
    for (int64_t s = 0; s < N; ++s) {
        const int32_t E = id_of_rep[rep[s]];
        T.cell_faces[s] = E;
        const int32_t K = (int32_t)(s / nf);
        const uint8_t e = (uint8_t)(s % nf);
        if (T.face_cells[2 * E] < 0) {
            T.face_cells[2 * E] = K;
            T.face_local[2 * E] = e;
            const int32_t fvs[4] = {fa[s], fb[s], fc[s], fd[s]};
            for (int q = 0; q < fv; ++q) T.face_verts[E * fv + q] = fvs[q];
        }
        else {
            T.face_cells[2 * E + 1] = K;
            T.face_local[2 * E + 1] = e;
        }
    }
    T.cell_bmask.assign(C, 0);
    T.boundary_faces = 0;
    for (int64_t E = 0; E < F; ++E)
        if (T.face_cells[2 * E + 1] < 0) {
            ++T.boundary_faces;
            const int32_t K = T.face_cells[2 * E];
            T.cell_bmask[K] |= (uint8_t)(1u << T.face_local[2 * E]);
        }
    T.face_measure.resize(F);
#pragma omp parallel for schedule(static)
    for (int64_t E = 0; E < F; ++E) {
        const double* P[4];
        for (int q = 0; q < fv; ++q) P[q] = coords + (int64_t)T.face_verts[E * fv + q] * dim;
        T.face_measure[E] = (cell && dim == 3) ? box_face_measure(P) : simplex_measure(P, fv - 1, dim);
    }
    return std::string();
}

void build_pattern(const HostTopology& T, int n, const uint8_t* tags, HostPattern& P)
{
    const int nf = T.nf;
    const int64_t F = T.F;
    P = HostPattern();
    P.n = n;
    P.rows = F * n;
    P.W = (T.C > 0) ? ((F > T.boundary_faces) ? (2 * nf - 1) * n - 1 : nf * n - 1) : 0;
    P.qmap.assign(F, 0);
    P.qdiag.assign(F, 0);
    P.row_len.assign(P.rows, 0);
    P.ell_cols.assign((size_t)P.W * P.rows, 0);
    const int64_t rows = P.rows;
    int64_t nnz = 0;
#pragma omp parallel for schedule(static) reduction(+ : nnz)
    for (int64_t E = 0; E < F; ++E) {
        const int32_t K0 = T.face_cells[2 * E], K1 = T.face_cells[2 * E + 1];
        int32_t list[12];
        int L = 0;
        for (int f = 0; f < nf; ++f) list[L++] = T.cell_faces[(int64_t)K0 * nf + f];
        if (K1 >= 0)
            for (int f = 0; f < nf; ++f) {
                const int32_t g = T.cell_faces[(int64_t)K1 * nf + f];
                if (g != (int32_t)E) list[L++] = g;
            }
        // at most 2 nf - 1 = 11 faces: insertion sort
        for (int x = 1; x < L; ++x)
            for (int y = x; y > 0 && list[y - 1] > list[y]; --y) std::swap(list[y - 1], list[y]);
        auto pos_of = [&](int32_t g) {
            for (int q = 0; q < L; ++q)
                if (list[q] == g) return q;
            return 0;
        };
        uint64_t qm = 0;
        for (int f = 0; f < nf; ++f) qm |= (uint64_t)pos_of(T.cell_faces[(int64_t)K0 * nf + f]) << (4 * f);
        if (K1 >= 0)
            for (int f = 0; f < nf; ++f)
                qm |= (uint64_t)pos_of(T.cell_faces[(int64_t)K1 * nf + f]) << (4 * (nf + f));
        P.qmap[E] = qm;
        const int qd = pos_of((int32_t)E);
        P.qdiag[E] = (uint8_t)qd;
        for (int i = 0; i < n; ++i) {
            const int64_t row = E * n + i;
            int len;
            int k = 0;
            const bool dirichlet = (K1 < 0) && tags[(int64_t)i * F + E] == 0;
            if (dirichlet) len = 1;
            else {
                len = L * n;
                for (int q = 0; q < L; ++q)
                    for (int j = 0; j < n; ++j) {
                        if (q == qd && j == i) continue;
                        P.ell_cols[(size_t)k * rows + row] = list[q] * n + j;
                        ++k;
                    }
            }
            for (; k < P.W; ++k) P.ell_cols[(size_t)k * rows + row] = (int32_t)row;
            P.row_len[row] = len;
            nnz += len;
        }
    }
    P.nnz = nnz;
}

}  // namespace mhfem
