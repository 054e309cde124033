#pragma once
// Cell- and face-local kernels of the MHFEM time step (sm_103a), templated
// on the cell type and the number of equations.  Instantiated for
// triangles and tetrahedra in k_local.cu and for rectangles and cuboids in
// k_local_box.cu (two translation units that compile in parallel).
//
//  - k_cell_local: one thread per cell.  Fuses the reference's b update
//    (MassMatrix::update, Solver.hpp:627-639), R (Solver.hpp:793-815), the
//    Q / dummy-row / LU / Q^-1 R solve (Solver.hpp:817-871) and the local
//    Schur entries A_ijKEF and RHS_iKE of SecondaryCoefficients.h:187-349
//    into one pass.  Everything stays in registers; the outputs are b, Q^-1 R
//    (needed by the reconstruction) and one assembly record per (cell, local
//    face) that the face-row assembly reads exactly once.
//  - k_upwind: mobility and explicit advective upwinding (Solver.hpp:663-769).
//  - k_reconstruct: Z_iK and v_iKe (Solver.hpp:1283-1313).
//  - k_face_average: initial face traces (Solver.hpp:319-339).
//
// GB300 has a low FP64 issue rate (about 0.6 T FMA/s, 1/57 of FP32), so the
// kernels keep FP64 operations to the minimum the formulas need: one
// reciprocal per LU pivot instead of per-entry divides, the mass matrix
// assembled without its common denominator and scaled once, and the shared
// inverse of the RT0 matrix reused for every (i, j) component pair; box
// cells take the closed-form inverse and skip its known zero entries.
#include "mhfem_internal.h"

namespace mhfem {

__device__ __forceinline__ double cget(const Coef& c, int64_t idx) { return c.p[c.full ? idx : 0]; }

// ---- cell types -----------------------------------------------------------
// A kernel template parameter, so that every per-cell array is sized at
// compile time: triangle and tetrahedron (faces opposite the vertices),
// rectangle and cuboid (TNL Quadrangle / Hexahedron face order).

enum { CT_TRI = 0, CT_TET = 1, CT_RECT = 2, CT_CUBOID = 3 };

__host__ __device__ constexpr int ct_nf(int ct) { return ct == CT_TRI ? 3 : ct == CT_CUBOID ? 6 : 4; }
__host__ __device__ constexpr int ct_dim(int ct) { return (ct == CT_TRI || ct == CT_RECT) ? 2 : 3; }
__host__ __device__ constexpr bool ct_box(int ct) { return ct >= CT_RECT; }
// MassMatrix<Cell>::size: packed upper triangle + row sums for simplices,
// one value per face orientation for boxes
__host__ __device__ constexpr int ct_S(int ct) { return ct == CT_TRI ? 9 : ct == CT_TET ? 14 : ct_dim(ct); }

// Orientation class of local face e of a box, the storage slot of its value
// (MassMatrix.h:216-227, 392-403): rectangle faces 0, 2 (normal y) -> 0 and
// 1, 3 (normal x) -> 1; cuboid faces 2, 4 (normal x) -> 0, 1, 3 (normal y)
// -> 1, 0, 5 (normal z) -> 2.
__host__ __device__ constexpr int box_class(int ct, int e)
{
    return ct == CT_RECT ? (e & 1) : (e == 2 || e == 4) ? 0 : (e == 1 || e == 3) ? 1 : 2;
}

// Whether entry (e, f) of the inverse RT0 mass matrix can be nonzero: always
// for simplices; for boxes only between faces of one orientation.  The
// arguments are constants after loop unrolling, so the test folds away and
// the known zeros cost no FP64 operations.
__host__ __device__ constexpr bool b_nonzero(int ct, int e, int f)
{
    return !ct_box(ct) || box_class(ct, e) == box_class(ct, f);
}

// Inverse RT0 mass matrix of an axis-aligned box cell, without D, in closed
// form (MassMatrix.h:171-186, 249-264, 340-362, 424-446): with the side
// lengths h from the lowest corner v0 to the opposite corner (v2 of a
// rectangle, v6 of a cuboid), orientation class c has the value
// s_c = 2 prod_{d != c'} h_d / h_c' (c' the axis normal to the class);
// entry (e, f) is 2 s on the diagonal and s between the two faces of one
// orientation (lumped: s on the diagonal only), row sums 3 s (lumped s).
template <int CT>
__device__ __forceinline__ void box_inverse(const DevProblem& P, int64_t K, double& meas, double (&sv)[3],
                                            double (&Binv)[ct_nf(CT)][ct_nf(CT)], double (&Brow)[ct_nf(CT)])
{
    constexpr int d = ct_dim(CT), NF = ct_nf(CT);
    const int32_t v0 = __ldg(P.cell_verts + K);
    const int32_t v1 = __ldg(P.cell_verts + (int64_t)(d == 2 ? 2 : 6) * P.C + K);
    double h[3];
#pragma unroll
    for (int k = 0; k < d; ++k) h[k] = __ldg(P.coords + (int64_t)v1 * d + k) - __ldg(P.coords + (int64_t)v0 * d + k);
    if constexpr (d == 2) {
        meas = fabs(h[0] * h[1]);
        sv[0] = 2 * h[0] / h[1];
        sv[1] = 2 * h[1] / h[0];
        sv[2] = 0;
    }
    else {
        meas = fabs(h[0] * h[1] * h[2]);
        sv[0] = 2 * h[1] * h[2] / h[0];
        sv[1] = 2 * h[0] * h[2] / h[1];
        sv[2] = 2 * h[0] * h[1] / h[2];
    }
#pragma unroll
    for (int e = 0; e < NF; ++e) {
        const double s = sv[box_class(CT, e)];
        Brow[e] = P.lumping ? s : 3 * s;
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            if (!b_nonzero(CT, e, f)) Binv[e][f] = 0;
            else if (e == f) Binv[e][f] = P.lumping ? s : 2 * s;
            else Binv[e][f] = P.lumping ? 0.0 : s;
        }
    }
}

// Stored b_ijKef / b_ijKe (the coefficient D included) read back from the
// per-cell storage bp (slot stride C): MassMatrix.h:600-631 for simplices,
// 188-227, 268-319, 364-403, 448-507 for boxes.
template <int CT>
__device__ __forceinline__ double b_ef_stored(const double* bp, int64_t C, int lumping, int e, int f)
{
    if constexpr (!ct_box(CT)) {
        const int lo = e < f ? e : f, hi = e < f ? f : e;
        return bp[(int64_t)(lo + hi * (hi + 1) / 2) * C];
    }
    else {
        const double s = bp[(int64_t)box_class(CT, e) * C];
        if (e == f) return lumping ? s : 2 * s;
        return lumping ? 0.0 : s;
    }
}

template <int CT>
__device__ __forceinline__ double b_e_stored(const double* bp, int64_t C, int lumping, int e)
{
    if constexpr (!ct_box(CT)) return bp[(int64_t)(ct_S(CT) - ct_nf(CT) + e) * C];
    else {
        const double s = bp[(int64_t)box_class(CT, e) * C];
        return lumping ? s : 3 * s;
    }
}

// ---- geometry -----------------------------------------------------------

template <int NF>
struct Cell {
    double X[NF][NF - 1];
};

template <int NF>
__device__ __forceinline__ void load_cell(const DevProblem& P, int64_t K, Cell<NF>& c)
{
    constexpr int d = NF - 1;
#pragma unroll
    for (int v = 0; v < NF; ++v) {
        const int32_t vid = __ldg(P.cell_verts + (int64_t)v * P.C + K);
#pragma unroll
        for (int k = 0; k < d; ++k) c.X[v][k] = __ldg(P.coords + (int64_t)vid * d + k);
    }
}

template <int NF>
__device__ __forceinline__ double cell_measure(const Cell<NF>& c)
{
    if constexpr (NF == 3) {
        const double ax = c.X[1][0] - c.X[0][0], ay = c.X[1][1] - c.X[0][1];
        const double bx = c.X[2][0] - c.X[0][0], by = c.X[2][1] - c.X[0][1];
        return 0.5 * fabs(ax * by - ay * bx);
    }
    else {
        double e[3][3];
#pragma unroll
        for (int v = 0; v < 3; ++v)
#pragma unroll
            for (int k = 0; k < 3; ++k) e[v][k] = c.X[v + 1][k] - c.X[0][k];
        const double det = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1])
                         - e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0])
                         + e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
        return fabs(det) * (1.0 / 6.0);
    }
}

template <int D>
__device__ __forceinline__ double dot(const double* a, const double* b)
{
    double s = a[0] * b[0];
#pragma unroll
    for (int k = 1; k < D; ++k) s = fma(a[k], b[k], s);
    return s;
}

// Numerator of the local RT0 mass matrix (MassMatrix.h:538-569, 661-692,
// 787-825, 932-962) and its common denominator.
template <int NF>
__device__ __forceinline__ void mass_numerator(const Cell<NF>& c, int lumping, double meas,
                                               double (&M)[NF][NF], double& den)
{
    constexpr int d = NF - 1;
    if constexpr (NF == 3) {
        if (!lumping) {
            double P0[2], P1[2];
#pragma unroll
            for (int k = 0; k < 2; ++k) { P0[k] = c.X[0][k] - c.X[2][k]; P1[k] = c.X[1][k] - c.X[2][k]; }
            const double P00 = dot<2>(P0, P0), P01 = dot<2>(P0, P1), P11 = dot<2>(P1, P1);
            M[0][0] = 3 * P00 + P11 - 3 * P01;
            M[1][1] = P00 + 3 * P11 - 3 * P01;
            M[2][2] = P00 + P11 + P01;
            M[0][1] = 3 * P01 - P00 - P11;
            M[0][2] = P11 - P00 - P01;
            M[1][2] = P00 - P11 - P01;
            den = 24 * meas;
        }
        else {
            double P01[2], P02[2], P12[2];
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                P01[k] = c.X[0][k] - c.X[1][k]; P02[k] = c.X[0][k] - c.X[2][k]; P12[k] = c.X[1][k] - c.X[2][k];
            }
            M[0][0] = dot<2>(P01, P01) + dot<2>(P02, P02);
            M[1][1] = dot<2>(P01, P01) + dot<2>(P12, P12);
            M[2][2] = dot<2>(P02, P02) + dot<2>(P12, P12);
            M[0][1] = dot<2>(P02, P12);
            M[0][2] = -dot<2>(P01, P12);
            M[1][2] = dot<2>(P01, P02);
            den = 12 * meas;
        }
    }
    else {
        if (!lumping) {
            double P[3][3];
#pragma unroll
            for (int v = 0; v < 3; ++v)
#pragma unroll
                for (int k = 0; k < 3; ++k) P[v][k] = c.X[v][k] - c.X[3][k];
            const double P00 = dot<3>(P[0], P[0]), P11 = dot<3>(P[1], P[1]), P22 = dot<3>(P[2], P[2]);
            const double P01 = dot<3>(P[0], P[1]), P02 = dot<3>(P[0], P[2]), P12 = dot<3>(P[1], P[2]);
            M[0][0] = 12 * P00 + 2 * P11 + 2 * P22 - 8 * P01 - 8 * P02 + 2 * P12;
            M[1][1] = 2 * P00 + 12 * P11 + 2 * P22 - 8 * P01 + 2 * P02 - 8 * P12;
            M[2][2] = 2 * P00 + 2 * P11 + 12 * P22 + 2 * P01 - 8 * P02 - 8 * P12;
            M[3][3] = 2 * (P00 + P11 + P22 + P01 + P02 + P12);
            M[0][1] = -3 * P00 - 3 * P11 + 2 * P22 + 12 * P01 - 3 * P02 - 3 * P12;
            M[0][2] = -3 * P00 + 2 * P11 - 3 * P22 - 3 * P01 + 12 * P02 - 3 * P12;
            M[1][2] = 2 * P00 - 3 * P11 - 3 * P22 - 3 * P01 - 3 * P02 + 12 * P12;
            M[0][3] = -3 * P00 + 2 * P11 + 2 * P22 - 3 * P01 - 3 * P02 + 2 * P12;
            M[1][3] = 2 * P00 - 3 * P11 + 2 * P22 - 3 * P01 + 2 * P02 - 3 * P12;
            M[2][3] = 2 * P00 + 2 * P11 - 3 * P22 + 2 * P01 - 3 * P02 - 3 * P12;
            den = 180 * meas;
        }
        else {
            double Pd[6][3];  // 01 02 03 12 13 23
            const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {1, 2, 3, 2, 3, 3};
#pragma unroll
            for (int q = 0; q < 6; ++q)
#pragma unroll
                for (int k = 0; k < 3; ++k) Pd[q][k] = c.X[pa[q]][k] - c.X[pb[q]][k];
            const double s01 = dot<3>(Pd[0], Pd[0]), s02 = dot<3>(Pd[1], Pd[1]), s03 = dot<3>(Pd[2], Pd[2]);
            const double s12 = dot<3>(Pd[3], Pd[3]), s13 = dot<3>(Pd[4], Pd[4]), s23 = dot<3>(Pd[5], Pd[5]);
            M[0][0] = s01 + s02 + s03;
            M[1][1] = s01 + s12 + s13;
            M[2][2] = s02 + s12 + s23;
            M[3][3] = s03 + s13 + s23;
            M[0][1] = dot<3>(Pd[1], Pd[3]) + dot<3>(Pd[2], Pd[4]);
            M[0][2] = -dot<3>(Pd[0], Pd[3]) + dot<3>(Pd[2], Pd[5]);
            M[0][3] = -dot<3>(Pd[0], Pd[4]) - dot<3>(Pd[1], Pd[5]);
            M[1][2] = dot<3>(Pd[0], Pd[1]) + dot<3>(Pd[4], Pd[5]);
            M[1][3] = dot<3>(Pd[0], Pd[2]) - dot<3>(Pd[3], Pd[5]);
            M[2][3] = dot<3>(Pd[1], Pd[2]) + dot<3>(Pd[3], Pd[4]);
            den = 36 * meas;
        }
    }
#pragma unroll
    for (int i = 0; i < NF; ++i)
#pragma unroll
        for (int j = 0; j < i; ++j) M[i][j] = M[j][i];
    (void)d;
}

// In-place symmetric inverse via Doolittle LU without pivoting, one FP64
// reciprocal per pivot; the result is scaled by `scale`.
template <int NF>
__device__ __forceinline__ void lu_inverse(double (&A)[NF][NF], double scale, double (&Inv)[NF][NF])
{
    double rp[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) {
#pragma unroll
        for (int j = k; j < NF; ++j) {
            double s = A[k][j];
#pragma unroll
            for (int q = 0; q < k; ++q) s = fma(-A[k][q], A[q][j], s);
            A[k][j] = s;
        }
        rp[k] = recip_newton(A[k][k]);
#pragma unroll
        for (int i = k + 1; i < NF; ++i) {
            double s = A[i][k];
#pragma unroll
            for (int q = 0; q < k; ++q) s = fma(-A[i][q], A[q][k], s);
            A[i][k] = s * rp[k];
        }
    }
#pragma unroll
    for (int col = 0; col < NF; ++col) {
        double v[NF];
#pragma unroll
        for (int i = 0; i < NF; ++i) {
            double s = (i == col) ? 1.0 : 0.0;
#pragma unroll
            for (int q = 0; q < i; ++q) s = fma(-A[i][q], v[q], s);
            v[i] = s;
        }
#pragma unroll
        for (int i = NF - 1; i >= 0; --i) {
            double s = v[i];
#pragma unroll
            for (int q = i + 1; q < NF; ++q) s = fma(-A[i][q], v[q], s);
            v[i] = s * rp[i];
        }
#pragma unroll
        for (int i = 0; i < NF; ++i) Inv[i][col] = v[i] * scale;
    }
}

// ---- the fused cell kernel ----------------------------------------------

enum { MODE_NO_ADV = 0, MODE_ADV = 1, MODE_CELL_DIRICHLET = 2, MODE_SKIP = 3 };

// The inverse of the RT0 mass matrix of cell K without D (Binv), its row
// sums (b_ijKe without D), the cell measure and, for boxes, the value of
// each face orientation (MassMatrix::update, MassMatrix.h:511-1050 and
// 152-508).
template <int CT>
__device__ __forceinline__ void cell_mass_inverse(const DevProblem& P, int64_t K, double& meas, double (&sv)[3],
                                                  double (&Binv)[ct_nf(CT)][ct_nf(CT)], double (&Brow)[ct_nf(CT)])
{
    constexpr int NF = ct_nf(CT);
    if constexpr (ct_box(CT)) {
        box_inverse<CT>(P, K, meas, sv, Binv, Brow);
    }
    else {
        Cell<NF> cell;
        load_cell<NF>(P, K, cell);
        meas = cell_measure<NF>(cell);
        // Binv = den * Mnum^-1
        double M[NF][NF];
        double den;
        mass_numerator<NF>(cell, P.lumping, meas, M, den);
        lu_inverse<NF>(M, den, Binv);
#pragma unroll
        for (int e = 0; e < NF; ++e) {
            double s = Binv[e][0];
#pragma unroll
            for (int f = 1; f < NF; ++f) s += Binv[e][f];
            Brow[e] = s;
        }
        (void)sv;
    }
}

template <int NE>
__device__ __forceinline__ void load_D(const DevProblem& P, int64_t K, double (&Dij)[NE][NE])
{
#pragma unroll
    for (int i = 0; i < NE; ++i)
#pragma unroll
        for (int j = 0; j < NE; ++j) Dij[i][j] = cget(P.D, ((int64_t)i * NE + j) * P.C + K);
}

// b_ijK_storage (i,j,s,K): simplices the packed upper triangle column by
// column, then the row sums; boxes one value per face orientation
template <int CT, int NE>
__device__ __forceinline__ void store_b(const DevProblem& P, int64_t K, const double (&sv)[3],
                                        const double (&Binv)[ct_nf(CT)][ct_nf(CT)], const double (&Brow)[ct_nf(CT)],
                                        const double (&Dij)[NE][NE])
{
    constexpr int NF = ct_nf(CT);
    constexpr int S = ct_S(CT);
    const int64_t C = P.C;
#pragma unroll
    for (int i = 0; i < NE; ++i)
#pragma unroll
        for (int j = 0; j < NE; ++j) {
            double* bp = P.b + ((int64_t)(i * NE + j) * S) * C + K;
            if constexpr (ct_box(CT)) {
#pragma unroll
                for (int c = 0; c < S; ++c) bp[(int64_t)c * C] = sv[c] * Dij[i][j];
            }
            else {
#pragma unroll
                for (int col = 0; col < NF; ++col)
#pragma unroll
                    for (int row = 0; row <= col; ++row)
                        bp[(int64_t)(col * (col + 1) / 2 + row) * C] = Binv[row][col] * Dij[i][j];
#pragma unroll
                for (int e = 0; e < NF; ++e) bp[(int64_t)(S - NF + e) * C] = Brow[e] * Dij[i][j];
            }
        }
}

// The b update alone (MassMatrix::update over all cells, Solver.hpp:627-639):
// the first launch of a step whose model updates its vector coefficients
// from this step's b (updateVectorCoefficients, Solver.hpp:641-652) before
// the rest of the cell work.
template <int CT, int NE>
__global__ void __launch_bounds__(128) k_update_b(const DevProblem P)
{
    constexpr int NF = ct_nf(CT);
    const int64_t K = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (K >= P.C) return;
    double meas, sv[3], Binv[NF][NF], Brow[NF], Dij[NE][NE];
    cell_mass_inverse<CT>(P, K, meas, sv, Binv, Brow);
    load_D<NE>(P, K, Dij);
    store_b<CT, NE>(P, K, sv, Binv, Brow, Dij);
}

template <int CT, int NE>
__global__ void __launch_bounds__(128) k_cell_local(const DevProblem P, const double rtau, const double src_scale)
{
    constexpr int NF = ct_nf(CT);
    const int64_t K = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (K >= P.C) return;
    const int64_t C = P.C;

    // inverse of the RT0 mass matrix (without D) and its row sums (b_ijKe without D)
    double meas;
    double Binv[NF][NF];
    double Brow[NF];
    double sv[3];  // box cells: the value of each face orientation
    cell_mass_inverse<CT>(P, K, meas, sv, Binv, Brow);
    double Dij[NE][NE];
    load_D<NE>(P, K, Dij);
    store_b<CT, NE>(P, K, sv, Binv, Brow, Dij);

    int32_t faces[NF];
#pragma unroll
    for (int e = 0; e < NF; ++e) faces[e] = __ldg(P.cell_faces + (int64_t)e * C + K);
    const uint32_t bmask = __ldg(P.cell_bmask + K);

    double mu[NE][NF];
#pragma unroll
    for (int i = 0; i < NE; ++i)
#pragma unroll
        for (int e = 0; e < NF; ++e)
            mu[i][e] = P.use_m_upw_array ? P.m_upw_read[(int64_t)faces[e] * NE + i] : P.m_upw_in.p[0];

    double ZK[NE];
#pragma unroll
    for (int i = 0; i < NE; ++i) ZK[i] = P.Z_iK[(int64_t)i * C + K];

    auto vel_at = [&](int i, int j, int e) -> double {
        const int64_t idx = (((int64_t)i * NE + j) * NF + e) * C + K;
        return cget(P.a, idx) + cget(P.u, idx);
    };

    // R_ijKe, R_iK (SecondaryCoefficients.h:50-127)
    double RQ[NE][NE][NF];
    double RK[NE];
    const double mtau = meas * rtau;
#pragma unroll
    for (int i = 0; i < NE; ++i) {
#pragma unroll
        for (int j = 0; j < NE; ++j)
#pragma unroll
            for (int e = 0; e < NF; ++e) {
                double R = 0;
#pragma unroll
                for (int f = 0; f < NF; ++f)
                    if (b_nonzero(CT, f, e)) R = fma(mu[i][f], Binv[f][e], R);
                R *= Dij[i][j];
                if (P.advection == MHFEM_IMPLICIT_UPWIND) {
                    const double vel = vel_at(i, j, e);
                    if (vel < 0) R -= 2 * vel;
                }
                else if (P.advection == MHFEM_IMPLICIT_TRACE) {
                    R -= vel_at(i, j, e);
                }
                RQ[i][j][e] = R;
            }
        double R = 0;
#pragma unroll
        for (int j = 0; j < NE; ++j) R = fma(cget(P.N, ((int64_t)i * NE + j) * C + K), ZK[j], R);
        R *= mtau;
        R = fma(meas, cget(P.f, (int64_t)i * C + K) + (P.psi.p ? src_scale * cget(P.psi, K) : 0.0), R);
#pragma unroll
        for (int e = 0; e < NF; ++e) R = fma(-mu[i][e], cget(P.w, ((int64_t)i * NF + e) * C + K), R);
        if (P.explicit_adv_active) {
            double aux = 0;
#pragma unroll
            for (int j = 0; j < NE; ++j)
#pragma unroll
                for (int e = 0; e < NF; ++e)
                    aux = fma(vel_at(i, j, e), P.Z_upw[((int64_t)faces[e] * NE + j) * NE + i], aux);
            R -= aux;
        }
        RK[i] = R;
    }

    // Q_ijK (SecondaryCoefficients.h:129-159), dummy rows, LU, Q^-1 R (Solver.hpp:817-871)
    double Q[NE][NE];
#pragma unroll
    for (int i = 0; i < NE; ++i) {
        bool singular = true;
#pragma unroll
        for (int j = 0; j < NE; ++j) {
            double q = 0;
#pragma unroll
            for (int e = 0; e < NF; ++e) {
                const int64_t idx = (((int64_t)i * NE + j) * NF + e) * C + K;
                q += fma(mu[i][e], Brow[e] * Dij[i][j], -cget(P.u, idx));
                if (P.advection == MHFEM_IMPLICIT_UPWIND) q += fabs(cget(P.a, idx) + cget(P.u, idx));
            }
            q += mtau * cget(P.N, ((int64_t)i * NE + j) * C + K) + meas * cget(P.r, ((int64_t)i * NE + j) * C + K);
            Q[i][j] = q;
            if (q != 0.0) singular = false;
        }
        if (singular) {
            Q[i][i] = 1.0;
            RK[i] += ZK[i];
        }
    }
    if constexpr (NE == 1) {
        const double rq = recip_newton(Q[0][0]);
        RK[0] *= rq;
#pragma unroll
        for (int e = 0; e < NF; ++e) RQ[0][0][e] *= rq;
    }
    else {
        // Doolittle LU without pivoting, in place (U on and above the
        // diagonal, L below), one reciprocal per pivot
        double rp[NE];
#pragma unroll
        for (int k = 0; k < NE; ++k) {
#pragma unroll
            for (int j = k; j < NE; ++j) {
                double u = Q[k][j];
#pragma unroll
                for (int q = 0; q < k; ++q) u = fma(-Q[k][q], Q[q][j], u);
                Q[k][j] = u;
            }
            rp[k] = recip_newton(Q[k][k]);
#pragma unroll
            for (int i = k + 1; i < NE; ++i) {
                double l = Q[i][k];
#pragma unroll
                for (int q = 0; q < k; ++q) l = fma(-Q[i][q], Q[q][k], l);
                Q[i][k] = l * rp[k];
            }
        }
        // x <- Q^-1 x for the NE components x[i] = X(i)
        auto solve = [&](auto&& X) {
#pragma unroll
            for (int i = 1; i < NE; ++i) {
                double y = X(i);
#pragma unroll
                for (int q = 0; q < i; ++q) y = fma(-Q[i][q], X(q), y);
                X(i) = y;
            }
#pragma unroll
            for (int i = NE - 1; i >= 0; --i) {
                double x = X(i);
#pragma unroll
                for (int q = i + 1; q < NE; ++q) x = fma(-Q[i][q], X(q), x);
                X(i) = x * rp[i];
            }
        };
        solve([&](int i) -> double& { return RK[i]; });
#pragma unroll
        for (int j = 0; j < NE; ++j)
#pragma unroll
            for (int e = 0; e < NF; ++e) solve([&](int i) -> double& { return RQ[i][j][e]; });
    }

#pragma unroll
    for (int i = 0; i < NE; ++i) {
        P.R_iK[(int64_t)i * C + K] = RK[i];
#pragma unroll
        for (int j = 0; j < NE; ++j)
#pragma unroll
            for (int e = 0; e < NF; ++e) P.R_ijKe[(((int64_t)i * NE + j) * NF + e) * C + K] = RQ[i][j][e];
    }

    // assembly records: A_ijKEF (row variant chosen per face) and RHS_iKE
#pragma unroll
    for (int e = 0; e < NF; ++e) {
        const bool bnd = (bmask >> e) & 1u;
#pragma unroll
        for (int i = 0; i < NE; ++i) {
            int mode;
            if (!bnd) mode = (P.advection == MHFEM_EXPLICIT_UPWIND) ? MODE_NO_ADV : MODE_ADV;
            else {
                const int tag = P.bc_tags[(int64_t)i * P.F + faces[e]];
                if (tag == MHFEM_BC_FIXED_VALUE) mode = MODE_SKIP;
                else if (tag == MHFEM_BC_FIXED_FLUX) mode = MODE_ADV;
                else if (tag == MHFEM_BC_FIXED_FLUX_NO_ADVECTION) mode = MODE_NO_ADV;
                else mode = (vel_at(i, i, e) >= 0) ? MODE_NO_ADV : MODE_CELL_DIRICHLET;
            }
            if (mode == MODE_SKIP) continue;
            double* rec = P.rec + ((K * NF + e) * NE + i) * (int64_t)P.rec_stride;
            double out[NE * NF + 1];
            if (mode == MODE_CELL_DIRICHLET) {
                // BoundaryConditions.hpp:34-37, 51-54
#pragma unroll
                for (int j = 0; j < NE; ++j)
#pragma unroll
                    for (int f = 0; f < NF; ++f) out[j * NF + f] = (i == j && f == e) ? 1.0 : 0.0;
                out[NE * NF] = ZK[i];
            }
            else {
                const bool adv = (mode == MODE_ADV);
                const double m = adv ? mu[i][e] : 1.0;
                double Sx[NE];
#pragma unroll
                for (int x = 0; x < NE; ++x) {
                    double s = m * Brow[e] * Dij[i][x];
                    if (adv && P.advection == MHFEM_IMPLICIT_UPWIND) s += fabs(vel_at(i, x, e));
                    Sx[x] = s;
                }
#pragma unroll
                for (int j = 0; j < NE; ++j)
#pragma unroll
                    for (int f = 0; f < NF; ++f) {
                        double T = b_nonzero(CT, e, f) ? m * Binv[e][f] * Dij[i][j] : 0.0;
                        if (adv && f == e) {
                            if (P.advection == MHFEM_IMPLICIT_UPWIND) {
                                const double vel = vel_at(i, j, e);
                                if (vel < 0) T -= 2 * vel;
                            }
                            else if (P.advection == MHFEM_IMPLICIT_TRACE) {
                                T -= vel_at(i, j, e);
                            }
                        }
                        double sq = 0;
#pragma unroll
                        for (int x = 0; x < NE; ++x) sq = fma(Sx[x], RQ[x][j][f], sq);
                        out[j * NF + f] = T - sq;
                    }
                double rhs = m * cget(P.w, ((int64_t)i * NF + e) * C + K);
#pragma unroll
                for (int j = 0; j < NE; ++j) {
                    rhs = fma(Sx[j], RK[j], rhs);
                    if (adv && P.explicit_adv_active)
                        rhs = fma(P.Z_upw[((int64_t)faces[e] * NE + j) * NE + i], vel_at(i, j, e), rhs);
                }
                out[NE * NF] = rhs;
            }
#pragma unroll
            for (int q = 0; q < NE * NF + 1; ++q) rec[q] = out[q];
        }
    }
}

template <int NF, int NE>
__global__ void k_upwind(const DevProblem P)
{
    const int64_t E = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (E >= P.F) return;
    const int2 kk = P.face_cells[E];
    const int e1 = P.face_local[2 * E];
    const int e2 = P.face_local[2 * E + 1];
    const int64_t C = P.C;
    if (P.mobility_upwind) {
#pragma unroll
        for (int i = 0; i < NE; ++i) {
            double m;
            if (kk.y < 0) {
                bool inflow = false;
#pragma unroll
                for (int j = 0; j < NE; ++j)
                    if (P.v_iKe[((int64_t)j * NF + e1) * C + kk.x] < 0) inflow = true;
                m = inflow ? cget(P.m_bnd, (int64_t)i * P.F + E) : cget(P.m, (int64_t)i * C + kk.x);
            }
            else {
                const double vel = P.v_iKe[((int64_t)i * NF + e1) * C + kk.x] - P.v_iKe[((int64_t)i * NF + e2) * C + kk.y];
                if (vel == 0) m = 0.5 * (cget(P.m, (int64_t)i * C + kk.x) + cget(P.m, (int64_t)i * C + kk.y));
                else if (vel > 0) m = cget(P.m, (int64_t)i * C + kk.x);
                else m = cget(P.m, (int64_t)i * C + kk.y);
            }
            P.m_upw[E * NE + i] = m;
        }
    }
    if (P.explicit_adv_active) {
#pragma unroll
        for (int j = 0; j < NE; ++j)
#pragma unroll
            for (int i = 0; i < NE; ++i) {
                const int64_t idx = (((int64_t)i * NE + j) * NF + e1) * C + kk.x;
                const double apu = cget(P.a, idx) + cget(P.u, idx);
                double z;
                if (apu > 0.0) z = P.Z_iK[(int64_t)j * C + kk.x];
                else if (apu == 0.0) z = 0;
                else if (kk.y >= 0) z = P.Z_iK[(int64_t)j * C + kk.y];
                else z = P.Z_iF[E * NE + j];
                P.Z_upw[(E * NE + j) * NE + i] = z;
            }
    }
}

template <int CT, int NE>
__global__ void k_reconstruct(const DevProblem P)
{
    constexpr int NF = ct_nf(CT);
    constexpr int S = ct_S(CT);
    const int64_t K = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (K >= P.C) return;
    const int64_t C = P.C;
    int32_t faces[NF];
#pragma unroll
    for (int e = 0; e < NF; ++e) faces[e] = __ldg(P.cell_faces + (int64_t)e * C + K);
    double ZF[NE][NF];
#pragma unroll
    for (int f = 0; f < NF; ++f)
#pragma unroll
        for (int j = 0; j < NE; ++j) ZF[j][f] = P.Z_iF[(int64_t)faces[f] * NE + j];
    double ZK[NE];
#pragma unroll
    for (int i = 0; i < NE; ++i) {
        double Z = 0;
#pragma unroll
        for (int f = 0; f < NF; ++f)
#pragma unroll
            for (int j = 0; j < NE; ++j) Z = fma(P.R_ijKe[(((int64_t)i * NE + j) * NF + f) * C + K], ZF[j][f], Z);
        Z += P.R_iK[(int64_t)i * C + K];
        ZK[i] = Z;
        P.Z_iK[(int64_t)i * C + K] = Z;
    }
    if (P.mobility_upwind) {
        // SecondaryCoefficients.h:16-48, two separate sums
#pragma unroll
        for (int i = 0; i < NE; ++i)
#pragma unroll
            for (int e = 0; e < NF; ++e) {
                double sK = 0, sE = 0;
#pragma unroll
                for (int j = 0; j < NE; ++j) {
                    const double* bp = P.b + ((int64_t)(i * NE + j) * S) * C + K;
                    sK = fma(b_e_stored<CT>(bp, C, P.lumping, e), ZK[j], sK);
#pragma unroll
                    for (int f = 0; f < NF; ++f)
                        if (b_nonzero(CT, e, f)) sE = fma(b_ef_stored<CT>(bp, C, P.lumping, e, f), ZF[j][f], sE);
                }
                P.v_iKe[((int64_t)i * NF + e) * C + K] = sK - sE + cget(P.w, ((int64_t)i * NF + e) * C + K);
            }
    }
}

template <int NE>
__global__ void k_face_average(const DevProblem P)
{
    const int64_t E = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (E >= P.F) return;
    const int2 kk = P.face_cells[E];
#pragma unroll
    for (int i = 0; i < NE; ++i) {
        const double z0 = P.Z_iK[(int64_t)i * P.C + kk.x];
        P.Z_iF[E * NE + i] = (kk.y < 0) ? z0 : 0.5 * (z0 + P.Z_iK[(int64_t)i * P.C + kk.y]);
    }
}

// ---- dispatch -------------------------------------------------------------

#define MHFEM_NE_DISPATCH(CTV, NEV, CALL)                                        \
    do {                                                                          \
        if ((NEV) == 1) { constexpr int CT = (CTV), NE = 1; constexpr int NF = ct_nf(CT); (void)NF; CALL; } \
        else if ((NEV) == 2) { constexpr int CT = (CTV), NE = 2; constexpr int NF = ct_nf(CT); (void)NF; CALL; } \
        else { constexpr int CT = (CTV), NE = 3; constexpr int NF = ct_nf(CT); (void)NF; CALL; } \
    } while (0)

static inline unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// box launchers (k_local_box.cu)
int launch_cell_local_box(const DevProblem& P, double rtau, double src_scale, cudaStream_t s);
int launch_update_b_box(const DevProblem& P, cudaStream_t s);
int launch_upwind_cuboid(const DevProblem& P, cudaStream_t s);
int launch_reconstruct_box(const DevProblem& P, cudaStream_t s);

}  // namespace mhfem
