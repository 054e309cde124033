/*
 * CPU oracle for the MHFEM per-time-step path: a plain C11 (+OpenMP)
 * restatement of the reference algorithm, used ONLY as test infrastructure
 * (parity checker in tests/, the smoke check and the timed CPU baseline of
 * bench.py).  The product path never links or calls this code.
 *
 * Parity status: UNPINNED.  The reference (TNL-MHFEM) ships no tests, no
 * golden vectors and no fixtures, and it cannot be compiled here (it needs
 * the external TNL library at commit 40f62622, which is absent).  The oracle
 * is pinned instead to known answers derived from mathematics and from the
 * reference's own formulas (RT0 basis quadrature of the mass matrix, the
 * linear patch test, local conservation, row structure); see tests/.
 *
 * Array layouts are the reference's CUDA permutations (BaseModel.h:18-125):
 * every per-cell array has the cell index K innermost, the face traces Z_iF
 * are face-major (F, i).
 */
#ifndef MHFEM_ORACLE_H
#define MHFEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One per-element coefficient: `full` = 0 means a single uniform value
 * (UniformCoefficient.h:8-52), otherwise a full array in the layout named
 * in the comment of each field of orc_problem. */
typedef struct {
    const double* p;
    int full;
} orc_coef;

typedef struct {
    /* static configuration (examples/config.h) */
    int dim;            /* 2 or 3 */
    int cell;           /* 0: simplices (triangles, tetrahedra); 1: boxes (rectangles, cuboids) */
    int nf;             /* faces per cell: dim + 1 (simplex), 2 dim (box) */
    int nv;             /* vertices per cell: dim + 1 (simplex), 2^dim (box) */
    int fv;             /* vertices per face: dim (simplex), 2^(dim-1) (box) */
    int n;              /* number of equations */
    int S;              /* MassMatrix::size: 9 (triangle), 14 (tetrahedron), 2 (rectangle), 3 (cuboid) */
    int lumping;        /* MassLumping::enabled = 1 */
    int advection;      /* 0 explicit_upwind, 1 implicit_upwind, 2 implicit_trace */
    int mobility_upwind;/* Model::do_mobility_upwind */

    int64_t V, C, F;
    const double* coords;      /* [V][dim] */
    const int32_t* cell_verts; /* [C][nf]  local vertex e is opposite local face e */
    const int32_t* cell_faces; /* [C][nf] */
    const int32_t* face_cells; /* [F][2], second = -1 on boundary faces */

    /* coefficients (layout: reference CUDA permutation) */
    orc_coef N;   /* (i,j,K)   */
    orc_coef u;   /* (i,j,e,K) */
    orc_coef m;   /* (i,K)     */
    orc_coef D;   /* (i,j,K)   */
    orc_coef w;   /* (i,e,K)   */
    orc_coef a;   /* (i,j,e,K) */
    orc_coef r;   /* (i,j,K)   */
    orc_coef f;   /* (i,K)     */
    orc_coef m_bnd; /* boundary mobility getBoundaryMobility, (i*F + E) */

    /* boundary conditions, (i*F + E) (BoundaryConditionsStorage.h) */
    const uint8_t* bc_tags;
    const double* bc_values;
    const double* bc_dirichlet;

    /* state and scheme data (owned by the caller) */
    double* Z_iF;      /* (F, i) */
    double* Z_iK;      /* (i, K) */
    double* v_iKe;     /* (i, e, K) */
    double* m_upw;     /* (E, i): computed if mobility_upwind, else an input */
    int m_upw_full;    /* only read when mobility_upwind == 0 */
    double* Z_upw;     /* (E, j, i) */
    double* b;         /* (i, j, s, K) */
    double* R_ijKe;    /* (i, j, e, K) */
    double* R_iK;      /* (i, K) */
} orc_problem;

/* Topology: faces numbered in order of first appearance when the cells are
 * visited in ascending order and their local faces e = 0..nf-1 in order.
 * Simplices: face e is the sub-simplex opposite local vertex e.  Boxes
 * (vertices in TNL's Quadrangle / Hexahedron order, v0 the lowest corner,
 * counterclockwise, bottom layer first): rectangle faces bottom, right, top,
 * left = (0,1), (1,2), (2,3), (3,0); cuboid faces bottom, front, right,
 * back, left, top = (0,1,2,3), (0,1,5,4), (1,2,6,5), (2,3,7,6), (3,0,4,7),
 * (4,5,6,7) (the orientations that MassMatrix.h:152-508 and
 * BasisFunctions_RTN0.h:55-126 name).  face_cells lists the adjacent cells
 * in ascending order.  Arrays must hold C*nf faces.  face_verts receives the
 * sorted vertex indices of each face ([F][fv]). */
int64_t orc_build_faces_ct(int dim, int cell, int64_t C, const int32_t* cell_verts,
                           int32_t* cell_faces, int32_t* face_cells, int32_t* face_verts);
/* the simplex case of orc_build_faces_ct */
int64_t orc_build_faces(int dim, int64_t C, const int32_t* cell_verts,
                        int32_t* cell_faces, int32_t* face_cells, int32_t* face_verts);

double orc_cell_measure(const orc_problem* p, int64_t K);
double orc_face_measure(const orc_problem* p, int64_t E, const int32_t* face_verts);

void orc_face_average(orc_problem* p);
void orc_update_b(orc_problem* p);
void orc_upwind(orc_problem* p, double t, double tau);
void orc_update_R(orc_problem* p, double tau);
void orc_update_Q(orc_problem* p, double tau);

/* Row lengths of the face-trace system, row index = E*n + i. */
void orc_row_lengths(const orc_problem* p, int32_t* rowlen);
/* Fills CSR (rowptr from orc_row_lengths) and the right-hand side.
 * face_verts is needed for the Neumann face measure. */
int orc_assemble(const orc_problem* p, const int32_t* face_verts, double t, double tau,
                 const int64_t* rowptr, int32_t* cols, double* vals, double* rhs);

/* BiCGStab with the identity (= Jacobi on a unit diagonal) preconditioner.
 * Returns 0 on convergence, 1 if max_iter was reached, 2 on breakdown. */
int orc_bicgstab(int64_t rows, const int64_t* rowptr, const int32_t* cols, const double* vals,
                 const double* rhs, double* x, double tol, int max_iter,
                 int* iters, double* residual);

void orc_reconstruct(orc_problem* p);
void orc_velocities(orc_problem* p);

/* One complete time step (control.h:64-102 loop body). */
int orc_step(orc_problem* p, const int32_t* face_verts, double t, double tau,
             const int64_t* rowptr, int32_t* cols, double* vals, double* rhs,
             double tol, int max_iter, int* iters, double* residual);

void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
