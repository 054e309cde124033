/*
 * mhfem.h - C ABI of the GB300-native MHFEM time-step library.
 *
 * The library implements the per-time-step hot path of TNL-MHFEM's CUDA
 * solver (TNL::MHFEM::Solver<Model, BoundaryModel, Matrix>, Solver.h:28-210)
 * on one GPU: local RT0 mass-matrix update, upwinding, local condensation,
 * in-place assembly of the hybridized face-trace system, its Krylov solve
 * (BiCGStab or restarted GMRES) and the reconstruction of the cell averages.  The reference's plugin API is
 * compile-time C++ (a Model class derived from BaseModel plus a
 * BoundaryModel); this header is the run-time C equivalent a maintainer binds
 * from C, C++, ctypes or any other FFI.
 *
 * Conventions
 *  - Every function returns an mhfem_status; mhfem_last_error() gives a
 *    message for the last failure on a handle.
 *  - All pointers are HOST pointers owned by the caller; the library owns
 *    all device memory.  A handle is not thread-safe; it uses one CUDA
 *    stream of its own.
 *  - Indices are int32 (examples/config.h:1-7: Index = int); reals are
 *    double (Real = double).
 *  - Array layouts follow the reference's CUDA permutations
 *    (BaseModel.h:18-125): per-cell arrays have the cell index K innermost,
 *    e.g. D_ijK at ((i*n + j)*C + K), a_ijKe at (((i*n + j)*f + e)*C + K),
 *    w_iKe at ((i*f + e)*C + K), m_iK at (i*C + K).  Face traces Z_iF are
 *    face-major: (E*n + i), which is also the DOF / row index
 *    (BaseModel.h:252-263).  Boundary-condition arrays are component-major:
 *    (i*F + E) (BoundaryModels/Stationary.h:21-36).
 */
#ifndef MHFEM_H
#define MHFEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t mhfem_status;
#define MHFEM_OK                        0
#define MHFEM_ERR_INVALID_ARGUMENT      1
#define MHFEM_ERR_STATE                 2   /* call made out of order */
#define MHFEM_ERR_CUDA                  3
#define MHFEM_ERR_NOT_CONVERGED         4   /* Solver.hpp:1259-1264 */
#define MHFEM_ERR_BREAKDOWN             5   /* Krylov breakdown (zero inner product) */
#define MHFEM_ERR_NONPOSITIVE_DIAGONAL  6   /* LinearSystem.h:153, BoundaryConditions.hpp:181 */
#define MHFEM_ERR_NO_DEVICE             7
#define MHFEM_ERR_OUT_OF_MEMORY         8
#define MHFEM_ERR_NOT_FINITE            9   /* NaN / Inf met in the solve */
#define MHFEM_ERR_TIMEOUT              10   /* host wall-clock limit on a solve */
#define MHFEM_ERR_UNSUPPORTED          11

typedef struct mhfem_solver_s* mhfem_t;

/* Advection discretization (BaseModel.h:12-16). */
#define MHFEM_EXPLICIT_UPWIND 0
#define MHFEM_IMPLICIT_UPWIND 1
#define MHFEM_IMPLICIT_TRACE  2

/* Solver forms. */
#define MHFEM_FORM_FP64    0   /* plain FP64 BiCGStab (the reference's path)          */
#define MHFEM_FORM_MIXED   1   /* FP32 inner BiCGStab + FP64 iterative refinement    */
#define MHFEM_FORM_LEARNED 2   /* FP64 BiCGStab warm-started by the message-passing net */

/* Boundary condition tags (BoundaryConditionsType.h:7-31). */
#define MHFEM_BC_FIXED_VALUE              0
#define MHFEM_BC_FIXED_FLUX               1
#define MHFEM_BC_ADVECTIVE_OUTFLOW        2
#define MHFEM_BC_FIXED_FLUX_NO_ADVECTION  3

/* Coefficient identifiers (BaseModel.h:267-275 and HeatEquationModel.h:114-133). */
#define MHFEM_COEF_N      0   /* (i,j,K)   */
#define MHFEM_COEF_U      1   /* (i,j,e,K) */
#define MHFEM_COEF_M      2   /* (i,K)     */
#define MHFEM_COEF_D      3   /* (i,j,K)   isotropic D, as in the reference */
#define MHFEM_COEF_W      4   /* (i,e,K)   */
#define MHFEM_COEF_A      5   /* (i,j,e,K) */
#define MHFEM_COEF_R      6   /* (i,j,K)   */
#define MHFEM_COEF_F      7   /* (i,K)     */
#define MHFEM_COEF_M_UPW  8   /* (E,i) upwinded mobility, a model input when mobility upwind is off */
#define MHFEM_COEF_M_BND  9   /* (i*F+E) getBoundaryMobility value on inflow boundary faces */
#define MHFEM_COEF_PSI   10   /* (K) spatial shape of the time-modulated source */

/* Arrays readable with mhfem_get_array. */
#define MHFEM_ARRAY_B       0  /* b_ijK_storage (i,j,s,K) */
#define MHFEM_ARRAY_R_IJKE  1  /* Q^-1 R_ijKe (i,j,e,K)   */
#define MHFEM_ARRAY_R_IK    2  /* Q^-1 R_iK (i,K)         */
#define MHFEM_ARRAY_M_UPW   3  /* m_iE_upw (E,i)          */
#define MHFEM_ARRAY_Z_UPW   4  /* Z_ijE_upw (E,j,i)       */
#define MHFEM_ARRAY_V       5  /* v_iKe (i,e,K)           */
#define MHFEM_ARRAY_RHS     6  /* scaled right-hand side, rows E*n+i */
#define MHFEM_ARRAY_Z_IF    7  /* face traces Z_iF (E,i)  */
#define MHFEM_ARRAY_Z_IK    8  /* cell values Z_iK (i,K)  */

typedef struct {
    int32_t dim;              /* 2: triangles or rectangles, 3: tetrahedra or cuboids (examples/config.h:13-21) */
    int32_t n_eq;             /* NumberOfEquations, 1 to 3 */
    int32_t mass_lumping;     /* MassLumping::enabled = 1 (MassMatrix.h:16-19) */
    int32_t advection;        /* MHFEM_*_UPWIND / MHFEM_IMPLICIT_TRACE */
    int32_t mobility_upwind;  /* Model::do_mobility_upwind (BaseModel.h:160-161) */
    int32_t form;             /* MHFEM_FORM_* */
    int32_t device;           /* CUDA device ordinal */
    int32_t cell;             /* MHFEM_CELL_SIMPLEX (triangles, tetrahedra) or MHFEM_CELL_BOX
                                 (rectangles, cuboids: the Quadrangle / Hexahedron topologies of
                                 examples/config.h:13-21, axis-aligned as MassMatrix.h:152-508 assumes) */
} mhfem_desc;

#define MHFEM_CELL_SIMPLEX 0
#define MHFEM_CELL_BOX     1

typedef struct {
    double  tol;              /* convergence-residue: relative residual ||b-Ax||/||b|| */
    int32_t max_iter;         /* max-iterations of the Krylov solver */
    double  inner_tol;        /* mixed form: relative tolerance of each FP32 sweep */
    int32_t max_sweeps;       /* mixed form: cap on refinement sweeps */
    int32_t check_every;      /* Krylov iterations between host convergence checks (systems
                                 above 2^18 rows; smaller FP64 BiCGStab solves run in one
                                 persistent launch and test every iteration) */
    double  timeout_s;        /* host wall-clock limit of one solve (<= 0: none) */
    int32_t inner_adaptive;   /* mixed form: relax the last sweeps' inner tolerance to what the outer
                                 tolerance still needs (never tighter than inner_tol) */
    int32_t linear_solver;    /* linear-solver (configSetup.h:32-38): MHFEM_SOLVER_BICGSTAB (default)
                                 or MHFEM_SOLVER_GMRES; the FP64 and learned forms' solve (the mixed
                                 form's inner solve is FP32 BiCGStab) */
    int32_t gmres_restart;    /* gmres-restarting-max: restart length, 1 to 32 (default 30) */
    int32_t gmres_variant;    /* gmres-variant: MHFEM_GMRES_CGS (default) or MHFEM_GMRES_CGSR
                                 (classical Gram-Schmidt with one reorthogonalization pass) */
    int32_t gmres_restart_min;      /* gmres-restarting-min: with gmres_restart_step_min > 0 and a
                                       value below gmres_restart, the restart length varies between
                                       the two from cycle to cycle (Baker, Jessup and Kolev's rule on
                                       the ratio of consecutive restart residuals); 0 (default): fixed
                                       at gmres_restart */
    int32_t gmres_restart_step_min; /* gmres-restarting-step-min: decrement of the restart length */
    int32_t gmres_restart_step_max; /* gmres-restarting-step-max: decrement after a well-converging
                                       cycle (at least gmres_restart_step_min) */
} mhfem_solver_opts;

#define MHFEM_SOLVER_BICGSTAB 0
#define MHFEM_SOLVER_GMRES    1
#define MHFEM_GMRES_CGS       0
#define MHFEM_GMRES_CGSR      1

typedef struct {
    int32_t iterations;       /* Krylov iterations (mixed: FP32 inner iterations, summed) */
    int32_t sweeps;           /* refinement sweeps (mixed form), else 1 */
    double  residual;         /* final relative residual in FP64 */
    int32_t guess_used;       /* learned form: 1 if the predicted initial guess was accepted */
    double  guess_residual;   /* learned form: relative residual of the predicted guess */
    double  warm_residual;    /* relative residual of the previous-step warm start */
    double  ms_pre, ms_assemble, ms_solve, ms_post;   /* device time per phase */
    double  ms_guess;         /* learned form: device time of the guess (features, network, gate
                                 residuals), included in ms_solve; 0 for the other forms */
    double  base_residual;    /* learned form: relative residual of the extrapolated base (-1: none) */
    int32_t guess_source;     /* learned form: the initial guess the solve started from:
                                 0 the warm start, 1 the network's guess, 2 the extrapolated base */
} mhfem_step_stats;

/* ---- lifecycle ---------------------------------------------------------- */

/* Replaces constructing Solver<Model,...> with its compile-time static
 * configuration (examples/config.h:1-61, examples/main.h:17). */
mhfem_status mhfem_create(const mhfem_desc* desc, mhfem_t* out);
/* Frees every device array the handle owns (the Solver owns mdd and its
 * arrays, Solver.h:182-207). */
mhfem_status mhfem_destroy(mhfem_t h);
/* Message of the last failure on the handle: the text the reference puts in
 * its exceptions (e.g. the non-convergence message of Solver.hpp:1259-1264). */
const char*  mhfem_last_error(mhfem_t h);
void         mhfem_default_solver_opts(mhfem_solver_opts* opts);

/* ---- setup -------------------------------------------------------------- */

/* Replaces Solver::setMesh (Solver.hpp:28-80) after MHFEM::init loaded the
 * mesh (control.h:15-47).  Simplices: cell_verts is [C][dim+1]; local
 * vertex e is opposite local face e (the convention MassMatrix.h:538 relies
 * on).  Boxes (desc.cell = MHFEM_CELL_BOX): cell_verts is [C][2^dim], the
 * vertices of TNL's Quadrangle / Hexahedron: axis-aligned, counterclockwise
 * from the lowest corner, the bottom face before the top one (the order
 * MassMatrix.h:171-186, 340-362 reads the side lengths from); another order
 * is refused with MHFEM_ERR_INVALID_ARGUMENT.  The library numbers the faces
 * in order of first appearance over the cells and their local faces. */
mhfem_status mhfem_set_mesh(mhfem_t h, int64_t num_vertices, const double* coords,
                            int64_t num_cells, const int32_t* cell_verts);

/* Sizes: vertices, cells, faces, rows (n*F, Solver::getDofs, Solver.hpp:560-569)
 * and non-zeros of the face system (the row capacities, Solver.hpp:449-484).
 * Any output pointer may be NULL. */
mhfem_status mhfem_get_sizes(mhfem_t h, int64_t* V, int64_t* C, int64_t* F,
                             int64_t* rows, int64_t* nnz);

/* Topology as built (getCellsForFace / getFacesForCell, mesh_helpers.h:49-160):
 * face_verts [F][vertices per face] (sorted vertex ids: d for simplices,
 * 2^(d-1) for boxes), face_cells [F][2] (ascending, -1 on the boundary),
 * cell_faces [C][faces per cell] (d+1 or 2d).  Any pointer may be NULL. */
mhfem_status mhfem_get_topology(mhfem_t h, int32_t* face_verts, int32_t* face_cells,
                                int32_t* cell_faces);

/* Replaces the model writing its coefficient arrays in Model::init
 * (HeatEquationModel.h:114-133).  count == 1 gives a uniform coefficient
 * (UniformCoefficient.h:8-52); otherwise count must equal the full size of
 * the layout listed beside the MHFEM_COEF_* identifier.  data may be host or
 * device memory (the copy is ordered on the handle's stream). */
mhfem_status mhfem_set_coeff(mhfem_t h, int32_t which, const double* data, int64_t count);

/* ---- model hooks (custom models) -----------------------------------------
 * The reference's models are compile-time C++ classes whose device
 * functions the Solver calls inside preIterate: updateNonLinearTerms per
 * cell before the mass-matrix update (Solver.hpp:616-625) and
 * updateVectorCoefficients after it (Solver.hpp:641-652); BaseModel's
 * preIterate / postIterate run around each step (BaseModel.h:147-166).
 * Here a model is host code that launches its own kernels: a hook is called
 * on the calling thread at a fixed point of the step with the handle's CUDA
 * stream, and updates the coefficient arrays on the device in place
 * (mhfem_coeff_device), reading the state (mhfem_array_device), with work
 * ordered on that stream.
 *  - MHFEM_HOOK_PRE_ITERATE is updateNonLinearTerms: the scalar
 *    coefficients (N, m, D, r, f) of this step, from the current state.
 *  - MHFEM_HOOK_VECTOR_COEFFICIENTS is updateVectorCoefficients: it runs
 *    after this step's b update (MHFEM_ARRAY_B holds the new b) and before
 *    upwinding, so the RT0 projections of u, w and a may read b, as in the
 *    reference.  With it registered the step launches the b update as a
 *    kernel of its own before the hook and the fused cell kernel after it;
 *    without it the cell kernel forms b and everything after it in one
 *    pass.  The cell kernel forms b again from D, so D changes belong in
 *    the PRE_ITERATE hook.
 *  - getBoundaryMobility (Solver.hpp:696) is the array MHFEM_COEF_M_BND
 *    (i*F+E), read on the inflow boundary faces by the mobility upwinding of
 *    the same step; a model with a time- or state-dependent boundary mobility
 *    rewrites it from either hook above (both run after the velocities v_iKe
 *    of the previous step's reconstruction and before the inflow test).
 *  - MHFEM_HOOK_POST_ITERATE runs after the reconstruction (BaseModel's
 *    postIterate).
 * Writes through these pointers bypass the host copies that mhfem_set_coeff
 * keeps: the learned form's static features keep the values last passed to
 * mhfem_set_coeff. */
typedef void (*mhfem_hook)(void* user, double t, double tau, void* stream);
#define MHFEM_HOOK_PRE_ITERATE          0  /* start of mhfem_pre_iterate, before the b update */
#define MHFEM_HOOK_POST_ITERATE         1  /* end of mhfem_post_iterate, after the reconstruction */
#define MHFEM_HOOK_VECTOR_COEFFICIENTS  2  /* after the b update, before upwinding (Solver.hpp:641-652) */
/* fn == NULL removes the hook. */
mhfem_status mhfem_set_hook(mhfem_t h, int32_t point, mhfem_hook fn, void* user);
/* The device array of a coefficient as currently stored (count 1: uniform,
 * a single value; pass a full array to mhfem_set_coeff first to make it
 * per-cell).  Asking for MHFEM_COEF_A or MHFEM_COEF_U switches the explicit
 * advection terms on for every later step (exact zeros leave the results
 * unchanged). */
mhfem_status mhfem_coeff_device(mhfem_t h, int32_t which, double** data, int64_t* count);
/* The device array of a scheme or state array (MHFEM_ARRAY_*).
 * Pointers from these two calls stay valid until the next mhfem_set_mesh,
 * mhfem_set_coeff of the same coefficient with another count, or
 * mhfem_destroy; MHFEM_ARRAY_RHS also moves when the linear system is set
 * up again (mhfem_setup_linear_system, or new boundary tags). */
mhfem_status mhfem_array_device(mhfem_t h, int32_t which, double** data, int64_t* count);

/* Time-modulated source (a model hook of updateNonLinearTerms,
 * Solver.hpp:616-625): before each step at time t,
 *   f_iK = f_base_iK + amplitude * sin(2*pi*t/period) * psi_K,
 * with f_base the MHFEM_COEF_F array and psi the MHFEM_COEF_PSI array.
 * amplitude == 0 switches it off. */
mhfem_status mhfem_set_source_modulation(mhfem_t h, double amplitude, double period);

/* Replaces BoundaryConditions::init from a BoundaryConditionsStorage
 * (BoundaryConditions.hpp:224-233; Solver.hpp:264-293).  Each array holds
 * n*F entries, index i*F + E. */
mhfem_status mhfem_set_bc(mhfem_t h, const uint8_t* tags, const double* values,
                          const double* dirichlet_values);

/* Replaces Solver::setInitialCondition (Solver.hpp:260-344): sets Z_iK
 * ((i,K), n*C values) and initializes Z_iF as the average of the adjacent
 * cells (Solver.hpp:319-339) and v_iKe = 0. */
mhfem_status mhfem_set_initial_condition(mhfem_t h, const double* Z_iK);

/* Sets both state arrays explicitly: a restart from saved Z_iK and Z_iF (the
 * reference restarts from the initial-condition file, Solver.hpp:296-306,
 * and averages Z_iF from it); Z_iF may be NULL: that face average. */
mhfem_status mhfem_set_state(mhfem_t h, const double* Z_iK, const double* Z_iF);

/* Replaces Solver::setup's solver selection (Solver.hpp:88-258) and the
 * iterative-solver keys of configSetup.h:32-62. */
mhfem_status mhfem_set_solver(mhfem_t h, const mhfem_solver_opts* opts);

/* Replaces Solver::setupLinearSystem (Solver.hpp:351-484): builds the fixed
 * sparsity pattern of the face system from the topology and the BC tags. */
mhfem_status mhfem_setup_linear_system(mhfem_t h);

/* ---- one time step (control.h:83-98) ------------------------------------ */

mhfem_status mhfem_pre_iterate(mhfem_t h, double t, double tau);     /* Solver.hpp:596-892  */
mhfem_status mhfem_assemble(mhfem_t h, double t, double tau);        /* Solver.hpp:894-962  */
mhfem_status mhfem_solve(mhfem_t h, mhfem_step_stats* stats);        /* Solver.hpp:979-1266 */
mhfem_status mhfem_post_iterate(mhfem_t h, double t, double tau);    /* Solver.hpp:1268-1324 */
/* All four phases; stats may be NULL. */
mhfem_status mhfem_step(mhfem_t h, double t, double tau, mhfem_step_stats* stats);

/* ---- results ------------------------------------------------------------ */

/* Z_iF (n*F, (E,i)) and Z_iK (n*C, (i,K)); either may be NULL.  What a
 * model's makeSnapshot reads (HeatEquationModel.h:164-231). */
mhfem_status mhfem_get_state(mhfem_t h, double* Z_iF, double* Z_iK);
/* One of the scheme arrays of BaseModel (BaseModel.h:280-286), MHFEM_ARRAY_*;
 * count must be its size. */
mhfem_status mhfem_get_array(mhfem_t h, int32_t which, double* out, int64_t count);

/* The assembled system in CSR (rowptr has rows+1 entries), with the unit
 * diagonal included, columns ascending in each row exactly as the
 * reference's row setters emit them (LinearSystem.h:66-256,
 * BoundaryConditions.hpp:132-222).  cols and vals hold nnz entries and rhs
 * rows entries (mhfem_get_sizes).  Any pointer may be NULL. */
mhfem_status mhfem_get_system(mhfem_t h, int64_t* rowptr, int32_t* cols, double* vals,
                              double* rhs);

/* The FP32 copy of the matrix values that the mixed form (and the learned
 * form's mixed solve) assembles beside the FP64 one: nnz entries in the CSR
 * order of mhfem_get_system, the unit diagonal as 1.0f; each value is the
 * FP64 value rounded to nearest (ties to even).  No counterpart in the
 * reference, whose matrix is FP64 only. */
mhfem_status mhfem_get_system32(mhfem_t h, float* vals32);

/* Cumulative counters as in Solver::writeEpilog (Solver.hpp:1326-1391),
 * plus the number of kernels this library launched on the handle. */
mhfem_status mhfem_get_totals(mhfem_t h, int64_t* iterations, int64_t* time_steps,
                              int64_t* kernel_launches);

/* ---- measurement (replaces the per-phase TNL::Timer of Solver.h:132-138) -- */

/* The handle's CUDA stream (a cudaStream_t), so a caller can record CUDA
 * events on the stream the kernels run on. */
mhfem_status mhfem_get_stream(mhfem_t h, void** stream);

/* Kernels that mhfem_time_kernel can time. */
#define MHFEM_KERNEL_CELL_LOCAL   0   /* fused b / R / Q^-1 R / local Schur records */
#define MHFEM_KERNEL_ASSEMBLE     1   /* face-row assembly */
#define MHFEM_KERNEL_SPMV_FP64    2   /* BiCGStab SpMV fused with a dot product, FP64 */
#define MHFEM_KERNEL_SPMV_FP32    3   /* the same in FP32 (mixed form) */
#define MHFEM_KERNEL_RECONSTRUCT  4   /* Z_iK (and v_iKe) reconstruction */
#define MHFEM_KERNEL_SPMV2_FP64       5   /* BiCGStab second SpMV fused with (t, s), (t, t), FP64 */
#define MHFEM_KERNEL_UPDATE_S_FP64    6   /* BiCGStab s = r - alpha v, FP64 */
#define MHFEM_KERNEL_UPDATE_XR_FP64   7   /* BiCGStab x += alpha p + omega s, r = s - omega t, (rh, r), FP64 */
#define MHFEM_KERNEL_UPDATE_P_FP64    8   /* BiCGStab p = r + beta (p - omega v), FP64 */

/* Times `reps` back-to-back launches of one kernel on the current system
 * with CUDA events on the handle's stream (after a step has run) and returns
 * the mean duration, the algorithmic bytes one launch must move (each array
 * counted once at its size) and its FP64 (or FP32) operation count.  The
 * Krylov kernels run on the solver's Krylov work vectors (overwritten; the
 * next solve initializes them again); the state Z_iF, Z_iK is left as it is. */
mhfem_status mhfem_time_kernel(mhfem_t h, int32_t kernel, int32_t reps, double* ms_per_launch,
                               double* bytes_per_launch, double* flops_per_launch);

/* Check of the bounded grid barrier that the small-system FP64 BiCGStab
 * (systems of at most 2^18 rows, one cooperative launch per solve) places
 * between its phases.  One cooperative launch of `ctas` CTAs on `device`
 * passes through the barrier once, every wait polling at most `max_polls`
 * times; CTA `skip_cta` (none if negative) never arrives, so the others'
 * waits run out, set the failure flag and return -- the kernel ends without
 * a fault or a hang and the context stays usable.  Returns the CTAs that
 * passed and that gave up, and the flag (the solve turns it into
 * MHFEM_ERR_CUDA).  The launch allocates a few bytes of device memory. */
mhfem_status mhfem_check_grid_barrier(int32_t device, int32_t ctas, int32_t skip_cta, int32_t max_polls,
                                      int32_t* ctas_passed, int32_t* ctas_gave_up, int32_t* failure_flag);

/* ---- learned warm start (MHFEM_FORM_LEARNED) ----------------------------
 * No counterpart in the reference: a message-passing network over the face
 * adjacency graph (3 layers, hidden width 64, BF16 weights, FP32
 * accumulation on the tensor cores) predicts the initial guess of each
 * solve (FP64 BiCGStab, or with `mixed_solve` the mixed-precision
 * refinement) as a correction to the polynomial extrapolation in time of the
 * last traces (order `extrapolation_order`, as far as the history reaches).
 * Of the previous-step warm start, the extrapolated base and the network's
 * guess, the one with the lowest relative residual starts the solve; the
 * solve always runs to the same FP64 tolerance.  The network is trained
 * online on the first `train_steps` steps, or takes parameters from
 * mhfem_learned_set_params.  Only n_eq = 1 and simplex cells are supported. */
typedef struct {
    int32_t train_steps;          /* online training steps (default 200)            */
    int32_t train_iters;          /* Adam iterations per training step (default 2)  */
    double  learning_rate;        /* Adam step size (default 1e-3)                  */
    int32_t use_during_training;  /* 1: also try the guess while still training     */
    uint64_t seed;                /* initial weights (0 keeps the current ones)     */
    double  lr_final;             /* learning rate at the last training step, as a
                                     fraction of learning_rate, reached by a cosine
                                     decay over the training steps (1: constant)     */
    int32_t mixed_solve;          /* 1: solve from the guess with the mixed-precision
                                     refinement of MHFEM_FORM_MIXED (FP32 inner
                                     BiCGStab, FP64 residuals, the same FP64
                                     tolerance) instead of FP64 BiCGStab; the handle
                                     then also keeps the FP32 copy of the matrix      */
    int32_t extrapolation_order;  /* 0 to 3: the base the network corrects, the polynomial
                                     extrapolation of the last order + 1 traces in time
                                     (0: the warm start itself; 1: 2 Zn - Zn1; 3: cubic) */
} mhfem_learned_opts;

#define MHFEM_LEARNED_FEATURES 16
mhfem_status mhfem_learned_set_options(mhfem_t h, const mhfem_learned_opts* opts);
/* FP32 master parameters, flat: W0 [16][64], b0 [64], then W_l [128][64], b_l [64]
 * for l = 1..3, then wd [64], bd [1]. */
mhfem_status mhfem_learned_get_params(mhfem_t h, float* params, int64_t count);
/* Parameters from elsewhere (e.g. a network trained on an earlier run of the
 * same model): the guess is tried from the next step on, trained or not. */
mhfem_status mhfem_learned_set_params(mhfem_t h, const float* params, int64_t count);
/* Network output for given features [F][16] on the handle's face graph. */
mhfem_status mhfem_learned_forward(mhfem_t h, const float* features, float* out);
/* Loss mean((out - target)^2) over the non-Dirichlet faces and its gradient
 * with respect to every parameter (layout as mhfem_learned_get_params). */
mhfem_status mhfem_learned_gradients(mhfem_t h, const float* features, const double* target, float* grads,
                                     double* loss);
mhfem_status mhfem_learned_status(mhfem_t h, int32_t* trained_steps, double* last_loss, int32_t* num_params);

/* ---- allocation-free solve -------------------------------------------------
 * No counterpart in the reference.  For callers whose device memory belongs
 * to their own pool allocator (a framework that hands out every buffer from
 * a pre-reserved arena and cannot have a library call cudaMalloc/cudaFree,
 * which bypass its accounting and synchronize the device): FP64 BiCGStab on
 * a caller-owned unit-diagonal system in the layout this library assembles
 * (ELL of the off-diagonal part, [width][rows], padding column = own row).
 * cols, vals, rhs and x are DEVICE pointers; x holds the initial guess and
 * receives the solution; stream is a cudaStream_t (NULL: default stream).
 * Every column index must lie in [0, rows): one pass checks them before the
 * solve and a system with any other index is refused with
 * MHFEM_ERR_INVALID_ARGUMENT (nothing else runs).
 * All work vectors live in one static device array of fixed size (about
 * 17 MB), so systems with more than MHFEM_NOALLOC_MAX_ROWS rows are
 * rejected with MHFEM_ERR_INVALID_ARGUMENT.  Under CUDA's default lazy module
 * loading that array is committed on a device at the FIRST call there (which
 * looks its address up with cudaGetSymbolAddress and may synchronize the
 * device), not when the library is loaded, and it stays until the process
 * exits: a pool-allocator user makes one warm-up call during its own
 * initialization, before any stream capture.  Every call shares the array:
 * calls that overlap on the GPU (other streams, other threads) race and must
 * be serialized by the caller.
 * The solve is the persistent small-system BiCGStab that mhfem_solve runs
 * for systems of this size (one cooperative launch per chunk of up to 256
 * iterations, the convergence test in every iteration), so the two entry
 * points return the same iterates.
 * The call blocks until the solve ends: at most max_iter iterations, and at
 * most timeout_s seconds of wall-clock time when timeout_s > 0 (checked
 * between chunks, after the queued work has drained; then
 * MHFEM_ERR_TIMEOUT).  Returns MHFEM_OK, MHFEM_ERR_NOT_CONVERGED,
 * MHFEM_ERR_BREAKDOWN or MHFEM_ERR_NOT_FINITE like mhfem_solve, and
 * MHFEM_ERR_CUDA if a grid barrier wait of the solve ran out (no fault: the
 * context stays usable).  *residual is the relative residual ||b - Ax|| /
 * ||b|| of the last iteration: on MHFEM_ERR_TIMEOUT that of the last
 * completed chunk. */
#define MHFEM_NOALLOC_MAX_ROWS 262144
mhfem_status mhfem_bicgstab_noalloc(const int32_t* cols, const double* vals, int32_t width, int64_t rows,
                                    const double* rhs, double* x, double tol, int32_t max_iter, double timeout_s,
                                    int32_t* iterations, double* residual, void* stream);

#ifdef __cplusplus
}
#endif
#endif
