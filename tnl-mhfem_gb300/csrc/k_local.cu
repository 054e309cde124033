// Launchers of the cell- and face-local kernels; the triangle and
// tetrahedron instances (the box instances are in k_local_box.cu).
#include "cell_kernels.cuh"

namespace mhfem {

int launch_cell_local(const DevProblem& P, double tau, cudaStream_t s)
{
    if (P.C == 0) return 0;
    const double src_scale = P.src_amp * sin(P.src_omega * P.src_time);
    if (P.cell) return launch_cell_local_box(P, 1.0 / tau, src_scale, s);
    const unsigned grid = blocks_for(P.C, 128);
    if (P.nf == 3) MHFEM_NE_DISPATCH(CT_TRI, P.n, (k_cell_local<CT, NE><<<grid, 128, 0, s>>>(P, 1.0 / tau, src_scale)));
    else MHFEM_NE_DISPATCH(CT_TET, P.n, (k_cell_local<CT, NE><<<grid, 128, 0, s>>>(P, 1.0 / tau, src_scale)));
    return 1;
}

int launch_update_b(const DevProblem& P, cudaStream_t s)
{
    if (P.C == 0) return 0;
    if (P.cell) return launch_update_b_box(P, s);
    const unsigned grid = blocks_for(P.C, 128);
    if (P.nf == 3) MHFEM_NE_DISPATCH(CT_TRI, P.n, (k_update_b<CT, NE><<<grid, 128, 0, s>>>(P)));
    else MHFEM_NE_DISPATCH(CT_TET, P.n, (k_update_b<CT, NE><<<grid, 128, 0, s>>>(P)));
    return 1;
}

// k_upwind depends on the number of faces per cell only: rectangles share
// the tetrahedron instances (4 faces), cuboids have their own.
int launch_upwind(const DevProblem& P, cudaStream_t s)
{
    if (P.F == 0 || !(P.mobility_upwind || P.explicit_adv_active)) return 0;
    if (P.nf == 6) return launch_upwind_cuboid(P, s);
    const unsigned grid = blocks_for(P.F, 256);
    if (P.nf == 3) MHFEM_NE_DISPATCH(CT_TRI, P.n, (k_upwind<NF, NE><<<grid, 256, 0, s>>>(P)));
    else MHFEM_NE_DISPATCH(CT_TET, P.n, (k_upwind<NF, NE><<<grid, 256, 0, s>>>(P)));
    return 1;
}

int launch_reconstruct(const DevProblem& P, cudaStream_t s)
{
    if (P.C == 0) return 0;
    if (P.cell) return launch_reconstruct_box(P, s);
    const unsigned grid = blocks_for(P.C, 256);
    if (P.nf == 3) MHFEM_NE_DISPATCH(CT_TRI, P.n, (k_reconstruct<CT, NE><<<grid, 256, 0, s>>>(P)));
    else MHFEM_NE_DISPATCH(CT_TET, P.n, (k_reconstruct<CT, NE><<<grid, 256, 0, s>>>(P)));
    return 1;
}

int launch_face_average(const DevProblem& P, cudaStream_t s)
{
    if (P.F == 0) return 0;
    if (P.n == 1) k_face_average<1><<<blocks_for(P.F, 256), 256, 0, s>>>(P);
    else if (P.n == 2) k_face_average<2><<<blocks_for(P.F, 256), 256, 0, s>>>(P);
    else k_face_average<3><<<blocks_for(P.F, 256), 256, 0, s>>>(P);
    return 1;
}

}  // namespace mhfem
