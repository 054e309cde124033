// Rectangle and cuboid instances of the cell- and face-local kernels
// (MassMatrix<Quadrangle> / MassMatrix<Hexahedron>, MassMatrix.h:152-508).
#include "cell_kernels.cuh"

namespace mhfem {

int launch_cell_local_box(const DevProblem& P, double rtau, double src_scale, cudaStream_t s)
{
    const unsigned grid = blocks_for(P.C, 128);
    if (P.dim == 2) MHFEM_NE_DISPATCH(CT_RECT, P.n, (k_cell_local<CT, NE><<<grid, 128, 0, s>>>(P, rtau, src_scale)));
    else MHFEM_NE_DISPATCH(CT_CUBOID, P.n, (k_cell_local<CT, NE><<<grid, 128, 0, s>>>(P, rtau, src_scale)));
    return 1;
}

int launch_update_b_box(const DevProblem& P, cudaStream_t s)
{
    const unsigned grid = blocks_for(P.C, 128);
    if (P.dim == 2) MHFEM_NE_DISPATCH(CT_RECT, P.n, (k_update_b<CT, NE><<<grid, 128, 0, s>>>(P)));
    else MHFEM_NE_DISPATCH(CT_CUBOID, P.n, (k_update_b<CT, NE><<<grid, 128, 0, s>>>(P)));
    return 1;
}

int launch_upwind_cuboid(const DevProblem& P, cudaStream_t s)
{
    MHFEM_NE_DISPATCH(CT_CUBOID, P.n, (k_upwind<NF, NE><<<blocks_for(P.F, 256), 256, 0, s>>>(P)));
    return 1;
}

int launch_reconstruct_box(const DevProblem& P, cudaStream_t s)
{
    const unsigned grid = blocks_for(P.C, 256);
    if (P.dim == 2) MHFEM_NE_DISPATCH(CT_RECT, P.n, (k_reconstruct<CT, NE><<<grid, 256, 0, s>>>(P)));
    else MHFEM_NE_DISPATCH(CT_CUBOID, P.n, (k_reconstruct<CT, NE><<<grid, 256, 0, s>>>(P)));
    return 1;
}

}  // namespace mhfem
