// In-place assembly of the hybridized face-trace system (sm_103a).
//
// One thread owns one row (E, i) (row index E*n + i, BaseModel.h:252-263),
// so the fixed pattern is filled without atomics.  The interior row follows
// LinearSystem::setMatrixElements (LinearSystem.h:66-256) and
// RightHandSide::getValue (RightHandSide.h:18-45); boundary rows follow
// BoundaryConditions::setMatrixElements (BoundaryConditions.hpp:335-508).
//
// Storage: every row is scaled to a unit diagonal (LinearSystem.h:196-201),
// so the diagonal is implicit and only the off-diagonal part is stored, in
// ELL form [slot][row] (column-major across rows: a warp's loads of one slot
// are one contiguous 256-byte segment).  The merged, ascending face order of
// the reference's row setters is precomputed once per mesh as a 4-bit
// position per (side, local face) ("qmap", one 32-bit word per face for
// up to 4 faces per cell, one 64-bit word for the 6 faces of a cuboid), so
// the kernel does no sorting.
// The local Schur entries come from the per-(cell, local face) records that
// k_cell_local wrote; each record is read by exactly one row.
#include <type_traits>

#include "fp_convert.h"
#include "mhfem_internal.h"

namespace mhfem {

// W32: also write the FP32 copy of the values (mixed form), rounded to
// nearest on the integer pipes (fp_convert.h): the hardware conversion issues
// on the FP64 pipe, which the row scaling already keeps busy.
template <int NF>
using QmapWord = std::conditional_t<(NF > 4), uint64_t, uint32_t>;

template <int NF, int NE, bool W32>
__global__ void __launch_bounds__(256) k_assemble(const DevProblem P, const QmapWord<NF>* __restrict__ qmap,
                                                  const uint8_t* __restrict__ qdiag, int W,
                                                  double* __restrict__ vals, float* __restrict__ vals32,
                                                  double* __restrict__ rhs)
{
    constexpr int RL = NE * NF + 1;
    const int64_t rows = P.rows;
    const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= rows) return;
    const int64_t E = row / NE;
    const int i = (int)(row - E * NE);
    const int2 kk = __ldg(&P.face_cells[E]);
    const int e0 = __ldg(P.face_local + 2 * E);
    const int e1 = __ldg(P.face_local + 2 * E + 1);
    const QmapWord<NF> qm = __ldg(qmap + E);
    const int dslot = __ldg(qdiag + E) * NE + i;

    auto put = [&](int q, int j, double v) {
        const int idx = q * NE + j;
        const int k = idx - (idx > dslot ? 1 : 0);
        vals[(int64_t)k * rows + row] = v;
        if constexpr (W32) vals32[(int64_t)k * rows + row] = f64_to_f32_rn(v);  // integer pipes, not FP64
    };
    // A record is read by one row only, but the 32-byte sectors it spans are
    // shared with the neighbouring records of the same cell, which other rows
    // read a little earlier or later: ordinary caching keeps those sectors in
    // L2 between the reads.  The stride is even, so records start on 16 bytes.
    auto rec_ptr = [&](int64_t K, int e) { return P.rec + ((K * NF + e) * NE + i) * (int64_t)P.rec_stride; };
    auto load_rec = [&](const double* rec, double (&A)[RL]) {
#pragma unroll
        for (int q = 0; q + 1 < RL; q += 2) {
            const double2 v = __ldg(reinterpret_cast<const double2*>(rec + q));
            A[q] = v.x;
            A[q + 1] = v.y;
        }
        if constexpr (RL % 2) A[RL - 1] = __ldg(rec + RL - 1);
    };

    if (kk.y < 0) {
        const int64_t bidx = (int64_t)i * P.F + E;
        const int tag = P.bc_tags[bidx];
        if (tag == MHFEM_BC_FIXED_VALUE) {
            rhs[row] = P.bc_dirichlet[bidx];  // BoundaryConditions.hpp:367-376
            return;
        }
        double A[RL];
        const double* r0 = rec_ptr(kk.x, e0);
        load_rec(r0, A);
        // the entries at run-time positions are re-read from the record (an
        // L1 hit), which keeps A in registers and costs no FP64 selects
        const double diag = __ldg(r0 + i * NF + e0);
        if (!positive_bits(diag)) atomicOr(P.err_flags, 1);
        const double rd = recip_newton(diag);
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const int q = (int)((qm >> (4 * f)) & 15u);
#pragma unroll
            for (int j = 0; j < NE; ++j) {
                if (j == i && f == e0) continue;
                put(q, j, A[j * NF + f] * rd);
            }
        }
        double bval = 0;
        if (tag != MHFEM_BC_ADVECTIVE_OUTFLOW) bval = -P.bc_values[bidx] * P.face_measure[E];
        bval += A[NE * NF];
        rhs[row] = bval * rd;
        return;
    }

    double A0[RL], A1[RL];
    const double* r0 = rec_ptr(kk.x, e0);
    const double* r1 = rec_ptr(kk.y, e1);
    load_rec(r0, A0);
    load_rec(r1, A1);
    // column e1 of the K1 record and the diagonal, re-read from the records
    // (L1 hits) at their run-time positions
    double a1e[NE];
#pragma unroll
    for (int j = 0; j < NE; ++j) a1e[j] = __ldg(r1 + j * NF + e1);
    const double diag = __ldg(r0 + i * NF + e0) + __ldg(r1 + i * NF + e1);
    if (!positive_bits(diag)) atomicOr(P.err_flags, 1);
    const double rd = recip_newton(diag);
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        const int q = (int)((qm >> (4 * f)) & 15u);
#pragma unroll
        for (int j = 0; j < NE; ++j) {
            if (f == e0) {
                if (j == i) continue;  // the unit diagonal (LinearSystem.h:196-201)
                put(q, j, (A0[j * NF + f] + a1e[j]) * rd);
            }
            else
                put(q, j, A0[j * NF + f] * rd);
        }
    }
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        if (f == e1) continue;
        const int q = (int)((qm >> (4 * (NF + f))) & 15u);
#pragma unroll
        for (int j = 0; j < NE; ++j) put(q, j, A1[j * NF + f] * rd);
    }
    rhs[row] = (A0[NE * NF] + A1[NE * NF]) * rd;
}

int launch_assemble(const DevProblem& P, const AssemblyMap& M, EllMatrix& A, double* rhs,
                    int write32, cudaStream_t s)
{
    if (P.rows == 0) return 0;
    const unsigned grid = (unsigned)((P.rows + 255) / 256);
#define MHFEM_ASSEMBLE_NF(NFV, W32, V32)                                                             \
    do {                                                                                             \
        if (P.n == 1) k_assemble<NFV, 1, W32><<<grid, 256, 0, s>>>(P, (const QmapWord<NFV>*)M.qmap, M.qdiag, A.width, A.vals, V32, rhs); \
        else if (P.n == 2) k_assemble<NFV, 2, W32><<<grid, 256, 0, s>>>(P, (const QmapWord<NFV>*)M.qmap, M.qdiag, A.width, A.vals, V32, rhs); \
        else k_assemble<NFV, 3, W32><<<grid, 256, 0, s>>>(P, (const QmapWord<NFV>*)M.qmap, M.qdiag, A.width, A.vals, V32, rhs); \
    } while (0)
#define MHFEM_ASSEMBLE(W32, V32)                          \
    do {                                                  \
        if (P.nf == 3) MHFEM_ASSEMBLE_NF(3, W32, V32);    \
        else if (P.nf == 4) MHFEM_ASSEMBLE_NF(4, W32, V32); \
        else MHFEM_ASSEMBLE_NF(6, W32, V32);              \
    } while (0)
    if (write32) MHFEM_ASSEMBLE(true, A.vals32);
    else MHFEM_ASSEMBLE(false, nullptr);
#undef MHFEM_ASSEMBLE
#undef MHFEM_ASSEMBLE_NF
    return 1;
}

}  // namespace mhfem
