// Stand-alone block-Jacobi PCG on a caller's 3x3-block CSR matrix (device pointers): the
// reference's bsm::solve_pcg (extern/BlockedSparseMatrix/include/BlockedSparseMatrix/solve_pcg.h:83)
// together with the block-diagonal preconditioner set-up that precedes it in
// NewtonsMethod::_solve_linear_system (symx/src/solver/NewtonsMethod.cpp:427-446).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace symxg {

// Outcome of one solve; the fields of bsm::PCGInfo (solve_pcg.h:21-27) plus the number of
// block rows that had no diagonal block (the solve does not start when it is nonzero).
struct BcsrPcgResult {
    int converged = 0;
    int iterations = 0;
    int indefinite = 0;
    int missing_diagonal = 0;
    double error = 0.0;
};

// Workspace of run_bcsr_pcg, in order, each part starting on a 256-byte boundary: the
// solver state (256 bytes), the completion tickets (8 unsigned), the reduction partials
// (2 x partials_per_part doubles), the preconditioner (12 values per block row) and six
// vectors (4 values per block row: x, r, z, p, p2, q).
constexpr size_t bcsr_pcg_round_up(size_t n) { return (n + 255) / 256 * 256; }
constexpr size_t bcsr_pcg_workspace_size(size_t n_blocks, size_t partials_per_part, size_t value_bytes)
{
    return 256 + bcsr_pcg_round_up(8 * 4) + bcsr_pcg_round_up(2 * partials_per_part * 8) +
           bcsr_pcg_round_up(12 * n_blocks * value_bytes) + 6 * bcsr_pcg_round_up(4 * n_blocks * value_bytes);
}

// Bytes of workspace run_bcsr_pcg needs for n_blocks block rows, with room for
// `partials_per_part` per-block partial sums per reduction (at least pcg_max_grid()).
template <typename T>
size_t bcsr_pcg_workspace_bytes(int n_blocks, unsigned partials_per_part)
{
    return bcsr_pcg_workspace_size(n_blocks < 0 ? 0 : (size_t)n_blocks, partials_per_part, sizeof(T));
}

// Solves A x = b, x starting at zero (the reference's Newton step passes a zero initial guess,
// NewtonsMethod.cpp:431-432), with PCG and a block-Jacobi preconditioner.  A: n_blocks block
// rows, row_ptr/cols int32, values component-major (component m of block k at
// vals[m * vals_stride + k]); b and x hold 3 values per block row.  Stops when
// sqrt(r.r / b.b) < abs_tol, when that error falls below rel_tol times its initial value, on
// p.Ap <= 0, or after max_iterations.  `workspace` (16-byte aligned, `workspace_bytes` long)
// holds every vector, the preconditioner, the reduction partials, the completion tickets and
// the solver state; nothing is allocated.  The call reads the state back to the host between
// chunks of iterations, so it returns with `s` synchronized.
template <typename T>
BcsrPcgResult run_bcsr_pcg(int n_blocks, const int32_t* row_ptr, const int32_t* cols, const T* vals,
                           int64_t vals_stride, const T* b, T* x, double abs_tol, double rel_tol, int max_iterations,
                           void* workspace, size_t workspace_bytes, unsigned partials_per_part, cudaStream_t s);

// run_bcsr_pcg<float> on a static device array instead of a caller's workspace, for callers
// that cannot allocate device memory (see bcsr_pcg_noalloc.cu for the rules of use).  At most
// bcsr_pcg_noalloc_max_blocks() block rows.
int bcsr_pcg_noalloc_max_blocks();
BcsrPcgResult run_bcsr_pcg_noalloc_f32(int n_blocks, const int32_t* row_ptr, const int32_t* cols, const float* vals,
                                       int64_t vals_stride, const float* b, float* x, double abs_tol, double rel_tol,
                                       int max_iterations, cudaStream_t s);

}  // namespace symxg
