// Host-side launchers of the hand-written device kernels of the solve path.
// All launches are asynchronous on the given stream; no launcher allocates.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace symxg {

// Number of kernels launched by this library since load (all handles, all streams).
int64_t launch_count();
void count_launch(int64_t n = 1);

// Device memory held by this library's own buffers (every cudaMalloc it makes for a solver,
// a Compiled<T> or a stand-alone PCG workspace), and its high-water mark since the last reset.
void note_device_alloc(int64_t bytes);
void note_device_free(int64_t bytes);
int64_t device_bytes_current();
int64_t device_bytes_peak(bool reset);

// Polls after which a bounded wait of the staged PCG kernels (a shared-memory stage's
// mbarrier, the persistent kernel's grid barrier) gives up and flags the solve
// (PcgState::wait_failed).  Process-wide, read at each launch; the default is
// kDefaultWaitPolls.  A small value makes the waits run out on purpose, which is how the
// error path is tested.  The drain of a block's bulk copies in flight before it exits always
// uses the default, so a block never exits with a copy still writing its shared memory.
constexpr long long kDefaultWaitPolls = 1ll << 22;
void set_wait_poll_limit(long long polls);  // < 0: the default
long long wait_poll_limit();

// Device-resident state of one PCG solve (read by the host between chunks of iterations).
struct PcgState {
    double bb;        // b.b
    double rz;        // r.z of the current iterate
    double pAp;
    double rr;
    double alpha, beta;
    double error, error0;
    double abs_tol, rel_tol;
    int iteration;
    int max_iterations;
    int done;         // 1 once converged, failed or out of iterations
    int converged;
    int indefinite;
    int wait_failed;  // 1 if a bounded wait inside a kernel gave up (the solve is invalid)
    // One-launch FP32 PCG: every replace_every iterations (0: never) the launch returns
    // unfinished and k_pcg_replace_residual replaces the recursive residual by b - A x
    // accumulated in FP64; `replacements` counts them.
    int replace_every;
    int replacements;
};

// Deterministic reductions: each launch uses a fixed grid, every block sums a fixed
// contiguous range, and the last block to finish combines the block partials in index
// order.  `partials` holds kReduceBlocks doubles, `ticket` one unsigned int (zeroed).
constexpr int kReduceBlocks = 304;  // 2 x 152 SMs
constexpr int kReduceThreads = 256;

// out[0] = sum(x[0..n))
void launch_sum(const double* x, int64_t n, double* partials, unsigned* ticket, double* out, cudaStream_t s);
// out[0] = max |x[i]|
void launch_max_abs(const double* x, int64_t n, double* partials, unsigned* ticket, double* out, cudaStream_t s);
// out[0] = sum a[i]*b[i] with a in T, b in double
template <typename T>
void launch_dot_mixed(const T* a, const double* b, int64_t n, double* partials, unsigned* ticket, double* out,
                      cudaStream_t s);

// Element-Hessian projection, in place, block-major storage, `count` matrices of N x N.
// not_converged: one int, set to 1 if any matrix hit the sweep cap.  With scratch (12 x 12
// only: `fallback` holds `count` indices, `n_fallback` one counter), translation-invariant
// matrices are projected in the 9-dimensional complement of the rigid translations and the
// others with the full decomposition in a second launch; without it, every matrix takes the
// full decomposition.
// 12 x 12 projection lists (each sized for every matrix of one launch): matrices that are not
// translation-invariant (full decomposition), and, when given, translation-invariant ones
// whose deflated part is not positive definite (deflated decomposition in full warps).
struct ProjectionScratch {
    int64_t* fallback = nullptr;
    unsigned long long* n_fallback = nullptr;
    int64_t* pending = nullptr;
    unsigned long long* n_pending = nullptr;
};
// sel: when given, project the `count` matrices H[sel[k]] instead of H[0 .. count).
template <typename T>
void launch_project_pd(T* H, int N, int64_t count, T eps, bool mirroring, int* not_converged, cudaStream_t s,
                       ProjectionScratch scratch = ProjectionScratch{}, const int64_t* sel = nullptr);

// 12 x 12 projection whose arithmetic is FP64-accurate for float or double storage: the
// sorting pass, then for the listed matrices an FP32 cyclic Jacobi refined by one FP64
// Ogita-Aishima step, the clamping applied as an FP64 correction and rounded once into H
// (symxg_dev::project_pd_refined).  Needs the sorting pass's lists in `scratch`.
template <typename T>
void launch_project_pd_refined12(T* H, int64_t count, double eps, bool mirroring, int* not_converged, cudaStream_t s,
                                 ProjectionScratch scratch, const int64_t* sel = nullptr);

// Progressive projection: flag (gflag[gblock] = 1) the element gradient blocks of the DoF
// blocks with max |grad| >= thr, counting the other blocks in *n_inactive; then list the
// elements of one potential not projected yet that touch a flagged block (all unprojected
// ones when gflag is null), marking them.
void launch_ppn_mark_blocks(int n_blocks, const double* grad, double thr, const int64_t* gptr, const int32_t* gcontrib,
                            uint8_t* gflag, unsigned long long* n_inactive, cudaStream_t s);
void launch_select_elements(int64_t n_el, int nb, const uint8_t* gflag, uint8_t* is_proj, int64_t* sel,
                            unsigned long long* n_sel, cudaStream_t s);

// BCSR values are stored component-major: component m (row-major inside the 3x3 block) of
// block k is vals[m * vstride + k], vstride >= nnzb.  vstride == kTiledBcsr selects the
// solver's tiled layout instead: tiles of 32 blocks, each nine component rows of 32 values,
// component m of block k at vals[(k / 32) * 288 + m * 32 + k % 32] (9 * nnzb rounded up to a
// whole tile).
constexpr int64_t kTiledBcsr = -1;
//
// Assembly: block s = sum over c in [slot_ptr[s], slot_ptr[s+1]) of blocks[contrib[c]]
// (element blocks: 9 consecutive values, row-major), summed in that fixed order.
template <typename T>
void launch_assemble_blocks(int64_t nnzb, const int64_t* slot_ptr, const int32_t* contrib, const T* blocks, T* vals,
                            int64_t vstride, cudaStream_t s);
// Gradient: g[3v+d] = sum over c in [ptr[v], ptr[v+1]) of gel[3*contrib[c]+d].
void launch_gather_gradient(int n_blocks, const int64_t* ptr, const int32_t* contrib, const double* gel, double* g,
                            cudaStream_t s);

// Block-Jacobi: Dinv[r] = inverse of the diagonal block vals[diag_slot[r]] (computed in
// double, stored as T).
template <typename T>
void launch_block_jacobi_setup(int n_blocks, const int32_t* diag_slot, const T* vals, int64_t vstride, T* Dinv,
                               cudaStream_t s);

// PCG over a 3x3-block CSR matrix (row_ptr/cols/vals), block-Jacobi preconditioner.
// Vectors in T, dot products accumulated in double, scalars in `state`.
// PCG vectors (x, r, z, p, p2, q) hold 4 values per block row (x, y, z, 0); Dinv holds
// the inverse diagonal blocks as 3 rows of 4 (12 values per block row).
template <typename T>
struct PcgBuffers {
    int n_blocks;
    const int32_t* row_ptr;
    const int32_t* cols;
    const T* vals;      // component-major with stride vals_stride, or tiled (vals_stride == kTiledBcsr)
    int64_t vals_stride;
    const T* Dinv;
    T* x;
    T* r;
    T* z;
    T* p;               // search directions, ping-pong between p and p2 across iterations
    T* p2;
    T* q;
    // Look-ahead PCG (float, k_pcg_solve_la; null: not used): six more vectors of 4 * n_blocks
    // values each, one after the other: z of the second gather set, mw = M^-1 A z of both
    // sets, mq = M^-1 q of both sets, w = A z.  z of the first set is `z` above.
    T* la = nullptr;
    double* partials;   // kPcgPartials doubles x 2
    unsigned* tickets;  // counters: 16 for the persistent kernel, 8 otherwise
    PcgState* state;
    // Staged SpMV (float, strided layout only; stages == 0: not used).  The producer copies
    // each stage's rows with bulk copies, which read these padded copies of row_ptr and cols.
    struct Staged {
        int stages = 0;          // shared-memory stages per block
        int stage_rows = 0;      // rows per stage (4 per consumer warp)
        int stage_cap = 0;       // values per component slot in a stage (multiple of 4)
        int rows_per_block = 0;  // multiple of stage_rows
        int grid = 0;
        size_t smem_bytes = 0;
        int persistent = 0;      // 1: the whole PCG loop can run as one cooperative launch
        int lookahead = 0;       // 1: ... also as the look-ahead form (k_pcg_solve_la), used when `la` is set
        size_t la_smem_bytes = 0;  // dynamic shared memory of the look-ahead form
        long long max_polls = kDefaultWaitPolls;  // set from wait_poll_limit() at each launch
        // one-launch PCG: chunk and block partials of p.Ap, r.r, r.z summed in FP64 (1) or in
        // float-float (0); the per-thread and per-warp sums are float-float in both
        int f64_sums = 1;
        const int32_t* row_ptr_ext = nullptr;  // row_ptr, then nnzb repeated to grid * rows_per_block + stage_rows + 8
        const int32_t* cols_ext = nullptr;     // cols, padded with zeros to a multiple of 4 plus 4
    } staged;
};
constexpr int kPcgMaxPartials = 1 << 16;

// Residual replacement of the one-launch FP32 PCG when it returned unfinished (no-op once the
// solve is done): r = b - A x with b = -grad, the products and sums in FP64 and r rounded once
// to float, z = M^-1 r, then r.r and r.z in FP64, the convergence test on the true residual,
// beta = r.z / r.z_old.  The next launch of the one-launch PCG continues from there.
void launch_pcg_replace_residual(const PcgBuffers<float>& B, const double* grad, cudaStream_t s);


// Set x = 0, r = b (b = -grad converted to T), z = M^-1 r, bb, rz, error0.
template <typename T>
void launch_pcg_init(const PcgBuffers<T>& B, const double* neg_rhs_source, cudaStream_t s);
// PCG iteration number `iteration` (0-based, counted on the host): the SpMV kernel forms the
// direction p = z + beta p_old in the ping-pong buffer and q = A p with p.q, the update kernel
// x, r, z with r.r and r.z.  Both are no-ops once state->done is set.
template <typename T>
void launch_pcg_iteration(const PcgBuffers<T>& B, int iteration, cudaStream_t s);
// The two launches of launch_pcg_iteration, separately (for per-kernel timing).
template <typename T>
void launch_pcg_spmv(const PcgBuffers<T>& B, int iteration, cudaStream_t s);
template <typename T>
void launch_pcg_update(const PcgBuffers<T>& B, int iteration, cudaStream_t s);

// y = A x over a 3x3-block CSR matrix with component-major values (the PCG's product, as a
// stand-alone launch).
template <typename T>
void launch_bcsr_spmv(int n_blocks, const int32_t* row_ptr, const int32_t* cols, const T* vals, int64_t vstride,
                      const T* x, T* y, cudaStream_t s);

// PCG on a right-hand side b with 3 values per block row (instead of a double gradient).
template <typename T>
void launch_pcg_init_rhs(const PcgBuffers<T>& B, const T* b3, cudaStream_t s);
// out3[3i+d] = in4[4i+d]
template <typename T>
void launch_rows4_to_vec3(int n_rows, const T* in4, T* out3, cudaStream_t s);
// Largest grid any PCG kernel launches with (the number of per-block partials it writes).
unsigned pcg_max_grid();

// Plan of the staged (bulk-copy) PCG SpMV for a float matrix with n_blocks rows whose
// row_ptr (host copy) is given: fills everything in `st` but the two device pointers, and
// returns the lengths the padded row_ptr and cols copies need (0, 0 when the staged kernel
// cannot run on this device or matrix, which then keeps the plain kernel).
struct StagedSizes {
    int64_t row_ptr_ext = 0, cols_ext = 0;
};
StagedSizes plan_staged_spmv(int n_blocks, const int32_t* row_ptr_host, PcgBuffers<float>::Staged& st);

// All PCG iterations (after launch_pcg_init) in one cooperative launch of the staged kernel:
// runs until convergence, p.Ap <= 0 or state->max_iterations, then sets state->done.  Only
// when B.staged.persistent; uses tickets[6..10] (cleared here): its grid barrier and the
// chunk counters of its dynamically scheduled product passes.
void launch_pcg_solve_persistent(const PcgBuffers<float>& B, cudaStream_t s);

// On the PCG solution du (4 values per block row) and double vectors with 3 per row:
// out = du . g;  out = max |du|;  x_out = x0 + step * du.
template <typename T>
void launch_dot_rows4(const T* du, const double* g, int n_rows, double* partials, unsigned* ticket, double* out,
                      cudaStream_t s);
template <typename T>
void launch_max_abs_rows4(const T* du, int n_rows, double* partials, unsigned* ticket, double* out, cudaStream_t s);
template <typename T>
void launch_axpy_rows4(int n_rows, const double* x0, double step, const T* du, double* x_out, cudaStream_t s);
// x_out = x0 + step * du (du in T, x in double)
template <typename T>
void launch_axpy_to(int64_t n, const double* x0, double step, const T* du, double* x_out, cudaStream_t s);
// y = (double) x
template <typename T>
void launch_convert_to_double(int64_t n, const T* x, double* y, cudaStream_t s);

}  // namespace symxg
