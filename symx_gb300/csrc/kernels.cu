// Hand-written device kernels of the second-order solve path (sm_103a).
//
// Reference loops they replace:
//   projection   symx/src/solver/second_order/ElementHessians.cpp:48-67 + project_to_PD.cpp:12-81
//   assembly     ElementHessians.cpp:224-256 + BlockedSparseMatrix.h:780-895 (mutex-per-row insertion)
//   gradient     SecondOrderCompiledPotential.cpp:158-169 + ParallelVector.h:185-197
//   reductions   ParallelNumber.h:129-137, bsm_vector_ops.h:52-225
//   SpMV         BlockedSparseMatrix.h:986-1138
//   block Jacobi BlockedSparseMatrix.h:1146-1361
//   PCG          solve_pcg.h:82-232
// Every sum here is taken in a fixed order (no floating-point atomics), so results are
// bitwise reproducible run to run.
#include "kernels.cuh"
#include "project_pd.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <type_traits>
#include <map>
#include <unordered_map>
#include <stdexcept>
#include <string>

namespace symxg {

namespace {

constexpr int kWarp = 32;

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide reduction of one value per thread (fixed tree order); result valid in thread 0.
template <bool IsMax>
__device__ double block_reduce(double v, double* sh)
{
    const int lane = threadIdx.x & (kWarp - 1), warp = threadIdx.x / kWarp;
    const int nwarps = (blockDim.x + kWarp - 1) / kWarp;
    v = IsMax ? warp_max(v) : warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = (lane < nwarps) ? sh[lane] : (IsMax ? 0.0 : 0.0);
        v = IsMax ? warp_max(v) : warp_sum(v);
    }
    return v;
}

// Store this block's partial; the last block to arrive combines all partials in index
// order and returns true in every one of its threads (result in *result of thread 0).
// `nparts` partial arrays of gridDim.x doubles each are handled together.
template <bool IsMax, int NPARTS>
__device__ bool last_block_combine(const double (&mine)[NPARTS], double* partials, unsigned* ticket,
                                   double (&result)[NPARTS])
{
    __shared__ double sh[32];
    __shared__ bool is_last;
    double blockv[NPARTS];
#pragma unroll
    for (int k = 0; k < NPARTS; ++k) blockv[k] = block_reduce<IsMax>(mine[k], sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NPARTS; ++k) partials[k * gridDim.x + blockIdx.x] = blockv[k];
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NPARTS; ++k) {
        double acc = 0.0;
        for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
            const double p = __ldcg(&partials[k * gridDim.x + i]);
            acc = IsMax ? fmax(acc, p) : acc + p;
        }
        result[k] = block_reduce<IsMax>(acc, sh);
    }
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

__device__ __forceinline__ void chunk_range(int64_t n, int64_t& begin, int64_t& end)
{
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    begin = chunk * blockIdx.x;
    end = begin + chunk < n ? begin + chunk : n;
}

__global__ void k_sum(const double* __restrict__ x, int64_t n, double* partials, unsigned* ticket, double* out)
{
    int64_t b, e;
    chunk_range(n, b, e);
    double acc = 0.0;
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) acc += x[i];
    double mine[1] = {acc}, res[1];
    if (last_block_combine<false, 1>(mine, partials, ticket, res) && threadIdx.x == 0) out[0] = res[0];
}

template <typename T>
__global__ void k_max_abs(const T* __restrict__ x, int64_t n, double* partials, unsigned* ticket, double* out)
{
    int64_t b, e;
    chunk_range(n, b, e);
    double acc = 0.0;
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const double v = (double)x[i];
        acc = fmax(acc, isnan(v) ? __longlong_as_double(0x7ff0000000000000LL) : fabs(v));
    }
    double mine[1] = {acc}, res[1];
    if (last_block_combine<true, 1>(mine, partials, ticket, res) && threadIdx.x == 0) out[0] = res[0];
}

template <typename T>
__global__ void k_dot_mixed(const T* __restrict__ a, const double* __restrict__ bv, int64_t n, double* partials,
                            unsigned* ticket, double* out)
{
    int64_t b, e;
    chunk_range(n, b, e);
    double acc = 0.0;
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) acc += (double)a[i] * bv[i];
    double mine[1] = {acc}, res[1];
    if (last_block_combine<false, 1>(mine, partials, ticket, res) && threadIdx.x == 0) out[0] = res[0];
}

// ---------------------------------------------------------------- projection
template <typename T, int N>
__global__ void __launch_bounds__(128) k_project_pd_unrolled(T* __restrict__ H, int64_t count, T eps, int mirroring,
                                                             int* not_converged, const int64_t* __restrict__ sel)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int64_t m = sel ? sel[k] : k;
    int nc = 0;
    T* h = H + m * (N * N);
    // Tet4-sized matrices of translation-invariant energies: 9 x 9 decomposition (the
    // scratch-free form of k_project_pd_deflated + k_project_pd_listed).
    if constexpr (N == 12) {
        if (symxg_dev::project_pd_deflated<T, N / 3>(h, eps, mirroring != 0, &nc) >= 0) {
            if (nc) *not_converged = 1;
            return;
        }
    }
    if constexpr (std::is_same<T, float>::value && N % 2 == 0)
        symxg_dev::project_pd_inplace_packed<N>(h, eps, mirroring != 0, &nc);
    else
        symxg_dev::project_pd_inplace<T, N>(h, eps, mirroring != 0, &nc);
    if (nc) *not_converged = 1;
}

// Translation-deflated projection (project_pd_deflated) of every matrix whose translation
// residual is rounding noise; the others are left unchanged and their indices appended to
// `fallback` (count in *n_fallback, zeroed before the launch) for k_project_pd_listed.
template <typename T, int N>
__global__ void __launch_bounds__(128) k_project_pd_deflated(T* __restrict__ H, int64_t count, T eps, int mirroring,
                                                             int* not_converged, int64_t* __restrict__ fallback,
                                                             unsigned long long* n_fallback,
                                                             const int64_t* __restrict__ sel)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int64_t m = sel ? sel[k] : k;
    int nc = 0;
    if (symxg_dev::project_pd_deflated<T, N / 3>(H + m * (N * N), eps, mirroring != 0, &nc) < 0)
        fallback[atomicAdd(n_fallback, 1ull)] = m;
    if (nc) *not_converged = 1;
}

// Sorting pass of the 12 x 12 projection: matrices whose deflated part is positive definite
// are done (left as they are: the projection would only lift their translation eigenvalues
// to eps); the others are listed, translation-invariant ones in `pending` for
// k_project_pd_deflated_listed and the rest in `fallback` for k_project_pd_listed (counts
// zeroed before the launch), so the eigen-decompositions run in full warps.
template <typename T, int N>
__global__ void __launch_bounds__(128) k_project_pd_sort(const T* __restrict__ H, int64_t count,
                                                         int64_t* __restrict__ fallback, unsigned long long* n_fallback,
                                                         const int64_t* __restrict__ sel, int64_t* __restrict__ pending,
                                                         unsigned long long* n_pending)
{
    constexpr int M = N - 3;
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int64_t m = sel ? sel[k] : k;
    T b[M * (M + 1) / 2];
    if (!symxg_dev::deflate_translations<T, N / 3>(H + m * (N * N), b)) fallback[atomicAdd(n_fallback, 1ull)] = m;
    else if (!symxg_dev::positive_definite_by_cholesky<T, M>(b)) pending[atomicAdd(n_pending, 1ull)] = m;
}

// The deflated eigen-decomposition of the matrices k_project_pd_sort listed as pending
// (grid-stride over the list).
template <typename T, int N>
__global__ void __launch_bounds__(128) k_project_pd_deflated_listed(T* __restrict__ H, const int64_t* __restrict__ list,
                                                                    const unsigned long long* n_list, T eps,
                                                                    int mirroring, int* not_converged)
{
    constexpr int M = N - 3;
    const int64_t n = (int64_t)*n_list;
    int nc = 0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        T* h = H + list[k] * (N * N);
        T b[M * (M + 1) / 2];
        if (symxg_dev::deflate_translations<T, N / 3>(h, b))
            symxg_dev::project_deflated_finish<T, N / 3>(h, b, eps, mirroring != 0, &nc);
    }
    if (nc) *not_converged = 1;
}

// Full projection of the matrices listed by k_project_pd_deflated (grid-stride over the list).
template <typename T, int N>
__global__ void __launch_bounds__(128) k_project_pd_listed(T* __restrict__ H, const int64_t* __restrict__ list,
                                                           const unsigned long long* n_list, T eps, int mirroring,
                                                           int* not_converged)
{
    const int64_t n = (int64_t)*n_list;
    int nc = 0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        T* h = H + list[k] * (N * N);
        if constexpr (std::is_same<T, float>::value && N % 2 == 0)
            symxg_dev::project_pd_inplace_packed<N>(h, eps, mirroring != 0, &nc);
        else
            symxg_dev::project_pd_inplace<T, N>(h, eps, mirroring != 0, &nc);
    }
    if (nc) *not_converged = 1;
}

// FP64-accurate projection (symxg_dev::project_pd_refined: FP32 Jacobi, one FP64 refinement
// step, clamping applied as an FP64 correction) of the matrices k_project_pd_sort listed,
// grid-stride over the list.  Deflate: the `pending` list (translation-invariant matrices),
// otherwise the `fallback` list (full decomposition).  One thread per matrix; the kernel is
// bound by the FP64 pipe, so a small block keeps the per-thread arrays in L1.
template <typename S, int N, bool Deflate>
__global__ void __launch_bounds__(64) k_project_pd_refined_listed(S* __restrict__ H, const int64_t* __restrict__ list,
                                                                  const unsigned long long* n_list, double eps,
                                                                  int mirroring, int* not_converged)
{
    const int64_t n = (int64_t)*n_list;
    int nc = 0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        symxg_dev::project_pd_refined<S, N / 3, Deflate>(H + list[k] * (N * N), eps, mirroring != 0, &nc);
    if (nc) *not_converged = 1;
}

// Progressive projection (NewtonsMethod.cpp:305-329): flag the element gradient blocks of
// every DoF block whose gradient max-abs is at least thr (gflag zeroed before); counts the
// other blocks in *n_inactive.
__global__ void k_ppn_mark_blocks(int n_blocks, const double* __restrict__ grad, double thr,
                                  const int64_t* __restrict__ gptr, const int32_t* __restrict__ gcontrib,
                                  uint8_t* __restrict__ gflag, unsigned long long* n_inactive)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_blocks) return;
    const double m = fmax(fabs(grad[3 * v]), fmax(fabs(grad[3 * v + 1]), fabs(grad[3 * v + 2])));
    if (!(m >= thr)) {
        atomicAdd(n_inactive, 1ull);
        return;
    }
    for (int64_t c = gptr[v]; c < gptr[v + 1]; ++c) gflag[gcontrib[c]] = 1;
}

// Elements of one potential not projected yet in this evaluation and touching a flagged
// gradient block (every unprojected one when gflag is null), as
// ElementHessians::_project_to_PD_for_update selects them (ElementHessians.cpp:104-131): marked
// projected and appended to sel (count in *n_sel).  The list order varies from run to run;
// each element's projection does not depend on it.
__global__ void k_select_elements(int64_t n_el, int nb, const uint8_t* __restrict__ gflag, uint8_t* __restrict__ is_proj,
                                  int64_t* __restrict__ sel, unsigned long long* n_sel)
{
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_el || is_proj[e]) return;
    bool take = gflag == nullptr;
    for (int a = 0; a < nb && !take; ++a) take = gflag[e * nb + a] != 0;
    if (!take) return;
    is_proj[e] = 1;
    sel[atomicAdd(n_sel, 1ull)] = e;
}

// Generic N (up to 30) with thread-private arrays; used for the element matrices the
// specialised kernels do not cover (Tet10: 30 x 30).
template <typename T>
__global__ void __launch_bounds__(64) k_project_pd_generic(T* __restrict__ H, int N, int64_t count, T eps,
                                                           int mirroring, int* not_converged,
                                                           const int64_t* __restrict__ sel)
{
    constexpr int NMAX = 30;
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int64_t m = sel ? sel[k] : k;
    T* h = H + m * (int64_t)N * N;
    const int nb = N / 3;
    auto bm = [nb](int i, int j) { return (((i / 3) * nb + (j / 3)) * 3 + (i % 3)) * 3 + (j % 3); };
    T A[NMAX * NMAX], V[NMAX * NMAX];
    T fro2 = T(0);
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
            const T v = h[bm(i, j)];
            A[i * NMAX + j] = v;
            V[i * NMAX + j] = (i == j) ? T(1) : T(0);
            fro2 += v * v;
        }
    int sweep = 0;
    for (; sweep < (2 * symxg_dev::JacobiTol<T>::max_double_sweeps); ++sweep) {
        T off = T(0);
        for (int p = 0; p < N; ++p)
            for (int q = p + 1; q < N; ++q) off += T(2) * A[p * NMAX + q] * A[p * NMAX + q];
        if (!(off > symxg_dev::JacobiTol<T>::rel2() * fro2)) break;
        for (int p = 0; p < N - 1; ++p)
            for (int q = p + 1; q < N; ++q) {
                const T apq = A[p * NMAX + q];
                if (apq == T(0)) continue;
                const T app = A[p * NMAX + p], aqq = A[q * NMAX + q];
                const T tau = (aqq - app) / (T(2) * apq);
                const T t = (tau >= T(0) ? T(1) : T(-1)) / (fabs(tau) + sqrt(T(1) + tau * tau));
                const T c = T(1) / sqrt(T(1) + t * t), s = t * c;
                for (int k = 0; k < N; ++k) {
                    const T akp = A[k * NMAX + p], akq = A[k * NMAX + q];
                    A[k * NMAX + p] = c * akp - s * akq;
                    A[k * NMAX + q] = s * akp + c * akq;
                }
                for (int k = 0; k < N; ++k) {
                    const T apk = A[p * NMAX + k], aqk = A[q * NMAX + k];
                    A[p * NMAX + k] = c * apk - s * aqk;
                    A[q * NMAX + k] = s * apk + c * aqk;
                }
                A[p * NMAX + q] = A[q * NMAX + p] = T(0);
                for (int k = 0; k < N; ++k) {
                    const T vkp = V[k * NMAX + p], vkq = V[k * NMAX + q];
                    V[k * NMAX + p] = c * vkp - s * vkq;
                    V[k * NMAX + q] = s * vkp + c * vkq;
                }
            }
    }
    if (sweep == (2 * symxg_dev::JacobiTol<T>::max_double_sweeps)) *not_converged = 1;
    bool changed = false;
    for (int i = 0; i < N; ++i) {
        T l = A[i * NMAX + i];
        if (l < eps) { changed = true; l = mirroring ? -l : eps; }
        A[i * NMAX + i] = l;
    }
    if (!changed) return;
    for (int i = 0; i < N; ++i)
        for (int j = i; j < N; ++j) {
            T s = T(0);
            for (int k = 0; k < N; ++k) s += V[i * NMAX + k] * A[k * NMAX + k] * V[j * NMAX + k];
            h[bm(i, j)] = s;
            h[bm(j, i)] = s;
        }
}

// Large element matrices (24 x 24 for Hex8): one warp per matrix, parallel cyclic Jacobi in
// the round-robin ("circle method") order: a sweep is N - 1 rounds of N / 2 disjoint index
// pairs, and one round applies all N / 2 rotations at once, A <- J^T A J with J block diagonal
// over the pairs.  Written per 2 x 2 block of pairs (k, l) this is B_kl <- R_k^T B_kl R_l, so
//   * lane k < N / 2 forms pair k's rotation from its diagonal block (same formula and
//     convergence test as the register kernels), updates that block in place and publishes
//     (c, s) in shared memory;
//   * the N/2 (N/2 - 1) / 2 off-diagonal blocks of the upper triangle are spread over the
//     lanes; each lane reads its four entries, applies both rotations and writes them back,
//     with the entry offsets of every round taken from a per-block table in shared memory;
//   * lane i keeps row i of the eigenvector matrix V in registers, its columns held in "slot"
//     order: in every round pair k occupies slots (2k, 2k + 1), and the round-robin step from
//     one round to the next is a fixed permutation of the slots (a rotation of the N - 1
//     moving ones), so the round loop stays rolled (the kernel fits the instruction cache)
//     while every register index is a compile-time constant.  After N - 1 rounds the slots
//     are back in their initial order, slot_index() below.
// Only the upper triangle of A in shared memory is kept up to date.  No two lanes touch the
// same entry within a round.
template <typename T, int N>
struct ProjPairsCfg {
    static constexpr int warps = sizeof(T) == 4 ? 8 : 4;
    // 24 x 24 float: 64 registers, 32 warps per SM; 30 x 30 (Tet10) holds 30 eigenvector
    // entries per lane and ~90 KB of shared memory per block: two blocks per SM
    static constexpr int min_blocks = N <= 24 ? 4 : 2;
    static constexpr int LD = N + 1;  // row stride of A and B (odd: conflict-free columns)
    static constexpr int VS = (N + 3) / 4 * 4;  // row stride of V in the reconstruction (16-byte rows)
    static constexpr int NP = N / 2, NR = N - 1, NOFF = NP * (NP - 1) / 2, SLOTS = (NOFF + 31) / 32;
    static constexpr int mat_elems = N * LD > N * VS ? N * LD : N * VS;
    // dynamic shared memory: A and B per warp, (c, s) per warp, the offset table
    static constexpr size_t off_B = (size_t)warps * mat_elems * sizeof(T);
    static constexpr size_t off_CS = off_B + (size_t)warps * mat_elems * sizeof(T);
    static constexpr size_t off_tab = (off_CS + (size_t)warps * NP * 2 * sizeof(T) + 15) / 16 * 16;
    static constexpr size_t smem_bytes = off_tab + (size_t)NR * SLOTS * 32 * sizeof(uint2);
};

// Pair k of round r as (a, b): position N - 1 is fixed, the others rotate.
template <int N>
__host__ __device__ __forceinline__ void rr_pair(int r, int k, int& a, int& b)
{
    a = r + k;
    if (a >= N - 1) a -= N - 1;
    b = N - 1;
    if (k != 0) {
        b = r - k + N - 1;
        if (b >= N - 1) b -= N - 1;
    }
}

// Index held by V slot s at the start of every sweep: pair k of round 0 is (k, N - 1 - k).
template <int N>
__host__ __device__ constexpr int slot_index(int s)
{
    return (s & 1) ? N - 1 - s / 2 : s / 2;
}

// Off-diagonal block b of the upper triangle over pairs, as (k, l), k < l (row-major order).
template <int NP>
__device__ __forceinline__ void off_block(int b, int& k, int& l)
{
    k = 0;
    l = 0;
    for (int kk = 0; kk < NP; ++kk) {
        const int n = NP - 1 - kk;
        if (b < n) {
            k = kk;
            l = kk + 1 + b;
            return;
        }
        b -= n;
    }
}

template <typename T>
struct Pair2;
template <>
struct Pair2<float> {
    using type = float2;
};
template <>
struct Pair2<double> {
    using type = double2;
};

// sum_{k < N} w[k] * row[k] with 16-byte shared-memory loads (row 16-byte aligned, padded
// to a multiple of 4 floats / 2 doubles)
template <int N>
__device__ __forceinline__ float row_dot(const float (&w)[N], const float* row)
{
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < N; k += 4) {
        const float4 r = *reinterpret_cast<const float4*>(row + k);
        acc = fmaf(w[k], r.x, acc);
        if (k + 1 < N) acc = fmaf(w[k + 1 < N ? k + 1 : k], r.y, acc);
        if (k + 2 < N) acc = fmaf(w[k + 2 < N ? k + 2 : k], r.z, acc);
        if (k + 3 < N) acc = fmaf(w[k + 3 < N ? k + 3 : k], r.w, acc);
    }
    return acc;
}
template <int N>
__device__ __forceinline__ double row_dot(const double (&w)[N], const double* row)
{
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < N; k += 2) {
        const double2 r = *reinterpret_cast<const double2*>(row + k);
        acc = fma(w[k], r.x, acc);
        if (k + 1 < N) acc = fma(w[k + 1 < N ? k + 1 : k], r.y, acc);
    }
    return acc;
}

template <typename T>
__device__ __forceinline__ T warp_allmax(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Warp test of one N x N element Hessian A (shared memory, row stride N + 1): true when A is
// translation-invariant (max |A t| <= tol max |A|) and Q^T A Q (Q the Helmert basis of the
// node space orthogonal to (1, ..., 1), (x) I3) has a Cholesky factorization with pivots above
// 16 M u of its largest diagonal entry.  A is then positive definite in the complement of the
// translations up to rounding, and the reference's projection would only lift the three
// translation eigenvalues from 0 to eps, a change below the rounding of A's entries.  B (the
// same shape) is scratch; every decision is taken by all lanes alike.
template <typename T, int N>
__device__ bool pairs_pd_shortcut(const T* __restrict__ A, T* __restrict__ B, int lane)
{
    constexpr int LD = N + 1, NB = N / 3, M = N - 3;
    // rows of A Q (lane i < N: row i): prefix sums over the node blocks; the full sums are
    // the translation residual of the row
    T amax = T(0), res = T(0);
    if (lane < N) {
        T acc[3] = {T(0), T(0), T(0)};
#pragma unroll
        for (int m = 0; m < NB; ++m)
#pragma unroll
            for (int e = 0; e < 3; ++e) {
                const T a = A[lane * LD + 3 * m + e];
                amax = fmax(amax, fabs(a));
                if (m >= 1) B[lane * LD + 3 * (m - 1) + e] = (acc[e] - T(m) * a) / sqrt(T(m * (m + 1)));
                acc[e] += a;
            }
        res = fmax(fabs(acc[0]), fmax(fabs(acc[1]), fabs(acc[2])));
    }
    amax = warp_allmax(amax);
    res = warp_allmax(res);
    if (!(res <= symxg_dev::DeflationTol<T>::value() * amax)) return false;
    __syncwarp();
    // columns of Q^T (A Q) (lane c < M: column c), written over rows 0 .. M-1 of the same column
    if (lane < M) {
        T acc[3] = {T(0), T(0), T(0)};
#pragma unroll
        for (int m = 0; m < NB; ++m)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const T t = B[(3 * m + d) * LD + lane];
                if (m >= 1) B[(3 * (m - 1) + d) * LD + lane] = (acc[d] - T(m) * t) / sqrt(T(m * (m + 1)));
                acc[d] += t;
            }
    }
    __syncwarp();
    // Cholesky (lower triangle, in place): lane i holds row i
    const T dmax = warp_allmax(lane < M ? B[lane * LD + lane] : T(0));
    const T tau = T(16 * M) * symxg_dev::UnitRoundoff<T>::value() * dmax;
    for (int j = 0; j < M; ++j) {
        const T d = B[j * LD + j];  // the same value in every lane
        if (!(d > tau)) return false;
        const T r = T(1) / sqrt(d);
        const bool mine = lane > j && lane < M;
        const T lij = mine ? B[lane * LD + j] * r : T(0);
        __syncwarp();
        if (mine) B[lane * LD + j] = lij;
        __syncwarp();
        if (mine)
            for (int k = j + 1; k <= lane; ++k) B[lane * LD + k] -= lij * B[k * LD + j];
        __syncwarp();
    }
    return true;
}

template <typename T, int N>
__global__ void __launch_bounds__(ProjPairsCfg<T, N>::warps * 32, ProjPairsCfg<T, N>::min_blocks)
    k_project_pd_pairs(T* __restrict__ H, int64_t count, T eps, int mirroring, int* not_converged,
                       const int64_t* __restrict__ sel)
{
    static_assert(N % 6 == 0 && N <= 30, "N a multiple of 6 up to 30 (3 x 3 blocks, pairs of indices)");
    using T2 = typename Pair2<T>::type;
    using Cfg = ProjPairsCfg<T, N>;
    constexpr int W = Cfg::warps, LD = Cfg::LD, VS = Cfg::VS;
    constexpr int NP = Cfg::NP, NR = Cfg::NR, NOFF = Cfg::NOFF, SLOTS = Cfg::SLOTS, nb = N / 3;
    // dynamic shared memory (Cfg::smem_bytes): per warp A and a deflated copy B (the
    // positive-definiteness test), (c, s) of the round's rotations, and per round, slot and
    // lane the 4 x 16-bit entry offsets of an off-diagonal pair block
    extern __shared__ __align__(16) unsigned char pairs_smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T* sA = reinterpret_cast<T*>(pairs_smem) + (size_t)w * Cfg::mat_elems;
    T* sB = reinterpret_cast<T*>(pairs_smem + Cfg::off_B) + (size_t)w * Cfg::mat_elems;
    T2* sCS = reinterpret_cast<T2*>(pairs_smem + Cfg::off_CS) + (size_t)w * NP;
    uint2* sTab = reinterpret_cast<uint2*>(pairs_smem + Cfg::off_tab);  // [NR][SLOTS][32]

    for (int e = threadIdx.x; e < NR * SLOTS * 32; e += blockDim.x) {
        const int r = e / (SLOTS * 32), j = (e / 32) % SLOTS, ln = e % 32, b = ln + 32 * j;
        uint2 v = make_uint2(0u, 0u);
        if (b < NOFF) {
            int k, l, ak, bk, al, bl;
            off_block<NP>(b, k, l);
            rr_pair<N>(r, k, ak, bk);
            rr_pair<N>(r, l, al, bl);
            auto up = [](int i, int jj) { return (unsigned)(i < jj ? i * LD + jj : jj * LD + i); };
            v.x = up(ak, al) | (up(ak, bl) << 16);
            v.y = up(bk, al) | (up(bk, bl) << 16);
        }
        sTab[(r * SLOTS + j) * 32 + ln] = v;
    }
    int bk[SLOTS], bl[SLOTS];
#pragma unroll
    for (int j = 0; j < SLOTS; ++j) off_block<NP>(lane + 32 * j < NOFF ? lane + 32 * j : 0, bk[j], bl[j]);
    __syncthreads();

    T* A = sA;
    T2* CS = sCS;
    int nc = 0;
    constexpr int max_sweeps = 2 * symxg_dev::JacobiTol<T>::max_double_sweeps;
    for (int64_t item = (int64_t)blockIdx.x * W + w; item < count; item += (int64_t)gridDim.x * W) {
        T* h = H + (sel ? sel[item] : item) * (int64_t)(N * N);
        T f = T(0);
        for (int idx = lane; idx < N * N; idx += 32) {  // block-major storage, read in order
            const int blk = idx / 9, r = idx % 9;
            const int i = (blk / nb) * 3 + r / 3, j = (blk % nb) * 3 + r % 3;
            const T v = h[idx];
            A[i * LD + j] = v;
            f += v * v;
        }
        __syncwarp();
        if (pairs_pd_shortcut<T, N>(A, sB, lane)) continue;  // H stays as it is
        T v[N];
#pragma unroll
        for (int s = 0; s < N; ++s) v[s] = lane == slot_index<N>(s) ? T(1) : T(0);
        // every lane takes the same decisions below: sums are reduced, then lane 0's broadcast
        f = (T)__shfl_sync(0xffffffffu, warp_sum(f), 0);
        __syncwarp();
        int sweep = 0;
        for (; sweep < max_sweeps; ++sweep) {
            T off = T(0);
            for (int idx = lane; idx < N * N; idx += 32) {
                const int i = idx / N, j = idx % N;
                if (i < j) off += A[i * LD + j] * A[i * LD + j];
            }
            off = T(2) * (T)__shfl_sync(0xffffffffu, warp_sum(off), 0);
            if (!(off > symxg_dev::JacobiTol<T>::rel2() * f)) break;
#pragma unroll 1
            for (int r = 0; r < NR; ++r) {
                if (lane < NP) {
                    int p, q;
                    rr_pair<N>(r, lane, p, q);
                    const int pq = p < q ? p * LD + q : q * LD + p;
                    const T app = A[p * LD + p], aqq = A[q * LD + q], apq = A[pq];
                    const T t = symxg_dev::jacobi_t(app, aqq, apq);
                    const T c = symxg_dev::inv_hypot1(t);
                    A[p * LD + p] = app - t * apq;
                    A[q * LD + q] = aqq + t * apq;
                    A[pq] = T(0);
                    T2 cs;
                    cs.x = c;
                    cs.y = t * c;
                    CS[lane] = cs;
                }
                __syncwarp();
#pragma unroll
                for (int j = 0; j < SLOTS; ++j) {
                    if ((j + 1) * 32 <= NOFF || lane + 32 * j < NOFF) {
                        const uint2 e = sTab[(r * SLOTS + j) * 32 + lane];
                        const T2 rk = CS[bk[j]], rl = CS[bl[j]];
                        const unsigned e00 = e.x & 0xffffu, e01 = e.x >> 16, e10 = e.y & 0xffffu, e11 = e.y >> 16;
                        const T b00 = A[e00], b01 = A[e01], b10 = A[e10], b11 = A[e11];
                        const T r00 = rk.x * b00 - rk.y * b10, r01 = rk.x * b01 - rk.y * b11;  // rows of pair k
                        const T r10 = rk.y * b00 + rk.x * b10, r11 = rk.y * b01 + rk.x * b11;
                        A[e00] = rl.x * r00 - rl.y * r01;  // columns of pair l
                        A[e01] = rl.y * r00 + rl.x * r01;
                        A[e10] = rl.x * r10 - rl.y * r11;
                        A[e11] = rl.y * r10 + rl.x * r11;
                    }
                }
#pragma unroll
                for (int k = 0; k < NP; ++k) {  // eigenvector columns: pair k in slots (2k, 2k + 1)
                    const T2 cs = CS[k];
                    const T vp = v[2 * k], vq = v[2 * k + 1];
                    v[2 * k] = cs.x * vp - cs.y * vq;
                    v[2 * k + 1] = cs.y * vp + cs.x * vq;
                }
                // next round's slot order: new[2k] = old[2k + 2], new[N - 2] = old[N - 1],
                // new[3] = old[0], new[2k + 1] = old[2k - 1] (k >= 2), slot 1 fixed
                const T v0 = v[0];
#pragma unroll
                for (int k = 0; k < NP - 1; ++k) v[2 * k] = v[2 * k + 2];
                v[N - 2] = v[N - 1];
#pragma unroll
                for (int k = NP - 1; k >= 2; --k) v[2 * k + 1] = v[2 * k - 1];
                v[3] = v0;
                __syncwarp();
            }
        }
        if (sweep == max_sweeps) nc = 1;
        T lam = T(0);
        bool mine = false;
        if (lane < N) {
            lam = A[lane * LD + lane];
            if (lam < eps) {
                mine = true;
                lam = mirroring ? -lam : eps;
            }
        }
        const bool changed = __any_sync(0xffffffffu, mine);
        if (changed) {
            __syncwarp();  // eigenvalues read before V overwrites A
            // rows of V with stride VS (a multiple of 4) for 16-byte row reads
            if (lane < N) {
#pragma unroll
                for (int s = 0; s < N; ++s) A[lane * VS + s] = v[s];
            }
#pragma unroll
            for (int s = 0; s < N; ++s) v[s] *= __shfl_sync(0xffffffffu, lam, slot_index<N>(s));  // V diag(lambda)
            __syncwarp();
            if (lane < N) {
                const int i = lane, bi = (i / 3) * nb, ri = (i % 3) * 3;
                for (int j = 0; j < N; ++j) h[(bi + j / 3) * 9 + ri + j % 3] = row_dot<N>(v, A + j * VS);
            }
        }
        __syncwarp();  // the next matrix reuses this warp's shared memory
    }
    if (nc) *not_converged = 1;
}

// ---------------------------------------------------------------- BCSR value layouts
// Component m (row-major inside the 3x3 block) of block k is vals[base(k) + m * step()].
// Strided (the C ABI's): base = k, step = vstride (component-major arrays).
// Tiled (the solver's own): blocks in tiles of 32, each tile nine component rows of 32
// values, base = (k / 32) * 288 + k % 32, step = 32.  A warp's loads stay coalesced as in the
// strided form, but the blocks of consecutive rows lie in one contiguous span of memory
// (one DRAM stream per warp instead of nine), and the component offsets are constants.
struct StridedBcsr {
    int64_t vs;
    __host__ __device__ __forceinline__ int64_t base(int64_t k) const { return k; }
    __host__ __device__ __forceinline__ int64_t step() const { return vs; }
};
struct TiledBcsr {
    __host__ __device__ __forceinline__ int64_t base(int64_t k) const { return (k >> 5) * 288 + (k & 31); }
    __host__ __device__ __forceinline__ static constexpr int64_t step() { return 32; }
};

// ---------------------------------------------------------------- assembly
template <typename T, typename L>
__global__ void k_assemble_blocks(int64_t nnzb, const int64_t* __restrict__ slot_ptr, const int32_t* __restrict__ contrib,
                                  const T* __restrict__ blocks, T* __restrict__ vals, L lay)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nnzb) return;
    T acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = T(0);
    for (int64_t c = slot_ptr[s]; c < slot_ptr[s + 1]; ++c) {
        const T* b = blocks + (int64_t)contrib[c] * 9;
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[k] += b[k];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) vals[lay.base(s) + k * lay.step()] = acc[k];
}

__global__ void k_gather_gradient(int n_blocks, const int64_t* __restrict__ ptr, const int32_t* __restrict__ contrib,
                                  const double* __restrict__ gel, double* __restrict__ g)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_blocks) return;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int64_t c = ptr[v]; c < ptr[v + 1]; ++c) {
        const double* b = gel + (int64_t)contrib[c] * 3;
        a0 += b[0];
        a1 += b[1];
        a2 += b[2];
    }
    g[3 * v] = a0;
    g[3 * v + 1] = a1;
    g[3 * v + 2] = a2;
}

// ---------------------------------------------------------------- block Jacobi
// Dinv holds, per block row, the inverse diagonal block as three rows of four (the fourth
// entry zero), so the preconditioner is applied with three 16-byte (float) loads.
template <typename T, typename L>
__global__ void k_block_jacobi_setup(int n_blocks, const int32_t* __restrict__ diag_slot, const T* __restrict__ vals,
                                     L lay, T* __restrict__ Dinv)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_blocks) return;
    const int64_t k = diag_slot[r];
    // symmetric 3x3 inverse from the upper triangle (cofactors / determinant)
    const T* __restrict__ v = vals + lay.base(k);
    const int64_t st = lay.step();
    const double a = v[0], b = v[st], c = v[2 * st], d = v[4 * st], e = v[5 * st], f = v[8 * st];
    const double c00 = d * f - e * e, c01 = c * e - b * f, c02 = b * e - c * d;
    const double det = a * c00 + b * c01 + c * c02;
    const double id = 1.0 / det;
    const double i00 = c00 * id, i01 = c01 * id, i02 = c02 * id;
    const double i11 = (a * f - c * c) * id, i12 = (b * c - a * e) * id, i22 = (a * d - b * b) * id;
    T* o = Dinv + (int64_t)r * 12;
    o[0] = (T)i00; o[1] = (T)i01; o[2] = (T)i02; o[3] = T(0);
    o[4] = (T)i01; o[5] = (T)i11; o[6] = (T)i12; o[7] = T(0);
    o[8] = (T)i02; o[9] = (T)i12; o[10] = (T)i22; o[11] = T(0);
}

// ---------------------------------------------------------------- SpMV / PCG
constexpr int kSpmvThreads = 256;  // 16 rows per block, 16 lanes per row
// Resident blocks per SM the SpMV kernels are compiled for: the full 2048 threads in float
// (the kernels are latency-bound, so occupancy beats the few registers it costs).
template <typename T>
struct SpmvMinBlocks {
    static constexpr int value = sizeof(T) == 4 ? 8 : 4;
};

// PCG vectors hold one block row as four values (x, y, z, 0): a gathered block column is
// one 16-byte load (float) instead of three 4-byte loads spread over 12 bytes.
template <typename T>
struct Row4 {
    T x, y, z, w;
};
__device__ __forceinline__ Row4<float> ld4(const float* __restrict__ p)
{
    const float4 v = *reinterpret_cast<const float4*>(p);
    return Row4<float>{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ Row4<double> ld4(const double* __restrict__ p)
{
    const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
    return Row4<double>{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void st4(float* __restrict__ p, const Row4<float>& v)
{
    *reinterpret_cast<float4*>(p) = make_float4(v.x, v.y, v.z, v.w);
}
__device__ __forceinline__ void st4(double* __restrict__ p, const Row4<double>& v)
{
    reinterpret_cast<double2*>(p)[0] = make_double2(v.x, v.y);
    reinterpret_cast<double2*>(p)[1] = make_double2(v.z, v.w);
}

// BCSR values in either layout above: each component load of a half-warp reads 16
// consecutive values.
//
// Per-lane partial products of two block rows at once, each over the 16 lanes of its
// half-warp, lane-strided over the row's blocks; both rows' loads are in flight together.
// xv(c) is the multiplied vector's block row c.  half_warp_transpose_sum reduces the
// partials; every lane of the warp must call both (rows past the end pass valid = false), so
// the full-mask shuffles are converged.
// The product loop of two_row_products on explicit block ranges [kbA, keA) and [kbB, keB)
// of `cols` / `vals` (global arrays, or a shared-memory stage indexed from its first block).
template <typename T, typename L, typename XV>
__device__ __forceinline__ void two_range_products(int kbA, int keA, int kbB, int keB, int lane16,
                                                   const int32_t* __restrict__ cols, const T* __restrict__ vals, L lay,
                                                   XV xv, T (&a)[3], T (&b)[3])
{
    const int64_t st = lay.step();
    a[0] = a[1] = a[2] = b[0] = b[1] = b[2] = T(0);
    for (int i = lane16;; i += 16) {
        const int kA = kbA + i, kB = kbB + i;
        const bool hA = kA < keA, hB = kB < keB;
        if (!hA && !hB) break;
        if (hA) {
            const Row4<T> v = xv(cols[kA]);
            const T* __restrict__ m = vals + lay.base(kA);
            a[0] += m[0] * v.x + m[st] * v.y + m[2 * st] * v.z;
            a[1] += m[3 * st] * v.x + m[4 * st] * v.y + m[5 * st] * v.z;
            a[2] += m[6 * st] * v.x + m[7 * st] * v.y + m[8 * st] * v.z;
        }
        if (hB) {
            const Row4<T> v = xv(cols[kB]);
            const T* __restrict__ m = vals + lay.base(kB);
            b[0] += m[0] * v.x + m[st] * v.y + m[2 * st] * v.z;
            b[1] += m[3 * st] * v.x + m[4 * st] * v.y + m[5 * st] * v.z;
            b[2] += m[6 * st] * v.x + m[7 * st] * v.y + m[8 * st] * v.z;
        }
    }
}

template <typename T, typename L, typename XV>
__device__ __forceinline__ void two_row_products(int rowA, bool vA, int rowB, bool vB, int lane16,
                                                 const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ cols,
                                                 const T* __restrict__ vals, L lay, XV xv, T (&a)[3], T (&b)[3])
{
    const int kbA = vA ? row_ptr[rowA] : 0, keA = vA ? row_ptr[rowA + 1] : 0;
    const int kbB = vB ? row_ptr[rowB] : 0, keB = vB ? row_ptr[rowB + 1] : 0;
    two_range_products<T>(kbA, keA, kbB, keB, lane16, cols, vals, lay, xv, a, b);
}

// Sum the six per-lane partials (a[0..2] of row A, b[0..2] of row B) over the 16 lanes of a
// half-warp with a transposing butterfly: at each level a lane keeps half of its values and
// sends the other half, so 8 shuffles do what 24 would do lane-by-lane.  On return lanes
// 2i and 2i+1 of the half-warp hold the total of value i (0..2: row A, 3..5: row B, 6..7:
// zero padding), summed in a fixed order.
template <typename T>
__device__ __forceinline__ T half_warp_transpose_sum(const T (&a)[3], const T (&b)[3], int lane16)
{
    T v[8] = {a[0], a[1], a[2], b[0], b[1], b[2], T(0), T(0)};
    const bool up8 = (lane16 & 8) != 0;
    T w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const T send = up8 ? v[i] : v[i + 4];
        const T keep = up8 ? v[i + 4] : v[i];
        w[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8, 16);
    }
    const bool up4 = (lane16 & 4) != 0;
    T u[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const T send = up4 ? w[i] : w[i + 2];
        const T keep = up4 ? w[i + 2] : w[i];
        u[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4, 16);
    }
    const bool up2 = (lane16 & 2) != 0;
    const T send = up2 ? u[0] : u[1];
    const T keep = up2 ? u[1] : u[0];
    const T t = keep + __shfl_xor_sync(0xffffffffu, send, 2, 16);
    return t + __shfl_xor_sync(0xffffffffu, t, 1, 16);
}

// y = A x (x and y with 3 values per block row, the C ABI layout); each warp takes four
// block rows per pass (two per half-warp).
template <typename T, typename L>
__global__ void __launch_bounds__(kSpmvThreads, SpmvMinBlocks<T>::value)
    k_bcsr_spmv(int n_blocks, const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ cols,
                const T* __restrict__ vals, L lay, const T* __restrict__ x, T* __restrict__ y)
{
    const int lane16 = threadIdx.x & 15;
    const int half = (threadIdx.x >> 4) & 1;
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int warps_total = (gridDim.x * blockDim.x) >> 5;
    auto xv = [x](int c) { return Row4<T>{x[3 * c], x[3 * c + 1], x[3 * c + 2], T(0)}; };
    for (int base = 4 * warp_global; base < n_blocks; base += 4 * warps_total) {
        const int rowA = base + half, rowB = base + 2 + half;
        const bool vA = rowA < n_blocks, vB = rowB < n_blocks;
        T a[3], b[3];
        two_row_products<T>(rowA, vA, rowB, vB, lane16, row_ptr, cols, vals, lay, xv, a, b);
        const T sum = half_warp_transpose_sum<T>(a, b, lane16);
        const int idx = lane16 >> 1;  // 0..2 row A, 3..5 row B
        if (!(lane16 & 1) && idx < 6) {
            const int row = idx < 3 ? rowA : rowB;
            if (idx < 3 ? vA : vB) y[3 * row + idx % 3] = sum;
        }
    }
}

// ---- float-float (double-single) accumulation for the FP32 PCG's dot products.
// Error-free transformations on the FP32 pipe (TwoSum, FMA-based TwoProd); the __f*_rn
// intrinsics keep the compiler from contracting or reordering them.  Relative accuracy is
// about 2^-44, with no FP64 instruction per vector entry (FP64 is 1/64 rate on this part).
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF ff_add(FF a, FF b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float h = __fadd_rn(s, e);
    return FF{h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ FF ff_prod(float x, float y)
{
    const float p = __fmul_rn(x, y);
    return FF{p, fmaf(x, y, -p)};
}
__device__ __forceinline__ FF ff_shfl_down(FF a, int o)
{
    return FF{__shfl_down_sync(0xffffffffu, a.hi, o), __shfl_down_sync(0xffffffffu, a.lo, o)};
}

// Accumulator of the PCG dot products: float-float for the FP32 PCG, double for FP64.
template <typename T>
struct DotAcc;
template <>
struct DotAcc<float> {
    FF v{0.f, 0.f};
    __device__ __forceinline__ void add_prod(float x, float y) { v = ff_add(v, ff_prod(x, y)); }
    // block-wide sum in fixed order; the result (as double) is valid in thread 0
    __device__ double block_sum(double* sh)
    {
        FF a = v;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a = ff_add(a, ff_shfl_down(a, o));
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        __syncthreads();
        float* shf = reinterpret_cast<float*>(sh);
        if (lane == 0) { shf[2 * warp] = a.hi; shf[2 * warp + 1] = a.lo; }
        __syncthreads();
        if (warp == 0) {
            a = lane < nw ? FF{shf[2 * lane], shf[2 * lane + 1]} : FF{0.f, 0.f};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a = ff_add(a, ff_shfl_down(a, o));
        }
        // FP64 only where the result is used (GB300's FP64 rate is 1/64 of FP32)
        return threadIdx.x == 0 ? (double)a.hi + (double)a.lo : 0.0;
    }
};
template <>
struct DotAcc<double> {
    double v = 0.0;
    __device__ __forceinline__ void add_prod(double x, double y) { v = fma(x, y, v); }
    __device__ double block_sum(double* sh) { return block_reduce<false>(v, sh); }
};

// Publish per-block partial sums (valid in thread 0) and let the last block combine them in
// index order (double).  Returns true in the threads of the last block.
template <int NPARTS>
__device__ bool publish_and_combine(const double (&blockv)[NPARTS], double* partials, unsigned* ticket,
                                    double (&result)[NPARTS])
{
    __shared__ double sh[32];
    __shared__ bool is_last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NPARTS; ++k) partials[k * gridDim.x + blockIdx.x] = blockv[k];
        __threadfence();
        is_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NPARTS; ++k) {
        double acc = 0.0;
        for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) acc += __ldcg(&partials[k * gridDim.x + i]);
        result[k] = block_reduce<false>(acc, sh);
    }
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// Direction of block row i: z + beta p_old (z on the first iteration); one helper so every
// thread computing a given row gets the same bits.
template <typename T>
__device__ __forceinline__ Row4<T> direction(const T* __restrict__ z, const T* __restrict__ p_old, T beta, bool first,
                                             int i)
{
    const Row4<T> zz = ld4(z + 4 * i);
    if (first) return zz;
    const Row4<T> pp = ld4(p_old + 4 * i);
    return Row4<T>{fma(beta, pp.x, zz.x), fma(beta, pp.y, zz.y), fma(beta, pp.z, zz.z), T(0)};
}
// The same with loads that bypass L1 (for vectors other blocks of the same launch wrote).
__device__ __forceinline__ Row4<float> ld4cg(const float* p)
{
    const float4 v = __ldcg(reinterpret_cast<const float4*>(p));
    return Row4<float>{v.x, v.y, v.z, v.w};
}
// The same cached in L1: the gathers of a product pass.  Neighbouring block rows share most of
// their columns, so a chunk of rows gathers a few thousand bytes many times over, and L1 serves
// the repeats instead of L2.  Valid for vectors written by other blocks before the last grid
// barrier: its GPU-scope acquire (grid_barrier) invalidates the SM's L1, and nothing writes the
// gathered vector during the pass.
__device__ __forceinline__ Row4<float> ld4ca(const float* p)
{
    const float4 v = __ldca(reinterpret_cast<const float4*>(p));
    return Row4<float>{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ Row4<float> direction_cg(const float* z, const float* p_old, float beta, bool first, int i)
{
    const Row4<float> zz = ld4cg(z + 4 * i);
    if (first) return zz;
    const Row4<float> pp = ld4cg(p_old + 4 * i);
    return Row4<float>{fmaf(beta, pp.x, zz.x), fmaf(beta, pp.y, zz.y), fmaf(beta, pp.z, zz.z), 0.f};
}

// PCG step 1: p = z + beta p_old (fused), q = A p, p.q.  Grid sized to the resident
// blocks; each warp takes four block rows per pass.
template <typename T, typename L>
__global__ void __launch_bounds__(kSpmvThreads, SpmvMinBlocks<T>::value)
    k_pcg_spmv(PcgBuffers<T> B, L lay, const T* __restrict__ p_old, T* __restrict__ p_new, int first)
{
    if (B.state->done) return;
    __shared__ double sh[32];
    const T beta = first ? T(0) : (T)B.state->beta;
    const bool f = first != 0;
    const int lane16 = threadIdx.x & 15;
    const int half = (threadIdx.x >> 4) & 1;
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int warps_total = (gridDim.x * blockDim.x) >> 5;
    const T* __restrict__ z = B.z;
    auto pv = [z, p_old, beta, f](int c) { return direction(z, p_old, beta, f, c); };
    DotAcc<T> pq;
    for (int base = 4 * warp_global; base < B.n_blocks; base += 4 * warps_total) {
        const int rowA = base + half, rowB = base + 2 + half;
        const bool vA = rowA < B.n_blocks, vB = rowB < B.n_blocks;
        T a[3], b[3];
        two_row_products<T>(rowA, vA, rowB, vB, lane16, B.row_ptr, B.cols, B.vals, lay, pv, a, b);
        const T qd = half_warp_transpose_sum<T>(a, b, lane16);
        // one lane per output component: p and q of that component, and its p.q term
        const int idx = lane16 >> 1;  // 0..2 row A, 3..5 row B
        if (!(lane16 & 1) && idx < 6) {
            const int row = idx < 3 ? rowA : rowB, d = idx % 3;
            if (idx < 3 ? vA : vB) {
                const int64_t o = 4 * (int64_t)row + d;
                const T pd = f ? z[o] : fma(beta, p_old[o], z[o]);  // the bits direction() gives
                p_new[o] = pd;
                B.q[o] = qd;
                pq.add_prod(pd, qd);
            }
        }
    }
    const double bpq[1] = {pq.block_sum(sh)};
    double res[1];
    if (publish_and_combine<1>(bpq, B.partials, B.tickets, res) && threadIdx.x == 0) {
        PcgState* st = B.state;
        st->pAp = res[0];
        if (!(res[0] > 0.0)) {  // indefinite (or NaN): stop as the reference does
            st->indefinite = 1;
            st->converged = 0;
            st->done = 1;
            st->iteration += 1;
        } else {
            st->alpha = st->rz / res[0];
        }
    }
}

// ---------------------------------------------------------------- staged SpMV (bulk copies)
// The same product as k_pcg_spmv (float, strided values), with the matrix streamed through
// shared memory.  Each block owns a contiguous range of rows, cut into stages of
// stage_rows rows; a producer thread copies a stage's block range (nine value components,
// the column indices, the stage's row_ptr entries) with cp.async.bulk into a ring of
// shared-memory stages, completion counted by an mbarrier per stage ("full"), while the
// consumer warps (4 rows each per stage, two per half-warp) work on earlier stages and
// release them through a second mbarrier ("empty").  The consumers' only global loads left
// on the critical path are the gathers of the direction rows, which hit L2.  Every wait is
// bounded: a wait that gives up marks the block aborted, the block stops issuing and
// consuming, waits (bounded) for the copies it issued, and the solve is flagged in
// PcgState::error.
constexpr int kStagedConsumerWarps = 7;
constexpr int kStagedThreads = 32 * (kStagedConsumerWarps + 1);  // warp 0: producer
constexpr int kStagedRowsPerWarp = 8;                             // one block row per quad of lanes
constexpr int kStagedRows = kStagedRowsPerWarp * kStagedConsumerWarps;
constexpr int kStagedMaxStages = 8;
// Bound of the drain waits (copies in flight before a block exits); the data waits use
// B.staged.max_polls (wait_poll_limit()).
constexpr long long kMaxBarrierPolls = kDefaultWaitPolls;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Wait for the phase of parity `parity` to complete; false after max_polls polls (none
// when max_polls is 0).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long max_polls = kMaxBarrierPolls)
{
    for (long long i = 0; i < max_polls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulk_copy_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
// L2 policy for data read once per pass (the matrix values and columns): its lines are the
// first to go, so the PCG vectors the pass gathers and the update phase rewrites stay in L2.
__device__ __forceinline__ uint64_t l2_evict_first_policy()
{
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ void bulk_copy_g2s_stream(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar,
                                                     uint64_t pol)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            dst),
        "l"(src), "r"(bytes), "r"(bar), "l"(pol)
        : "memory");
}

// Bytes of one shared-memory stage: nine value slots and one column slot of `cap` entries,
// then stage_rows + 4 row_ptr entries, rounded to 128.
__host__ __device__ __forceinline__ size_t staged_stage_bytes(int cap, int stage_rows)
{
    return ((size_t)10 * cap * 4 + (size_t)(stage_rows + 4) * 4 + 127) / 128 * 128;
}

// Shared-memory layout of a staged block: full barriers, empty barriers (kStagedMaxStages
// each), the chunk held by each ring slot, the per-chunk partial sums of the consumer warps
// (kStagedPartSlots chunks in flight at most, with a count of the warps that stored theirs),
// then the ring of stages.  The chunk slots and partials are used by the persistent kernel.
constexpr int kStagedPartSlots = 2 * kStagedMaxStages;

constexpr size_t kStagedHeaderBytes =
    (16 * kStagedMaxStages + 4 * kStagedMaxStages + 4 * kStagedPartSlots +
     8 * kStagedPartSlots * kStagedConsumerWarps + 127) / 128 * 128;
struct StagedShared {
    uint64_t* full;
    uint64_t* empty;
    int* chunk;        // [kStagedMaxStages] chunk index of the stage in each slot, -1: end of a pass
    unsigned* wcount;  // [kStagedPartSlots] consumer warps that stored their partial
    float2* wpart;     // [kStagedPartSlots][kStagedConsumerWarps] float-float warp partials
    unsigned char* stage0;
};
__device__ __forceinline__ StagedShared staged_shared(unsigned char* smem)
{
    StagedShared ss;
    ss.full = reinterpret_cast<uint64_t*>(smem);
    ss.empty = ss.full + kStagedMaxStages;
    ss.chunk = reinterpret_cast<int*>(smem + 16 * kStagedMaxStages);
    ss.wcount = reinterpret_cast<unsigned*>(smem + 20 * kStagedMaxStages);
    ss.wpart = reinterpret_cast<float2*>(smem + 20 * kStagedMaxStages + 4 * kStagedPartSlots);
    ss.stage0 = smem + kStagedHeaderBytes;
    return ss;
}
__device__ __forceinline__ void staged_init_barriers(const StagedShared& ss, int stages)
{
    if (threadIdx.x < kStagedPartSlots) ss.wcount[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(smem_addr(&ss.full[s]), 1);
            mbar_init(smem_addr(&ss.empty[s]), kStagedConsumerWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
}

// Consumer side of the staged passes: the four lanes of a quad (q = lane & 3) take one block
// row of a stage.  Lane q multiplies blocks q, q + 4, ... of the row (its range [kb, ke) of
// the stage's value and column slots), four at a time with the four gathers in flight
// together, and a transposing sum over the quad leaves component q of the row's product in
// lane q (q < 3; lane 3 holds 0).  Per row this is a handful of warp instructions, where a
// half-warp per row spent most of its instructions on the 16-lane sum and per-stage
// bookkeeping.  Every lane of the warp must call it (the loop bound and the shuffles are
// warp-wide); rows without blocks pass kb == ke.  The sum of component j is taken in one
// fixed order.
template <typename XV>
__device__ __forceinline__ float quad_row_product(int kb, int ke, int q, const int32_t* __restrict__ scols,
                                                  const float* __restrict__ svals, int CAP, XV xv)
{
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    for (int base = kb + q; __any_sync(0xffffffffu, base < ke); base += 16) {
        Row4<float> x[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) x[i] = base + 4 * i < ke ? xv(scols[base + 4 * i]) : Row4<float>{};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int k = base + 4 * i;
            if (k < ke) {
                a0 += svals[k] * x[i].x + svals[CAP + k] * x[i].y + svals[2 * CAP + k] * x[i].z;
                a1 += svals[3 * CAP + k] * x[i].x + svals[4 * CAP + k] * x[i].y + svals[5 * CAP + k] * x[i].z;
                a2 += svals[6 * CAP + k] * x[i].x + svals[7 * CAP + k] * x[i].y + svals[8 * CAP + k] * x[i].z;
            }
        }
    }
    const bool b2 = (q & 2) != 0, b1 = (q & 1) != 0;
    const float w0 = (b2 ? a2 : a0) + __shfl_xor_sync(0xffffffffu, b2 ? a0 : a2, 2);
    const float w1 = (b2 ? 0.f : a1) + __shfl_xor_sync(0xffffffffu, b2 ? a1 : 0.f, 2);
    return (b1 ? w1 : w0) + __shfl_xor_sync(0xffffffffu, b1 ? w0 : w1, 1);
}

// Position of a consumer in the ring: stage number g, its slot and the parity of the slot's
// phase, advanced without dividing by the stage count.
struct RingCursor {
    unsigned g, slot, parity;
    __device__ __forceinline__ RingCursor(unsigned g0, int stages) : g(g0)
    {
        slot = g0 % (unsigned)stages;
        parity = (g0 / (unsigned)stages) & 1u;
    }
    __device__ __forceinline__ void advance(int stages)
    {
        ++g;
        if (++slot == (unsigned)stages) {
            slot = 0;
            parity ^= 1u;
        }
    }
};

// One pass of the staged product over this block's rows: p = z + beta p_old (fused into
// the gathers; the owning lane stores p_new), q = A p, and this thread's share of p.q.
// Stages are numbered over the whole launch (pass after pass; the matrix does not change):
// `seq` is the first stage of this pass and advances by the pass's stage count in every
// thread; `issued` (producer thread) counts the stages copied so far.  With run_ahead the
// producer goes on into the next pass's stages until the ring is full, so the next pass
// starts on stages already in shared memory; the caller then waits for them before the
// block exits (staged_drain).  kCg: read the direction vectors through L2 only (they were
// written by other blocks of the same launch).  Sets *abort_flag when a wait gives up.
template <bool kCg>
__device__ __forceinline__ void staged_spmv_pass(const PcgBuffers<float>& B, const StagedShared& ss,
                                                 const float* __restrict__ p_old, float* __restrict__ p_new, bool first,
                                                 float beta, unsigned& seq, unsigned& issued, bool run_ahead,
                                                 volatile int* abort_flag, DotAcc<float>& pq)
{
    const int S = B.staged.stage_rows, CAP = B.staged.stage_cap, NS = B.staged.stages;
    const size_t stage_bytes = staged_stage_bytes(CAP, S);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row_begin = blockIdx.x * B.staged.rows_per_block;
    const int row_end = min(row_begin + B.staged.rows_per_block, B.n_blocks);
    const int n_stages = B.staged.rows_per_block / S;
    if (warp == 0) {
        if (lane == 0) {
            const unsigned last = seq + n_stages + (run_ahead ? NS : 0);  // one past the last stage to copy now
            // block range of stage g, loaded one stage ahead so that the load overlaps the
            // wait for the ring slot
            auto range = [&](unsigned g, int& kb, int& ke) {
                const int r0 = row_begin + (int)(g % (unsigned)n_stages) * S;
                kb = B.staged.row_ptr_ext[r0];
                ke = B.staged.row_ptr_ext[r0 + S];
            };
            const uint64_t pol = l2_evict_first_policy();
            int next_kb = 0, next_ke = 0;
            if (issued < last) range(issued, next_kb, next_ke);
            for (unsigned g = issued; g < last && !*abort_flag; ++g) {
                const unsigned s = g % NS, use = g / NS;
                const int j = (int)(g % (unsigned)n_stages);
                const int kb = next_kb, ke = next_ke;
                if (g + 1 < last) range(g + 1, next_kb, next_ke);
                if (use > 0 && !mbar_wait(smem_addr(&ss.empty[s]), (use - 1) & 1, B.staged.max_polls)) {
                    *abort_flag = 1;
                    break;
                }
                const int r0 = row_begin + j * S;
                const int kb4 = kb & ~3, ke4 = (ke + 3) & ~3;
                const uint32_t span = (uint32_t)(ke4 - kb4) * 4u;
                unsigned char* st = ss.stage0 + s * stage_bytes;
                const uint32_t fb = smem_addr(&ss.full[s]);
                mbar_arrive_expect_tx(fb, 10u * span + (uint32_t)(S + 4) * 4u);
                if (span) {
                    for (int m = 0; m < 9; ++m)
                        bulk_copy_g2s_stream(smem_addr(st + (size_t)m * CAP * 4), B.vals + m * B.vals_stride + kb4,
                                             span, fb, pol);
                    bulk_copy_g2s_stream(smem_addr(st + (size_t)9 * CAP * 4), B.staged.cols_ext + kb4, span, fb, pol);
                }
                bulk_copy_g2s(smem_addr(st + (size_t)10 * CAP * 4), B.staged.row_ptr_ext + r0, (uint32_t)(S + 4) * 4u, fb);
                issued = g + 1;
            }
        }
    } else {
        const int cw = warp - 1, q = lane & 3, lr = kStagedRowsPerWarp * cw + (lane >> 2);
        const float* __restrict__ z = B.z;
        auto pv = [z, p_old, beta, first](int c) {
            return kCg ? direction_cg(z, p_old, beta, first, c) : direction(z, p_old, beta, first, c);
        };
        RingCursor rc(seq, NS);
        for (int j = 0; j < n_stages; ++j) {
            // one decision per warp: the product below shuffles over the full warp
            const bool stop = __any_sync(
                0xffffffffu, *abort_flag || !mbar_wait(smem_addr(&ss.full[rc.slot]), rc.parity, B.staged.max_polls));
            if (stop) {
                *abort_flag = 1;
                break;
            }
            const unsigned char* st = ss.stage0 + rc.slot * stage_bytes;
            const int32_t* rp = reinterpret_cast<const int32_t*>(st + (size_t)10 * CAP * 4);
            const int kb4 = rp[0] & ~3;
            const int row = row_begin + j * S + lr;
            const bool valid = row < row_end;
            const int kb = valid ? rp[lr] - kb4 : 0, ke = valid ? rp[lr + 1] - kb4 : 0;
            const int32_t* __restrict__ scols = reinterpret_cast<const int32_t*>(st + (size_t)9 * CAP * 4);
            const float* __restrict__ svals = reinterpret_cast<const float*>(st);
            const bool own = valid && q < 3;  // the lane that finishes component q of the row
            const int64_t o = 4 * (int64_t)row + q;
            float zo = 0.f, po = 0.f;
            if (own) {
                zo = kCg ? __ldcg(z + o) : z[o];
                po = first ? 0.0f : (kCg ? __ldcg(p_old + o) : p_old[o]);
            }
            // the stage is released after its values are read, when its loads have returned
            const float qd = quad_row_product(kb, ke, q, scols, svals, CAP, pv);
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_addr(&ss.empty[rc.slot]));
            if (own) {
                const float pd = first ? zo : fmaf(beta, po, zo);  // direction()'s bits
                p_new[o] = pd;
                B.q[o] = qd;
                pq.add_prod(pd, qd);
            }
            rc.advance(NS);
        }
    }
    seq += n_stages;
}

// Producer thread: wait (bounded) until the last stages it copied have landed, so no bulk
// copy is still writing this block's shared memory when it exits.  Only the last `stages`
// copies can be in flight (a slot is reused only after its previous stage was consumed), and
// each is the latest use of its slot, so waiting on its own phase parity is exact.
__device__ __forceinline__ void staged_drain(const PcgBuffers<float>& B, const StagedShared& ss, unsigned issued)
{
    if (threadIdx.x != 0) return;
    const unsigned NS = (unsigned)B.staged.stages;
    for (unsigned g = issued > NS ? issued - NS : 0; g < issued; ++g)
        mbar_wait(smem_addr(&ss.full[g % NS]), (g / NS) & 1);
}

// ---- dynamic schedule of the look-ahead kernel's product pass
// The rows are cut into chunks of stage_rows rows (one stage each).  In every pass the
// blocks claim chunks, kClaimChunks at a time, from a counter of that pass (atomicAdd; a
// value past the last chunk ends the block's pass), so a block on a slower SM simply takes
// fewer chunks and all blocks reach the grid barrier together.  The producer thread issues
// the claim of its next unit when it starts the first stage of the current one, so the
// claim's round trip, and the load of the next unit's row range after it, overlap the waits
// for ring slots.  After the end marker of pass li it runs on into pass li + 1 until the
// ring is full; it never claims from a pass beyond li + 1.  Three counters rotate (pass k
// uses ctr[k % 3]); ctr[(li + 2) % 3] is cleared by block 0 during pass li, when no block can
// still claim from pass li - 1 and none can claim from pass li + 2 yet.
//
// The sums stay bitwise reproducible: each consumer warp sums its products of a chunk in a
// fixed shuffle tree, the last warp to finish a chunk adds the warp sums in a fixed order and
// stores the chunk's partials, and after the barrier every block adds them in chunk order.
// None of it depends on which block took which chunk.
constexpr int kClaimChunks = 1;
struct DynProducer {
    int it = 0;         // pass of the next stage to issue
    int c = -1;         // its chunk, or -1: the end marker of pass `it`
    int unit0 = 0;      // first chunk of the claimed unit holding c, and one past its last
    int unit_end = 0;
    int rp[kClaimChunks + 1];  // row_ptr at the unit's chunk boundaries
    bool have = false;  // false: nothing claimed yet for pass `it`
    bool pending = false;   // a claim for the unit after this one is in flight
    int next_it = 0;
    unsigned next_v = 0;
    int end_it = -1;    // pass of the last end marker issued, and the stage numbers of the
    unsigned end_g = 0, end_g_prev = 0;  // last two end markers
};

// Take the claim value v of pass `it` as the current unit (loads its row range).
__device__ __forceinline__ void dyn_take(const PcgBuffers<float>& B, int n_chunks, int it, unsigned v, DynProducer& P)
{
    P.it = it;
    P.have = true;
    if (v >= (unsigned)n_chunks) {
        P.c = -1;
        return;
    }
    P.c = P.unit0 = (int)v;
    P.unit_end = min((int)v + kClaimChunks, n_chunks);
    const int S = B.staged.stage_rows;
#pragma unroll
    for (int k = 0; k <= kClaimChunks; ++k)
        if (P.unit0 + k <= P.unit_end) P.rp[k] = __ldcg(B.staged.row_ptr_ext + (P.unit0 + k) * S);
}

// Producer thread of a dynamically scheduled pass li (see above): claims chunks, copies each
// into the next free ring slot and publishes its chunk index (-1: the pass's end marker).
__device__ __forceinline__ void dyn_produce(const PcgBuffers<float>& B, const StagedShared& ss, int li, unsigned* ctr,
                                            int n_chunks, unsigned& issued, DynProducer& P, volatile int* abort_flag)
{
    const int S = B.staged.stage_rows, CAP = B.staged.stage_cap, NS = B.staged.stages;
    const size_t stage_bytes = staged_stage_bytes(CAP, S);
    const uint64_t pol = l2_evict_first_policy();
    while (!*abort_flag) {
        // once the end marker of pass li is out (in this pass or, running ahead, in the
        // previous one), stop when every ring slot that pass li's consumers free is taken
        if (P.end_it >= li) {
            const unsigned e = P.end_it == li ? P.end_g : P.end_g_prev;
            if (issued > e + (unsigned)NS) break;
        }
        if (!P.have) {  // nothing claimed ahead (launch start, or after a stop)
            if (P.it > li + 1) break;
            dyn_take(B, n_chunks, P.it, atomicAdd(&ctr[P.it % 3], (unsigned)kClaimChunks), P);
        }
        // claim the unit after this one now: its round trip overlaps the slot waits
        if (!P.pending && (P.c < 0 || P.c == P.unit0)) {
            const int nit = P.c < 0 ? P.it + 1 : P.it;
            if (nit <= li + 1) {
                P.next_it = nit;
                P.next_v = atomicAdd(&ctr[nit % 3], (unsigned)kClaimChunks);
                P.pending = true;
            }
        }
        const unsigned g = issued, s = g % NS, use = g / NS;
        if (use > 0 && !mbar_wait(smem_addr(&ss.empty[s]), (use - 1) & 1, B.staged.max_polls)) {
            *abort_flag = 1;
            break;
        }
        ss.chunk[s] = P.c;  // published to the consumers by the arrive's release
        const uint32_t fb = smem_addr(&ss.full[s]);
        if (P.c >= 0) {
            const int r0 = P.c * S, j = P.c - P.unit0;
            int kb = P.rp[0], ke = P.rp[1];  // constant indices only: P stays in registers
#pragma unroll
            for (int k = 1; k < kClaimChunks; ++k)
                if (j == k) {
                    kb = P.rp[k];
                    ke = P.rp[k + 1];
                }
            const int kb4 = kb & ~3, ke4 = (ke + 3) & ~3;
            const uint32_t span = (uint32_t)(ke4 - kb4) * 4u;
            unsigned char* st = ss.stage0 + s * stage_bytes;
            mbar_arrive_expect_tx(fb, 10u * span + (uint32_t)(S + 4) * 4u);
            if (span) {
                for (int m = 0; m < 9; ++m)
                    bulk_copy_g2s_stream(smem_addr(st + (size_t)m * CAP * 4), B.vals + m * B.vals_stride + kb4,
                                         span, fb, pol);
                bulk_copy_g2s_stream(smem_addr(st + (size_t)9 * CAP * 4), B.staged.cols_ext + kb4, span, fb,
                                     pol);
            }
            bulk_copy_g2s(smem_addr(st + (size_t)10 * CAP * 4), B.staged.row_ptr_ext + r0,
                          (uint32_t)(S + 4) * 4u, fb);
        } else {
            mbar_arrive(fb);
        }
        issued = g + 1;
        if (P.c < 0) {
            P.end_it = P.it;
            P.end_g_prev = P.end_g;
            P.end_g = g;
        }
        // next stage: the unit's next chunk, else the claimed unit, else claim at the top
        if (P.c >= 0 && P.c + 1 < P.unit_end) {
            P.c += 1;
        } else if (P.pending) {
            P.pending = false;
            dyn_take(B, n_chunks, P.next_it, P.next_v, P);
        } else {
            P.it = P.c < 0 ? P.it + 1 : P.it;
            P.have = false;
        }
    }
}

// One pass of the persistent kernel's product over this block's own rows [row_begin,
// row_end) (an even split; stages of S rows, the last one shorter), z gathered alone: the
// owning lane forms p = z + beta p_old and q = A z + beta q_old (A p_old = q_old), half the
// gathered bytes of forming A (z + beta p_old) directly.  Equal in exact arithmetic; in float
// the recursive q differs from A p by rounding carried over iterations, which the outer Newton
// loop's FP64 residual corrects like the rest of the FP32 solve's error.  The producer runs
// on into the next pass's stages (the same rows: the matrix does not change) until the ring is
// full, so a pass starts on stages already in shared memory.  Contiguous rows per block keep
// the z rows gathered by consecutive stages overlapping, so many gathers hit L1.  Each thread
// accumulates its share of p.q; nothing is published per stage, so the loop holds no fence.
__device__ __forceinline__ void staged_pass_rows(const PcgBuffers<float>& B, const StagedShared& ss, int row_begin,
                                                 int row_end, const float* __restrict__ p_old,
                                                 float* __restrict__ p_new, bool first, float beta, unsigned& seq,
                                                 unsigned& issued, volatile int* abort_flag, DotAcc<float>& pq)
{
    const int S = B.staged.stage_rows, CAP = B.staged.stage_cap, NS = B.staged.stages;
    const size_t stage_bytes = staged_stage_bytes(CAP, S);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_stages = (row_end - row_begin + S - 1) / S;
    if (n_stages <= 0) return;
    if (warp == 0) {
        if (lane == 0) {
            const unsigned last = seq + n_stages + NS;  // one past the last stage to copy now
            auto range = [&](unsigned g, int& r0, int& kb, int& ke) {
                r0 = row_begin + (int)(g % (unsigned)n_stages) * S;
                kb = B.staged.row_ptr_ext[r0];
                ke = B.staged.row_ptr_ext[min(r0 + S, row_end)];
            };
            const uint64_t pol = l2_evict_first_policy();
            int next_r0 = 0, next_kb = 0, next_ke = 0;
            if (issued < last) range(issued, next_r0, next_kb, next_ke);
            for (unsigned g = issued; g < last && !*abort_flag; ++g) {
                const unsigned s = g % NS, use = g / NS;
                const int r0 = next_r0, kb = next_kb, ke = next_ke;
                if (g + 1 < last) range(g + 1, next_r0, next_kb, next_ke);  // overlaps the slot wait
                if (r0 & 3) {  // row_ptr copies need a 16-byte aligned start (pcg_block_rows)
                    *abort_flag = 1;
                    break;
                }
                if (use > 0 && !mbar_wait(smem_addr(&ss.empty[s]), (use - 1) & 1, B.staged.max_polls)) {
                    *abort_flag = 1;
                    break;
                }
                const int kb4 = kb & ~3, ke4 = (ke + 3) & ~3;
                const uint32_t span = (uint32_t)(ke4 - kb4) * 4u;
                unsigned char* st = ss.stage0 + s * stage_bytes;
                const uint32_t fb = smem_addr(&ss.full[s]);
                mbar_arrive_expect_tx(fb, 10u * span + (uint32_t)(S + 4) * 4u);
                if (span) {
                    for (int m = 0; m < 9; ++m)
                        bulk_copy_g2s_stream(smem_addr(st + (size_t)m * CAP * 4), B.vals + m * B.vals_stride + kb4,
                                             span, fb, pol);
                    bulk_copy_g2s_stream(smem_addr(st + (size_t)9 * CAP * 4), B.staged.cols_ext + kb4, span, fb, pol);
                }
                bulk_copy_g2s(smem_addr(st + (size_t)10 * CAP * 4), B.staged.row_ptr_ext + r0, (uint32_t)(S + 4) * 4u, fb);
                issued = g + 1;
            }
        }
    } else {
        const int cw = warp - 1, q = lane & 3, lr = kStagedRowsPerWarp * cw + (lane >> 2);
        const float* __restrict__ z = B.z;
        auto pv = [z](int c) { return ld4ca(z + 4 * c); };
        RingCursor rc(seq, NS);
        for (int j = 0; j < n_stages; ++j) {
            // one decision per warp: the product below shuffles over the full warp
            const bool stop = __any_sync(
                0xffffffffu, *abort_flag || !mbar_wait(smem_addr(&ss.full[rc.slot]), rc.parity, B.staged.max_polls));
            if (stop) {
                *abort_flag = 1;
                break;
            }
            const unsigned char* st = ss.stage0 + rc.slot * stage_bytes;
            const int32_t* rp = reinterpret_cast<const int32_t*>(st + (size_t)10 * CAP * 4);
            const int kb4 = rp[0] & ~3;
            const int row = row_begin + j * S + lr;
            const bool valid = row < row_end && lr < S;
            const int kb = valid ? rp[lr] - kb4 : 0, ke = valid ? rp[lr + 1] - kb4 : 0;
            const int32_t* __restrict__ scols = reinterpret_cast<const int32_t*>(st + (size_t)9 * CAP * 4);
            const float* __restrict__ svals = reinterpret_cast<const float*>(st);
            const bool own = valid && q < 3;  // the lane that finishes component q of the row
            const int64_t o = 4 * (int64_t)row + q;
            float zo = 0.f, po = 0.f, qo = 0.f;
            if (own) {
                zo = __ldcg(z + o);
                if (!first) {
                    po = __ldcg(p_old + o);
                    qo = __ldcg(B.q + o);
                }
            }
            // the stage is released after its values are read, when its loads have returned
            const float wd = quad_row_product(kb, ke, q, scols, svals, CAP, pv);
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_addr(&ss.empty[rc.slot]));
            if (own) {
                const float pd = first ? zo : fmaf(beta, po, zo);
                const float qd = first ? wd : fmaf(beta, qo, wd);
                p_new[o] = pd;
                B.q[o] = qd;  // only this lane reads and writes component o of q in a pass
                pq.add_prod(pd, qd);
            }
            rc.advance(NS);
        }
    }
    seq += n_stages;  // every thread, producer included: the next pass's first stage
}

// Block-wide float-float sums of two values per thread in a fixed tree; valid in thread 0.
__device__ __forceinline__ void block_sum2_ff(FF a, FF b, double* sh, FF& ra, FF& rb)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a = ff_add(a, ff_shfl_down(a, o));
        b = ff_add(b, ff_shfl_down(b, o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float* shf = reinterpret_cast<float*>(sh);  // 4 floats per warp
    __syncthreads();
    if (lane == 0) {
        shf[4 * warp] = a.hi;
        shf[4 * warp + 1] = a.lo;
        shf[4 * warp + 2] = b.hi;
        shf[4 * warp + 3] = b.lo;
    }
    __syncthreads();
    if (warp == 0) {
        a = lane < nw ? FF{shf[4 * lane], shf[4 * lane + 1]} : FF{0.f, 0.f};
        b = lane < nw ? FF{shf[4 * lane + 2], shf[4 * lane + 3]} : FF{0.f, 0.f};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a = ff_add(a, ff_shfl_down(a, o));
            b = ff_add(b, ff_shfl_down(b, o));
        }
    }
    ra = a;
    rb = b;
}

// Sums of two arrays of gridDim.x float-float block partials, in one fixed order (the same
// in every block), returned to every thread.
__device__ void sum_grid_partials2_ff(const float2* pa, const float2* pb, double* sh, double& a, double& b)
{
    FF va{0.f, 0.f}, vb{0.f, 0.f};
    for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
        const float2 x = __ldcg(pa + i), y = __ldcg(pb + i);
        va = ff_add(va, FF{x.x, x.y});
        vb = ff_add(vb, FF{y.x, y.y});
    }
    FF ra, rb;
    block_sum2_ff(va, vb, sh, ra, rb);
    __shared__ double result[2];
    if (threadIdx.x == 0) {
        result[0] = (double)ra.hi + (double)ra.lo;
        result[1] = (double)rb.hi + (double)rb.lo;
    }
    __syncthreads();
    a = result[0];
    b = result[1];
}

// Sum of the n float-float chunk partials in one fixed order (the same in every block),
// returned to every thread.
__device__ double sum_chunk_partials(const float2* part, int n, double* sh)
{
    FF a{0.f, 0.f};
    int i = threadIdx.x;
    constexpr int U = 8;  // loads in flight per thread
    for (; i + (U - 1) * (int)blockDim.x < n; i += U * blockDim.x) {
        float2 v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) v[u] = __ldcg(part + i + u * blockDim.x);
#pragma unroll
        for (int u = 0; u < U; ++u) a = ff_add(a, FF{v[u].x, v[u].y});
    }
    for (; i < n; i += blockDim.x) {
        const float2 v = __ldcg(part + i);
        a = ff_add(a, FF{v.x, v.y});
    }
    DotAcc<float> acc;
    acc.v = a;
    const double r = acc.block_sum(sh);
    __shared__ double result;
    if (threadIdx.x == 0) result = r;
    __syncthreads();
    return result;
}

// Sum of n FP64 partials in one fixed order (the same in every block), returned to every
// thread.
__device__ double sum_partials_f64(const double* p, int n, double* sh)
{
    double a = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) a += __ldcg(p + i);
    const double r = block_reduce<false>(a, sh);
    __shared__ double result;
    if (threadIdx.x == 0) result = r;
    __syncthreads();
    return result;
}

__global__ void __launch_bounds__(kStagedThreads, 1)
    k_pcg_spmv_staged(PcgBuffers<float> B, const float* __restrict__ p_old, float* __restrict__ p_new, int first)
{
    if (B.state->done) return;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ double sh[32];
    __shared__ int aborted;
    const StagedShared ss = staged_shared(smem);
    if (threadIdx.x == 0) aborted = 0;
    staged_init_barriers(ss, B.staged.stages);
    __syncthreads();
    volatile int* abort_flag = &aborted;
    DotAcc<float> pq;
    unsigned seq = 0, issued = 0;
    staged_spmv_pass<false>(B, ss, p_old, p_new, first != 0, first ? 0.f : (float)B.state->beta, seq, issued, false,
                            abort_flag, pq);
    if (*abort_flag) staged_drain(B, ss, issued);
    const double bpq[1] = {pq.block_sum(sh)};
    __syncthreads();
    const int block_aborted = *abort_flag;
    double res[1];
    if (publish_and_combine<1>(bpq, B.partials, B.tickets, res) && threadIdx.x == 0) {
        PcgState* st = B.state;
        st->pAp = res[0];
        if (!(res[0] > 0.0)) {  // indefinite (or NaN): stop as the reference does
            st->indefinite = 1;
            st->converged = 0;
            st->done = 1;
            st->iteration += 1;
        } else {
            st->alpha = st->rz / res[0];
        }
    }
    if (block_aborted && threadIdx.x == 0) {
        B.state->wait_failed = 1;
        B.state->converged = 0;
        B.state->done = 1;
    }
}

// z = M^-1 r for one block row
template <typename T>
__device__ __forceinline__ Row4<T> apply_block_jacobi(const T* __restrict__ Dinv, int i, const Row4<T>& r)
{
    const Row4<T> m0 = ld4(Dinv + 12 * (int64_t)i), m1 = ld4(Dinv + 12 * (int64_t)i + 4),
                  m2 = ld4(Dinv + 12 * (int64_t)i + 8);
    return Row4<T>{m0.x * r.x + m0.y * r.y + m0.z * r.z, m1.x * r.x + m1.y * r.y + m1.z * r.z,
                   m2.x * r.x + m2.y * r.y + m2.z * r.z, T(0)};
}

// PCG step 2: x += alpha p, r -= alpha q, z = M^-1 r, r.r and r.z; convergence test and beta.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_update(PcgBuffers<T> B, const T* __restrict__ p)
{
    if (B.state->done) return;
    __shared__ double sh[32];
    const T alpha = (T)B.state->alpha;
    DotAcc<T> rr, rz;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n_blocks; i += gridDim.x * blockDim.x) {
        Row4<T> x = ld4(B.x + 4 * i), r = ld4(B.r + 4 * i);
        const Row4<T> pp = ld4(p + 4 * i), q = ld4(B.q + 4 * i);
        x.x = fma(alpha, pp.x, x.x);
        x.y = fma(alpha, pp.y, x.y);
        x.z = fma(alpha, pp.z, x.z);
        r.x = fma(-alpha, q.x, r.x);
        r.y = fma(-alpha, q.y, r.y);
        r.z = fma(-alpha, q.z, r.z);
        const Row4<T> z = apply_block_jacobi(B.Dinv, i, r);
        st4(B.x + 4 * i, x);
        st4(B.r + 4 * i, r);
        st4(B.z + 4 * i, z);
        rr.add_prod(r.x, r.x);
        rr.add_prod(r.y, r.y);
        rr.add_prod(r.z, r.z);
        rz.add_prod(r.x, z.x);
        rz.add_prod(r.y, z.y);
        rz.add_prod(r.z, z.z);
    }
    const double bv[2] = {rr.block_sum(sh), rz.block_sum(sh)};
    double res[2];
    if (publish_and_combine<2>(bv, B.partials, B.tickets + 1, res) && threadIdx.x == 0) {
        PcgState* st = B.state;
        st->iteration += 1;
        st->rr = res[0];
        st->error = sqrt(res[0] / st->bb);
        if (st->error < st->abs_tol || st->error / st->error0 < st->rel_tol) {
            st->converged = 1;
            st->done = 1;
        } else if (st->iteration >= st->max_iterations) {
            st->converged = 0;
            st->done = 1;
        } else {
            st->beta = res[1] / st->rz;
            st->rz = res[1];
        }
    }
}

// ---------------------------------------------------------------- persistent PCG
// The whole PCG loop in one cooperative launch (all blocks resident): per iteration the
// staged product pass over the block's own rows (staged_pass_rows; an even split in units of
// four rows), a grid barrier, p.Ap from the block partials (every block sums them itself in
// one fixed order, so all blocks hold the same alpha), the update of the same rows (x, r, z,
// r.r, r.z), a second grid barrier, and the convergence test and beta, computed identically
// in every block.  The iteration and its stopping rules are those
// of k_pcg_spmv + k_pcg_update.  Plain (L1-cached) loads are safe across iterations: the
// barrier's acquire at GPU scope, ordered before every thread of the block by __syncthreads,
// makes the other blocks' writes visible to them (the guarantee a grid synchronization
// gives).  Grid barrier word bar[0] counts arrivals over the whole launch (zero at launch):
// barrier k is passed when it reaches k * gridDim.x.  Every wait is bounded; a block that
// gives up flags PcgState::wait_failed and leaves the loop.
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ bool grid_barrier(unsigned* bar, unsigned& generation, volatile int* ok_flag, long long max_polls)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned target = (generation + 1) * gridDim.x;
        __threadfence();
        red_release_add(&bar[0], 1u);
        bool ok = true;
        for (long long polls = 0; ld_acquire(&bar[0]) < target; ++polls) {
            if (polls > max_polls) {
                ok = false;
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
        *ok_flag = ok ? 1 : 0;
    }
    __syncthreads();
    generation += 1;
    return *ok_flag != 0;
}

// Per-iteration decisions of a persistent PCG block, taken by thread 0 alone and read by the
// others after a __syncthreads: the scalar recurrence runs in FP64, and on GB300 (FP64 at
// 1/64 of the FP32 rate) every thread of every block repeating its divisions and square root
// would cost more than the rest of an iteration's arithmetic.
struct PcgCtl {
    float alpha, beta;  // the coefficients the next pass / update use
    int stop;           // 1: leave the iteration loop
    // thread 0's FP64 recurrence and outcome (in shared memory, so the other threads hold no
    // registers for it)
    double rz, alpha64, beta64, pAp, rr, error;
    double thr_abs, thr_rel;  // the convergence test on r.r (no square root per iteration)
    int iteration, converged, indefinite, paused;
    int have_rr;  // rr holds a residual of this launch
};

// Rows [row_begin, row_end) of block b of G in the persistent kernel: an even split in units of
// four rows, so every stage of S rows (S a multiple of four) starts on a 16-byte boundary of
// row_ptr, as its bulk copy requires.
__host__ __device__ __forceinline__ void pcg_block_rows(int64_t b, int64_t G, int64_t n, int& row_begin, int& row_end)
{
    const int64_t units = (n + 3) / 4;
    const int64_t rb = 4 * (b * units / G), re = 4 * ((b + 1) * units / G);
    row_begin = (int)(rb < n ? rb : n);
    row_end = (int)(re < n ? re : n);
}

// Chunks of the persistent kernel's product pass (one stage of rows each).
__host__ __device__ __forceinline__ int pcg_chunks(int n_blocks, int stage_rows)
{
    return (n_blocks + stage_rows - 1) / stage_rows;
}


template <bool kF64Sums>
__global__ void __launch_bounds__(kStagedThreads, 2) k_pcg_solve_staged(PcgBuffers<float> B)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ double sh[32];
    __shared__ int aborted, barrier_ok;
    __shared__ PcgState st0;  // as k_pcg_init left it (an earlier launch)
    if (threadIdx.x == 0) st0 = *B.state;
    __syncthreads();
    if (st0.done) return;
    const StagedShared ss = staged_shared(smem);
    if (threadIdx.x == 0) aborted = 0;
    staged_init_barriers(ss, B.staged.stages);
    __syncthreads();
    volatile int* abort_flag = &aborted;
    unsigned* bar = B.tickets + 6;
    unsigned generation = 0, seq = 0, issued = 0;
    const unsigned G = gridDim.x;
    // block partials (FF sums: float2, FP64 sums: double; 8 bytes each): p.Ap, r.r, r.z
    float2* part_pq = reinterpret_cast<float2*>(B.partials);
    float2* part_rr = part_pq + G;
    float2* part_rz = part_rr + G;
    double* part_pq64 = B.partials;
    double* part_rr64 = B.partials + G;
    double* part_rz64 = B.partials + 2 * G;
    int row_begin, row_end;
    pcg_block_rows(blockIdx.x, G, B.n_blocks, row_begin, row_end);
    // a launch after a residual replacement continues the recurrence: beta from the state
    // the FP64 recurrence is thread 0's (PcgCtl); every thread counts the iterations
    __shared__ PcgCtl ctl;
    if (threadIdx.x == 0) {
        ctl.rz = st0.rz;
        ctl.alpha64 = 0.0;
        ctl.beta64 = st0.iteration > 0 ? st0.beta : 0.0;
        ctl.pAp = ctl.rr = 0.0;
        ctl.error = st0.error;
        ctl.iteration = st0.iteration;
        ctl.converged = ctl.indefinite = ctl.paused = ctl.have_rr = 0;
        ctl.beta = (float)ctl.beta64;
        // sqrt(rr / bb) < abs_tol  and  sqrt(rr / bb) / error0 < rel_tol, as comparisons of rr
        ctl.thr_abs = st0.abs_tol * st0.abs_tol * st0.bb;
        ctl.thr_rel = st0.rel_tol * st0.error0 * st0.rel_tol * st0.error0 * st0.bb;
    }
    __syncthreads();
    int iteration = st0.iteration;
    bool failed = false;
    float beta_f = ctl.beta;
    for (int li = 0;; ++li) {
        float* p_old = (iteration & 1) ? B.p : B.p2;
        float* p_new = (iteration & 1) ? B.p2 : B.p;
        const bool first = iteration == 0;
        DotAcc<float> pqa;
        staged_pass_rows(B, ss, row_begin, row_end, p_old, p_new, first, first ? 0.f : beta_f, seq, issued, abort_flag,
                         pqa);
        {
            FF bpq, unused;
            block_sum2_ff(pqa.v, FF{0.f, 0.f}, sh, bpq, unused);  // valid in thread 0
            if (threadIdx.x == 0) {
                if (kF64Sums) part_pq64[blockIdx.x] = (double)bpq.hi + (double)bpq.lo;
                else part_pq[blockIdx.x] = make_float2(bpq.hi, bpq.lo);
            }
        }
        if (!grid_barrier(bar, generation, &barrier_ok, B.staged.max_polls) || *abort_flag) {
            failed = true;
            break;
        }
        const double pAp = kF64Sums ? sum_partials_f64(part_pq64, (int)G, sh) : sum_chunk_partials(part_pq, (int)G, sh);
        if (threadIdx.x == 0) {
            ctl.stop = 0;
            ctl.pAp = pAp;
            if (!(pAp > 0.0)) {  // indefinite (or NaN): stop as the reference does
                ctl.indefinite = 1;
                ctl.iteration = iteration + 1;
                ctl.stop = 1;
            } else {
                ctl.alpha64 = ctl.rz / pAp;
                ctl.alpha = (float)ctl.alpha64;
            }
        }
        __syncthreads();
        if (ctl.stop) break;
        const float a = ctl.alpha;
        DotAcc<float> rra, rza;
        // two rows per thread and pass (rows i and i + blockDim.x, summed in that order, as a
        // row-by-row loop would), all their loads (preconditioner blocks included) issued
        // before their math
        for (int i = row_begin + (int)threadIdx.x; i < row_end; i += 2 * blockDim.x) {
            const int i2 = i + (int)blockDim.x;
            const bool h2 = i2 < row_end;
            Row4<float> x[2], r[2], pp[2], q[2], m0[2], m1[2], m2[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int k = u ? i2 : i;
                if (u == 0 || h2) {
                    x[u] = ld4(B.x + 4 * k);
                    r[u] = ld4(B.r + 4 * k);
                    pp[u] = ld4(p_new + 4 * k);
                    q[u] = ld4(B.q + 4 * k);
                    m0[u] = ld4(B.Dinv + 12 * (int64_t)k);
                    m1[u] = ld4(B.Dinv + 12 * (int64_t)k + 4);
                    m2[u] = ld4(B.Dinv + 12 * (int64_t)k + 8);
                }
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (u == 1 && !h2) break;
                const int k = u ? i2 : i;
                x[u].x = fmaf(a, pp[u].x, x[u].x);
                x[u].y = fmaf(a, pp[u].y, x[u].y);
                x[u].z = fmaf(a, pp[u].z, x[u].z);
                r[u].x = fmaf(-a, q[u].x, r[u].x);
                r[u].y = fmaf(-a, q[u].y, r[u].y);
                r[u].z = fmaf(-a, q[u].z, r[u].z);
                const Row4<float> z{m0[u].x * r[u].x + m0[u].y * r[u].y + m0[u].z * r[u].z,
                                    m1[u].x * r[u].x + m1[u].y * r[u].y + m1[u].z * r[u].z,
                                    m2[u].x * r[u].x + m2[u].y * r[u].y + m2[u].z * r[u].z, 0.0f};
                st4(B.x + 4 * k, x[u]);
                st4(B.r + 4 * k, r[u]);
                st4(B.z + 4 * k, z);
                rra.add_prod(r[u].x, r[u].x);
                rra.add_prod(r[u].y, r[u].y);
                rra.add_prod(r[u].z, r[u].z);
                rza.add_prod(r[u].x, z.x);
                rza.add_prod(r[u].y, z.y);
                rza.add_prod(r[u].z, z.z);
            }
        }
        FF brr, brz;
        block_sum2_ff(rra.v, rza.v, sh, brr, brz);
        if (threadIdx.x == 0) {
            if (kF64Sums) {
                part_rr64[blockIdx.x] = (double)brr.hi + (double)brr.lo;
                part_rz64[blockIdx.x] = (double)brz.hi + (double)brz.lo;
            } else {
                part_rr[blockIdx.x] = make_float2(brr.hi, brr.lo);
                part_rz[blockIdx.x] = make_float2(brz.hi, brz.lo);
            }
        }
        if (!grid_barrier(bar, generation, &barrier_ok, B.staged.max_polls)) {
            failed = true;
            break;
        }
        double rr, rz_new;
        if (kF64Sums) {
            rr = sum_partials_f64(part_rr64, (int)G, sh);
            rz_new = sum_partials_f64(part_rz64, (int)G, sh);
        } else {
            sum_grid_partials2_ff(part_rr, part_rz, sh, rr, rz_new);
        }
        iteration += 1;
        if (threadIdx.x == 0) {
            ctl.stop = 1;
            ctl.iteration = iteration;
            ctl.rr = rr;
            ctl.have_rr = 1;
            if (rr < ctl.thr_abs || rr < ctl.thr_rel) {
                ctl.converged = 1;
            } else if (iteration >= st0.max_iterations) {
            } else if (st0.replace_every > 0 && iteration % st0.replace_every == 0) {
                ctl.paused = 1;  // rz stays that of the last iterate: the replacement forms beta
            } else {
                ctl.beta64 = rz_new / ctl.rz;
                ctl.rz = rz_new;
                ctl.beta = (float)ctl.beta64;
                ctl.stop = 0;
            }
        }
        __syncthreads();
        if (ctl.stop) break;
        beta_f = ctl.beta;
    }
    staged_drain(B, ss, issued);  // stages copied ahead for a pass that will not run
    if (failed && threadIdx.x == 0) atomicExch(&B.state->wait_failed, 1);
    if (blockIdx.x == 0 && threadIdx.x == 0 && !failed) {
        PcgState* st = B.state;
        st->iteration = ctl.iteration;
        st->converged = ctl.converged;
        st->indefinite = ctl.indefinite;
        st->done = ctl.paused ? 0 : 1;
        st->pAp = ctl.pAp;
        st->alpha = ctl.alpha64;
        st->beta = ctl.beta64;
        st->rz = ctl.rz;
        st->rr = ctl.rr;
        st->error = ctl.have_rr ? sqrt(ctl.rr / st0.bb) : st0.error;
    }
}

// ---------------------------------------------------------------- look-ahead PCG
// The same iteration as k_pcg_solve_staged (the reference's block-Jacobi PCG, solve_pcg.h:82-232),
// reorganised so that one grid barrier per iteration suffices: the update of x, r and z is
// folded into the next product pass, and the pass forms the product of the next z directly.
// With w_k = A z_k, mw_k = M^-1 w_k, mq_k = M^-1 q_k, iteration k of the pass computes, per
// block row (the owning lane of each component):
//     p_{k-1} = z_{k-1} + beta_{k-1} p_{k-2}        q_{k-1} = w_{k-1} + beta_{k-1} q_{k-2}
//     x_k = x_{k-1} + alpha_{k-1} p_{k-1}           r_k = r_{k-1} - alpha_{k-1} q_{k-1}
//     z_k = M^-1 r_k      mq_{k-1} = M^-1 q_{k-1}   w_k = A z_k      mw_k = M^-1 w_k
// where each gathered column c of z_k is formed from (z_{k-1}, mw_{k-1}, mq_{k-2}) of row c as
// z_{k-1} - alpha_{k-1} (mw_{k-1} + beta_{k-1} mq_{k-2}), equal to M^-1 r_k up to the rounding
// of that one step: the stored z and mq are formed from r and q in every pass, so no rounding
// accumulates in them (a recursively updated z loses its agreement with r once r falls below
// the FP32 resolution of its first value, and the residual then stops decreasing).  The pass
// leaves
// per-chunk partials of r.r, r.z, z.w, z.q + p.w and p.q; after the barrier every block
// sums them in one fixed order and forms beta_k = rz_k / rz_{k-1} and
//     p_k.A p_k = z.w + beta_k (z.q + p.w) + beta_k^2 p.q       (p_k = z_k + beta_k p_{k-1})
// without any orthogonality assumption, so the iterates are those of the two-barrier form up
// to rounding (the same iteration counts on the Tet4 systems of this path).  The convergence
// test on r_k runs after the pass that formed x_k; a converged solve has done one product more
// than the two-barrier form.  The first pass of a launch (entry) gathers z as it is (after
// k_pcg_init or a residual replacement), forms w and mw and, when earlier iterations exist,
// mq = M^-1 q of the last direction.  The gathered vectors (z, mw, mq) alternate between two
// sets by pass parity, the per-chunk partials between two halves, so no pass writes what
// another block may still read from the previous one.
constexpr int kLaSums = 5;  // r.r, r.z, z.w, z.q + p.w, p.q
// Shared-memory layout of a look-ahead block: full and empty barriers (one per stage), the
// consumer warps' partials of stages + 1 chunks in flight (a warp publishes a chunk after
// releasing its stage, so the warps are at most `stages` chunks apart), the chunk index of each
// ring slot, the per-slot count of warps that published, then the ring of stages.
__host__ __device__ __forceinline__ size_t la_header_bytes(int stages)
{
    return ((size_t)16 * stages + (size_t)8 * kLaSums * kStagedConsumerWarps * (stages + 1) + 4 * (size_t)stages +
            4 * (size_t)(stages + 1) + 127) / 128 * 128;
}
__device__ __forceinline__ StagedShared la_shared(unsigned char* smem, int stages)
{
    StagedShared ss;
    ss.full = reinterpret_cast<uint64_t*>(smem);
    ss.empty = ss.full + stages;
    ss.wpart = reinterpret_cast<float2*>(smem + 16 * stages);
    unsigned char* tail = smem + 16 * stages + (size_t)8 * kLaSums * kStagedConsumerWarps * (stages + 1);
    ss.chunk = reinterpret_cast<int*>(tail);
    ss.wcount = reinterpret_cast<unsigned*>(tail + 4 * stages);
    ss.stage0 = smem + la_header_bytes(stages);
    return ss;
}
struct LaVectors {
    const float* z;  // gathered set: z, mw, mq
    const float* mw;
    const float* mq;
    float* zo;  // the set this pass writes
    float* mwo;
    float* mqo;
    float* w;
};
__device__ __forceinline__ LaVectors la_vectors(const PcgBuffers<float>& B, int set_in)
{
    const int64_t vs = 4 * (int64_t)B.n_blocks;
    float* z1 = B.la;
    float* mw0 = B.la + vs;
    float* mw1 = B.la + 2 * vs;
    float* mq0 = B.la + 3 * vs;
    float* mq1 = B.la + 4 * vs;
    LaVectors v;
    v.z = set_in ? z1 : B.z;
    v.mw = set_in ? mw1 : mw0;
    v.mq = set_in ? mq1 : mq0;
    v.zo = set_in ? B.z : z1;
    v.mwo = set_in ? mw0 : mw1;
    v.mqo = set_in ? mq0 : mq1;
    v.w = B.la + 5 * vs;
    return v;
}
// z_k of one component from (z_{k-1}, mw_{k-1}, mq_{k-2}): the owner and every gather use this
__device__ __forceinline__ float la_znext(float z, float mw, float mq, float alpha, float beta)
{
    return __fmaf_rn(-alpha, __fmaf_rn(beta, mq, mw), z);
}

// Sums of eight float-float values over groups of W lanes (W = 32 or 16) in a fixed tree that
// transposes as it goes: at each of the first three levels a lane keeps half of its values and
// sends the other half, so each lane ends with one value, the total of value j in lane
// j * W / 8 of its group (the other lanes hold partial or repeated sums).  Each total is the
// same fixed sequence of float-float additions on every run.
__device__ __forceinline__ FF ff_shfl_xor(FF a, int o)
{
    return FF{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
}
template <int W>
__device__ __forceinline__ FF ff_transpose_sum8(const FF (&v)[8], int lane)
{
    constexpr int h = W / 2;
    FF w[4], u[2];
    const bool b2 = (lane & h) != 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] = ff_add(b2 ? v[i + 4] : v[i], ff_shfl_xor(b2 ? v[i] : v[i + 4], h));
    const bool b1 = (lane & (h / 2)) != 0;
#pragma unroll
    for (int i = 0; i < 2; ++i) u[i] = ff_add(b1 ? w[i + 2] : w[i], ff_shfl_xor(b1 ? w[i] : w[i + 2], h / 2));
    const bool b0 = (lane & (h / 4)) != 0;
    FF t = ff_add(b0 ? u[1] : u[0], ff_shfl_xor(b0 ? u[0] : u[1], h / 4));
#pragma unroll
    for (int o = h / 8; o > 0; o >>= 1) t = ff_add(t, ff_shfl_xor(t, o));
    return t;
}

// Chunk partial of the kLaSums float-float sums of one consumer warp: a fixed transposing
// tree over the warp, then the last of the 15 warps to finish the chunk adds the 15 warp sums
// in a fixed tree over 16 lanes and stores the chunk's partials (value-major:
// part[k * n_chunks + c]).
template <bool kF64Sums>
__device__ __forceinline__ void la_publish(const FF (&v)[kLaSums], const StagedShared& ss, unsigned ps, int cw, int c,
                                           int n_chunks, double* part)
{
    const int lane = threadIdx.x & 31;
    FF v8[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v8[k] = k < kLaSums ? v[k] : FF{0.f, 0.f};
    const FF t = ff_transpose_sum8<32>(v8, lane);  // value lane / 4 in lanes 0, 4, ..., 16
    float2* wp = ss.wpart + (size_t)ps * kStagedConsumerWarps * kLaSums;
    if ((lane & 3) == 0 && lane < 4 * kLaSums) wp[cw * kLaSums + (lane >> 2)] = make_float2(t.hi, t.lo);
    __syncwarp();
    unsigned last = 0;
    if (lane == 0) {
        __threadfence_block();
        last = atomicAdd(&ss.wcount[ps], 1u) == kStagedConsumerWarps - 1 ? 1u : 0u;
    }
    if (!__shfl_sync(0xffffffffu, last, 0)) return;
    __threadfence_block();
    __syncwarp();
    FF s8[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        if (k < kLaSums && lane < kStagedConsumerWarps) {
            const volatile float* x = reinterpret_cast<volatile float*>(&wp[lane * kLaSums + k]);
            s8[k] = FF{x[0], x[1]};
        } else {
            s8[k] = FF{0.f, 0.f};
        }
    }
    const FF s = ff_transpose_sum8<16>(s8, lane);  // value lane / 2 in lanes 0, 2, ..., 8
    if (lane == 0) ss.wcount[ps] = 0;
    if ((lane & 1) == 0 && lane < 2 * kLaSums) {
        const int k = lane >> 1;
        if constexpr (kF64Sums) part[(size_t)k * n_chunks + c] = (double)s.hi + (double)s.lo;
        else reinterpret_cast<float2*>(part)[(size_t)k * n_chunks + c] = make_float2(s.hi, s.lo);
    }
}

// Consumer warps of one look-ahead pass (kEntry: the first pass of a launch).  Per stage a warp
// takes four rows (two per half-warp), issues the owner's loads and the gathers together, then
// reads the stage's values from shared memory and releases the stage (no global load is in
// flight at the release), forms the products, the owners' updates and this chunk's partials.
template <bool kF64Sums, bool kEntry>
__device__ __forceinline__ void la_consume(const PcgBuffers<float>& B, const StagedShared& ss, const LaVectors& V,
                                           int n_chunks, float alpha, float beta, bool first, double* part,
                                           unsigned& seq, volatile int* abort_flag)
{
    const int S = B.staged.stage_rows, CAP = B.staged.stage_cap, NS = B.staged.stages;
    const size_t stage_bytes = staged_stage_bytes(CAP, S);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cw = warp - 1, q = lane & 3, lr = kStagedRowsPerWarp * cw + (lane >> 2);
    const int qb = lane & ~3;  // first lane of this quad: components 0..2 of its row in qb .. qb + 2
    const int n = B.n_blocks;
    auto gather = [&](int c) {
        if constexpr (kEntry) {
            return ld4ca(V.z + 4 * c);
        } else {
            const Row4<float> z = ld4ca(V.z + 4 * c), mw = ld4ca(V.mw + 4 * c), mq = ld4ca(V.mq + 4 * c);
            return Row4<float>{la_znext(z.x, mw.x, mq.x, alpha, beta), la_znext(z.y, mw.y, mq.y, alpha, beta),
                               la_znext(z.z, mw.z, mq.z, alpha, beta), 0.f};
        }
    };
    RingCursor rc(seq, NS);
    for (;;) {
        // one decision per warp: the product below shuffles over the full warp
        const bool stop = __any_sync(
            0xffffffffu, *abort_flag || !mbar_wait(smem_addr(&ss.full[rc.slot]), rc.parity, B.staged.max_polls));
        if (stop) {
            *abort_flag = 1;
            break;
        }
        const int c = *(volatile int*)&ss.chunk[rc.slot];
        if (c < 0) {  // end of this pass
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_addr(&ss.empty[rc.slot]));
            rc.advance(NS);
            break;
        }
        const int row = c * S + lr;
        const bool valid = row < n;
        const bool own = valid && q < 3;  // the lane that finishes component q of the row
        const int64_t o = 4 * (int64_t)row + q;
        const unsigned char* st = ss.stage0 + rc.slot * stage_bytes;
        const int32_t* rp = reinterpret_cast<const int32_t*>(st + (size_t)10 * CAP * 4);
        const int kb4 = rp[0] & ~3;
        const int kb = valid ? rp[lr] - kb4 : 0, ke = valid ? rp[lr + 1] - kb4 : 0;
        const int32_t* __restrict__ scols = reinterpret_cast<const int32_t*>(st + (size_t)9 * CAP * 4);
        const float* __restrict__ svals = reinterpret_cast<const float*>(st);
        // the owner's row values (written by other blocks in the previous pass: L2 loads)
        float zp = 0.f, po = 0.f, qo = 0.f, wo = 0.f, xo = 0.f, ro = 0.f;
        Row4<float> dv{}, qrow{};
        if (own) {
            dv = ld4(B.Dinv + 12 * (int64_t)row + 4 * q);
            zp = __ldcg(V.z + o);
            if constexpr (kEntry) {
                if (!first) {
                    po = __ldcg(B.p + o);
                    qrow = ld4cg(B.q + 4 * (int64_t)row);
                }
            } else {
                po = __ldcg(B.p + o);
                qo = __ldcg(B.q + o);
                wo = __ldcg(V.w + o);
                xo = __ldcg(B.x + o);
                ro = __ldcg(B.r + o);
            }
        }
        // the stage is released after its values are read, when its loads have returned
        const float wd = quad_row_product(kb, ke, q, scols, svals, CAP, gather);
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(&ss.empty[rc.slot]));
        const float w0 = __shfl_sync(0xffffffffu, wd, qb), w1 = __shfl_sync(0xffffffffu, wd, qb + 1),
                    w2 = __shfl_sync(0xffffffffu, wd, qb + 2);
        FF t[kLaSums];
#pragma unroll
        for (int k = 0; k < kLaSums; ++k) t[k] = FF{0.f, 0.f};
        float sv[7];  // the owner's stores, issued after the partials are published
        if constexpr (kEntry) {
            if (own) {
                const float mwd = dv.x * w0 + dv.y * w1 + dv.z * w2;
                const float mqd = first ? 0.f : dv.x * qrow.x + dv.y * qrow.y + dv.z * qrow.z;
                const float qd = first ? 0.f : (q == 0 ? qrow.x : q == 1 ? qrow.y : qrow.z);
                t[2] = ff_prod(zp, wd);
                t[3] = ff_add(ff_prod(zp, qd), ff_prod(po, wd));
                t[4] = ff_prod(po, qd);
                sv[0] = zp;
                sv[1] = mwd;
                sv[2] = mqd;
            }
        } else {
            // every lane takes part in the shuffles (non-owners carry zeros)
            const float pd = __fmaf_rn(beta, po, zp);
            const float qd = __fmaf_rn(beta, qo, wo);
            const float xd = __fmaf_rn(alpha, pd, xo);
            const float rd = __fmaf_rn(-alpha, qd, ro);
            const float r0 = __shfl_sync(0xffffffffu, rd, qb), r1 = __shfl_sync(0xffffffffu, rd, qb + 1),
                        r2 = __shfl_sync(0xffffffffu, rd, qb + 2);
            const float q0 = __shfl_sync(0xffffffffu, qd, qb), q1 = __shfl_sync(0xffffffffu, qd, qb + 1),
                        q2 = __shfl_sync(0xffffffffu, qd, qb + 2);
            if (own) {
                const float mwd = dv.x * w0 + dv.y * w1 + dv.z * w2;
                const float zd = dv.x * r0 + dv.y * r1 + dv.z * r2;
                const float mqd = dv.x * q0 + dv.y * q1 + dv.z * q2;
                sv[0] = zd;
                sv[1] = mwd;
                sv[2] = mqd;
                sv[3] = pd;
                sv[4] = qd;
                sv[5] = xd;
                sv[6] = rd;
                t[0] = ff_prod(rd, rd);
                t[1] = ff_prod(rd, zd);
                t[2] = ff_prod(zd, wd);
                t[3] = ff_add(ff_prod(zd, qd), ff_prod(pd, wd));
                t[4] = ff_prod(pd, qd);
            }
        }
        // publish first: its block-scope fence then waits for no store of this stage
        la_publish<kF64Sums>(t, ss, rc.g % (unsigned)(NS + 1), cw, c, n_chunks, part);
        if (own) {
            V.zo[o] = sv[0];
            V.mwo[o] = sv[1];
            V.mqo[o] = sv[2];
            V.w[o] = wd;
            if constexpr (kEntry) {
                if (first) {  // no earlier direction: p = q = 0 for the first update
                    B.p[o] = 0.f;
                    B.q[o] = 0.f;
                }
            } else {
                B.p[o] = sv[3];
                B.q[o] = sv[4];
                B.x[o] = sv[5];
                B.r[o] = sv[6];
            }
        }
        rc.advance(NS);
    }
    seq = rc.g;
}

// Fixed-order sums of the kLaSums chunk partial arrays (value-major, n each), returned to every
// thread.  sh: kLaSums * 2 floats per warp.
template <bool kF64Sums>
__device__ void la_sum_partials(const double* part, int n, double* sh, double (&out)[kLaSums])
{
    __shared__ double result[kLaSums];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if constexpr (kF64Sums) {
#pragma unroll
        for (int k = 0; k < kLaSums; ++k) {
            double a = 0.0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) a += __ldcg(part + (size_t)k * n + i);
            const double r = block_reduce<false>(a, sh);
            if (threadIdx.x == 0) result[k] = r;
        }
    } else {
        const float2* p2 = reinterpret_cast<const float2*>(part);
        FF a[kLaSums];
#pragma unroll
        for (int k = 0; k < kLaSums; ++k) a[k] = FF{0.f, 0.f};
        int i = threadIdx.x;
        constexpr int U = 4;  // chunks per thread in flight (kLaSums loads each)
        for (; i + (U - 1) * (int)blockDim.x < n; i += U * blockDim.x) {
            float2 v[U][kLaSums];
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int k = 0; k < kLaSums; ++k) v[u][k] = __ldcg(p2 + (size_t)k * n + i + u * blockDim.x);
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int k = 0; k < kLaSums; ++k) a[k] = ff_add(a[k], FF{v[u][k].x, v[u][k].y});
        }
        for (; i < n; i += blockDim.x) {
            float2 v[kLaSums];
#pragma unroll
            for (int k = 0; k < kLaSums; ++k) v[k] = __ldcg(p2 + (size_t)k * n + i);
#pragma unroll
            for (int k = 0; k < kLaSums; ++k) a[k] = ff_add(a[k], FF{v[k].x, v[k].y});
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int k = 0; k < kLaSums; ++k) a[k] = ff_add(a[k], ff_shfl_down(a[k], o));
        float* shf = reinterpret_cast<float*>(sh);
        __syncthreads();
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < kLaSums; ++k) {
                shf[(warp * kLaSums + k) * 2] = a[k].hi;
                shf[(warp * kLaSums + k) * 2 + 1] = a[k].lo;
            }
        __syncthreads();
        if (warp == 0) {
#pragma unroll
            for (int k = 0; k < kLaSums; ++k)
                a[k] = lane < nw ? FF{shf[(lane * kLaSums + k) * 2], shf[(lane * kLaSums + k) * 2 + 1]} : FF{0.f, 0.f};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int k = 0; k < kLaSums; ++k) a[k] = ff_add(a[k], ff_shfl_down(a[k], o));
            if (lane == 0)
#pragma unroll
                for (int k = 0; k < kLaSums; ++k) result[k] = (double)a[k].hi + (double)a[k].lo;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kLaSums; ++k) out[k] = result[k];
}

template <bool kF64Sums>
__global__ void __launch_bounds__(kStagedThreads, 2) k_pcg_solve_la(PcgBuffers<float> B)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ double sh[kLaSums * (kStagedThreads / 32)];  // la_sum_partials: 2 floats per value and warp
    __shared__ int aborted, barrier_ok;
    __shared__ PcgState st0;  // as k_pcg_init or the residual replacement left it
    if (threadIdx.x == 0) st0 = *B.state;
    __syncthreads();
    if (st0.done) return;
    const int NS = B.staged.stages;
    const StagedShared ss = la_shared(smem, NS);
    if (threadIdx.x == 0) aborted = 0;
    if (threadIdx.x <= NS) ss.wcount[threadIdx.x] = 0;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(smem_addr(&ss.full[s]), 1);
            mbar_init(smem_addr(&ss.empty[s]), kStagedConsumerWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    volatile int* abort_flag = &aborted;
    unsigned* bar = B.tickets + 6;
    unsigned* ctr = B.tickets + 8;  // chunk counters of three consecutive passes
    unsigned generation = 0, seq = 0, issued = 0;
    DynProducer P;
    const int n_chunks = pcg_chunks(B.n_blocks, B.staged.stage_rows);
    const bool first = st0.iteration == 0;
    // after a residual replacement the state holds the new r.z and beta (k_pcg_replace_residual);
    // the FP64 recurrence is thread 0's (PcgCtl)
    __shared__ PcgCtl ctl;
    if (threadIdx.x == 0) {
        ctl.rz = st0.rz;
        ctl.alpha64 = 0.0;
        ctl.beta64 = first ? 0.0 : st0.beta;
        ctl.pAp = ctl.rr = 0.0;
        ctl.error = st0.error;
        ctl.iteration = st0.iteration;
        ctl.converged = ctl.indefinite = ctl.paused = ctl.have_rr = 0;
        ctl.thr_abs = st0.abs_tol * st0.abs_tol * st0.bb;
        ctl.thr_rel = st0.rel_tol * st0.error0 * st0.rel_tol * st0.error0 * st0.bb;
    }
    bool failed = false;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int li = 0;; ++li) {
        // no block claims from pass li - 1 any more, none from pass li + 2 before the barrier
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(&ctr[(li + 2) % 3], 0u);
        const LaVectors V = la_vectors(B, li & 1);
        double* part = B.partials + (size_t)(li & 1) * kLaSums * n_chunks;
        if (warp == 0) {
            if (lane == 0) dyn_produce(B, ss, li, ctr, n_chunks, issued, P, abort_flag);
        } else if (li == 0) {
            la_consume<kF64Sums, true>(B, ss, V, n_chunks, 0.f, 0.f, first, part, seq, abort_flag);
        } else {
            la_consume<kF64Sums, false>(B, ss, V, n_chunks, ctl.alpha, ctl.beta, false, part, seq, abort_flag);
        }
        if (!grid_barrier(bar, generation, &barrier_ok, B.staged.max_polls) || *abort_flag) {
            failed = true;
            break;
        }
        double sums[kLaSums];
        la_sum_partials<kF64Sums>(part, n_chunks, sh, sums);
        if (threadIdx.x == 0) {
            ctl.stop = 1;
            bool go = true;
            if (li > 0) {  // the pass formed x_k and r_k: the reference's test after its update
                ctl.iteration += 1;
                ctl.rr = sums[0];
                ctl.have_rr = 1;
                if (ctl.rr < ctl.thr_abs || ctl.rr < ctl.thr_rel) {
                    ctl.converged = 1;
                    go = false;
                } else if (ctl.iteration >= st0.max_iterations) {
                    go = false;
                } else if (st0.replace_every > 0 && ctl.iteration % st0.replace_every == 0) {
                    ctl.paused = 1;  // rz stays that of the last iterate: the replacement forms beta
                    go = false;
                } else {
                    ctl.beta64 = sums[1] / ctl.rz;
                    ctl.rz = sums[1];
                }
            }
            if (go) {
                const double beta = ctl.beta64;
                ctl.pAp = sums[2] + beta * sums[3] + beta * beta * sums[4];
                if (!(ctl.pAp > 0.0)) {  // indefinite (or NaN): stop as the reference does
                    ctl.indefinite = 1;
                    ctl.iteration += 1;
                } else {
                    ctl.alpha64 = ctl.rz / ctl.pAp;
                    ctl.alpha = (float)ctl.alpha64;
                    ctl.beta = (float)beta;
                    ctl.stop = 0;
                }
            }
        }
        __syncthreads();
        if (ctl.stop) break;
    }
    staged_drain(B, ss, issued);  // stages copied ahead for a pass that will not run
    if (failed && threadIdx.x == 0) atomicExch(&B.state->wait_failed, 1);
    if (blockIdx.x == 0 && threadIdx.x == 0 && !failed) {
        PcgState* st = B.state;
        st->iteration = ctl.iteration;
        st->converged = ctl.converged;
        st->indefinite = ctl.indefinite;
        st->done = ctl.paused ? 0 : 1;
        st->pAp = ctl.pAp;
        st->alpha = ctl.alpha64;
        st->beta = ctl.beta64;
        st->rz = ctl.rz;
        st->rr = ctl.rr;
        st->error = ctl.have_rr ? sqrt(ctl.rr / st0.bb) : st0.error;
    }
}

// Residual replacement (see launch_pcg_replace_residual): one half-warp per block row,
// lane-strided over the row's blocks, products and sums in FP64.
__global__ void __launch_bounds__(256) k_pcg_replace_residual(PcgBuffers<float> B, const double* __restrict__ grad)
{
    if (B.state->done) return;
    __shared__ double sh[32];
    const int lane16 = threadIdx.x & 15, half = (threadIdx.x >> 4) & 1;
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, warps_total = (gridDim.x * blockDim.x) >> 5;
    const int64_t st = B.vals_stride;
    double rr = 0.0, rz = 0.0;
    // two rows per warp and pass; the loop bound is warp-uniform, so the full-mask shuffles
    // below are converged (a half-warp past the last row adds zeros)
    for (int base = 2 * warp_global; base < B.n_blocks; base += 2 * warps_total) {
        const int row = base + half;
        const bool valid = row < B.n_blocks;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        const int kb = valid ? B.row_ptr[row] : 0, ke = valid ? B.row_ptr[row + 1] : 0;
        for (int k = kb + lane16; k < ke; k += 16) {
            const Row4<float> x = ld4(B.x + 4 * B.cols[k]);
            const float* __restrict__ m = B.vals + k;
            const double x0 = x.x, x1 = x.y, x2 = x.z;
            a0 = fma((double)m[0], x0, fma((double)m[st], x1, fma((double)m[2 * st], x2, a0)));
            a1 = fma((double)m[3 * st], x0, fma((double)m[4 * st], x1, fma((double)m[5 * st], x2, a1)));
            a2 = fma((double)m[6 * st], x0, fma((double)m[7 * st], x1, fma((double)m[8 * st], x2, a2)));
        }
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {
            a0 += __shfl_xor_sync(0xffffffffu, a0, o, 16);
            a1 += __shfl_xor_sync(0xffffffffu, a1, o, 16);
            a2 += __shfl_xor_sync(0xffffffffu, a2, o, 16);
        }
        if (valid && lane16 == 0) {
            const Row4<float> r{(float)(-grad[3 * row] - a0), (float)(-grad[3 * row + 1] - a1),
                                (float)(-grad[3 * row + 2] - a2), 0.0f};
            const Row4<float> z = apply_block_jacobi(B.Dinv, row, r);
            st4(B.r + 4 * row, r);
            st4(B.z + 4 * row, z);
            rr = fma((double)r.x, (double)r.x, fma((double)r.y, (double)r.y, fma((double)r.z, (double)r.z, rr)));
            rz = fma((double)r.x, (double)z.x, fma((double)r.y, (double)z.y, fma((double)r.z, (double)z.z, rz)));
        }
    }
    const double bv[2] = {block_reduce<false>(rr, sh), block_reduce<false>(rz, sh)};
    double res[2];
    if (publish_and_combine<2>(bv, B.partials, B.tickets + 1, res) && threadIdx.x == 0) {
        PcgState* s = B.state;
        s->replacements += 1;
        s->rr = res[0];
        s->error = sqrt(res[0] / s->bb);
        if (s->error < s->abs_tol || s->error / s->error0 < s->rel_tol) {
            s->converged = 1;
            s->done = 1;
        } else if (s->iteration >= s->max_iterations) {
            s->done = 1;
        } else {
            s->beta = res[1] / s->rz;
            s->rz = res[1];
        }
    }
}

// r = b = -grad (as T), x = 0, z = M^-1 r; b.b (double, from the FP64 gradient) and r.z.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_init(PcgBuffers<T> B, const double* __restrict__ grad)
{
    __shared__ double sh[32];
    double bb = 0.0;
    DotAcc<T> rz;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n_blocks; i += gridDim.x * blockDim.x) {
        const double b0 = -grad[3 * i], b1 = -grad[3 * i + 1], b2 = -grad[3 * i + 2];
        bb = fma(b0, b0, fma(b1, b1, fma(b2, b2, bb)));
        const Row4<T> r{(T)b0, (T)b1, (T)b2, T(0)};
        const Row4<T> z = apply_block_jacobi(B.Dinv, i, r);
        st4(B.r + 4 * i, r);
        st4(B.x + 4 * i, Row4<T>{T(0), T(0), T(0), T(0)});
        st4(B.z + 4 * i, z);
        rz.add_prod(r.x, z.x);
        rz.add_prod(r.y, z.y);
        rz.add_prod(r.z, z.z);
    }
    const double bv[2] = {block_reduce<false>(bb, sh), rz.block_sum(sh)};
    double res[2];
    if (publish_and_combine<2>(bv, B.partials, B.tickets + 2, res) && threadIdx.x == 0) {
        PcgState* st = B.state;
        st->bb = res[0];
        st->rz = res[1];
        st->iteration = 0;
        st->indefinite = 0;
        st->converged = 0;
        st->done = 0;
        if (res[0] < st->abs_tol * st->abs_tol) {  // zero right-hand side: x = 0
            st->error = 0.0;
            st->converged = 1;
            st->done = 1;
        } else {
            st->error0 = 1.0;  // x0 = 0, so r = b exactly: sqrt(r.r / b.b) = 1
            st->error = 1.0;
            if (st->error < st->abs_tol) { st->converged = 1; st->done = 1; }
        }
    }
}

// Same as k_pcg_init for a right-hand side b given in T with 3 values per block row.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_init_rhs(PcgBuffers<T> B, const T* __restrict__ b3)
{
    __shared__ double sh[32];
    double bb = 0.0;
    DotAcc<T> rz;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n_blocks; i += gridDim.x * blockDim.x) {
        const Row4<T> r{b3[3 * i], b3[3 * i + 1], b3[3 * i + 2], T(0)};
        bb = fma((double)r.x, (double)r.x, fma((double)r.y, (double)r.y, fma((double)r.z, (double)r.z, bb)));
        const Row4<T> z = apply_block_jacobi(B.Dinv, i, r);
        st4(B.r + 4 * i, r);
        st4(B.x + 4 * i, Row4<T>{T(0), T(0), T(0), T(0)});
        st4(B.z + 4 * i, z);
        rz.add_prod(r.x, z.x);
        rz.add_prod(r.y, z.y);
        rz.add_prod(r.z, z.z);
    }
    const double bv[2] = {block_reduce<false>(bb, sh), rz.block_sum(sh)};
    double res[2];
    if (publish_and_combine<2>(bv, B.partials, B.tickets + 2, res) && threadIdx.x == 0) {
        PcgState* st = B.state;
        st->bb = res[0];
        st->rz = res[1];
        st->iteration = 0;
        st->indefinite = 0;
        st->converged = 0;
        st->done = 0;
        if (res[0] < st->abs_tol * st->abs_tol) {
            st->error = 0.0;
            st->converged = 1;
            st->done = 1;
        } else {
            st->error0 = 1.0;
            st->error = 1.0;
            if (st->error < st->abs_tol) { st->converged = 1; st->done = 1; }
        }
    }
}

template <typename T>
__global__ void k_rows4_to_vec3(int n_rows, const T* __restrict__ in4, T* __restrict__ out3)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 3 * (int64_t)n_rows) return;
    const int64_t i = k / 3, d = k - 3 * i;
    out3[k] = in4[4 * i + d];
}

// ---- Newton helpers on the PCG solution (4 values per block row)
template <typename T>
__global__ void k_dot_rows4(const T* __restrict__ du, const double* __restrict__ g, int n_rows, double* partials,
                            unsigned* ticket, double* out)
{
    int64_t b, e;
    chunk_range(n_rows, b, e);
    double acc = 0.0;
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x)
        acc += (double)du[4 * i] * g[3 * i] + (double)du[4 * i + 1] * g[3 * i + 1] + (double)du[4 * i + 2] * g[3 * i + 2];
    double mine[1] = {acc}, res[1];
    if (last_block_combine<false, 1>(mine, partials, ticket, res) && threadIdx.x == 0) out[0] = res[0];
}

template <typename T>
__global__ void k_max_abs_rows4(const T* __restrict__ du, int n_rows, double* partials, unsigned* ticket, double* out)
{
    int64_t b, e;
    chunk_range(n_rows, b, e);
    float acc = 0.f;
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x)
        for (int d = 0; d < 3; ++d) {
            const float v = (float)du[4 * i + d];
            acc = fmaxf(acc, isnan(v) ? __int_as_float(0x7f800000) : fabsf(v));
        }
    double mine[1] = {(double)acc}, res[1];
    if (last_block_combine<true, 1>(mine, partials, ticket, res) && threadIdx.x == 0) out[0] = res[0];
}

template <typename T>
__global__ void k_axpy_rows4(int n_rows, const double* __restrict__ x0, double step, const T* __restrict__ du,
                             double* __restrict__ x)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 3 * (int64_t)n_rows) return;
    const int64_t i = k / 3, d = k - 3 * i;
    x[k] = x0[k] + step * (double)du[4 * i + d];
}

template <typename T>
__global__ void k_axpy_to(int64_t n, const double* __restrict__ x0, double step, const T* __restrict__ du,
                          double* __restrict__ x)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = x0[i] + step * (double)du[i];
}

template <typename T>
__global__ void k_convert(int64_t n, const T* __restrict__ x, double* __restrict__ y)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = (double)x[i];
}

std::atomic<int64_t> g_launches{0};

inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

void check_launch(const char* what)
{
    g_launches.fetch_add(1, std::memory_order_relaxed);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(std::string("symx_gb300: launch of ") + what + " failed: " + cudaGetErrorString(e));
}

// Blocks of `kernel` resident at once on the whole device (cached per kernel).
template <typename K>
unsigned resident_grid(K kernel, int threads)
{
    static std::mutex m;
    static std::map<std::pair<const void*, int>, unsigned> cache;  // per (kernel, device)
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(m);
    const auto key = std::make_pair((const void*)kernel, dev);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
    const unsigned g = (unsigned)std::max(1, sms * std::max(1, per_sm));
    cache[key] = g;
    return g;
}

}  // namespace

int64_t launch_count() { return g_launches.load(); }
std::atomic<long long> g_wait_polls{kDefaultWaitPolls};
void set_wait_poll_limit(long long polls) { g_wait_polls.store(polls < 0 ? kDefaultWaitPolls : polls); }
long long wait_poll_limit() { return g_wait_polls.load(); }
void count_launch(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
std::atomic<int64_t> g_dev_bytes{0}, g_dev_peak{0};
void note_device_alloc(int64_t bytes)
{
    const int64_t now = g_dev_bytes.fetch_add(bytes) + bytes;
    int64_t peak = g_dev_peak.load();
    while (now > peak && !g_dev_peak.compare_exchange_weak(peak, now)) {
    }
}
void note_device_free(int64_t bytes) { g_dev_bytes.fetch_sub(bytes); }
int64_t device_bytes_current() { return g_dev_bytes.load(); }
int64_t device_bytes_peak(bool reset)
{
    const int64_t p = g_dev_peak.load();
    if (reset) g_dev_peak.store(g_dev_bytes.load());
    return p;
}

void launch_sum(const double* x, int64_t n, double* partials, unsigned* ticket, double* out, cudaStream_t s)
{
    k_sum<<<kReduceBlocks, kReduceThreads, 0, s>>>(x, n, partials, ticket, out);
    check_launch("sum");
}

void launch_max_abs(const double* x, int64_t n, double* partials, unsigned* ticket, double* out, cudaStream_t s)
{
    k_max_abs<double><<<kReduceBlocks, kReduceThreads, 0, s>>>(x, n, partials, ticket, out);
    check_launch("max_abs");
}

template <typename T>
void launch_dot_mixed(const T* a, const double* b, int64_t n, double* partials, unsigned* ticket, double* out,
                      cudaStream_t s)
{
    k_dot_mixed<T><<<kReduceBlocks, kReduceThreads, 0, s>>>(a, b, n, partials, ticket, out);
    check_launch("dot");
}

// Warp-per-matrix projection (k_project_pd_pairs) of N x N matrices, N = 18, 24 or 30: a
// persistent grid of the resident blocks, dynamic shared memory set up once per device.
template <typename T, int N>
void launch_project_pd_pairs(T* H, int64_t count, T eps, bool mirroring, int* not_converged, const int64_t* sel,
                             cudaStream_t s)
{
    using Cfg = ProjPairsCfg<T, N>;
    constexpr int threads = Cfg::warps * 32;
    static std::mutex m;
    static std::map<int, bool> configured;
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lock(m);
        if (!configured[dev]) {
            const cudaError_t e = cudaFuncSetAttribute(k_project_pd_pairs<T, N>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::smem_bytes);
            if (e != cudaSuccess)
                throw std::runtime_error(std::string("symx_gb300: projection shared memory: ") + cudaGetErrorString(e));
            configured[dev] = true;
        }
    }
    int per_sm = 0, sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_project_pd_pairs<T, N>, threads, Cfg::smem_bytes);
    const unsigned grid = (unsigned)std::max(1, sms * std::max(1, per_sm));
    const unsigned need = blocks_for(count, Cfg::warps);
    k_project_pd_pairs<T, N><<<need < grid ? need : grid, threads, Cfg::smem_bytes, s>>>(H, count, eps, mirroring,
                                                                                        not_converged, sel);
}

template <typename T>
void launch_project_pd(T* H, int N, int64_t count, T eps, bool mirroring, int* not_converged, cudaStream_t s,
                       ProjectionScratch scratch, const int64_t* sel)
{
    if (count <= 0) return;
    if (N == 12 && scratch.fallback && scratch.n_fallback) {
        const bool split = scratch.pending && scratch.n_pending;
        const cudaError_t e = cudaMemsetAsync(scratch.n_fallback, 0, sizeof(unsigned long long), s);
        if (e != cudaSuccess) throw std::runtime_error(std::string("symx_gb300: memset: ") + cudaGetErrorString(e));
        if (split) {
            const cudaError_t e2 = cudaMemsetAsync(scratch.n_pending, 0, sizeof(unsigned long long), s);
            if (e2 != cudaSuccess) throw std::runtime_error(std::string("symx_gb300: memset: ") + cudaGetErrorString(e2));
        }
        if (split) {
            k_project_pd_sort<T, 12><<<blocks_for(count, 128), 128, 0, s>>>(H, count, scratch.fallback, scratch.n_fallback,
                                                                           sel, scratch.pending, scratch.n_pending);
            check_launch("project_pd_sort");
        } else {
            k_project_pd_deflated<T, 12><<<blocks_for(count, 128), 128, 0, s>>>(H, count, eps, mirroring, not_converged,
                                                                                  scratch.fallback, scratch.n_fallback, sel);
            check_launch("project_pd_deflated");
        }
        if (split) {
            const unsigned pending_grid = resident_grid(k_project_pd_deflated_listed<T, 12>, 128);
            k_project_pd_deflated_listed<T, 12><<<pending_grid, 128, 0, s>>>(H, scratch.pending, scratch.n_pending, eps,
                                                                           mirroring, not_converged);
            check_launch("project_pd_deflated_listed");
        }
        const unsigned listed_grid = resident_grid(k_project_pd_listed<T, 12>, 128);
        k_project_pd_listed<T, 12><<<listed_grid, 128, 0, s>>>(H, scratch.fallback, scratch.n_fallback, eps, mirroring,
                                                               not_converged);
        check_launch("project_pd_listed");
        return;
    }
    switch (N) {
        case 3: k_project_pd_unrolled<T, 3><<<blocks_for(count, 128), 128, 0, s>>>(H, count, eps, mirroring, not_converged, sel); break;
        case 6: k_project_pd_unrolled<T, 6><<<blocks_for(count, 128), 128, 0, s>>>(H, count, eps, mirroring, not_converged, sel); break;
        case 9: k_project_pd_unrolled<T, 9><<<blocks_for(count, 128), 128, 0, s>>>(H, count, eps, mirroring, not_converged, sel); break;
        case 12: k_project_pd_unrolled<T, 12><<<blocks_for(count, 128), 128, 0, s>>>(H, count, eps, mirroring, not_converged, sel); break;
        case 18: launch_project_pd_pairs<T, 18>(H, count, eps, mirroring, not_converged, sel, s); break;
        case 24: launch_project_pd_pairs<T, 24>(H, count, eps, mirroring, not_converged, sel, s); break;
        case 30: launch_project_pd_pairs<T, 30>(H, count, eps, mirroring, not_converged, sel, s); break;
        default:
            if (N > 30 || N % 3 != 0) throw std::runtime_error("symx_gb300: projection supports N = 3k <= 30");
            k_project_pd_generic<T><<<blocks_for(count, 64), 64, 0, s>>>(H, N, count, eps, mirroring, not_converged, sel);
    }
    check_launch("project_pd");
}

template <typename T>
void launch_project_pd_refined12(T* H, int64_t count, double eps, bool mirroring, int* not_converged, cudaStream_t s,
                                 ProjectionScratch scratch, const int64_t* sel)
{
    if (count <= 0) return;
    if (!scratch.fallback || !scratch.n_fallback || !scratch.pending || !scratch.n_pending)
        throw std::runtime_error("symx_gb300: the refined projection needs the sorting pass's lists");
    for (unsigned long long* c : {scratch.n_fallback, scratch.n_pending}) {
        const cudaError_t e = cudaMemsetAsync(c, 0, sizeof(unsigned long long), s);
        if (e != cudaSuccess) throw std::runtime_error(std::string("symx_gb300: memset: ") + cudaGetErrorString(e));
    }
    k_project_pd_sort<T, 12><<<blocks_for(count, 128), 128, 0, s>>>(H, count, scratch.fallback, scratch.n_fallback, sel,
                                                                   scratch.pending, scratch.n_pending);
    check_launch("project_pd_sort");
    const unsigned pending_grid = resident_grid(k_project_pd_refined_listed<T, 12, true>, 64);
    k_project_pd_refined_listed<T, 12, true><<<pending_grid, 64, 0, s>>>(H, scratch.pending, scratch.n_pending, eps,
                                                                         mirroring, not_converged);
    check_launch("project_pd_refined_listed");
    const unsigned fallback_grid = resident_grid(k_project_pd_refined_listed<T, 12, false>, 64);
    k_project_pd_refined_listed<T, 12, false><<<fallback_grid, 64, 0, s>>>(H, scratch.fallback, scratch.n_fallback, eps,
                                                                           mirroring, not_converged);
    check_launch("project_pd_refined_fallback");
}

template <typename T>
void launch_assemble_blocks(int64_t nnzb, const int64_t* slot_ptr, const int32_t* contrib, const T* blocks, T* vals,
                            int64_t vstride, cudaStream_t s)
{
    if (nnzb <= 0) return;
    if (vstride == kTiledBcsr)
        k_assemble_blocks<T><<<blocks_for(nnzb, 256), 256, 0, s>>>(nnzb, slot_ptr, contrib, blocks, vals, TiledBcsr{});
    else
        k_assemble_blocks<T><<<blocks_for(nnzb, 256), 256, 0, s>>>(nnzb, slot_ptr, contrib, blocks, vals,
                                                                    StridedBcsr{vstride});
    check_launch("assemble");
}

void launch_gather_gradient(int n_blocks, const int64_t* ptr, const int32_t* contrib, const double* gel, double* g,
                            cudaStream_t s)
{
    k_gather_gradient<<<blocks_for(n_blocks, 256), 256, 0, s>>>(n_blocks, ptr, contrib, gel, g);
    check_launch("gather_gradient");
}

void launch_ppn_mark_blocks(int n_blocks, const double* grad, double thr, const int64_t* gptr, const int32_t* gcontrib,
                            uint8_t* gflag, unsigned long long* n_inactive, cudaStream_t s)
{
    if (n_blocks <= 0) return;
    k_ppn_mark_blocks<<<blocks_for(n_blocks, 256), 256, 0, s>>>(n_blocks, grad, thr, gptr, gcontrib, gflag, n_inactive);
    check_launch("ppn_mark_blocks");
}

void launch_select_elements(int64_t n_el, int nb, const uint8_t* gflag, uint8_t* is_proj, int64_t* sel,
                            unsigned long long* n_sel, cudaStream_t s)
{
    if (n_el <= 0) return;
    k_select_elements<<<blocks_for(n_el, 256), 256, 0, s>>>(n_el, nb, gflag, is_proj, sel, n_sel);
    check_launch("select_elements");
}

template <typename T>
void launch_block_jacobi_setup(int n_blocks, const int32_t* diag_slot, const T* vals, int64_t vstride, T* Dinv,
                               cudaStream_t s)
{
    if (vstride == kTiledBcsr)
        k_block_jacobi_setup<T><<<blocks_for(n_blocks, 256), 256, 0, s>>>(n_blocks, diag_slot, vals, TiledBcsr{}, Dinv);
    else
        k_block_jacobi_setup<T><<<blocks_for(n_blocks, 256), 256, 0, s>>>(n_blocks, diag_slot, vals,
                                                                           StridedBcsr{vstride}, Dinv);
    check_launch("block_jacobi_setup");
}


template <typename T>
void launch_pcg_init(const PcgBuffers<T>& B, const double* grad, cudaStream_t s)
{
    const unsigned g = std::min<unsigned>(blocks_for(B.n_blocks, 256), resident_grid(k_pcg_init<T>, 256));
    k_pcg_init<T><<<g, 256, 0, s>>>(B, grad);
    check_launch("pcg_init");
}

template <typename T, typename L>
void launch_pcg_spmv_l(const PcgBuffers<T>& B, L lay, int iteration, cudaStream_t s)
{
    const unsigned gs = std::min<unsigned>(blocks_for((int64_t)B.n_blocks * 8, kSpmvThreads),
                                           resident_grid(k_pcg_spmv<T, L>, kSpmvThreads));
    T* p_old = (iteration & 1) ? B.p : B.p2;
    T* p_new = (iteration & 1) ? B.p2 : B.p;
    k_pcg_spmv<T, L><<<gs, kSpmvThreads, 0, s>>>(B, lay, p_old, p_new, iteration == 0 ? 1 : 0);
    check_launch("pcg_spmv");
}

template <typename T>
void launch_pcg_spmv(const PcgBuffers<T>& B, int iteration, cudaStream_t s)
{
    if constexpr (std::is_same<T, float>::value) {
        if (B.staged.stages > 0 && B.vals_stride != kTiledBcsr) {
            float* p_old = (iteration & 1) ? B.p : B.p2;
            float* p_new = (iteration & 1) ? B.p2 : B.p;
            PcgBuffers<float> arg = B;
            arg.staged.max_polls = wait_poll_limit();
            k_pcg_spmv_staged<<<B.staged.grid, kStagedThreads, B.staged.smem_bytes, s>>>(arg, p_old, p_new,
                                                                                        iteration == 0 ? 1 : 0);
            check_launch("pcg_spmv_staged");
            return;
        }
    }
    if (B.vals_stride == kTiledBcsr) launch_pcg_spmv_l<T>(B, TiledBcsr{}, iteration, s);
    else launch_pcg_spmv_l<T>(B, StridedBcsr{B.vals_stride}, iteration, s);
}

void launch_pcg_solve_persistent(const PcgBuffers<float>& B, cudaStream_t s)
{
    if (!B.staged.persistent) throw std::runtime_error("symx_gb300: persistent PCG not planned for this matrix");
    const cudaError_t e = cudaMemsetAsync(B.tickets + 6, 0, 5 * sizeof(unsigned), s);
    if (e != cudaSuccess) throw std::runtime_error(std::string("symx_gb300: memset: ") + cudaGetErrorString(e));
    PcgBuffers<float> arg = B;
    arg.staged.max_polls = wait_poll_limit();
    void* args[] = {&arg};
    const bool la = B.staged.lookahead && B.la;
    const void* fn = la ? (B.staged.f64_sums ? (const void*)k_pcg_solve_la<true> : (const void*)k_pcg_solve_la<false>)
                        : (B.staged.f64_sums ? (const void*)k_pcg_solve_staged<true>
                                             : (const void*)k_pcg_solve_staged<false>);
    const cudaError_t l = cudaLaunchCooperativeKernel(fn, dim3(B.staged.grid), dim3(kStagedThreads), args,
                                                      la ? B.staged.la_smem_bytes : B.staged.smem_bytes, s);
    if (l != cudaSuccess)
        throw std::runtime_error(std::string("symx_gb300: cooperative launch of the PCG failed: ") + cudaGetErrorString(l));
    check_launch("pcg_solve_staged");
}

void launch_pcg_replace_residual(const PcgBuffers<float>& B, const double* grad, cudaStream_t s)
{
    k_pcg_replace_residual<<<kReduceBlocks, 256, 0, s>>>(B, grad);
    check_launch("pcg_replace_residual");
}

StagedSizes plan_staged_spmv(int n, const int32_t* rp, PcgBuffers<float>::Staged& st)
{
    st = PcgBuffers<float>::Staged{};
    StagedSizes none;
    if (n <= 0) return none;
    int dev = 0, sms = 0, optin = 0, per_sm_bytes = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return none;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&per_sm_bytes, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    const int S = kStagedRows;
    const int64_t nnzb = rp[n];
    for (int per_sm : {2, 1}) {
        const int64_t grid = (int64_t)sms * per_sm;
        const int64_t rows = ((n + grid - 1) / grid + S - 1) / S * S;
        int64_t cap = 4;
        for (int64_t r0 = 0; r0 < grid * rows; r0 += S) {  // chunks (dynamic schedule, fixed ranges)
            const int64_t kb = rp[std::min<int64_t>(r0, n)], ke = rp[std::min<int64_t>(r0 + S, n)];
            cap = std::max<int64_t>(cap, ((ke + 3) & ~int64_t(3)) - (kb & ~int64_t(3)));
        }
        for (int64_t b = 0; b < grid; ++b) {  // stages of the even row split (persistent kernel)
            int rb, re;
            pcg_block_rows(b, grid, n, rb, re);
            for (int64_t r0 = rb; r0 < re; r0 += S) {
                const int64_t kb = rp[r0], ke = rp[std::min<int64_t>(r0 + S, re)];
                cap = std::max<int64_t>(cap, ((ke + 3) & ~int64_t(3)) - (kb & ~int64_t(3)));
            }
        }
        const size_t stage_bytes = staged_stage_bytes((int)cap, S);
        const int64_t budget =
            std::min<int64_t>(optin, per_sm_bytes / per_sm - 1024) - (int64_t)kStagedHeaderBytes - 1024;  // static smem
        const int stages = (int)std::min<int64_t>(kStagedMaxStages, budget / (int64_t)stage_bytes);
        if (stages < 2 || cap > (1 << 24)) continue;
        const size_t smem = kStagedHeaderBytes + (size_t)stages * stage_bytes;
        if (cudaFuncSetAttribute(k_pcg_spmv_staged, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        int resident = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_pcg_spmv_staged, kStagedThreads, smem) !=
                cudaSuccess ||
            resident < per_sm) {
            cudaGetLastError();
            continue;
        }
        // the persistent form needs every block resident at once (cooperative launch)
        int coop = 0, resident_ff = 0, resident_f64 = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        if (coop &&
            cudaFuncSetAttribute(k_pcg_solve_staged<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
                cudaSuccess &&
            cudaFuncSetAttribute(k_pcg_solve_staged<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
                cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident_ff, k_pcg_solve_staged<false>, kStagedThreads,
                                                          smem) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident_f64, k_pcg_solve_staged<true>, kStagedThreads,
                                                          smem) == cudaSuccess &&
            resident_ff >= per_sm && resident_f64 >= per_sm &&
            3 * grid <= 2 * kPcgMaxPartials)
            st.persistent = 1;
        cudaGetLastError();
        // the look-ahead form: its own header, the same ring; partials of two passes
        const size_t la_smem = la_header_bytes(stages) + (size_t)stages * stage_bytes;
        const int64_t la_budget = std::min<int64_t>(optin, per_sm_bytes / per_sm - 1024) - 1024;  // static smem
        int resident_la0 = 0, resident_la1 = 0;
        if (st.persistent && (int64_t)la_smem <= la_budget &&
            cudaFuncSetAttribute(k_pcg_solve_la<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)la_smem) ==
                cudaSuccess &&
            cudaFuncSetAttribute(k_pcg_solve_la<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)la_smem) ==
                cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident_la0, k_pcg_solve_la<false>, kStagedThreads,
                                                          la_smem) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident_la1, k_pcg_solve_la<true>, kStagedThreads,
                                                          la_smem) == cudaSuccess &&
            resident_la0 >= per_sm && resident_la1 >= per_sm &&
            (int64_t)2 * kLaSums * pcg_chunks(n, S) <= 2 * (int64_t)kPcgMaxPartials) {
            st.lookahead = 1;
            st.la_smem_bytes = la_smem;
        }
        cudaGetLastError();
        st.stages = stages;
        st.stage_rows = S;
        st.stage_cap = (int)cap;
        st.rows_per_block = (int)rows;
        st.grid = (int)grid;
        st.smem_bytes = smem;
        StagedSizes z;
        z.row_ptr_ext = grid * rows + S + 8;
        z.cols_ext = ((nnzb + 3) & ~int64_t(3)) + 4;
        return z;
    }
    return none;
}

template <typename T>
void launch_pcg_update(const PcgBuffers<T>& B, int iteration, cudaStream_t s)
{
    T* p_new = (iteration & 1) ? B.p2 : B.p;
    const unsigned gu = std::min<unsigned>(blocks_for(B.n_blocks, 256), resident_grid(k_pcg_update<T>, 256));
    k_pcg_update<T><<<gu, 256, 0, s>>>(B, p_new);
    check_launch("pcg_update");
}

template <typename T>
void launch_pcg_iteration(const PcgBuffers<T>& B, int iteration, cudaStream_t s)
{
    launch_pcg_spmv<T>(B, iteration, s);
    launch_pcg_update<T>(B, iteration, s);
}

template <typename T>
void launch_bcsr_spmv(int n_blocks, const int32_t* row_ptr, const int32_t* cols, const T* vals, int64_t vstride,
                      const T* x, T* y, cudaStream_t s)
{
    if (n_blocks <= 0) return;
    const unsigned blocks = blocks_for((int64_t)n_blocks * 8, kSpmvThreads);
    if (vstride == kTiledBcsr) {
        const unsigned g = std::min<unsigned>(blocks, resident_grid(k_bcsr_spmv<T, TiledBcsr>, kSpmvThreads));
        k_bcsr_spmv<T><<<g, kSpmvThreads, 0, s>>>(n_blocks, row_ptr, cols, vals, TiledBcsr{}, x, y);
    } else {
        const unsigned g = std::min<unsigned>(blocks, resident_grid(k_bcsr_spmv<T, StridedBcsr>, kSpmvThreads));
        k_bcsr_spmv<T><<<g, kSpmvThreads, 0, s>>>(n_blocks, row_ptr, cols, vals, StridedBcsr{vstride}, x, y);
    }
    check_launch("bcsr_spmv");
}

template <typename T>
void launch_pcg_init_rhs(const PcgBuffers<T>& B, const T* b3, cudaStream_t s)
{
    const unsigned g = std::min<unsigned>(blocks_for(B.n_blocks, 256), resident_grid(k_pcg_init_rhs<T>, 256));
    k_pcg_init_rhs<T><<<g, 256, 0, s>>>(B, b3);
    check_launch("pcg_init_rhs");
}

template <typename T>
void launch_rows4_to_vec3(int n_rows, const T* in4, T* out3, cudaStream_t s)
{
    k_rows4_to_vec3<T><<<blocks_for(3 * (int64_t)n_rows, 256), 256, 0, s>>>(n_rows, in4, out3);
    check_launch("rows4_to_vec3");
}

unsigned pcg_max_grid()
{
    return std::max({resident_grid(k_pcg_spmv<float, TiledBcsr>, kSpmvThreads),
                     resident_grid(k_pcg_spmv<float, StridedBcsr>, kSpmvThreads),
                     resident_grid(k_pcg_spmv<double, TiledBcsr>, kSpmvThreads),
                     resident_grid(k_pcg_spmv<double, StridedBcsr>, kSpmvThreads), resident_grid(k_pcg_update<float>, 256),
                     resident_grid(k_pcg_init<float>, 256), resident_grid(k_pcg_init_rhs<float>, 256),
                     resident_grid(k_pcg_update<double>, 256),
                     resident_grid(k_pcg_init<double>, 256), resident_grid(k_pcg_init_rhs<double>, 256)});
}

template <typename T>
void launch_dot_rows4(const T* du, const double* g, int n_rows, double* partials, unsigned* ticket, double* out,
                      cudaStream_t s)
{
    k_dot_rows4<T><<<kReduceBlocks, kReduceThreads, 0, s>>>(du, g, n_rows, partials, ticket, out);
    check_launch("dot_rows4");
}

template <typename T>
void launch_max_abs_rows4(const T* du, int n_rows, double* partials, unsigned* ticket, double* out, cudaStream_t s)
{
    k_max_abs_rows4<T><<<kReduceBlocks, kReduceThreads, 0, s>>>(du, n_rows, partials, ticket, out);
    check_launch("max_abs_rows4");
}

template <typename T>
void launch_axpy_rows4(int n_rows, const double* x0, double step, const T* du, double* x_out, cudaStream_t s)
{
    k_axpy_rows4<T><<<blocks_for(3 * (int64_t)n_rows, 256), 256, 0, s>>>(n_rows, x0, step, du, x_out);
    check_launch("axpy_rows4");
}

template <typename T>
void launch_axpy_to(int64_t n, const double* x0, double step, const T* du, double* x_out, cudaStream_t s)
{
    k_axpy_to<T><<<blocks_for(n, 256), 256, 0, s>>>(n, x0, step, du, x_out);
    check_launch("axpy");
}

template <typename T>
void launch_convert_to_double(int64_t n, const T* x, double* y, cudaStream_t s)
{
    k_convert<T><<<blocks_for(n, 256), 256, 0, s>>>(n, x, y);
    check_launch("convert");
}

#define SYMXG_INSTANTIATE(T)                                                                                          \
    template void launch_dot_mixed<T>(const T*, const double*, int64_t, double*, unsigned*, double*, cudaStream_t);  \
    template void launch_project_pd_refined12<T>(T*, int64_t, double, bool, int*, cudaStream_t, ProjectionScratch,    \
                                                 const int64_t*);                                                     \
    template void launch_project_pd<T>(T*, int, int64_t, T, bool, int*, cudaStream_t, ProjectionScratch,               \
                                       const int64_t*);                                                                 \
    template void launch_assemble_blocks<T>(int64_t, const int64_t*, const int32_t*, const T*, T*, int64_t, cudaStream_t); \
    template void launch_block_jacobi_setup<T>(int, const int32_t*, const T*, int64_t, T*, cudaStream_t);              \
    template void launch_pcg_init<T>(const PcgBuffers<T>&, const double*, cudaStream_t);                               \
    template void launch_pcg_iteration<T>(const PcgBuffers<T>&, int, cudaStream_t);                                   \
    template void launch_pcg_spmv<T>(const PcgBuffers<T>&, int, cudaStream_t);                                        \
    template void launch_pcg_update<T>(const PcgBuffers<T>&, int, cudaStream_t);                                      \
    template void launch_bcsr_spmv<T>(int, const int32_t*, const int32_t*, const T*, int64_t, const T*, T*, cudaStream_t); \
    template void launch_axpy_to<T>(int64_t, const double*, double, const T*, double*, cudaStream_t);                  \
    template void launch_dot_rows4<T>(const T*, const double*, int, double*, unsigned*, double*, cudaStream_t);        \
    template void launch_pcg_init_rhs<T>(const PcgBuffers<T>&, const T*, cudaStream_t);                                \
    template void launch_rows4_to_vec3<T>(int, const T*, T*, cudaStream_t);                                            \
    template void launch_max_abs_rows4<T>(const T*, int, double*, unsigned*, double*, cudaStream_t);                   \
    template void launch_axpy_rows4<T>(int, const double*, double, const T*, double*, cudaStream_t);                   \
    template void launch_convert_to_double<T>(int64_t, const T*, double*, cudaStream_t);
SYMXG_INSTANTIATE(float)
SYMXG_INSTANTIATE(double)

}  // namespace symxg
