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
                                                             int* not_converged)
{
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= count) return;
    int nc = 0;
    symxg_dev::project_pd_inplace<T, N>(H + m * (N * N), eps, mirroring != 0, &nc);
    if (nc) *not_converged = 1;
}

// Generic N (up to 24) with thread-private arrays; used for large element matrices.
template <typename T>
__global__ void __launch_bounds__(64) k_project_pd_generic(T* __restrict__ H, int N, int64_t count, T eps,
                                                           int mirroring, int* not_converged)
{
    constexpr int NMAX = 24;
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= count) return;
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

// ---------------------------------------------------------------- assembly
template <typename T>
__global__ void k_assemble_blocks(int64_t nnzb, const int64_t* __restrict__ slot_ptr, const int32_t* __restrict__ contrib,
                                  const T* __restrict__ blocks, T* __restrict__ vals, int64_t vstride)
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
    for (int k = 0; k < 9; ++k) vals[k * vstride + s] = acc[k];
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
template <typename T>
__global__ void k_block_jacobi_setup(int n_blocks, const int32_t* __restrict__ diag_slot, const T* __restrict__ vals,
                                     int64_t vstride, T* __restrict__ Dinv)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_blocks) return;
    const int64_t k = diag_slot[r];
    // symmetric 3x3 inverse from the upper triangle (cofactors / determinant)
    const double a = vals[k], b = vals[vstride + k], c = vals[2 * vstride + k], d = vals[4 * vstride + k],
                 e = vals[5 * vstride + k], f = vals[8 * vstride + k];
    const double c00 = d * f - e * e, c01 = c * e - b * f, c02 = b * e - c * d;
    const double det = a * c00 + b * c01 + c * c02;
    const double id = 1.0 / det;
    T* o = Dinv + (int64_t)r * 9;
    o[0] = (T)(c00 * id);
    o[1] = (T)(c01 * id);
    o[2] = (T)(c02 * id);
    o[3] = o[1];
    o[4] = (T)((a * f - c * c) * id);
    o[5] = (T)((b * c - a * e) * id);
    o[6] = o[2];
    o[7] = o[5];
    o[8] = (T)((a * d - b * b) * id);
}

// ---------------------------------------------------------------- SpMV / PCG
constexpr int kSpmvThreads = 256;  // 16 rows per block, 16 lanes per row

// BCSR storage: the nine components of 3x3 block k (row-major inside the block) are
// vals[m * vstride + k], m = 0..8 (component-major), so each load of a half-warp reads 16
// consecutive values.
//
// Products of two block rows at once, each over the 16 lanes of its half-warp, lane-strided
// over the row's blocks; both rows' loads are in flight together.  xv(c, d) is component d of
// the multiplied vector at block column c.  The sums are reduced across the 16 lanes in a
// fixed butterfly order; every lane of the warp must call this (rows past the end pass
// valid = false), so the full-mask shuffles are converged.
template <typename T, typename XV>
__device__ __forceinline__ void two_row_products(int rowA, bool vA, int rowB, bool vB, int lane16,
                                                 const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ cols,
                                                 const T* __restrict__ vals, int64_t vs, XV xv, T (&a)[3], T (&b)[3])
{
    a[0] = a[1] = a[2] = b[0] = b[1] = b[2] = T(0);
    const int kbA = vA ? row_ptr[rowA] : 0, keA = vA ? row_ptr[rowA + 1] : 0;
    const int kbB = vB ? row_ptr[rowB] : 0, keB = vB ? row_ptr[rowB + 1] : 0;
    for (int i = lane16;; i += 16) {
        const int kA = kbA + i, kB = kbB + i;
        const bool hA = kA < keA, hB = kB < keB;
        if (!hA && !hB) break;
        if (hA) {
            const int c = cols[kA];
            const T x0 = xv(c, 0), x1 = xv(c, 1), x2 = xv(c, 2);
            a[0] += vals[kA] * x0 + vals[vs + kA] * x1 + vals[2 * vs + kA] * x2;
            a[1] += vals[3 * vs + kA] * x0 + vals[4 * vs + kA] * x1 + vals[5 * vs + kA] * x2;
            a[2] += vals[6 * vs + kA] * x0 + vals[7 * vs + kA] * x1 + vals[8 * vs + kA] * x2;
        }
        if (hB) {
            const int c = cols[kB];
            const T x0 = xv(c, 0), x1 = xv(c, 1), x2 = xv(c, 2);
            b[0] += vals[kB] * x0 + vals[vs + kB] * x1 + vals[2 * vs + kB] * x2;
            b[1] += vals[3 * vs + kB] * x0 + vals[4 * vs + kB] * x1 + vals[5 * vs + kB] * x2;
            b[2] += vals[6 * vs + kB] * x0 + vals[7 * vs + kB] * x1 + vals[8 * vs + kB] * x2;
        }
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            a[d] += __shfl_xor_sync(0xffffffffu, a[d], o, 16);
            b[d] += __shfl_xor_sync(0xffffffffu, b[d], o, 16);
        }
    }
}

// y = A x; each warp takes four block rows per pass (two per half-warp).
template <typename T>
__global__ void __launch_bounds__(kSpmvThreads) k_bcsr_spmv(int n_blocks, const int32_t* __restrict__ row_ptr,
                                                            const int32_t* __restrict__ cols, const T* __restrict__ vals,
                                                            int64_t vs, const T* __restrict__ x, T* __restrict__ y)
{
    const int lane16 = threadIdx.x & 15;
    const int half = (threadIdx.x >> 4) & 1;
    const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int warps_total = (gridDim.x * blockDim.x) >> 5;
    auto xv = [x](int c, int d) { return x[3 * c + d]; };
    for (int base = 4 * warp_global; base < n_blocks; base += 4 * warps_total) {
        const int rowA = base + half, rowB = base + 2 + half;
        const bool vA = rowA < n_blocks, vB = rowB < n_blocks;
        T a[3], b[3];
        two_row_products<T>(rowA, vA, rowB, vB, lane16, row_ptr, cols, vals, vs, xv, a, b);
        if (lane16 == 0) {
            if (vA) { y[3 * rowA] = a[0]; y[3 * rowA + 1] = a[1]; y[3 * rowA + 2] = a[2]; }
            if (vB) { y[3 * rowB] = b[0]; y[3 * rowB + 1] = b[1]; y[3 * rowB + 2] = b[2]; }
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
        return (double)a.hi + (double)a.lo;
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

// p_new = z + beta * p_old (p_new = z on the first iteration); one helper so every thread
// computing a given entry gets the same bits.
template <typename T>
__device__ __forceinline__ T direction(const T* __restrict__ z, const T* __restrict__ p_old, T beta, bool first, int i)
{
    return first ? z[i] : fma(beta, p_old[i], z[i]);
}

// PCG step 1: p = z + beta p_old (fused), q = A p, p.q.  Grid sized to the resident
// blocks; each warp takes four block rows per pass.
template <typename T>
__global__ void __launch_bounds__(kSpmvThreads) k_pcg_spmv(PcgBuffers<T> B, const T* __restrict__ p_old,
                                                           T* __restrict__ p_new, int first)
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
    auto pv = [z, p_old, beta, f](int c, int d) { return direction(z, p_old, beta, f, 3 * c + d); };
    DotAcc<T> pq;
    for (int base = 4 * warp_global; base < B.n_blocks; base += 4 * warps_total) {
        const int rowA = base + half, rowB = base + 2 + half;
        const bool vA = rowA < B.n_blocks, vB = rowB < B.n_blocks;
        T a[3], b[3];
        two_row_products<T>(rowA, vA, rowB, vB, lane16, B.row_ptr, B.cols, B.vals, B.vals_stride, pv, a, b);
        if (lane16 == 0) {
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                const int row = rr ? rowB : rowA;
                if (!(rr ? vB : vA)) continue;
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const T pd = pv(row, d);
                    const T qd = rr ? b[d] : a[d];
                    p_new[3 * row + d] = pd;
                    B.q[3 * row + d] = qd;
                    pq.add_prod(pd, qd);
                }
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

// PCG step 2: x += alpha p, r -= alpha q, z = M^-1 r, r.r and r.z; convergence test and beta.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_update(PcgBuffers<T> B, const T* __restrict__ p)
{
    if (B.state->done) return;
    __shared__ double sh[32];
    const T alpha = (T)B.state->alpha;
    DotAcc<T> rr, rz;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n_blocks; i += gridDim.x * blockDim.x) {
        T r[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int k = 3 * i + d;
            B.x[k] = fma(alpha, p[k], B.x[k]);
            r[d] = fma(-alpha, B.q[k], B.r[k]);
            B.r[k] = r[d];
        }
        const T* m = B.Dinv + (int64_t)i * 9;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const T z = m[3 * d] * r[0] + m[3 * d + 1] * r[1] + m[3 * d + 2] * r[2];
            B.z[3 * i + d] = z;
            rr.add_prod(r[d], r[d]);
            rz.add_prod(r[d], z);
        }
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

// Float PCG step 2 on four block rows per thread with 16-byte loads: the vectors are padded
// to a multiple of four block rows (zero tails), so rows 4t..4t+3 are 12 consecutive floats
// (three float4) and their preconditioner blocks 36 floats (nine float4).
__global__ void __launch_bounds__(256) k_pcg_update_f32x4(PcgBuffers<float> B, const float* __restrict__ p)
{
    if (B.state->done) return;
    __shared__ double sh[32];
    const float alpha = (float)B.state->alpha;
    DotAcc<float> rr, rz;
    const int groups = B.n_pad / 4;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < groups; t += gridDim.x * blockDim.x) {
        float xs[12], ps[12], rs[12], qs[12], zs[12], m[36];
        const float4* X4 = reinterpret_cast<const float4*>(B.x) + 3 * t;
        const float4* P4 = reinterpret_cast<const float4*>(p) + 3 * t;
        const float4* R4 = reinterpret_cast<const float4*>(B.r) + 3 * t;
        const float4* Q4 = reinterpret_cast<const float4*>(B.q) + 3 * t;
        const float4* M4 = reinterpret_cast<const float4*>(B.Dinv) + 9 * t;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float4 a = X4[j], b = P4[j], c = R4[j], d = Q4[j];
            xs[4 * j] = a.x; xs[4 * j + 1] = a.y; xs[4 * j + 2] = a.z; xs[4 * j + 3] = a.w;
            ps[4 * j] = b.x; ps[4 * j + 1] = b.y; ps[4 * j + 2] = b.z; ps[4 * j + 3] = b.w;
            rs[4 * j] = c.x; rs[4 * j + 1] = c.y; rs[4 * j + 2] = c.z; rs[4 * j + 3] = c.w;
            qs[4 * j] = d.x; qs[4 * j + 1] = d.y; qs[4 * j + 2] = d.z; qs[4 * j + 3] = d.w;
        }
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const float4 a = M4[j];
            m[4 * j] = a.x; m[4 * j + 1] = a.y; m[4 * j + 2] = a.z; m[4 * j + 3] = a.w;
        }
#pragma unroll
        for (int k = 0; k < 12; ++k) {
            xs[k] = fmaf(alpha, ps[k], xs[k]);
            rs[k] = fmaf(-alpha, qs[k], rs[k]);
        }
#pragma unroll
        for (int row = 0; row < 4; ++row)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const float* mm = m + 9 * row + 3 * d;
                zs[3 * row + d] = mm[0] * rs[3 * row] + mm[1] * rs[3 * row + 1] + mm[2] * rs[3 * row + 2];
            }
#pragma unroll
        for (int k = 0; k < 12; ++k) {
            rr.add_prod(rs[k], rs[k]);
            rz.add_prod(rs[k], zs[k]);
        }
        float4* Xo = reinterpret_cast<float4*>(B.x) + 3 * t;
        float4* Ro = reinterpret_cast<float4*>(B.r) + 3 * t;
        float4* Zo = reinterpret_cast<float4*>(B.z) + 3 * t;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            Xo[j] = make_float4(xs[4 * j], xs[4 * j + 1], xs[4 * j + 2], xs[4 * j + 3]);
            Ro[j] = make_float4(rs[4 * j], rs[4 * j + 1], rs[4 * j + 2], rs[4 * j + 3]);
            Zo[j] = make_float4(zs[4 * j], zs[4 * j + 1], zs[4 * j + 2], zs[4 * j + 3]);
        }
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

// r = b = -grad (as T), x = 0, z = M^-1 r; b.b (double, from the FP64 gradient) and r.z.
template <typename T>
__global__ void __launch_bounds__(256) k_pcg_init(PcgBuffers<T> B, const double* __restrict__ grad)
{
    __shared__ double sh[32];
    double bb = 0.0;
    DotAcc<T> rz;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < B.n_blocks; i += gridDim.x * blockDim.x) {
        T r[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double b = -grad[3 * i + d];
            r[d] = (T)b;
            B.r[3 * i + d] = r[d];
            B.x[3 * i + d] = T(0);
            bb = fma(b, b, bb);
        }
        const T* m = B.Dinv + (int64_t)i * 9;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const T z = m[3 * d] * r[0] + m[3 * d + 1] * r[1] + m[3 * d + 2] * r[2];
            B.z[3 * i + d] = z;
            rz.add_prod(r[d], z);
        }
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

}  // namespace

int64_t launch_count() { return g_launches.load(); }
void count_launch(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

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

template <typename T>
void launch_project_pd(T* H, int N, int64_t count, T eps, bool mirroring, int* not_converged, cudaStream_t s)
{
    if (count <= 0) return;
    switch (N) {
        case 3: k_project_pd_unrolled<T, 3><<<blocks_for(count, 128), 128, 0, s>>>(H, count, eps, mirroring, not_converged); break;
        case 6: k_project_pd_unrolled<T, 6><<<blocks_for(count, 128), 128, 0, s>>>(H, count, eps, mirroring, not_converged); break;
        case 9: k_project_pd_unrolled<T, 9><<<blocks_for(count, 128), 128, 0, s>>>(H, count, eps, mirroring, not_converged); break;
        case 12: k_project_pd_unrolled<T, 12><<<blocks_for(count, 128), 128, 0, s>>>(H, count, eps, mirroring, not_converged); break;
        default:
            if (N > 24 || N % 3 != 0) throw std::runtime_error("symx_gb300: projection supports N = 3k <= 24");
            k_project_pd_generic<T><<<blocks_for(count, 64), 64, 0, s>>>(H, N, count, eps, mirroring, not_converged);
    }
    check_launch("project_pd");
}

template <typename T>
void launch_assemble_blocks(int64_t nnzb, const int64_t* slot_ptr, const int32_t* contrib, const T* blocks, T* vals,
                            int64_t vstride, cudaStream_t s)
{
    if (nnzb <= 0) return;
    k_assemble_blocks<T><<<blocks_for(nnzb, 256), 256, 0, s>>>(nnzb, slot_ptr, contrib, blocks, vals, vstride);
    check_launch("assemble");
}

void launch_gather_gradient(int n_blocks, const int64_t* ptr, const int32_t* contrib, const double* gel, double* g,
                            cudaStream_t s)
{
    k_gather_gradient<<<blocks_for(n_blocks, 256), 256, 0, s>>>(n_blocks, ptr, contrib, gel, g);
    check_launch("gather_gradient");
}

template <typename T>
void launch_block_jacobi_setup(int n_blocks, const int32_t* diag_slot, const T* vals, int64_t vstride, T* Dinv,
                               cudaStream_t s)
{
    k_block_jacobi_setup<T><<<blocks_for(n_blocks, 256), 256, 0, s>>>(n_blocks, diag_slot, vals, vstride, Dinv);
    check_launch("block_jacobi_setup");
}

// Blocks of `kernel` resident at once on the whole device (cached per kernel).
template <typename K>
unsigned resident_grid(K kernel, int threads)
{
    static std::mutex m;
    static std::unordered_map<const void*, unsigned> cache;
    std::lock_guard<std::mutex> lock(m);
    auto it = cache.find((const void*)kernel);
    if (it != cache.end()) return it->second;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
    const unsigned g = (unsigned)std::max(1, sms * std::max(1, per_sm));
    cache[(const void*)kernel] = g;
    return g;
}

template <typename T>
void launch_pcg_init(const PcgBuffers<T>& B, const double* grad, cudaStream_t s)
{
    const unsigned g = std::min<unsigned>(blocks_for(B.n_blocks, 256), resident_grid(k_pcg_init<T>, 256));
    k_pcg_init<T><<<g, 256, 0, s>>>(B, grad);
    check_launch("pcg_init");
}

template <typename T>
void launch_pcg_spmv(const PcgBuffers<T>& B, int iteration, cudaStream_t s)
{
    const unsigned gs = std::min<unsigned>(blocks_for((int64_t)B.n_blocks * 8, kSpmvThreads),
                                           resident_grid(k_pcg_spmv<T>, kSpmvThreads));
    T* p_old = (iteration & 1) ? B.p : B.p2;
    T* p_new = (iteration & 1) ? B.p2 : B.p;
    k_pcg_spmv<T><<<gs, kSpmvThreads, 0, s>>>(B, p_old, p_new, iteration == 0 ? 1 : 0);
    check_launch("pcg_spmv");
}

template <typename T>
void launch_pcg_update(const PcgBuffers<T>& B, int iteration, cudaStream_t s)
{
    T* p_new = (iteration & 1) ? B.p2 : B.p;
    if constexpr (std::is_same<T, float>::value) {
        const unsigned gu = std::min<unsigned>(blocks_for(B.n_pad / 4, 256), resident_grid(k_pcg_update_f32x4, 256));
        k_pcg_update_f32x4<<<gu, 256, 0, s>>>(B, p_new);
    } else {
        const unsigned gu = std::min<unsigned>(blocks_for(B.n_blocks, 256), resident_grid(k_pcg_update<T>, 256));
        k_pcg_update<T><<<gu, 256, 0, s>>>(B, p_new);
    }
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
    const unsigned g = std::min<unsigned>(blocks_for((int64_t)n_blocks * 8, kSpmvThreads),
                                          resident_grid(k_bcsr_spmv<T>, kSpmvThreads));
    k_bcsr_spmv<T><<<g, kSpmvThreads, 0, s>>>(n_blocks, row_ptr, cols, vals, vstride, x, y);
    check_launch("bcsr_spmv");
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
    template void launch_project_pd<T>(T*, int, int64_t, T, bool, int*, cudaStream_t);                                 \
    template void launch_assemble_blocks<T>(int64_t, const int64_t*, const int32_t*, const T*, T*, int64_t, cudaStream_t); \
    template void launch_block_jacobi_setup<T>(int, const int32_t*, const T*, int64_t, T*, cudaStream_t);              \
    template void launch_pcg_init<T>(const PcgBuffers<T>&, const double*, cudaStream_t);                               \
    template void launch_pcg_iteration<T>(const PcgBuffers<T>&, int, cudaStream_t);                                   \
    template void launch_pcg_spmv<T>(const PcgBuffers<T>&, int, cudaStream_t);                                        \
    template void launch_pcg_update<T>(const PcgBuffers<T>&, int, cudaStream_t);                                      \
    template void launch_bcsr_spmv<T>(int, const int32_t*, const int32_t*, const T*, int64_t, const T*, T*, cudaStream_t); \
    template void launch_axpy_to<T>(int64_t, const double*, double, const T*, double*, cudaStream_t);                  \
    template void launch_convert_to_double<T>(int64_t, const T*, double*, cudaStream_t);
SYMXG_INSTANTIATE(float)
SYMXG_INSTANTIATE(double)

}  // namespace symxg
