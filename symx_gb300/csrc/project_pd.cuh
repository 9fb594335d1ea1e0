// Batched projection of symmetric element Hessians to positive definite.
//
// Semantics of the reference's project_to_PD_inplace
// (symx/src/solver/second_order/project_to_PD.cpp:12-32): eigenvalues below `eps` are
// replaced by `eps` (or by their negation when mirroring), and the matrix is rebuilt as
// V diag(lambda) V^T only if some eigenvalue changed.
//
// The eigen-decomposition is cyclic Jacobi (Golub & Van Loan, Matrix Computations,
// Sec. 8.5) on the upper triangle, one thread per matrix, every index known at compile
// time so that A (N(N+1)/2 values) and V (N*N values) live in registers for N = 12.
// The number of sweeps is capped; a matrix that has not converged by then is still
// rebuilt from the current rotation and flagged in `status`.
//
// Element Hessians are stored block-major: the 3x3 block (a, b) of an N x N matrix
// (N = 3 * nb) starts at ((a * nb + b) * 9) and is row-major inside.
#pragma once

#ifndef SYMXG_DEVICE
#define SYMXG_DEVICE __device__ __forceinline__
#endif

namespace symxg_dev {

template <int N>
SYMXG_DEVICE constexpr int bm_index(int i, int j)
{
    return (((i / 3) * (N / 3) + (j / 3)) * 3 + (i % 3)) * 3 + (j % 3);
}

template <int N>
SYMXG_DEVICE constexpr int tri(int i, int j)
{
    return (i <= j) ? (i * N - (i * (i - 1)) / 2 + (j - i)) : (j * N - (j * (j - 1)) / 2 + (i - j));
}

template <typename T>
struct JacobiTol;
// Stop when the off-diagonal Frobenius norm is below 32 ulp of the matrix norm: rotations
// leave rounding-level off-diagonal entries behind, so a tighter test would never pass.
template <>
struct JacobiTol<float> {
    static SYMXG_DEVICE float rel2() { return 1.4551915e-11f; }  // (32 * 2^-23)^2
    static constexpr int max_sweeps = 15;
};
template <>
struct JacobiTol<double> {
    static SYMXG_DEVICE double rel2() { return 5.048709793414476e-29; }  // (32 * 2^-52)^2
    static constexpr int max_sweeps = 20;
};

template <typename T>
SYMXG_DEVICE T sq(T x) { return x * x; }

// Project the matrix H (block-major, N x N) in place.  Returns 1 if the matrix changed,
// and sets *not_converged when the sweep cap was reached.
template <typename T, int N>
SYMXG_DEVICE int project_pd_inplace(T* __restrict__ H, T eps, bool mirroring, int* not_converged)
{
    constexpr int NT = N * (N + 1) / 2;
    T a[NT];
    T v[N * N];
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = i; j < N; ++j) a[tri<N>(i, j)] = H[bm_index<N>(i, j)];
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) v[i * N + j] = (i == j) ? T(1) : T(0);

    T fro2 = T(0);
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = i; j < N; ++j) fro2 += (i == j ? T(1) : T(2)) * sq(a[tri<N>(i, j)]);

    int sweep = 0;
    for (; sweep < JacobiTol<T>::max_sweeps; ++sweep) {
        T off = T(0);
#pragma unroll
        for (int p = 0; p < N; ++p)
#pragma unroll
            for (int q = p + 1; q < N; ++q) off += sq(a[tri<N>(p, q)]);
        if (!(off > JacobiTol<T>::rel2() * fro2)) break;
#pragma unroll
        for (int p = 0; p < N - 1; ++p) {
#pragma unroll
            for (int q = p + 1; q < N; ++q) {
                const T apq = a[tri<N>(p, q)];
                const T app = a[tri<N>(p, p)];
                const T aqq = a[tri<N>(q, q)];
                const T tau = (aqq - app) / (T(2) * apq);
                T t = (tau >= T(0) ? T(1) : T(-1)) / (fabs(tau) + sqrt(T(1) + tau * tau));
                t = (apq != T(0)) ? t : T(0);
                const T c = T(1) / sqrt(T(1) + t * t);
                const T s = t * c;
                a[tri<N>(p, p)] = app - t * apq;
                a[tri<N>(q, q)] = aqq + t * apq;
                a[tri<N>(p, q)] = T(0);
#pragma unroll
                for (int k = 0; k < N; ++k) {
                    if (k == p || k == q) continue;
                    const T akp = a[tri<N>(k, p)];
                    const T akq = a[tri<N>(k, q)];
                    a[tri<N>(k, p)] = c * akp - s * akq;
                    a[tri<N>(k, q)] = s * akp + c * akq;
                }
#pragma unroll
                for (int k = 0; k < N; ++k) {
                    const T vkp = v[k * N + p];
                    const T vkq = v[k * N + q];
                    v[k * N + p] = c * vkp - s * vkq;
                    v[k * N + q] = s * vkp + c * vkq;
                }
            }
        }
    }
    if (sweep == JacobiTol<T>::max_sweeps && not_converged) *not_converged = 1;

    bool changed = false;
    T lam[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        T l = a[tri<N>(i, i)];
        if (l < eps) {
            changed = true;
            l = mirroring ? -l : eps;
        }
        lam[i] = l;
    }
    if (!changed) return 0;
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = i; j < N; ++j) {
            T s = T(0);
#pragma unroll
            for (int k = 0; k < N; ++k) s += v[i * N + k] * lam[k] * v[j * N + k];
            H[bm_index<N>(i, j)] = s;
            H[bm_index<N>(j, i)] = s;
        }
    return 1;
}

}  // namespace symxg_dev
