// Batched projection of symmetric element Hessians to positive definite.
//
// Semantics of the reference's project_to_PD_inplace
// (symx/src/solver/second_order/project_to_PD.cpp:12-32): eigenvalues below `eps` are
// replaced by `eps` (or by their negation when mirroring), and the matrix is rebuilt as
// V diag(lambda) V^T only if some eigenvalue changed.
//
// Eigen-decomposition: cyclic Jacobi (Golub & Van Loan, Matrix Computations, Sec. 8.5),
// one thread per matrix with A (upper triangle) and V in registers.  To keep the code small
// enough for the instruction cache while every register index stays a compile-time
// constant, one "step" rotates the pairs (0, q), q = 1..N-1 (unrolled), and then relabels
// the indices cyclically (i -> i-1 mod N) by register moves.  N steps bring the labels back
// and rotate every pair twice, i.e. they are two cyclic sweeps.  Convergence is tested every
// few steps; the number of steps is capped and a matrix that reaches the cap is still rebuilt
// from the current rotation and flagged.
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

// Stop when the off-diagonal Frobenius norm is below 32 ulp of the matrix norm: rotations
// leave rounding-level off-diagonal entries behind, so a tighter test would never pass.
template <typename T>
struct JacobiTol;
template <>
struct JacobiTol<float> {
    static SYMXG_DEVICE float rel2() { return 1.4551915e-11f; }  // (32 * 2^-23)^2
    static constexpr int max_double_sweeps = 8;
};
template <>
struct JacobiTol<double> {
    static SYMXG_DEVICE double rel2() { return 5.048709793414476e-29; }  // (32 * 2^-52)^2
    static constexpr int max_double_sweeps = 10;
};

template <typename T>
SYMXG_DEVICE T sq(T x) { return x * x; }

// tan of the Jacobi angle that zeroes a_pq: t = 2 a_pq sgn(d) / (|d| + sqrt(d^2 + 4 a_pq^2)),
// d = a_qq - a_pp; t = 0 when a_pq = 0.  This form cannot overflow.
SYMXG_DEVICE float jacobi_t(float app, float aqq, float apq)
{
    const float d = aqq - app;
    const float r = d * d + 4.0f * apq * apq;
    const float den = fabsf(d) + (r > 0.0f ? r * rsqrtf(r) : 0.0f);
    const float num = 2.0f * apq * (d >= 0.0f ? 1.0f : -1.0f);
    return den > 0.0f ? num * __frcp_rn(den) : 0.0f;
}
SYMXG_DEVICE double jacobi_t(double app, double aqq, double apq)
{
    const double d = aqq - app;
    const double r = d * d + 4.0 * apq * apq;
    const double den = fabs(d) + sqrt(r);
    const double num = 2.0 * apq * (d >= 0.0 ? 1.0 : -1.0);
    return den > 0.0 ? num / den : 0.0;
}
SYMXG_DEVICE float inv_hypot1(float t) { return rsqrtf(1.0f + t * t); }
SYMXG_DEVICE double inv_hypot1(double t) { return 1.0 / sqrt(1.0 + t * t); }

// Rotate the pairs (0, q), q = 1..N-1, then relabel i -> i-1 (mod N).
template <typename T, int N>
SYMXG_DEVICE void jacobi_step(T (&a)[N * (N + 1) / 2], T (&v)[N * N])
{
#pragma unroll
    for (int q = 1; q < N; ++q) {
        const T apq = a[tri<N>(0, q)];
        const T app = a[tri<N>(0, 0)];
        const T aqq = a[tri<N>(q, q)];
        const T t = jacobi_t(app, aqq, apq);
        const T c = inv_hypot1(t);
        const T s = t * c;
        a[tri<N>(0, 0)] = app - t * apq;
        a[tri<N>(q, q)] = aqq + t * apq;
        a[tri<N>(0, q)] = T(0);
#pragma unroll
        for (int k = 1; k < N; ++k) {
            if (k == q) continue;
            const T akp = a[tri<N>(k, 0)];
            const T akq = a[tri<N>(k, q)];
            a[tri<N>(k, 0)] = c * akp - s * akq;
            a[tri<N>(k, q)] = s * akp + c * akq;
        }
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const T vkp = v[k * N + 0];
            const T vkq = v[k * N + q];
            v[k * N + 0] = c * vkp - s * vkq;
            v[k * N + q] = s * vkp + c * vkq;
        }
    }
    // relabel: new index i is old index i+1 (mod N)
    T na[N * (N + 1) / 2];
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = i; j < N; ++j) na[tri<N>(i, j)] = a[tri<N>((i + 1) % N, (j + 1) % N)];
#pragma unroll
    for (int k = 0; k < N * (N + 1) / 2; ++k) a[k] = na[k];
#pragma unroll
    for (int r = 0; r < N; ++r) {
        const T first = v[r * N + 0];
#pragma unroll
        for (int j = 0; j + 1 < N; ++j) v[r * N + j] = v[r * N + j + 1];
        v[r * N + N - 1] = first;
    }
}

// One classic cyclic sweep over all pairs (p, q), p < q, fully unrolled.  Used for double,
// where the FP64 pipe, not instruction fetch, bounds the kernel and the relabeling moves of
// jacobi_step would only add spills.
template <typename T, int N>
SYMXG_DEVICE void jacobi_double_sweep_cyclic(T (&a)[N * (N + 1) / 2], T (&v)[N * N])
{
#pragma unroll 1
    for (int rep = 0; rep < 2; ++rep) {
#pragma unroll
        for (int p = 0; p < N - 1; ++p) {
#pragma unroll
            for (int q = p + 1; q < N; ++q) {
                const T apq = a[tri<N>(p, q)];
                const T app = a[tri<N>(p, p)];
                const T aqq = a[tri<N>(q, q)];
                const T t = jacobi_t(app, aqq, apq);
                const T c = inv_hypot1(t);
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
}

#if defined(SYMXG_PACKED_FP32X2) || (defined(__CUDACC__) && (!defined(__CUDA_ARCH__) || __CUDA_ARCH__ >= 1000))
#define SYMXG_HAVE_PACKED_PROJECTION 1
// float, even N, on sm_100 and later: the eigenvector matrix is held as pairs of rows in
// float2 registers, vv[kp * N + j] = (V[2kp][j], V[2kp+1][j]), and updated with the packed
// FP32x2 instructions (__ffma2_rn / __fmul2_rn), two rows per instruction.  Same rotations,
// same order as jacobi_step.
template <int N>
SYMXG_DEVICE void jacobi_step_packed(float (&a)[N * (N + 1) / 2], float2 (&vv)[(N / 2) * N])
{
#pragma unroll
    for (int q = 1; q < N; ++q) {
        const float apq = a[tri<N>(0, q)];
        const float app = a[tri<N>(0, 0)];
        const float aqq = a[tri<N>(q, q)];
        const float t = jacobi_t(app, aqq, apq);
        const float c = inv_hypot1(t);
        const float s = t * c;
        a[tri<N>(0, 0)] = app - t * apq;
        a[tri<N>(q, q)] = aqq + t * apq;
        a[tri<N>(0, q)] = 0.0f;
#pragma unroll
        for (int k = 1; k < N; ++k) {
            if (k == q) continue;
            const float akp = a[tri<N>(k, 0)];
            const float akq = a[tri<N>(k, q)];
            a[tri<N>(k, 0)] = c * akp - s * akq;
            a[tri<N>(k, q)] = s * akp + c * akq;
        }
        const float2 c2 = make_float2(c, c), s2 = make_float2(s, s), ns2 = make_float2(-s, -s);
#pragma unroll
        for (int kp = 0; kp < N / 2; ++kp) {
            const float2 P = vv[kp * N + 0];
            const float2 Q = vv[kp * N + q];
            vv[kp * N + 0] = __ffma2_rn(c2, P, __fmul2_rn(ns2, Q));
            vv[kp * N + q] = __ffma2_rn(s2, P, __fmul2_rn(c2, Q));
        }
    }
    float na[N * (N + 1) / 2];
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = i; j < N; ++j) na[tri<N>(i, j)] = a[tri<N>((i + 1) % N, (j + 1) % N)];
#pragma unroll
    for (int k = 0; k < N * (N + 1) / 2; ++k) a[k] = na[k];
#pragma unroll
    for (int kp = 0; kp < N / 2; ++kp) {
        const float2 first = vv[kp * N + 0];
#pragma unroll
        for (int j = 0; j + 1 < N; ++j) vv[kp * N + j] = vv[kp * N + j + 1];
        vv[kp * N + N - 1] = first;
    }
}

template <int N>
SYMXG_DEVICE int project_pd_inplace_packed(float* __restrict__ H, float eps, bool mirroring, int* not_converged)
{
    constexpr int NT = N * (N + 1) / 2;
    float a[NT];
    float2 vv[(N / 2) * N];
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = i; j < N; ++j) a[tri<N>(i, j)] = H[bm_index<N>(i, j)];
#pragma unroll
    for (int kp = 0; kp < N / 2; ++kp)
#pragma unroll
        for (int j = 0; j < N; ++j) vv[kp * N + j] = make_float2(j == 2 * kp ? 1.0f : 0.0f, j == 2 * kp + 1 ? 1.0f : 0.0f);
    float fro2 = 0.0f;
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = i; j < N; ++j) fro2 += (i == j ? 1.0f : 2.0f) * sq(a[tri<N>(i, j)]);
    constexpr int kGroup = N < 4 ? N : 4;
    constexpr int kMaxGroups = JacobiTol<float>::max_double_sweeps * ((N + kGroup - 1) / kGroup);
    int grp = 0;
    for (; grp < kMaxGroups; ++grp) {
        float off = 0.0f;
#pragma unroll
        for (int p = 0; p < N; ++p)
#pragma unroll
            for (int q = p + 1; q < N; ++q) off += sq(a[tri<N>(p, q)]);
        if (!(off > JacobiTol<float>::rel2() * fro2)) break;
#pragma unroll 1
        for (int step = 0; step < kGroup; ++step) jacobi_step_packed<N>(a, vv);
    }
    if (grp == kMaxGroups && not_converged) *not_converged = 1;
    bool changed = false;
    float lam[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        float l = a[tri<N>(i, i)];
        if (l < eps) {
            changed = true;
            l = mirroring ? -l : eps;
        }
        lam[i] = l;
    }
    if (!changed) return 0;
    // H = V diag(lam) V^T, two rows of H per packed accumulator
#pragma unroll
    for (int ip = 0; ip < N / 2; ++ip)
#pragma unroll
        for (int j = 2 * ip; j < N; ++j) {
            float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int k = 0; k < N; ++k) {
                const float2 vj = vv[(j / 2) * N + k];
                const float w = lam[k] * ((j & 1) ? vj.y : vj.x);
                acc = __ffma2_rn(vv[ip * N + k], make_float2(w, w), acc);
            }
            H[bm_index<N>(2 * ip, j)] = acc.x;
            H[bm_index<N>(j, 2 * ip)] = acc.x;
            if (j >= 2 * ip + 1) {
                H[bm_index<N>(2 * ip + 1, j)] = acc.y;
                H[bm_index<N>(j, 2 * ip + 1)] = acc.y;
            }
        }
    return 1;
}
#endif

// Cyclic Jacobi on the symmetric matrix a (upper triangle) with eigenvectors accumulated in
// v (v = I on entry): on return the diagonal of a holds the eigenvalues and column k of v
// the eigenvector of a[k][k].  Convergence is tested every kGroup relabel steps (float) or
// every double sweep (double); the off-diagonal norm and V diag(lambda) V^T do not depend on
// the labelling, so stopping between full double sweeps is exact.  Returns false when the
// sweep cap was reached.
template <typename T, int N>
SYMXG_DEVICE bool jacobi_eigen(T (&a)[N * (N + 1) / 2], T (&v)[N * N])
{
    T fro2 = T(0);
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = i; j < N; ++j) fro2 += (i == j ? T(1) : T(2)) * sq(a[tri<N>(i, j)]);
    constexpr int kGroup = (sizeof(T) == 4) ? (N < 4 ? N : 4) : N;
    constexpr int kMaxGroups = JacobiTol<T>::max_double_sweeps * ((N + kGroup - 1) / kGroup);
    int grp = 0;
    for (; grp < kMaxGroups; ++grp) {
        T off = T(0);
#pragma unroll
        for (int p = 0; p < N; ++p)
#pragma unroll
            for (int q = p + 1; q < N; ++q) off += sq(a[tri<N>(p, q)]);
        if (!(off > JacobiTol<T>::rel2() * fro2)) break;
        if (sizeof(T) == 4) {
#pragma unroll 1
            for (int step = 0; step < kGroup; ++step) jacobi_step<T, N>(a, v);
        } else {
            jacobi_double_sweep_cyclic<T, N>(a, v);
        }
    }
    return grp < kMaxGroups;
}

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
    if (!jacobi_eigen<T, N>(a, v) && not_converged) *not_converged = 1;

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

// ---- translation deflation
//
// An element energy that depends on its nodes only through their differences (every elastic
// energy) has a Hessian that annihilates the three rigid translations t_d = (e_d, ..., e_d) /
// sqrt(NB) of its NB nodes; in floating point H t_d is rounding noise.  For such a matrix
// the projection is done in the complement of the translations: with Q = B (x) I3, B the
// Helmert basis of the node space orthogonal to (1, ..., 1) (column m = 1..NB-1:
// 1/sqrt(m(m+1)) for the nodes before m, -m/sqrt(m(m+1)) for node m, 0 after), H equals
// Q (Q^T H Q) Q^T, the translation eigenvalues are 0, and the eigen-decomposition shrinks
// from N x N to (N-3) x (N-3) (Jacobi work grows as n^3: 0.42x for a Tet4).  The result is
// the reference's V diag(lambda') V^T with the translation eigenvalues 0 -> eps (0 when
// mirroring).  A matrix whose translation residual max |H t| exceeds tol * max |H| is left
// alone and reported (returns -1): the caller projects it with the full decomposition.
template <typename T>
struct DeflationTol;
template <>
struct DeflationTol<float> {
    static SYMXG_DEVICE float value() { return 1e-5f; }   // ~80 ulp of the largest entry
};
template <>
struct DeflationTol<double> {
    static SYMXG_DEVICE double value() { return 1e-12; }
};

// Helmert basis entry B[i][m] (m = 1..NB-1), with c[m] = 1/sqrt(m(m+1)).
template <typename T, int NB>
SYMXG_DEVICE T helmert(const T (&c)[NB], int i, int m)
{
    return i < m ? c[m] : (i == m ? -T(m) * c[m] : T(0));
}

// True when the symmetric M x M matrix b (upper triangle) has a Cholesky factorization whose
// pivots all exceed 16 M u of its largest diagonal entry (u the unit roundoff of T): it is
// then positive definite up to rounding, with every eigenvalue above -(rounding of b).
template <typename T>
struct UnitRoundoff;
template <>
struct UnitRoundoff<float> {
    static SYMXG_DEVICE float value() { return 5.9604645e-8f; }  // 2^-24
};
template <>
struct UnitRoundoff<double> {
    static SYMXG_DEVICE double value() { return 1.1102230246251565e-16; }  // 2^-53
};
template <typename T, int M>
SYMXG_DEVICE bool positive_definite_by_cholesky(const T (&b)[M * (M + 1) / 2])
{
    T dmax = T(0);
#pragma unroll
    for (int i = 0; i < M; ++i) dmax = fmax(dmax, b[tri<M>(i, i)]);
    const T tau = T(16 * M) * UnitRoundoff<T>::value() * dmax;
    T u[M * (M + 1) / 2];  // U = L^T: u(k, i) = L(i, k), k <= i
#pragma unroll
    for (int j = 0; j < M; ++j) {
        T d = b[tri<M>(j, j)];
#pragma unroll
        for (int k = 0; k < j; ++k) d -= u[tri<M>(k, j)] * u[tri<M>(k, j)];
        if (!(d > tau)) return false;
        const T r = T(1) / sqrt(d);
#pragma unroll
        for (int i = j + 1; i < M; ++i) {
            T x = b[tri<M>(j, i)];
#pragma unroll
            for (int k = 0; k < j; ++k) x -= u[tri<M>(k, i)] * u[tri<M>(k, j)];
            u[tri<M>(j, i)] = x * r;
        }
    }
    return true;
}

// Upper triangle of the symmetric block-major matrix H into a, and max |entry| into hmax.  A
// 16-byte aligned float matrix is read with 16-byte loads in storage order (N * N / 4 of
// them instead of N (N + 1) / 2 scalar loads).
template <typename T, int N>
SYMXG_DEVICE void load_upper(const T* __restrict__ H, T (&a)[N * (N + 1) / 2], T& hmax)
{
#ifdef __CUDA_ARCH__
    if constexpr (sizeof(T) == 4 && (N * N) % 4 == 0) {
        if ((reinterpret_cast<unsigned long long>(H) & 15ull) == 0ull) {
            const float4* H4 = reinterpret_cast<const float4*>(H);
#pragma unroll
            for (int q = 0; q < N * N / 4; ++q) {
                const float4 v = __ldg(H4 + q);
                const T vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int idx = 4 * q + t, blk = idx / 9, r = idx % 9;
                    const int i = (blk / (N / 3)) * 3 + r / 3, j = (blk % (N / 3)) * 3 + r % 3;
                    if (i <= j) a[tri<N>(i, j)] = vv[t];
                    hmax = fmax(hmax, fabs(vv[t]));
                }
            }
            return;
        }
    }
#endif
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = i; j < N; ++j) {
            a[tri<N>(i, j)] = H[bm_index<N>(i, j)];
            hmax = fmax(hmax, fabs(a[tri<N>(i, j)]));
        }
}

// b = Q^T H Q (upper triangle) of a translation-invariant H; returns false (b unset) when the
// translation residual max |H t| exceeds tol * max |H|.
template <typename T, int NB>
SYMXG_DEVICE bool deflate_translations(const T* __restrict__ H, T (&b)[(3 * NB - 3) * (3 * NB - 2) / 2])
{
    constexpr int N = 3 * NB;
    constexpr int M = N - 3;
    T c[NB];
    c[0] = T(0);
#pragma unroll
    for (int m = 1; m < NB; ++m) c[m] = T(1) / sqrt(T(m * (m + 1)));
    T a[N * (N + 1) / 2];
    T hmax = T(0);
    load_upper<T, N>(H, a, hmax);
    // translation residual: (H t_e) at row (i, d), up to the factor 1/sqrt(NB)
    T res = T(0);
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            T r = T(0);
#pragma unroll
            for (int jn = 0; jn < NB; ++jn) r += a[tri<N>(i, 3 * jn + e)];
            res = fmax(res, fabs(r));
        }
    if (!(res <= DeflationTol<T>::value() * hmax)) return false;
    // b = Q^T H Q (upper triangle), row (m, d) of b = row 3 (m - 1) + d
#pragma unroll
    for (int p = 0; p < M; ++p)
#pragma unroll
        for (int q = p; q < M; ++q) {
            const int m = p / 3 + 1, d = p % 3, l = q / 3 + 1, e = q % 3;
            T s = T(0);
#pragma unroll
            for (int i = 0; i <= m; ++i) {
                T t = T(0);
#pragma unroll
                for (int j = 0; j <= l; ++j) t += helmert<T, NB>(c, j, l) * a[tri<N>(3 * i + d, 3 * j + e)];
                s += helmert<T, NB>(c, i, m) * t;
            }
            b[tri<M>(p, q)] = s;
        }
    return true;
}

// Eigen-decomposition of b = Q^T H Q, clamping, and H = Q W Q^T + lam_t / NB (1 1^T (x) I3).
// Returns 1 when H changed.
template <typename T, int NB>
SYMXG_DEVICE int project_deflated_finish(T* __restrict__ H, T (&b)[(3 * NB - 3) * (3 * NB - 2) / 2], T eps,
                                         bool mirroring, int* not_converged)
{
    constexpr int N = 3 * NB;
    constexpr int M = N - 3;
    T c[NB];
    c[0] = T(0);
#pragma unroll
    for (int m = 1; m < NB; ++m) c[m] = T(1) / sqrt(T(m * (m + 1)));
    T v[M * M];
#pragma unroll
    for (int i = 0; i < M; ++i)
#pragma unroll
        for (int j = 0; j < M; ++j) v[i * M + j] = (i == j) ? T(1) : T(0);
    if (!jacobi_eigen<T, M>(b, v) && not_converged) *not_converged = 1;

    bool changed = false;
    T lam[M];
#pragma unroll
    for (int k = 0; k < M; ++k) {
        T l = b[tri<M>(k, k)];
        if (l < eps) {
            changed = true;
            l = mirroring ? -l : eps;
        }
        lam[k] = l;
    }
    T lam_t = T(0);  // the three translation eigenvalues
    if (T(0) < eps) {
        changed = true;
        lam_t = mirroring ? T(0) : eps;
    }
    if (!changed) return 0;
    // W = V diag(lam) V^T (upper triangle, reusing b), then H = Q W Q^T + lam_t / NB (1 1^T (x) I3)
#pragma unroll
    for (int p = 0; p < M; ++p)
#pragma unroll
        for (int q = p; q < M; ++q) {
            T s = T(0);
#pragma unroll
            for (int k = 0; k < M; ++k) s += v[p * M + k] * lam[k] * v[q * M + k];
            b[tri<M>(p, q)] = s;
        }
    const T diag_t = lam_t / T(NB);
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = i; j < N; ++j) {
            const int in = i / 3, d = i % 3, jn = j / 3, e = j % 3;
            T s = (d == e) ? diag_t : T(0);
#pragma unroll
            for (int m = 1; m < NB; ++m) {
                if (m < in) continue;  // B[in][m] = 0 for in > m
                T t = T(0);
#pragma unroll
                for (int l = 1; l < NB; ++l) {
                    if (l < jn) continue;
                    t += helmert<T, NB>(c, jn, l) * b[tri<M>(3 * (m - 1) + d, 3 * (l - 1) + e)];
                }
                s += helmert<T, NB>(c, in, m) * t;
            }
            H[bm_index<N>(i, j)] = s;
            H[bm_index<N>(j, i)] = s;
        }
    return 1;
}

// Q^T H Q positive definite (the usual case for an elastic element near its rest shape): the
// projection keeps its eigenvalues and only lifts the three translation eigenvalues from 0 to
// eps (the term eps / NB (1 1^T (x) I3)), a change far below the rounding of H's entries, so
// H is left as it is and the eigen-decomposition is skipped.
template <typename T, int NB>
SYMXG_DEVICE int project_pd_deflated(T* __restrict__ H, T eps, bool mirroring, int* not_converged)
{
    constexpr int M = 3 * NB - 3;
    T b[M * (M + 1) / 2];
    if (!deflate_translations<T, NB>(H, b)) return -1;
    if (positive_definite_by_cholesky<T, M>(b)) return 0;
    return project_deflated_finish<T, NB>(H, b, eps, mirroring, not_converged);
}

// ---- FP64-accurate projection from an FP32 eigen-decomposition
//
// The cyclic Jacobi above converges in FP32 for a small fraction of its FP64 cost (GB300's
// FP64 rate is 1/64 of FP32).  Its eigenvectors X (orthonormal and exact to ~1e-6) are then
// refined in FP64 with one step of Ogita and Aishima's iterative refinement for the symmetric
// eigenvalue problem (T. Ogita, K. Aishima, "Iterative refinement for symmetric eigenvalue
// decomposition", Japan J. Indust. Appl. Math. 35 (2018) 1007-1035, Algorithm 1):
//   R = I - X^T X,  S = X^T A X,  lam_i = s_ii / (1 - r_ii),
//   delta = 2 (|S - diag(lam)| + |A| |R|)            (Frobenius norms bound the 2-norms),
//   E_ij = (s_ij + lam_j r_ij) / (lam_j - lam_i) when |lam_i - lam_j| > delta, else r_ij / 2,
//   X' = X + X E,
// which squares the eigenvector error (one step takes FP32 vectors to ~1e-12 relative).  The
// clamping is then applied as a correction to A itself, A + sum_k (lam'_k - lam_k) x'_k x'_k^T
// over the clamped eigenvalues only, so the eigenpairs that do not change do not enter the
// result at all and the correction carries the (small) clamped eigenvalues' accuracy.
//
// A is the upper triangle in FP64, X the FP32 eigenvectors (column k = eigenvector k).  dW
// (upper triangle) receives the correction; returns true when some eigenvalue was clamped.
template <int M>
SYMXG_DEVICE bool refine_clamp_correction(const double (&A)[M * (M + 1) / 2], const float (&X)[M * M], double eps,
                                          bool mirroring, double (&dW)[M * (M + 1) / 2])
{
    constexpr int MT = M * (M + 1) / 2;
    double S[MT], R[MT];
#pragma unroll 1
    for (int j = 0; j < M; ++j) {
        double y[M];  // A x_j
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double t = 0.0;
#pragma unroll
            for (int k = 0; k < M; ++k) t = fma(A[tri<M>(i, k)], (double)X[k * M + j], t);
            y[i] = t;
        }
#pragma unroll
        for (int i = 0; i < M; ++i) {
            if (i > j) continue;
            double s = 0.0, r = 0.0;
#pragma unroll
            for (int k = 0; k < M; ++k) {
                const double xi = (double)X[k * M + i];
                s = fma(xi, y[k], s);
                r = fma(xi, (double)X[k * M + j], r);
            }
            S[tri<M>(i, j)] = s;
            R[tri<M>(i, j)] = (i == j ? 1.0 : 0.0) - r;
        }
    }
    double lam[M];
#pragma unroll
    for (int i = 0; i < M; ++i) lam[i] = S[tri<M>(i, i)] / (1.0 - R[tri<M>(i, i)]);
    double nsd = 0.0, na = 0.0, nr = 0.0;
#pragma unroll
    for (int i = 0; i < M; ++i)
#pragma unroll
        for (int j = i; j < M; ++j) {
            const double w = i == j ? 1.0 : 2.0;
            const double sd = i == j ? S[tri<M>(i, i)] - lam[i] : S[tri<M>(i, j)];
            nsd = fma(w * sd, sd, nsd);
            na = fma(w * A[tri<M>(i, j)], A[tri<M>(i, j)], na);
            nr = fma(w * R[tri<M>(i, j)], R[tri<M>(i, j)], nr);
        }
    const double delta = 2.0 * (sqrt(nsd) + sqrt(na) * sqrt(nr));
#pragma unroll
    for (int k = 0; k < MT; ++k) dW[k] = 0.0;
    bool changed = false;
#pragma unroll 1
    for (int k = 0; k < M; ++k) {
        const double l = lam[k];
        if (!(l < eps)) continue;
        changed = true;
        const double c = (mirroring ? -l : eps) - l;
        double x[M];  // x'_k = x_k + X E[:, k]
#pragma unroll
        for (int r = 0; r < M; ++r) x[r] = (double)X[r * M + k];
#pragma unroll
        for (int i = 0; i < M; ++i) {
            const double rik = R[tri<M>(i, k)];
            double e;
            if (i == k) e = 0.5 * rik;
            else if (fabs(lam[i] - l) > delta) e = (S[tri<M>(i, k)] + l * rik) / (l - lam[i]);
            else e = 0.5 * rik;
#pragma unroll
            for (int r = 0; r < M; ++r) x[r] = fma((double)X[r * M + i], e, x[r]);
        }
#pragma unroll
        for (int p = 0; p < M; ++p)
#pragma unroll
            for (int q = p; q < M; ++q) dW[tri<M>(p, q)] = fma(c * x[p], x[q], dW[tri<M>(p, q)]);
    }
    return changed;
}

// Projection of one stored matrix H (S = float or double storage) with the FP32 Jacobi and
// the FP64 refinement above.  Deflate: H is translation-invariant (an elastic element's
// Hessian, as k_project_pd_sort found it): the decomposition is of b = Q^T H Q (Q the
// Helmert basis of the translations' complement, (3 NB - 3) x (3 NB - 3)), and the result is
// H + Q dW Q^T + lam_t / NB (1 1^T (x) I3) with the translation eigenvalues 0 -> eps (0 when
// mirroring), as project_deflated_finish has it.  Otherwise the full N x N matrix is
// decomposed and H + dW is stored.  Every sum is formed in FP64 and rounded once into S.
// Returns 1 when H changed; sets *not_converged when the FP32 Jacobi hit its sweep cap.
template <typename S, int NB, bool Deflate>
SYMXG_DEVICE int project_pd_refined(S* __restrict__ H, double eps, bool mirroring, int* not_converged)
{
    constexpr int N = 3 * NB;
    constexpr int M = Deflate ? N - 3 : N;
    constexpr int MT = M * (M + 1) / 2;
    double c[NB];
    c[0] = 0.0;
#pragma unroll
    for (int m = 1; m < NB; ++m) c[m] = 1.0 / sqrt((double)(m * (m + 1)));
    double b[MT];
    if constexpr (Deflate) {
        // b = Q^T H Q, row (m, d) of b = row 3 (m - 1) + d; H read entry by entry (L1 hits)
#pragma unroll
        for (int p = 0; p < M; ++p)
#pragma unroll
            for (int q = p; q < M; ++q) {
                const int m = p / 3 + 1, d = p % 3, l = q / 3 + 1, e = q % 3;
                double s = 0.0;
#pragma unroll
                for (int i = 0; i <= m; ++i) {
                    double t = 0.0;
#pragma unroll
                    for (int j = 0; j <= l; ++j)
                        t = fma(helmert<double, NB>(c, j, l), (double)H[bm_index<N>(3 * i + d, 3 * j + e)], t);
                    s = fma(helmert<double, NB>(c, i, m), t, s);
                }
                b[tri<M>(p, q)] = s;
            }
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
            for (int j = i; j < N; ++j) b[tri<M>(i, j)] = (double)H[bm_index<N>(i, j)];
    }
    float a32[MT], v[M * M];
#pragma unroll
    for (int k = 0; k < MT; ++k) a32[k] = (float)b[k];
#pragma unroll
    for (int i = 0; i < M; ++i)
#pragma unroll
        for (int j = 0; j < M; ++j) v[i * M + j] = (i == j) ? 1.0f : 0.0f;
    if (!jacobi_eigen<float, M>(a32, v) && not_converged) *not_converged = 1;
    double dW[MT];
    bool changed = refine_clamp_correction<M>(b, v, eps, mirroring, dW);
    double lam_t = 0.0;
    if (Deflate && 0.0 < eps) {
        changed = true;
        lam_t = mirroring ? 0.0 : eps;
    }
    if (!changed) return 0;
    if constexpr (Deflate) {
        const double diag_t = lam_t / (double)NB;
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
            for (int j = i; j < N; ++j) {
                const int in = i / 3, d = i % 3, jn = j / 3, e = j % 3;
                double s = (d == e) ? diag_t : 0.0;
#pragma unroll
                for (int m = 1; m < NB; ++m) {
                    if (m < in) continue;  // B[in][m] = 0 for in > m
                    double t = 0.0;
#pragma unroll
                    for (int l = 1; l < NB; ++l) {
                        if (l < jn) continue;
                        t = fma(helmert<double, NB>(c, jn, l), dW[tri<M>(3 * (m - 1) + d, 3 * (l - 1) + e)], t);
                    }
                    s = fma(helmert<double, NB>(c, in, m), t, s);
                }
                const S out = (S)((double)H[bm_index<N>(i, j)] + s);
                H[bm_index<N>(i, j)] = out;
                H[bm_index<N>(j, i)] = out;
            }
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
            for (int j = i; j < N; ++j) {
                const S out = (S)((double)H[bm_index<N>(i, j)] + dW[tri<M>(i, j)]);
                H[bm_index<N>(i, j)] = out;
                H[bm_index<N>(j, i)] = out;
            }
    }
    return 1;
}

}  // namespace symxg_dev
