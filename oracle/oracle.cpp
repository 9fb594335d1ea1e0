// ORACLE -- test infrastructure, not product code.
//
// CPU restatement (C++17 + OpenMP) of the reference SymX second-order solve path,
// used only as the checker by tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg.  The product (symx_gb300) never links, loads or calls it.
//
// Parity of this restatement is pinned against outputs of the unmodified reference
// (oracle/_ref, built by oracle/Makefile.ref) committed under tests/golden/.
//
// What is restated (reference file:line):
//   * Neo-Hookean element energy/gradient/Hessian with the FEM quadrature:
//       examples/elasticity_potentials.h:7-13, symx/src/solver/fem_integrators.cpp:41-133.
//       The reference differentiates symbolically; here the closed-form first and second
//       Piola-Kirchhoff derivatives are used (same function, independent derivation).
//       log(J) for J <= 0 is -inf as in the reference's generated code
//       (symx/src/compile/Compilation.cpp:426-428), so inverted elements have E = +inf.
//   * Inertia (examples/dynamic_elasticity_with_contact.cpp:86-103) and penalty Dirichlet
//       (examples/rubber_extrusion.cpp:94-107) potentials.
//   * project_to_PD_inplace (symx/src/solver/second_order/project_to_PD.cpp:12-32):
//       eigenvalues < eps become eps (or -lambda when mirroring), A = V diag V^T only if
//       something changed.  The eigen-decomposition here is Householder tridiagonalization +
//       implicit symmetric QR (Golub & Van Loan, Matrix Computations, 8.3), the algorithm class
//       of the reference's Eigen::SelfAdjointEigenSolver, written out here.
//   * Assembly of all element blocks, both triangles (ElementHessians.cpp:224-256).
//   * Block-Jacobi preconditioner: symmetric 3x3 inverse of the diagonal blocks
//       (BlockedSparseMatrix.h:1146-1278) and its application (:1280-1361).
//   * bsm::solve_pcg (solve_pcg.h:82-232): x0 = 0, stop when sqrt(r.r/b.b) < abs_tol or
//       error/error_0 < rel_tol, stop on p.Ap <= 0.
//   * Quasistatic form (dt <= 0): gravity as the potential -m g.x instead of the inertia term
//       (the GPU library's convention; the reference expresses it the same way as a user
//       potential).
//   * NewtonsMethod::solve with ProjectedNewton (NewtonsMethod.cpp:28-252), forcing term
//       (:423-424), descent check (:159-171), step tolerance (:208-215), Armijo line search
//       (:459-641), residual = max |grad| (solver_utils.h:127).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using Clock = std::chrono::steady_clock;
double seconds_since(Clock::time_point t0) { return std::chrono::duration<double>(Clock::now() - t0).count(); }

struct M3 { double a[3][3]; };

inline double det3(const M3& m)
{
    return m.a[0][0] * (m.a[1][1] * m.a[2][2] - m.a[1][2] * m.a[2][1])
         - m.a[0][1] * (m.a[1][0] * m.a[2][2] - m.a[1][2] * m.a[2][0])
         + m.a[0][2] * (m.a[1][0] * m.a[2][1] - m.a[1][1] * m.a[2][0]);
}

// Inverse-transpose of F via the cofactor matrix divided by det.
inline M3 inv_transpose(const M3& m, double d)
{
    M3 r;
    r.a[0][0] = (m.a[1][1] * m.a[2][2] - m.a[1][2] * m.a[2][1]) / d;
    r.a[0][1] = -(m.a[1][0] * m.a[2][2] - m.a[1][2] * m.a[2][0]) / d;
    r.a[0][2] = (m.a[1][0] * m.a[2][1] - m.a[1][1] * m.a[2][0]) / d;
    r.a[1][0] = -(m.a[0][1] * m.a[2][2] - m.a[0][2] * m.a[2][1]) / d;
    r.a[1][1] = (m.a[0][0] * m.a[2][2] - m.a[0][2] * m.a[2][0]) / d;
    r.a[1][2] = -(m.a[0][0] * m.a[2][1] - m.a[0][1] * m.a[2][0]) / d;
    r.a[2][0] = (m.a[0][1] * m.a[1][2] - m.a[0][2] * m.a[1][1]) / d;
    r.a[2][1] = -(m.a[0][0] * m.a[1][2] - m.a[0][2] * m.a[1][0]) / d;
    r.a[2][2] = (m.a[0][0] * m.a[1][1] - m.a[0][1] * m.a[1][0]) / d;
    return r;
}

// Quadrature of one element type: per point, dN/dxi (nodes x 3) and weight
// (fem_integrators.cpp:52-81; shape functions fem_integrators.h:26-99).
struct Rule {
    int nodes = 0;
    std::vector<double> w;
    std::vector<std::vector<double>> dNdxi;  // per qp: nodes*3
};

Rule make_rule(int nodes)
{
    Rule r;
    r.nodes = nodes;
    if (nodes == 4) {
        r.w = {1.0 / 6.0};
        r.dNdxi = {{-1, -1, -1, 1, 0, 0, 0, 1, 0, 0, 0, 1}};
    } else if (nodes == 10) {
        // quadratic tetrahedron (fem_integrators.h:56-76), 4-point rule with the reference's
        // rounded weights and points (fem_integrators.cpp:60-68)
        const double w = 0.041666667, a = 0.58541020, b = 0.13819660;
        const double pts[4][3] = {{a, b, b}, {b, a, b}, {b, b, a}, {b, b, b}};
        for (int q = 0; q < 4; ++q) {
            const double x0 = pts[q][0], x1 = pts[q][1], x2 = pts[q][2];
            const double n[4] = {1.0 - x0 - x1 - x2, x0, x1, x2};
            const double dn[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};  // d n_i / d xi_k
            const int edge[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
            std::vector<double> d(30);
            for (int c = 0; c < 4; ++c)
                for (int k = 0; k < 3; ++k) d[3 * c + k] = (4.0 * n[c] - 1.0) * dn[c][k];
            for (int m = 0; m < 6; ++m) {
                const int i = edge[m][0], j = edge[m][1];
                for (int k = 0; k < 3; ++k) d[3 * (4 + m) + k] = 4.0 * (dn[i][k] * n[j] + n[i] * dn[j][k]);
            }
            r.w.push_back(w);
            r.dNdxi.push_back(d);
        }
    } else {
        const double p = 1.0 / std::sqrt(3.0);
        const double s[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                {-1, -1, 1}, {1, -1, 1}, {1, 1, 1}, {-1, 1, 1}};
        for (int q = 0; q < 8; ++q) {
            const double xi[3] = {s[q][0] * p, s[q][1] * p, s[q][2] * p};
            std::vector<double> d(24);
            for (int a = 0; a < 8; ++a) {
                const double f0 = 0.5 * (1 + s[a][0] * xi[0]), f1 = 0.5 * (1 + s[a][1] * xi[1]),
                             f2 = 0.5 * (1 + s[a][2] * xi[2]);
                d[3 * a + 0] = 0.5 * s[a][0] * f1 * f2;
                d[3 * a + 1] = 0.5 * s[a][1] * f0 * f2;
                d[3 * a + 2] = 0.5 * s[a][2] * f0 * f1;
            }
            r.w.push_back(1.0);
            r.dNdxi.push_back(d);
        }
    }
    return r;
}

// Neo-Hookean element: E = sum_q w_q det(JX_q) psi(F_q),
// psi = mu/2 (tr F^T F - 3) - mu ln J + lambda/2 (ln J)^2.
// P = mu (F - F^-T) + lambda ln J F^-T;
// dP_ij/dF_kl = mu d_ik d_jl + (mu - lambda ln J) Finv^T_il Finv^T_kj + lambda Finv^T_ij Finv^T_kl.
// With B_a = grad_X N_a: g_(a,i) += c P_ij B_aj, H_(a,i),(b,k) += c dP_ij/dF_kl B_aj B_bl.
void nh_element(const Rule& rule, const double* x, const double* X, double mu, double lam,
                double* E_out, double* g, double* H, bool want_grad, bool want_hess)
{
    const int nn = rule.nodes, n = 3 * nn;
    double E = 0.0;
    if (want_grad) std::fill(g, g + n, 0.0);
    if (want_hess) std::fill(H, H + n * n, 0.0);
    std::vector<double> B(nn * 3);
    for (size_t q = 0; q < rule.w.size(); ++q) {
        const double* dN = rule.dNdxi[q].data();
        M3 JX{}, Jx{};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double sX = 0, sx = 0;
                for (int a = 0; a < nn; ++a) { sX += X[3 * a + i] * dN[3 * a + j]; sx += x[3 * a + i] * dN[3 * a + j]; }
                JX.a[i][j] = sX; Jx.a[i][j] = sx;
            }
        const double detJX = det3(JX);
        const M3 JXit = inv_transpose(JX, detJX);  // JX^-T
        for (int a = 0; a < nn; ++a)
            for (int i = 0; i < 3; ++i) {
                double s = 0;
                for (int j = 0; j < 3; ++j) s += JXit.a[i][j] * dN[3 * a + j];
                B[3 * a + i] = s;
            }
        M3 F{};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double s = 0;
                for (int a = 0; a < nn; ++a) s += x[3 * a + i] * B[3 * a + j];
                F.a[i][j] = s;
            }
        const double J = det3(F);
        const double c = rule.w[q] * detJX;
        if (!(J > 0.0)) { E = std::numeric_limits<double>::infinity(); continue; }
        const double lnJ = std::log(J);
        double Ic = 0;
        for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) Ic += F.a[i][j] * F.a[i][j];
        E += c * (0.5 * mu * (Ic - 3.0) - mu * lnJ + 0.5 * lam * lnJ * lnJ);
        if (!want_grad && !want_hess) continue;
        const M3 Fit = inv_transpose(F, J);
        double P[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) P[i][j] = mu * (F.a[i][j] - Fit.a[i][j]) + lam * lnJ * Fit.a[i][j];
        if (want_grad)
            for (int a = 0; a < nn; ++a)
                for (int i = 0; i < 3; ++i) {
                    double s = 0;
                    for (int j = 0; j < 3; ++j) s += P[i][j] * B[3 * a + j];
                    g[3 * a + i] += c * s;
                }
        if (want_hess) {
            const double k1 = mu - lam * lnJ;
            // dP[i][j][k][l]
            double dP[3][3][3][3];
            for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) for (int l = 0; l < 3; ++l)
                    dP[i][j][k][l] = (i == k && j == l ? mu : 0.0) + k1 * Fit.a[i][l] * Fit.a[k][j]
                                   + lam * Fit.a[i][j] * Fit.a[k][l];
            for (int a = 0; a < nn; ++a)
                for (int b = 0; b < nn; ++b)
                    for (int i = 0; i < 3; ++i)
                        for (int k = 0; k < 3; ++k) {
                            double s = 0;
                            for (int j = 0; j < 3; ++j)
                                for (int l = 0; l < 3; ++l) s += dP[i][j][k][l] * B[3 * a + j] * B[3 * b + l];
                            H[(3 * a + i) * n + 3 * b + k] += c * s;
                        }
        }
    }
    *E_out = E;
}

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (row-major, in A).
// On return diag(A) holds the eigenvalues and V (row-major) the eigenvectors as columns.
void jacobi_eig(int n, double* A, double* V)
{
    for (int i = 0; i < n * n; ++i) V[i] = 0.0;
    for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
    double norm = 0.0;
    for (int i = 0; i < n * n; ++i) norm += A[i] * A[i];
    if (norm == 0.0) return;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < n; ++p) for (int q = p + 1; q < n; ++q) off += A[p * n + q] * A[p * n + q];
        if (off <= 1e-34 * norm) break;
        for (int p = 0; p < n - 1; ++p) {
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[p * n + q];
                if (apq == 0.0) continue;
                const double app = A[p * n + p], aqq = A[q * n + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                A[p * n + q] = A[q * n + p] = 0.0;
                for (int k = 0; k < n; ++k) {
                    const double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
        }
    }
}

// Symmetric eigen-decomposition by Householder tridiagonalization (Golub & Van Loan,
// Matrix Computations, Alg. 8.3.1) followed by implicit symmetric QR steps with the
// Wilkinson shift (Alg. 8.3.2), accumulating all transformations.  The same algorithm class
// as the reference's Eigen::SelfAdjointEigenSolver.  On return lam holds the eigenvalues and
// Q (row-major) the eigenvectors as columns.  Returns false if the QR iteration did not
// converge.
bool symmetric_eig(int n, const double* A_in, double* lam, double* Q)
{
    std::vector<double> A(A_in, A_in + n * n), v(n), p(n), w(n);
    for (int i = 0; i < n * n; ++i) Q[i] = 0.0;
    for (int i = 0; i < n; ++i) Q[i * n + i] = 1.0;
    for (int k = 0; k + 2 < n; ++k) {
        // Householder vector for x = A[k+1:n, k]
        double alpha = 0.0;
        for (int i = k + 1; i < n; ++i) alpha += A[i * n + k] * A[i * n + k];
        alpha = std::sqrt(alpha);
        if (alpha == 0.0) continue;
        const double x0 = A[(k + 1) * n + k];
        const double r = x0 >= 0.0 ? -alpha : alpha;  // reflect x onto r e1
        for (int i = 0; i < n; ++i) v[i] = 0.0;
        v[k + 1] = x0 - r;
        for (int i = k + 2; i < n; ++i) v[i] = A[i * n + k];
        double vv = 0.0;
        for (int i = k + 1; i < n; ++i) vv += v[i] * v[i];
        if (vv == 0.0) continue;
        const double beta = 2.0 / vv;
        // p = beta A v, w = p - (beta p.v / 2) v, A -= v w^T + w v^T (trailing block incl. column k)
        for (int i = k; i < n; ++i) {
            double s = 0.0;
            for (int j = k + 1; j < n; ++j) s += A[i * n + j] * v[j];
            p[i] = beta * s;
        }
        double pv = 0.0;
        for (int i = k + 1; i < n; ++i) pv += p[i] * v[i];
        for (int i = k; i < n; ++i) w[i] = p[i] - 0.5 * beta * pv * v[i];
        for (int i = k + 1; i < n; ++i)
            for (int j = k + 1; j < n; ++j) A[i * n + j] -= v[i] * w[j] + w[i] * v[j];
        A[(k + 1) * n + k] = A[k * n + k + 1] = r;
        for (int i = k + 2; i < n; ++i) A[i * n + k] = A[k * n + i] = 0.0;
        // Q = Q (I - beta v v^T)
        for (int i = 0; i < n; ++i) {
            double s = 0.0;
            for (int j = k + 1; j < n; ++j) s += Q[i * n + j] * v[j];
            s *= beta;
            for (int j = k + 1; j < n; ++j) Q[i * n + j] -= s * v[j];
        }
    }
    std::vector<double> d(n), e(n, 0.0);
    for (int i = 0; i < n; ++i) d[i] = A[i * n + i];
    for (int i = 0; i + 1 < n; ++i) e[i] = A[i * n + i + 1];
    const double eps = std::numeric_limits<double>::epsilon();
    int hi = n - 1, guard = 0;
    while (hi > 0) {
        if (++guard > 60 * n) return false;
        // deflate converged trailing off-diagonals
        if (std::fabs(e[hi - 1]) <= eps * (std::fabs(d[hi - 1]) + std::fabs(d[hi]))) {
            e[hi - 1] = 0.0;
            --hi;
            continue;
        }
        int lo = hi - 1;
        while (lo > 0 && std::fabs(e[lo - 1]) > eps * (std::fabs(d[lo - 1]) + std::fabs(d[lo]))) --lo;
        // Wilkinson shift from the trailing 2x2 block
        const double dd = 0.5 * (d[hi - 1] - d[hi]);
        const double b2 = e[hi - 1] * e[hi - 1];
        const double mu = d[hi] - b2 / (dd + (dd >= 0.0 ? 1.0 : -1.0) * std::sqrt(dd * dd + b2));
        // implicit QR step on rows/cols lo..hi (bulge chase with Givens rotations)
        double x = d[lo] - mu, z = e[lo];
        for (int k = lo; k < hi; ++k) {
            const double rr = std::hypot(x, z);
            const double c = x / rr, sn = -z / rr;
            if (k > lo) e[k - 1] = rr;
            const double a11 = d[k], a22 = d[k + 1], a12 = e[k];
            d[k] = c * c * a11 - 2.0 * c * sn * a12 + sn * sn * a22;
            d[k + 1] = sn * sn * a11 + 2.0 * c * sn * a12 + c * c * a22;
            e[k] = c * sn * (a11 - a22) + (c * c - sn * sn) * a12;
            if (k + 1 < hi) {
                x = e[k];
                z = -sn * e[k + 1];
                e[k + 1] = c * e[k + 1];
            }
            for (int i = 0; i < n; ++i) {
                const double qk = Q[i * n + k], qk1 = Q[i * n + k + 1];
                Q[i * n + k] = c * qk - sn * qk1;
                Q[i * n + k + 1] = sn * qk + c * qk1;
            }
        }
    }
    for (int i = 0; i < n; ++i) lam[i] = d[i];
    return true;
}

bool project_pd(int n, double* M, double eps, bool mirroring)
{
    std::vector<double> V(n * n), lam(n);
    if (!symmetric_eig(n, M, lam.data(), V.data())) {
        // fall back to Jacobi for the (never observed) non-converging case
        std::vector<double> A(M, M + n * n);
        jacobi_eig(n, A.data(), V.data());
        for (int i = 0; i < n; ++i) lam[i] = A[i * n + i];
    }
    bool changed = false;
    for (int i = 0; i < n; ++i) {
        if (lam[i] < eps) { changed = true; lam[i] = mirroring ? -lam[i] : eps; }
    }
    if (!changed) return false;
    for (int i = 0; i < n; ++i)
        for (int j = i; j < n; ++j) {
            double s = 0;
            for (int k = 0; k < n; ++k) s += V[i * n + k] * lam[k] * V[j * n + k];
            M[i * n + j] = M[j * n + i] = s;
        }
    return true;
}

// ---------------------------------------------------------------------------------
struct Problem {
    int nv = 0, ne = 0, nodes = 0, nbc = 0, n_threads = 1;
    std::vector<int32_t> conn, bc_idx;
    std::vector<double> X, x0, v0, x, mass, mu, lam, bc_target;
    double dt = 0, g[3] = {0, 0, 0}, k_bc = 0;
    Rule rule;
    // BCSR sparsity (3x3 blocks, sorted columns, both triangles)
    std::vector<int32_t> rowptr, cols;
    std::vector<double> vals;      // nnzb*9, row-major within a block
    std::vector<int32_t> elem_slot; // ne*nodes*nodes slot of each element block
    std::vector<int32_t> diag_slot; // nv
    std::vector<double> Dinv;       // nv*9
    // element storage
    std::vector<double> Eel, gel, Hel;
};

void build_sparsity(Problem& P)
{
    const int nn = P.nodes;
    std::vector<std::vector<int32_t>> adj(P.nv);
    for (int v = 0; v < P.nv; ++v) adj[v].push_back(v);
    for (int e = 0; e < P.ne; ++e)
        for (int a = 0; a < nn; ++a)
            for (int b = 0; b < nn; ++b) adj[P.conn[e * nn + a]].push_back(P.conn[e * nn + b]);
    P.rowptr.assign(P.nv + 1, 0);
    for (int v = 0; v < P.nv; ++v) {
        auto& r = adj[v];
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end()), r.end());
        P.rowptr[v + 1] = P.rowptr[v] + (int32_t)r.size();
    }
    P.cols.resize(P.rowptr[P.nv]);
    for (int v = 0; v < P.nv; ++v) std::copy(adj[v].begin(), adj[v].end(), P.cols.begin() + P.rowptr[v]);
    auto find = [&](int r, int c) {
        auto b = P.cols.begin() + P.rowptr[r], e = P.cols.begin() + P.rowptr[r + 1];
        return (int32_t)(std::lower_bound(b, e, c) - P.cols.begin());
    };
    P.elem_slot.resize((size_t)P.ne * nn * nn);
    for (int e = 0; e < P.ne; ++e)
        for (int a = 0; a < nn; ++a)
            for (int b = 0; b < nn; ++b)
                P.elem_slot[((size_t)e * nn + a) * nn + b] = find(P.conn[e * nn + a], P.conn[e * nn + b]);
    P.diag_slot.resize(P.nv);
    for (int v = 0; v < P.nv; ++v) P.diag_slot[v] = find(v, v);
    P.vals.assign((size_t)P.cols.size() * 9, 0.0);
}

// E (and gradient) of all potentials at P.x.  Element contributions are summed in the
// order potentials were defined (elastic, inertia, boundary), elements in index order.
double evaluate(Problem& P, double* grad, bool want_hess, double* t_eval)
{
    auto t0 = Clock::now();
    const int nn = P.nodes, n = 3 * nn;
    const bool want_grad = grad != nullptr;
    P.Eel.resize(P.ne);
    if (want_grad) P.gel.resize((size_t)P.ne * n);
    if (want_hess) P.Hel.resize((size_t)P.ne * n * n);
#pragma omp parallel for schedule(static) num_threads(P.n_threads)
    for (int e = 0; e < P.ne; ++e) {
        double xe[30], Xe[30];
        for (int a = 0; a < nn; ++a)
            for (int d = 0; d < 3; ++d) {
                xe[3 * a + d] = P.x[3 * P.conn[e * nn + a] + d];
                Xe[3 * a + d] = P.X[3 * P.conn[e * nn + a] + d];
            }
        nh_element(P.rule, xe, Xe, P.mu[e], P.lam[e], &P.Eel[e], want_grad ? &P.gel[(size_t)e * n] : nullptr,
                   want_hess ? &P.Hel[(size_t)e * n * n] : nullptr, want_grad, want_hess);
    }
    double E = 0.0;
    for (int e = 0; e < P.ne; ++e) E += P.Eel[e];
    // dt > 0: backward-Euler inertia; dt <= 0: quasistatic, gravity as the potential -m g.x
    const bool quasistatic = !(P.dt > 0.0);
    const double idt2 = quasistatic ? 0.0 : 1.0 / (P.dt * P.dt);
    double Ein = 0.0;
    for (int v = 0; v < P.nv; ++v) {
        if (quasistatic) {
            Ein -= P.mass[v] * (P.g[0] * P.x[3 * v] + P.g[1] * P.x[3 * v + 1] + P.g[2] * P.x[3 * v + 2]);
            continue;
        }
        double s = 0;
        for (int d = 0; d < 3; ++d) {
            const double xh = P.x0[3 * v + d] + P.dt * P.v0[3 * v + d] + P.dt * P.dt * P.g[d];
            const double dv = P.x[3 * v + d] - xh;
            s += dv * dv;
        }
        Ein += 0.5 * P.mass[v] * s * idt2;
    }
    double Ebc = 0.0;
    for (int i = 0; i < P.nbc; ++i) {
        double s = 0;
        for (int d = 0; d < 3; ++d) {
            const double dv = P.x[3 * P.bc_idx[i] + d] - P.bc_target[3 * i + d];
            s += dv * dv;
        }
        Ebc += 0.5 * P.k_bc * s;
    }
    E = E + Ein + Ebc;
    if (want_grad) {
        std::fill(grad, grad + 3 * (size_t)P.nv, 0.0);
        for (int e = 0; e < P.ne; ++e)
            for (int a = 0; a < nn; ++a)
                for (int d = 0; d < 3; ++d) grad[3 * P.conn[e * nn + a] + d] += P.gel[(size_t)e * n + 3 * a + d];
        for (int v = 0; v < P.nv; ++v)
            for (int d = 0; d < 3; ++d) {
                if (quasistatic) {
                    grad[3 * v + d] -= P.mass[v] * P.g[d];
                    continue;
                }
                const double xh = P.x0[3 * v + d] + P.dt * P.v0[3 * v + d] + P.dt * P.dt * P.g[d];
                grad[3 * v + d] += P.mass[v] * (P.x[3 * v + d] - xh) * idt2;
            }
        for (int i = 0; i < P.nbc; ++i)
            for (int d = 0; d < 3; ++d)
                grad[3 * P.bc_idx[i] + d] += P.k_bc * (P.x[3 * P.bc_idx[i] + d] - P.bc_target[3 * i + d]);
    }
    if (t_eval) *t_eval += seconds_since(t0);
    return E;
}

void project_all(Problem& P, double eps, bool mirroring, double* t)
{
    auto t0 = Clock::now();
    const int n = 3 * P.nodes;
#pragma omp parallel for schedule(dynamic, 64) num_threads(P.n_threads)
    for (int e = 0; e < P.ne; ++e) project_pd(n, &P.Hel[(size_t)e * n * n], eps, mirroring);
    if (t) *t += seconds_since(t0);
}

// Projection of the element Hessians not yet projected in this evaluation: all of them
// (active == nullptr), or those with a node whose block row is active
// (ElementHessians.cpp:69-182).  Slots [0, ne) of is_proj are the elastic elements, then one
// per vertex (inertia or gravity) and one per boundary vertex; `count` adds the elements
// projected.
void project_selected(Problem& P, double eps, bool mirroring, std::vector<uint8_t>& is_proj, const uint8_t* active,
                      long long& count)
{
    const int nn = P.nodes, n = 3 * nn;
    std::vector<uint8_t> pick(P.ne, 0);
    for (int e = 0; e < P.ne; ++e) {
        if (is_proj[e]) continue;
        bool take = active == nullptr;
        for (int a = 0; a < nn && !take; ++a) take = active[P.conn[e * nn + a]] != 0;
        if (take) {
            pick[e] = 1;
            is_proj[e] = 1;
            ++count;
        }
    }
#pragma omp parallel for schedule(dynamic, 64) num_threads(P.n_threads)
    for (int e = 0; e < P.ne; ++e)
        if (pick[e]) project_pd(n, &P.Hel[(size_t)e * n * n], eps, mirroring);
    for (int v = 0; v < P.nv; ++v) {
        const size_t k = (size_t)P.ne + v;
        if (!is_proj[k] && (active == nullptr || active[v])) { is_proj[k] = 1; ++count; }
    }
    for (int i = 0; i < P.nbc; ++i) {
        const size_t k = (size_t)P.ne + P.nv + i;
        if (!is_proj[k] && (active == nullptr || active[P.bc_idx[i]])) { is_proj[k] = 1; ++count; }
    }
}

// Block-Jacobi preconditioner (BlockedSparseMatrix.h:1146-1278): the symmetric 3x3
// inverse of each diagonal block via the cofactors of its upper triangle.
void block_jacobi_setup(Problem& P)
{
    P.Dinv.resize((size_t)P.nv * 9);
    for (int v = 0; v < P.nv; ++v) {
        const double* m = &P.vals[(size_t)P.diag_slot[v] * 9];
        const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[8];
        const double c00 = d * f - e * e, c01 = c * e - b * f, c02 = b * e - c * d;
        const double det = a * c00 + b * c01 + c * c02;
        const double id = 1.0 / det;
        double* r = &P.Dinv[(size_t)v * 9];
        r[0] = c00 * id; r[1] = c01 * id; r[2] = c02 * id;
        r[3] = r[1]; r[4] = (a * f - c * c) * id; r[5] = (b * c - a * e) * id;
        r[6] = r[2]; r[7] = r[5]; r[8] = (a * d - b * b) * id;
    }
}

void assemble(Problem& P, double* t)
{
    auto t0 = Clock::now();
    const int nn = P.nodes, n = 3 * nn;
    std::fill(P.vals.begin(), P.vals.end(), 0.0);
    for (int e = 0; e < P.ne; ++e)
        for (int a = 0; a < nn; ++a)
            for (int b = 0; b < nn; ++b) {
                double* blk = &P.vals[(size_t)P.elem_slot[((size_t)e * nn + a) * nn + b] * 9];
                const double* h = &P.Hel[(size_t)e * n * n];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 3; ++j) blk[3 * i + j] += h[(3 * a + i) * n + 3 * b + j];
            }
    const double idt2 = P.dt > 0.0 ? 1.0 / (P.dt * P.dt) : 0.0;  // quasistatic: gravity has no Hessian
    for (int v = 0; v < P.nv; ++v) {
        double* blk = &P.vals[(size_t)P.diag_slot[v] * 9];
        for (int d = 0; d < 3; ++d) blk[4 * d] += P.mass[v] * idt2;
    }
    for (int i = 0; i < P.nbc; ++i) {
        double* blk = &P.vals[(size_t)P.diag_slot[P.bc_idx[i]] * 9];
        for (int d = 0; d < 3; ++d) blk[4 * d] += P.k_bc;
    }
    block_jacobi_setup(P);
    if (t) *t += seconds_since(t0);
}

void spmv(const Problem& P, const double* x, double* y)
{
#pragma omp parallel for schedule(static) num_threads(P.n_threads)
    for (int r = 0; r < P.nv; ++r) {
        double s0 = 0, s1 = 0, s2 = 0;
        for (int k = P.rowptr[r]; k < P.rowptr[r + 1]; ++k) {
            const double* b = &P.vals[(size_t)k * 9];
            const double* xc = x + 3 * (size_t)P.cols[k];
            s0 += b[0] * xc[0] + b[1] * xc[1] + b[2] * xc[2];
            s1 += b[3] * xc[0] + b[4] * xc[1] + b[5] * xc[2];
            s2 += b[6] * xc[0] + b[7] * xc[1] + b[8] * xc[2];
        }
        y[3 * r] = s0; y[3 * r + 1] = s1; y[3 * r + 2] = s2;
    }
}

double dot(const Problem& P, const double* a, const double* b, size_t n)
{
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static) num_threads(P.n_threads)
    for (long long i = 0; i < (long long)n; ++i) s += a[i] * b[i];
    return s;
}

void precond(const Problem& P, const double* r, double* z)
{
#pragma omp parallel for schedule(static) num_threads(P.n_threads)
    for (int v = 0; v < P.nv; ++v) {
        const double* m = &P.Dinv[(size_t)v * 9];
        for (int i = 0; i < 3; ++i) z[3 * v + i] = m[3 * i] * r[3 * v] + m[3 * i + 1] * r[3 * v + 1] + m[3 * i + 2] * r[3 * v + 2];
    }
}

struct PCGOut { int iters = 0; bool converged = false; };

PCGOut pcg(const Problem& P, double* x, const double* b, double abs_tol, double rel_tol, int max_iter)
{
    const size_t n = 3 * (size_t)P.nv;
    PCGOut out;
    std::fill(x, x + n, 0.0);
    const double bb = dot(P, b, b, n);
    if (bb < abs_tol * abs_tol) { out.converged = true; return out; }
    std::vector<double> r(b, b + n), z(n), p(n), Ap(n);
    double error = std::sqrt(dot(P, r.data(), r.data(), n) / bb);
    const double error0 = error;
    if (error < abs_tol) { out.converged = true; return out; }
    precond(P, r.data(), z.data());
    p = z;
    double rz = dot(P, r.data(), z.data(), n);
    for (int it = 1; it <= max_iter; ++it) {
        spmv(P, p.data(), Ap.data());
        const double pAp = dot(P, p.data(), Ap.data(), n);
        if (pAp <= 0.0) { out.iters = it; out.converged = false; return out; }
        const double alpha = rz / pAp;
#pragma omp parallel for schedule(static) num_threads(P.n_threads)
        for (long long i = 0; i < (long long)n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
        error = std::sqrt(dot(P, r.data(), r.data(), n) / bb);
        if (error < abs_tol || error / error0 < rel_tol) { out.iters = it; out.converged = true; return out; }
        precond(P, r.data(), z.data());
        const double rz_old = rz;
        rz = dot(P, r.data(), z.data(), n);
        const double beta = rz / rz_old;
#pragma omp parallel for schedule(static) num_threads(P.n_threads)
        for (long long i = 0; i < (long long)n; ++i) p[i] = z[i] + beta * p[i];
    }
    out.iters = max_iter;
    return out;
}

}  // namespace

extern "C" {

// Settings and statistics of one Newton solve (mirror of NewtonSettings/SolveStats for
// the subset the configurations use).
struct oracle_settings {
    int max_iterations;
    int min_iterations;
    double residual_tolerance_abs;
    double residual_tolerance_rel;
    double step_tolerance;
    int max_iterations_as_success;
    double projection_eps;
    int mirroring;
    int cg_max_iterations;
    double cg_abs_tolerance;
    double cg_rel_tolerance;
    double armijo_beta;
    int max_armijo;
    double bailout_residual;
    // ProjectionToPD (solver_utils.h:137-142): 0 Newton, 1 ProjectedNewton, 2 ProjectOnDemand,
    // 3 Progressive; and their parameters (solver_utils.h:219-228)
    int projection_mode;
    int project_on_demand_countdown;
    double ppn_tightening_factor;
    double ppn_release_factor;
};

struct oracle_stats {
    int solver_return;   // 0 ok, 2 too many its, 4 linear solve failure, 5 no descent, 6 armijo failure
    int newton_iterations;
    int cg_iterations;
    int ls_bt_iterations;
    double final_residual;
    double final_energy;
    double t_eval, t_project, t_assembly, t_linear_solve, t_line_search, t_total;
    // element Hessians evaluated / projected over the solve, the inertia (or gravity) and
    // boundary potentials' one-vertex elements included (NewtonsMethod.cpp:219-227)
    long long n_hessians, n_projected_hessians;
};

void oracle_default_settings(oracle_settings* s)
{
    s->max_iterations = std::numeric_limits<int>::max();
    s->min_iterations = 0;
    s->residual_tolerance_abs = 1e-6;
    s->residual_tolerance_rel = 0.0;
    s->step_tolerance = 0.0;
    s->max_iterations_as_success = 0;
    s->projection_eps = 1e-10;
    s->mirroring = 0;
    s->cg_max_iterations = 10000;
    s->cg_abs_tolerance = 1e-12;
    s->cg_rel_tolerance = 1e-4;
    s->armijo_beta = 1e-4;
    s->max_armijo = 20;
    s->bailout_residual = 1e-10;
    s->projection_mode = 1;
    s->project_on_demand_countdown = 4;
    s->ppn_tightening_factor = 0.5;
    s->ppn_release_factor = 2.0;
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// Per-element Neo-Hookean [E, g, H] for a batch (nodes 4 or 8); x, X: n*nodes*3.
int oracle_nh_element_batch(int nodes, int n, const double* x, const double* X, const double* mu,
                            const double* lam, double* E, double* g, double* H)
{
    if (nodes != 4 && nodes != 8 && nodes != 10) return 1;
    const Rule rule = make_rule(nodes);
    const int m = 3 * nodes;
#pragma omp parallel for schedule(static)
    for (int e = 0; e < n; ++e)
        nh_element(rule, x + (size_t)e * m, X + (size_t)e * m, mu[e], lam[e], E + e, g ? g + (size_t)e * m : nullptr,
                   H ? H + (size_t)e * m * m : nullptr, g != nullptr, H != nullptr);
    return 0;
}

int oracle_project_pd_batch(int n, int count, double* mats, double eps, int mirroring, uint8_t* changed)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < count; ++i) {
        const bool c = project_pd(n, mats + (size_t)i * n * n, eps, mirroring != 0);
        if (changed) changed[i] = c ? 1 : 0;
    }
    return 0;
}

void* oracle_create(int nv, int ne, int nodes, const int32_t* conn, const double* X, const double* x0,
                    const double* v0, const double* x_init, const double* mass, const double* mu, const double* lam,
                    int nbc, const int32_t* bc_idx, const double* bc_target, double dt, const double* gravity,
                    double k_bc, int n_threads)
{
    if (nodes != 4 && nodes != 8 && nodes != 10) return nullptr;
    Problem* P = new Problem();
    P->nv = nv; P->ne = ne; P->nodes = nodes; P->nbc = nbc;
    P->n_threads = n_threads > 0 ? n_threads : oracle_num_threads();
    P->conn.assign(conn, conn + (size_t)ne * nodes);
    P->X.assign(X, X + 3 * (size_t)nv);
    P->x0.assign(x0, x0 + 3 * (size_t)nv);
    P->v0.assign(v0, v0 + 3 * (size_t)nv);
    P->x.assign(x_init, x_init + 3 * (size_t)nv);
    P->mass.assign(mass, mass + nv);
    P->mu.assign(mu, mu + ne);
    P->lam.assign(lam, lam + ne);
    P->bc_idx.assign(bc_idx, bc_idx + nbc);
    P->bc_target.assign(bc_target, bc_target + 3 * (size_t)nbc);
    P->dt = dt; P->g[0] = gravity[0]; P->g[1] = gravity[1]; P->g[2] = gravity[2]; P->k_bc = k_bc;
    P->rule = make_rule(nodes);
    build_sparsity(*P);
    return P;
}

void oracle_destroy(void* h) { delete static_cast<Problem*>(h); }

// Step inputs x0 (previous positions) and v0 (velocities), 3 per vertex.
int oracle_set_state(void* h, const double* x0, const double* v0)
{
    Problem& P = *static_cast<Problem*>(h);
    if (x0) P.x0.assign(x0, x0 + 3 * (size_t)P.nv);
    if (v0) P.v0.assign(v0, v0 + 3 * (size_t)P.nv);
    return 0;
}

int oracle_set_x(void* h, const double* x)
{
    Problem& P = *static_cast<Problem*>(h);
    std::copy(x, x + 3 * (size_t)P.nv, P.x.begin());
    return 0;
}

int oracle_get_x(void* h, double* x)
{
    Problem& P = *static_cast<Problem*>(h);
    std::copy(P.x.begin(), P.x.end(), x);
    return 0;
}

// Energy and gradient at the current x (grad may be null).
int oracle_evaluate(void* h, double* E, double* grad)
{
    Problem& P = *static_cast<Problem*>(h);
    *E = evaluate(P, grad, false, nullptr);
    return 0;
}

// Element Hessians of the elastic potential (optionally projected) and the assembled
// BCSR matrix.  Pass null outputs to query sizes: nnzb.
int oracle_assemble(void* h, int project, double eps, int32_t* nnzb, int32_t* rowptr, int32_t* cols, double* vals,
                    double* elem_hess)
{
    Problem& P = *static_cast<Problem*>(h);
    *nnzb = (int32_t)P.cols.size();
    if (!vals) return 0;
    std::vector<double> g(3 * (size_t)P.nv);
    evaluate(P, g.data(), true, nullptr);
    if (project) project_all(P, eps, false, nullptr);
    if (elem_hess) std::copy(P.Hel.begin(), P.Hel.end(), elem_hess);
    assemble(P, nullptr);
    std::copy(P.rowptr.begin(), P.rowptr.end(), rowptr);
    std::copy(P.cols.begin(), P.cols.end(), cols);
    std::copy(P.vals.begin(), P.vals.end(), vals);
    return 0;
}

int oracle_solve(void* h, const oracle_settings* s, oracle_stats* st)
{
    Problem& P = *static_cast<Problem*>(h);
    auto t_start = Clock::now();
    std::memset(st, 0, sizeof(*st));
    const size_t n = 3 * (size_t)P.nv;
    std::vector<double> grad(n), du(n), rhs(n), x_before(n);
    double res0 = std::numeric_limits<double>::max();
    int result = -1;  // running
    int it = -1;
    double E0 = 0.0, residual = 0.0;
    const int mode = s->projection_mode;
    int pdn_countdown = 0;
    double ppn_threshold = -1.0;
    std::vector<uint8_t> is_proj((size_t)P.ne + P.nv + P.nbc), active(P.nv);
    const long long n_all_hessians = (long long)P.ne + P.nv + P.nbc;
    long long n_proj = 0;
    while (result < 0) {
        ++it;
        if (it == s->max_iterations) { result = s->max_iterations_as_success ? 0 : 2; break; }
        E0 = evaluate(P, grad.data(), true, &st->t_eval);
        residual = 0.0;
        for (size_t i = 0; i < n; ++i) residual = std::max(residual, std::fabs(grad[i]));
        if (it == 0) res0 = residual;
        if (residual < s->bailout_residual) { result = 0; break; }
        if (it >= s->min_iterations) {
            if (residual < s->residual_tolerance_abs) { result = 0; break; }
            if (it > 0 && residual / res0 < s->residual_tolerance_rel) { result = 0; break; }
        }
        // projection and solve until the direction descends or nothing is left to project
        // (NewtonsMethod.cpp:133-186, _project_and_assemble :257-341, _increase_projection
        // :343-358, _decrease_projection :359-373).  Element Hessians of this evaluation start
        // unprojected; the inertia/gravity and boundary potentials' one-vertex elements are
        // counted like the reference's (their projection changes nothing the oracle keeps).
        std::fill(is_proj.begin(), is_proj.end(), 0);
        double du_dot_g = 0.0, du_max = 0.0;
        while (true) {
            bool all_projected = false;
            const auto tp = Clock::now();
            if (mode == 1 || (mode == 2 && pdn_countdown > 0)) {
                project_selected(P, s->projection_eps, s->mirroring != 0, is_proj, nullptr, n_proj);
                all_projected = true;
            } else if (mode == 3 && ppn_threshold > 0.0) {
                if (ppn_threshold < 1e-12) ppn_threshold = 0.0;
                all_projected = true;
                for (int v = 0; v < P.nv; ++v) {
                    const double m = std::max(std::fabs(grad[3 * v]), std::max(std::fabs(grad[3 * v + 1]), std::fabs(grad[3 * v + 2])));
                    active[v] = m >= ppn_threshold ? 1 : 0;
                    if (!active[v]) all_projected = false;
                }
                project_selected(P, s->projection_eps, s->mirroring != 0, is_proj, active.data(), n_proj);
            }
            st->t_project += seconds_since(tp);
            assemble(P, &st->t_assembly);
            auto tl = Clock::now();
            const double forcing = std::min(1e-2, residual * std::min(0.5, std::sqrt(residual)));
            const double abs_tol = std::max(forcing, s->cg_abs_tolerance);
            for (size_t i = 0; i < n; ++i) rhs[i] = -grad[i];
            PCGOut po = pcg(P, du.data(), rhs.data(), abs_tol, s->cg_rel_tolerance, s->cg_max_iterations);
            st->t_linear_solve += seconds_since(tl);
            st->cg_iterations += po.iters;
            const bool can_project_more = mode != 0 && !all_projected;
            if (!po.converged && !can_project_more) { result = 4; break; }
            bool descends = false;
            if (po.converged) {
                du_dot_g = 0.0;
                for (size_t i = 0; i < n; ++i) du_dot_g += du[i] * grad[i];
                descends = du_dot_g < 0.0;
                if (!descends && !can_project_more) { result = 5; break; }
            }
            if (po.converged && descends) break;
            if (mode == 2) pdn_countdown = s->project_on_demand_countdown;
            if (mode == 3) {
                if (ppn_threshold < 0.0) ppn_threshold = residual;
                ppn_threshold *= s->ppn_tightening_factor;
                // Deviation: a zero threshold cannot tighten and the reference would retry the
                // same solve forever; a threshold below 1e-12 projects everything next time.
                if (ppn_threshold == 0.0) ppn_threshold = 1e-13;
            }
        }
        if (result >= 0) break;
        st->n_hessians += n_all_hessians;  // counted once the direction is found
        st->n_projected_hessians += n_proj;
        n_proj = 0;
        if (mode == 2) pdn_countdown--;
        if (mode == 3) ppn_threshold *= s->ppn_release_factor;
        for (size_t i = 0; i < n; ++i) du_max = std::max(du_max, std::fabs(du[i]));
        if (it >= s->min_iterations && du_max < s->step_tolerance) { result = 0; break; }
        // Armijo backtracking (no step cap, no max-step or validity callbacks)
        auto tls = Clock::now();
        x_before = P.x;
        double step = 1.0;
        auto apply = [&](double sc) { for (size_t i = 0; i < n; ++i) P.x[i] = x_before[i] + sc * du[i]; };
        apply(step);
        const double expected = s->armijo_beta * du_dot_g;
        double E_thr = E0 + expected * step;
        int a = 0;
        for (; a < s->max_armijo; ++a) {
            const double E1 = evaluate(P, nullptr, false, nullptr);
            if (E1 < E_thr) break;
            step *= 0.5;
            apply(step);
            E_thr = E0 + expected * step;
            st->ls_bt_iterations++;
        }
        st->t_line_search += seconds_since(tls);
        if (a == s->max_armijo) { result = 6; break; }
    }
    st->solver_return = result;
    st->newton_iterations = it;
    st->final_residual = residual;
    st->final_energy = E0;
    st->t_total = seconds_since(t_start);
    return 0;
}

// bsm::solve_pcg (solve_pcg.h:82-232) with the block-diagonal preconditioner on a given
// 3x3-block CSR matrix (row-major blocks); x0 = 0.  Every row must hold its diagonal block
// (returns -1 otherwise).
int oracle_bcsr_pcg(int32_t n_blocks, const int32_t* rowptr, const int32_t* cols, const double* vals, const double* b,
                    double* x, double abs_tol, double rel_tol, int32_t max_iter, int32_t* iterations,
                    int32_t* converged)
{
    Problem P;
    P.nv = n_blocks;
    P.n_threads = 1;
    P.rowptr.assign(rowptr, rowptr + n_blocks + 1);
    P.cols.assign(cols, cols + rowptr[n_blocks]);
    P.vals.assign(vals, vals + (size_t)rowptr[n_blocks] * 9);
    P.diag_slot.assign(n_blocks, -1);
    for (int r = 0; r < n_blocks; ++r)
        for (int k = rowptr[r]; k < rowptr[r + 1]; ++k)
            if (cols[k] == r) { P.diag_slot[r] = k; break; }
    for (int r = 0; r < n_blocks; ++r)
        if (P.diag_slot[r] < 0) return -1;
    block_jacobi_setup(P);
    const PCGOut o = pcg(P, x, b, abs_tol, rel_tol, max_iter);
    *iterations = o.iters;
    *converged = o.converged ? 1 : 0;
    return 0;
}

}  // extern "C"
