// CPU tests of the symx_gb300 C++ API (symbolic front end, differentiation, code
// generation, NVRTC compilation).  Built and driven by tests/test_cpp_api.py.
//
//   test_cpu_api nh_elem <in.bin> <out.bin>   NH Tet4 [E, g, H] through the symbolic API
//   test_cpu_api nvrtc <cache_dir>            generate + NVRTC-compile the elastic-step kernels
//   test_cpu_api selftest                     closed-form derivative checks
#include <symx>

#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "../../symx_gb300/csrc/cuda_module.h"

using namespace symx;

static int fails = 0;
static void expect_close(const char* what, double got, double want, double tol = 1e-12)
{
    const double err = std::fabs(got - want) / std::max(1.0, std::fabs(want));
    if (!(err <= tol)) {
        std::printf("FAIL %s: got %.17g want %.17g\n", what, got, want);
        ++fails;
    }
}

static int selftest()
{
    Workspace ws;
    Scalar x = ws.make_scalar(), y = ws.make_scalar();
    x.set_value(0.7);
    y.set_value(-1.3);
    // d/dx (x^3 y + sin(x) / y) = 3 x^2 y + cos(x) / y
    Scalar f = x.powN(3) * y + sin(x) / y;
    expect_close("diff poly/trig", diff(f, x).eval(), 3 * 0.49 * -1.3 + std::cos(0.7) / -1.3);
    // d2/dxdy
    expect_close("mixed second derivative", diff(diff(f, x), y).eval(), 3 * 0.49 - std::cos(0.7) / (1.69));
    // log guard: log of a non-positive value is -inf
    Scalar g = log(y);
    if (!(std::isinf(g.eval()) && g.eval() < 0)) { std::printf("FAIL log guard\n"); ++fails; }
    // sqrt, exp, branch-based abs
    Scalar h = sqrt(x * x + 1.0) * exp(x) + abs(y);
    const double hx = (0.7 / std::sqrt(1.49)) * std::exp(0.7) + std::sqrt(1.49) * std::exp(0.7);
    expect_close("sqrt/exp derivative", diff(h, x).eval(), hx);
    expect_close("abs branch derivative", diff(h, y).eval(), -1.0);
    // hash-consing: rebuilding an expression returns the same node
    Scalar a1 = x * y + 2.0, a2 = x * y + 2.0;
    if (a1.expr_id != a2.expr_id) { std::printf("FAIL hash-consing\n"); ++fails; }
    // 3x3 determinant / inverse
    Matrix M = ws.make_matrix({3, 3});
    const double mv[9] = {2, 0.5, 0.1, 0.3, 3, 0.2, 0.4, 0.6, 4};
    for (int i = 0; i < 9; ++i) M.values()[i].set_value(mv[i]);
    const double det = 2 * (12 - 0.12) - 0.5 * (1.2 - 0.08) + 0.1 * (0.18 - 1.2);
    expect_close("det", M.det().eval(), det);
    Matrix I = M * M.inv();
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) expect_close("M*inv(M)", I(i, j).eval(), i == j ? 1.0 : 0.0, 1e-14);
    // symmetric Hessian mirrors the upper triangle
    Matrix H = hessian(f, {x, y});
    if (H(1, 0).expr_id != H(0, 1).expr_id) { std::printf("FAIL symmetric hessian\n"); ++fails; }
    std::printf(fails ? "selftest FAILED (%d)\n" : "selftest PASS\n", fails);
    return fails ? 1 : 0;
}

static int nh_elem(const char* in, const char* out)
{
    std::ifstream f(in, std::ios::binary);
    int64_t n = 0;
    f.read(reinterpret_cast<char*>(&n), sizeof(n));
    std::vector<double> rows(26 * n);
    f.read(reinterpret_cast<char*>(rows.data()), sizeof(double) * rows.size());
    Workspace ws;
    std::vector<Vector> x = ws.make_vectors(3, 4), X = ws.make_vectors(3, 4);
    Scalar mu = ws.make_scalar(), lam = ws.make_scalar();
    auto jac = [&](const std::vector<Vector>& v) {
        Matrix J = ws.get_identity_matrix(3);
        J.set_col(0, v[1] - v[0]);
        J.set_col(1, v[2] - v[0]);
        J.set_col(2, v[3] - v[0]);
        return J;
    };
    Matrix F = jac(x) * jac(X).inv();
    Matrix C = F.transpose() * F;
    Scalar logJ = log(F.det());
    Scalar E = (0.5 * mu * (C.trace() - 3.0) - mu * logJ + 0.5 * lam * logJ.powN(2)) * jac(X).det() * (1.0 / 6.0);
    std::vector<Scalar> vgh = value_gradient_hessian(E, collect_scalars(x));
    std::vector<double> res(157 * n);
    for (int64_t e = 0; e < n; ++e) {
        const double* r = &rows[26 * e];
        for (int v = 0; v < 4; ++v)
            for (int d = 0; d < 3; ++d) {
                x[v][d].set_value(r[3 * v + d]);
                X[v][d].set_value(r[12 + 3 * v + d]);
            }
        mu.set_value(r[24]);
        lam.set_value(r[25]);
        for (int k = 0; k < 157; ++k) res[157 * e + k] = vgh[k].eval();
    }
    std::ofstream o(out, std::ios::binary);
    o.write(reinterpret_cast<const char*>(res.data()), sizeof(double) * res.size());
    return 0;
}

// Neo-Hookean Hex27 element, E and dE/dx summed over get_integration_rule(Hex27), evaluated on
// the host.  in: int64 n, n x 164 rows [x (81), X (81), mu, lambda]; out: n x 82 [E, g(81)].
static int nh_elem27(const char* in, const char* out)
{
    std::ifstream f(in, std::ios::binary);
    int64_t n = 0;
    f.read(reinterpret_cast<char*>(&n), sizeof(n));
    std::vector<double> rows(164 * n);
    f.read(reinterpret_cast<char*>(rows.data()), sizeof(double) * rows.size());
    Workspace ws;
    std::vector<Vector> x = ws.make_vectors(3, 27), X = ws.make_vectors(3, 27);
    Vector xi = ws.make_vectors(3, 1)[0];
    Scalar mu = ws.make_scalar(), lam = ws.make_scalar();
    Matrix Jx = fem_jacobian(FEM_Element::Hex27, x, xi), JX = fem_jacobian(FEM_Element::Hex27, X, xi);
    Matrix F = Jx * JX.inv();
    Scalar logJ = log(F.det());
    Scalar psi = 0.5 * mu * ((F.transpose() * F).trace() - 3.0) - mu * logJ + 0.5 * lam * logJ.powN(2);
    std::vector<Scalar> vg = value_gradient(psi * JX.det(), collect_scalars(x));
    const auto rule = get_integration_rule(FEM_Element::Hex27);
    std::vector<double> res(82 * n, 0.0);
    for (int64_t e = 0; e < n; ++e) {
        const double* r = &rows[164 * e];
        for (int v = 0; v < 27; ++v)
            for (int d = 0; d < 3; ++d) {
                x[v][d].set_value(r[3 * v + d]);
                X[v][d].set_value(r[81 + 3 * v + d]);
            }
        mu.set_value(r[162]);
        lam.set_value(r[163]);
        for (const auto& q : rule) {
            for (int d = 0; d < 3; ++d) xi[d].set_value(q[1 + d]);
            for (int k = 0; k < 82; ++k) res[82 * e + k] += q[0] * vg[k].eval();
        }
    }
    std::ofstream o(out, std::ios::binary);
    o.write(reinterpret_cast<const char*>(res.data()), sizeof(double) * res.size());
    return 0;
}

static int nvrtc(const char* cache_dir)
{
    (void)cache_dir;
    // a 2-tet mesh with the same three potentials as the elastic step
    std::vector<std::array<double, 3>> x = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 1}};
    std::vector<std::array<double, 3>> X = x, x0 = x, v0(5, {0, 0, 0});
    std::vector<int32_t> tets = {0, 0, 1, 2, 3, 1, 1, 2, 3, 4};
    std::vector<double> mu = {1.0, 1.0}, lam = {1.0, 1.0}, mass(5, 1.0);
    std::vector<std::array<int32_t, 1>> verts = {{0}, {1}, {2}, {3}, {4}};
    double dt = 0.01;
    std::array<double, 3> grav{0, -9.81, 0};
    auto G = GlobalPotential::create();
    G->add_potential("nh", tets, 5, [&](MappedWorkspace<double>& mws, Element& e) {
        std::vector<Vector> xs = mws.make_vectors(x, e.slice(1, 5));
        std::vector<Vector> Xs = mws.make_vectors(X, e.slice(1, 5));
        Scalar m = mws.make_scalar(mu, e[0]);
        Scalar l = mws.make_scalar(lam, e[0]);
        return fem_integrator(mws, FEM_Element::Tet4, [&](Scalar& w, Vector& xi) {
            Matrix F = fem_jacobian(FEM_Element::Tet4, xs, xi) * fem_jacobian(FEM_Element::Tet4, Xs, xi).inv();
            Scalar lj = log(F.det());
            return (0.5 * m * (F.frobenius_norm_sq() - 3.0) - m * lj + 0.5 * l * lj.powN(2)) *
                   fem_jacobian(FEM_Element::Tet4, Xs, xi).det() * w;
        });
    });
    G->add_potential("inertia", verts, [&](MappedWorkspace<double>& mws, Element& e) {
        Vector a = mws.make_vector(x, e[0]), b = mws.make_vector(x0, e[0]), v = mws.make_vector(v0, e[0]);
        Scalar m = mws.make_scalar(mass, e[0]), h = mws.make_scalar(dt);
        Vector g = mws.make_vector(grav);
        return 0.5 * m * (a - (b + h * v + h * h * g)).squared_norm() / h.powN(2);
    });
    G->add_dof(x);
    const std::vector<std::string> src = generate_element_kernel_sources(*G);
    for (size_t i = 0; i < src.size(); ++i) {
        const std::string cubin = symxg::compile_cubin(src[i], {});
        std::printf("potential %zu: %zu source bytes -> %zu cubin bytes\n", i, src[i].size(), cubin.size());
        if (cubin.size() < 1000) { std::printf("FAIL cubin too small\n"); return 1; }
    }
    // mixed-derivative (adjoint) kernels for every bound non-DoF input
    const std::vector<std::uintptr_t> params = {reinterpret_cast<std::uintptr_t>(&mu), reinterpret_cast<std::uintptr_t>(&lam),
                                                reinterpret_cast<std::uintptr_t>(&x0), reinterpret_cast<std::uintptr_t>(&v0),
                                                reinterpret_cast<std::uintptr_t>(&mass)};
    for (std::uintptr_t prm : params) {
        const std::vector<std::string> ms = generate_mixed_kernel_sources(*G, prm);
        if (ms.size() != 1) { std::printf("FAIL expected one mixed kernel per parameter, got %zu\n", ms.size()); return 1; }
        const std::string cubin = symxg::compile_cubin(ms[0], {});
        std::printf("mixed kernel: %zu source bytes -> %zu cubin bytes\n", ms[0].size(), cubin.size());
        if (cubin.size() < 1000) { std::printf("FAIL cubin too small\n"); return 1; }
    }
    // a Hex8 element: eight quadrature points, so the mixed E+g+H kernel takes one lane per point
    {
        std::vector<std::array<double, 3>> hx;
        for (int k = 0; k < 8; ++k) hx.push_back({double(k & 1), double((k >> 1) & 1), double((k >> 2) & 1)});
        std::vector<std::array<double, 3>> hX = hx;
        std::vector<int32_t> hexes = {0, 0, 1, 3, 2, 4, 5, 7, 6};
        std::vector<double> hmu = {1.0}, hlam = {1.0};
        auto G2 = GlobalPotential::create();
        G2->add_potential("nh_hex", hexes, 9, [&](MappedWorkspace<double>& mws, Element& e) {
            std::vector<Vector> xs = mws.make_vectors(hx, e.slice(1, 9));
            std::vector<Vector> Xs = mws.make_vectors(hX, e.slice(1, 9));
            Scalar m = mws.make_scalar(hmu, e[0]);
            Scalar l = mws.make_scalar(hlam, e[0]);
            return fem_integrator(mws, FEM_Element::Hex8, [&](Scalar& w, Vector& xi) {
                Matrix F = fem_jacobian(FEM_Element::Hex8, xs, xi) * fem_jacobian(FEM_Element::Hex8, Xs, xi).inv();
                Scalar lj = log(F.det());
                return (0.5 * m * (F.frobenius_norm_sq() - 3.0) - m * lj + 0.5 * l * lj.powN(2)) *
                       fem_jacobian(FEM_Element::Hex8, Xs, xi).det() * w;
            });
        });
        G2->add_dof(hx);
        const std::vector<std::string> hs = generate_element_kernel_sources(*G2);
        if (hs.size() != 1 || hs[0].find("symxg_eval_h_f32_q") == std::string::npos) {
            std::printf("FAIL the Hex8 source has no quadrature-parallel Hessian function\n");
            return 1;
        }
        const std::string cubin = symxg::compile_cubin(hs[0], {});
        std::printf("hex8 potential: %zu source bytes -> %zu cubin bytes\n", hs[0].size(), cubin.size());
        if (cubin.size() < 1000) { std::printf("FAIL cubin too small\n"); return 1; }
    }
    std::printf("nvrtc PASS\n");
    return 0;
}

// Writes generate_cuboid_mesh's output: int64 {n_vertices, n_elements, stride}, the vertices
// (FLOAT), the connectivity (int32).  prec is "d" or "f".
template <typename FLOAT>
int write_mesh(int type, const std::array<int32_t, 3>& n, const std::array<FLOAT, 3>& size, const char* path)
{
    const symx::FEMMesh<FLOAT> m = symx::generate_cuboid_mesh(static_cast<symx::FEM_Element>(type), size, n);
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return 1;
    const int64_t hdr[3] = {(int64_t)m.vertices.size(), (int64_t)m.n_elements, (int64_t)m.connectivity_stride};
    std::fwrite(hdr, sizeof(hdr), 1, f);
    for (const auto& v : m.vertices) std::fwrite(v.data(), sizeof(FLOAT), 3, f);
    std::fwrite(m.connectivity.data(), sizeof(int), m.connectivity.size(), f);
    std::fclose(f);
    return 0;
}

int mesh(char** a)
{
    const int type = std::atoi(a[1]);
    const std::array<int32_t, 3> n = {std::atoi(a[2]), std::atoi(a[3]), std::atoi(a[4])};
    if (std::string(a[0]) == "f")
        return write_mesh<float>(type, n, {(float)std::atof(a[5]), (float)std::atof(a[6]), (float)std::atof(a[7])}, a[8]);
    return write_mesh<double>(type, n, {std::atof(a[5]), std::atof(a[6]), std::atof(a[7])}, a[8]);
}

// reorder_connectivity_RCM on a connectivity file: in int64 {stride, n_elements, num_nodes},
// int32 conn; out int32 old_to_new, int32 conn.
int rcm(const char* in, const char* out, bool reorder_elements)
{
    std::FILE* f = std::fopen(in, "rb");
    if (!f) return 1;
    int64_t hdr[3];
    if (std::fread(hdr, sizeof(hdr), 1, f) != 1) return 1;
    std::vector<int> conn((size_t)(hdr[0] * hdr[1]));
    if (std::fread(conn.data(), sizeof(int), conn.size(), f) != conn.size()) return 1;
    std::fclose(f);
    const symx::ReorderResult r =
        symx::reorder_connectivity_RCM(conn.data(), (int)hdr[0], (int)hdr[1], (int)hdr[2], reorder_elements);
    f = std::fopen(out, "wb");
    if (!f) return 1;
    std::fwrite(r.old_to_new.data(), sizeof(int), r.old_to_new.size(), f);
    std::fwrite(conn.data(), sizeof(int), conn.size(), f);
    std::fclose(f);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    const std::string mode = argv[1];
    try {
        if (mode == "selftest") return selftest();
        if (mode == "nh_elem" && argc >= 4) return nh_elem(argv[2], argv[3]);
        if (mode == "nh_elem27" && argc >= 4) return nh_elem27(argv[2], argv[3]);
        if (mode == "nvrtc") return nvrtc(argc >= 3 ? argv[2] : "");
        if (mode == "mesh" && argc >= 11) return mesh(argv + 2);  // prec type nx ny nz sx sy sz out
        if (mode == "rcm" && argc >= 5) return rcm(argv[2], argv[3], std::atoi(argv[4]) != 0);
    } catch (const std::exception& e) {
        std::printf("exception: %s\n", e.what());
        return 3;
    }
    return 2;
}
