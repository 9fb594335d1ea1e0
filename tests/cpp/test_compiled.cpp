// Compiled<T> (GPU) against host evaluation of the same expressions, following the
// reference's compilation tests (tests/test_compilation.cpp:16-460 and the compiled
// sections of tests/test_scalar.cpp:280-300, 620-640).  Usage:
//   test_compiled nogpu <folder>                       code generation and files without a device
//   test_compiled gpu <folder> <nh_in.bin> <nh_ref.bin>  every case on the GPU
#include <symx>

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

using namespace symx;

static int fails = 0;
#define REQUIRE(c)                                                            \
    do {                                                                      \
        if (!(c)) {                                                           \
            std::printf("FAIL line %d: %s\n", __LINE__, #c);                  \
            ++fails;                                                          \
        }                                                                     \
    } while (0)

static bool approx(double a, double b, double tol = 1e-12) { return std::abs(a - b) < tol; }
static bool file_exists(const std::string& p) { return std::ifstream(p).good(); }

// tests/test_compilation.cpp:16-93: a chain through every operation, double and float
static void chain(const std::string& dir)
{
    Workspace ws;
    Scalar a = ws.make_scalar(), b = ws.make_scalar(), c = ws.make_scalar();
    const double A = 5.76, B = 1.47, C = 0.79;
    Scalar x = a + b;
    x -= c;
    x *= a;
    x /= b;
    x = powN(x, 2);
    x = powF(x, 3.1);
    x = x.inv();
    x = sqrt(x);
    x = log(x);
    x = exp(x);
    x = sin(x);
    x = cos(x);
    x = tan(x);
    x *= asin(c);
    x *= acos(c);
    x = atan(x);
    const std::string checksum = x.get_checksum();
    std::vector<Scalar> expr = {x};
    a.set_value(A);
    b.set_value(B);
    c.set_value(C);
    const double sol = expr[0].eval();
    {
        Compiled<double> f(expr, "f_double", dir, checksum);
        f.set(a, A);
        f.set(b, B);
        f.set(c, C);
        REQUIRE(approx(sol, f.run()[0]));
    }
    {
        Compiled<float> f(expr, "f_float", dir, checksum);
        f.set(a, (float)A);
        f.set(b, (float)B);
        f.set(c, (float)C);
        REQUIRE(std::abs(sol - (double)f.run()[0]) < 1e-2);
    }
}

// tests/test_compilation.cpp:96-167
static void multi_expression(const std::string& dir)
{
    Workspace ws;
    Scalar x = ws.make_scalar(), y = ws.make_scalar();
    std::vector<Scalar> exprs = {x + y, x * y - 0.5, sin(x) + cos(y), sqrt(x * x + y * y)};
    const double X = 1.2, Y = 2.1;
    x.set_value(X);
    y.set_value(Y);
    std::vector<double> expected;
    for (auto& e : exprs) expected.push_back(e.eval());
    const std::string checksum = exprs[0].get_checksum();
    {
        Compiled<double> f(exprs, "multi_type_test_double", dir, checksum);
        f.set(x, X);
        f.set(y, Y);
        const View<double> r = f.run();
        REQUIRE(r.size() == 4);
        for (int i = 0; i < 4; ++i) REQUIRE(approx(expected[i], r[i]));
    }
    {
        Compiled<float> f(exprs, "multi_type_test_float", dir, checksum);
        f.set(x, (float)X);
        f.set(y, (float)Y);
        const View<float> r = f.run();
        for (int i = 0; i < 4; ++i) REQUIRE(approx(expected[i], (double)r[i], 1e-5));
    }
}

// tests/test_compilation.cpp:170-248
static void branches(const std::string& dir)
{
    Workspace ws;
    Scalar a = ws.make_scalar(), b = ws.make_scalar(), c = ws.make_scalar();
    Scalar e = branch(a > b, a * c + sin(b), b * c - cos(a));
    {
        Compiled<double> f({e}, "branch_true", dir, e.get_checksum());
        f.set(a, 2.0);
        f.set(b, 1.0);
        f.set(c, 0.5);
        REQUIRE(approx(f.run()[0], 2.0 * 0.5 + std::sin(1.0)));
    }
    {
        Compiled<double> f({e}, "branch_false", dir, e.get_checksum());
        f.set(a, 1.0);
        f.set(b, 2.0);
        f.set(c, 0.5);
        REQUIRE(approx(f.run()[0], 2.0 * 0.5 - std::cos(1.0)));
    }
    {
        Scalar d = ws.make_scalar();
        Scalar inner = branch(c > 0.0, c.powN(2), c.sqrt());
        Scalar nested = branch(a > b, a * inner, b + inner);
        Compiled<double> f({nested}, "nested_branch", dir, nested.get_checksum());
        f.set(a, 3.0);
        f.set(b, 1.0);
        f.set(c, 4.0);
        f.set(d, 0.1);
        REQUIRE(approx(f.run()[0], 3.0 * 16.0));
    }
    // tests/test_scalar.cpp:620-634: log of a negative value is -inf
    {
        Scalar xl = ws.make_scalar();
        Compiled<double> f({log(xl)}, "log_edge_test", dir);
        f.set(xl, -1.0);
        const View<double> r = f.run();
        REQUIRE(std::isinf(r[0]) && std::signbit(r[0]));
    }
}

// tests/test_compilation.cpp:251-312
static void caching(const std::string& dir)
{
    Workspace ws;
    Scalar a = ws.make_scalar(), b = ws.make_scalar();
    Scalar expr = a * b + sin(a);
    const std::string checksum = expr.get_checksum();
    Compiled<double> f1;
    f1.compile({expr}, "cache_test", dir, checksum);
    REQUIRE(f1.is_valid() && !f1.was_cached());
    Compiled<double> f2;
    REQUIRE(f2.load_if_cached("cache_test", dir, checksum));
    REQUIRE(f2.was_cached());
    Compiled<double> f3;
    REQUIRE(!f3.load_if_cached("cache_test", dir, checksum + "_other"));
    REQUIRE(!f3.is_valid());
    Compiled<float> f4;  // same name and id, other type: a miss
    REQUIRE(!f4.load_if_cached("cache_test", dir, checksum));
    f1.set(a, 1.5);
    f1.set(b, 2.3);
    f2.set(a, 1.5);
    f2.set(b, 2.3);
    REQUIRE(f1.run()[0] == f2.run()[0]);
    REQUIRE(approx(f2.run()[0], 1.5 * 2.3 + std::sin(1.5)));

    Scalar other = a + b * cos(a);
    REQUIRE(other.get_checksum() != checksum);
    REQUIRE(get_checksum({expr}) == get_checksum({a * b + sin(a)}));

    // try_load_otherwise_compile: a miss compiles, a hit loads
    Compiled<double> g1;
    g1.try_load_otherwise_compile({other}, "try_load_test", dir, other.get_checksum() + "_miss");
    Compiled<double> g2;
    g2.try_load_otherwise_compile({other}, "try_load_test", dir, other.get_checksum() + "_miss");
    REQUIRE(g2.was_cached() && g2.get_name() == "try_load_test");
    // with loading disabled the same call compiles again
    enable_load_compiled(false);
    Compiled<double> g3({other}, "try_load_test", dir, other.get_checksum() + "_miss");
    REQUIRE(!g3.was_cached());
    enable_load_compiled(true);
    const Compilation::Info info = g3.get_compilation_info();
    REQUIRE(info.n_inputs == 2 && info.n_outputs == 1 && info.compiled_type == FloatType::Double);
    REQUIRE(info.runtime_compilation > 0.0 && info.n_bytes_symbols > 0);
    g3.set(a, 1.0);
    g3.set(b, 2.0);
    REQUIRE(approx(g3.run()[0], 1.0 + 2.0 * std::cos(1.0)));
}

// tests/test_compilation.cpp:315-367 and 369-427: thread buffers and matrix inputs
static void threads_and_matrices(const std::string& dir)
{
    Workspace ws;
    Scalar a = ws.make_scalar(), b = ws.make_scalar();
    Scalar expr = a * a + b * b + sin(a) * cos(b);
    Compiled<double> f({expr}, "multi_thread", dir, expr.get_checksum());
    REQUIRE(f.get_n_threads() == 1);
    f.set_n_threads(4);
    REQUIRE(f.get_n_threads() == 4);
    const double A[4] = {1.0, 2.0, 3.0, 4.0}, B[4] = {0.5, 1.5, 2.5, 3.5};
    for (int t = 0; t < 4; ++t) {
        f.set(a, A[t], t);
        f.set(b, B[t], t);
    }
    for (int t = 0; t < 4; ++t) REQUIRE(approx(f.run(t)[0], A[t] * A[t] + B[t] * B[t] + std::sin(A[t]) * std::cos(B[t])));
    REQUIRE(approx(f.run()[0], 1.0 + 0.25 + std::sin(1.0) * std::cos(0.5)));
    bool threw = false;
    try {
        f.run(4);
    } catch (const std::out_of_range&) {
        threw = true;
    }
    REQUIRE(threw);

    Matrix m = Matrix::zero({2, 2}, ws.make_scalar());
    m(0, 0) = ws.make_scalar();
    m(0, 1) = ws.make_scalar();
    m(1, 0) = ws.make_scalar();
    m(1, 1) = ws.make_scalar();
    Compiled<double> g({m.det(), m.trace()}, "matrix_thread_test", dir, m.det().get_checksum());
    g.set_n_threads(2);
    const double m1[4] = {2.0, 1.0, 1.0, 3.0};
    struct RowMajor {
        double v[4];
        double operator()(int i, int j) const { return v[2 * i + j]; }
    } m2{{1.0, -1.0, 2.0, 0.0}};
    g.set(m, &m1[0], 0);
    g.set(m, m2, 1);
    const View<double> r1 = g.run(0);
    REQUIRE(approx(r1[0], 5.0) && approx(r1[1], 5.0));
    const View<double> r2 = g.run(1);
    REQUIRE(approx(r2[0], 2.0) && approx(r2[1], 1.0));
    std::vector<double> v = {0.25, 0.75};
    Vector vec({a, b});
    f.set(vec, v, 2);
    REQUIRE(approx(f.run(2)[0], 0.0625 + 0.5625 + std::sin(0.25) * std::cos(0.75)));
}

// Check mode (reference Compiled.cpp:126-190): NaN inputs and outputs throw.
static void check_mode(const std::string& dir)
{
    Workspace ws;
    Scalar a = ws.make_scalar();
    Scalar e = sqrt(a);
    Compiled<double> f({e}, "nan_check", dir, e.get_checksum());
    f.set(a, -1.0);
    REQUIRE(std::isnan(f.run()[0]));  // off by default
    check_mode_ON(true);
    REQUIRE(get_check_mode_ON());
    bool out_threw = false, in_threw = false;
    try {
        f.run();
    } catch (const std::runtime_error& ex) {
        out_threw = std::string(ex.what()).find("NaN detected in output #0") != std::string::npos;
    }
    f.set(a, std::nan(""));
    try {
        f.run();
    } catch (const std::runtime_error& ex) {
        in_threw = std::string(ex.what()).find("NaN detected in input #0") != std::string::npos;
    }
    check_mode_ON(false);
    REQUIRE(out_threw && in_threw);
    Compiled<double> invalid;
    bool invalid_threw = false;
    try {
        invalid.run();
    } catch (const std::runtime_error& ex) {
        invalid_threw = std::string(ex.what()).find("Cannot run invalid compilation") != std::string::npos;
    }
    REQUIRE(invalid_threw);
}

// Batches: run_all over many input sets and run_device over a symbol-major device batch.
static void batches(const std::string& dir)
{
    Workspace ws;
    Scalar x = ws.make_scalar(), y = ws.make_scalar(), z = ws.make_scalar();
    std::vector<Scalar> exprs = {x * y * z + exp(-x * x), branch(x > y, log(z), atan(x - y)), powF(z, 1.7) / (1.0 + y * y)};
    Compiled<double> f(exprs, "batch_test", dir, get_checksum(exprs));
    const int n = 1000;
    f.set_n_threads(n);
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> u(0.1, 2.0);
    std::vector<double> in(3 * n);
    for (auto& v : in) v = u(rng);
    for (int t = 0; t < n; ++t) {
        f.set(x, in[3 * t], t);
        f.set(y, in[3 * t + 1], t);
        f.set(z, in[3 * t + 2], t);
    }
    f.run_all();
    double worst = 0.0;
    for (int t = 0; t < n; ++t) {
        x.set_value(in[3 * t]);
        y.set_value(in[3 * t + 1]);
        z.set_value(in[3 * t + 2]);
        for (int k = 0; k < 3; ++k) worst = std::max(worst, std::abs(f.get_output_buffer(t)[k] - exprs[k].eval()));
    }
    REQUIRE(worst < 1e-12);

    // device batch, symbol-major: in[i * n + t], out[k * n + t]
    std::vector<double> soa(3 * n), out(3 * n, 0.0);
    for (int t = 0; t < n; ++t)
        for (int i = 0; i < 3; ++i) soa[i * n + t] = in[3 * t + i];
    double *d_in = nullptr, *d_out = nullptr;
    REQUIRE(cudaMalloc(&d_in, sizeof(double) * 3 * n) == cudaSuccess);
    REQUIRE(cudaMalloc(&d_out, sizeof(double) * 3 * n) == cudaSuccess);
    cudaMemcpy(d_in, soa.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice);
    f.run_device(d_in, d_out, n, 1, n, 1, n, nullptr);
    REQUIRE(cudaMemcpy(out.data(), d_out, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost) == cudaSuccess);
    cudaFree(d_in);
    cudaFree(d_out);
    double worst_dev = 0.0;
    for (int t = 0; t < n; ++t)
        for (int k = 0; k < 3; ++k) worst_dev = std::max(worst_dev, std::abs(out[k * n + t] - f.get_output_buffer(t)[k]));
    REQUIRE(worst_dev == 0.0);
}

// Neo-Hookean Tet4 [E, g, H] through Compiled<double> against the reference's own outputs
// (golden fixture elem_nh_tet4: 26 inputs and 157 outputs per element).
static void nh_tet4(const std::string& dir, const char* in_path, const char* ref_path)
{
    std::ifstream fi(in_path, std::ios::binary), fr(ref_path, std::ios::binary);
    int64_t n = 0;
    fi.read(reinterpret_cast<char*>(&n), sizeof(n));
    std::vector<double> rows(26 * n), ref(157 * n);
    fi.read(reinterpret_cast<char*>(rows.data()), sizeof(double) * rows.size());
    fr.read(reinterpret_cast<char*>(ref.data()), sizeof(double) * ref.size());
    REQUIRE(fi.good() && fr.good() && n > 0);
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
    Scalar logJ = log(F.det());
    Scalar E = (0.5 * mu * ((F.transpose() * F).trace() - 3.0) - mu * logJ + 0.5 * lam * logJ.powN(2)) * jac(X).det() *
               (1.0 / 6.0);
    std::vector<Scalar> vgh = value_gradient_hessian(E, collect_scalars(x));
    Compiled<double> f(vgh, "nh_tet4_egh", dir);
    REQUIRE(f.get_n_inputs() == 26 && f.get_n_outputs() == 157);
    f.set_n_threads((int)n);
    for (int64_t e = 0; e < n; ++e) {
        const double* r = &rows[26 * e];
        for (int v = 0; v < 4; ++v) {
            f.set(x[v], std::vector<double>(r + 3 * v, r + 3 * v + 3), (int)e);
            f.set(X[v], std::vector<double>(r + 12 + 3 * v, r + 12 + 3 * v + 3), (int)e);
        }
        f.set(mu, r[24], (int)e);
        f.set(lam, r[25], (int)e);
    }
    f.run_all();
    // per block (E, g, H): max error relative to the block's largest magnitude
    const int lo[3] = {0, 1, 13}, hi[3] = {1, 13, 157};
    for (int blk = 0; blk < 3; ++blk) {
        double err = 0.0, scale = 0.0;
        for (int64_t e = 0; e < n; ++e)
            for (int k = lo[blk]; k < hi[blk]; ++k) {
                err = std::max(err, std::abs(f.get_output_buffer((int)e)[k] - ref[157 * e + k]));
                scale = std::max(scale, std::abs(ref[157 * e + k]));
            }
        std::printf("nh_tet4 block %d: max error %.3g of scale %.3g\n", blk, err, scale);
        REQUIRE(err <= 1e-12 * scale);
    }
    // one element through run() agrees with the batch bit for bit
    Compiled<double> g;
    REQUIRE(g.load_if_cached("nh_tet4_egh", dir, get_checksum(vgh)));
    for (int i = 0; i < 26; ++i) g.get_input_buffer()[i] = f.get_input_buffer(3)[i];
    const View<double> one = g.run();
    bool same = true;
    for (int k = 0; k < 157; ++k) same = same && one[k] == f.get_output_buffer(3)[k];
    REQUIRE(same);
}

// Without a CUDA device: the kernel is still generated and compiled (NVRTC), its files are
// written, and loading fails with a clear error.
static void nogpu(const std::string& dir)
{
    Workspace ws;
    Scalar a = ws.make_scalar(), b = ws.make_scalar();
    Scalar e = a * b + sin(a);
    bool threw = false;
    try {
        Compiled<double> f({e}, "nogpu_test", dir, e.get_checksum());
    } catch (const std::runtime_error& ex) {
        threw = std::string(ex.what()).find("failed to load the compiled kernel of 'nogpu_test'") != std::string::npos;
        if (!threw) std::printf("unexpected error: %s\n", ex.what());
    }
    REQUIRE(threw);
    REQUIRE(file_exists(dir + "/nogpu_test.cu") && file_exists(dir + "/nogpu_test.cubin") &&
            file_exists(dir + "/nogpu_test.symxg"));
    REQUIRE(e.get_checksum() == get_checksum({e}));
    REQUIRE(e.get_checksum() != (a + b).get_checksum());
    bool empty_id_threw = false;
    try {
        Compiled<double> f;
        f.load_if_cached("nogpu_test", dir, "");
    } catch (const std::invalid_argument&) {
        empty_id_threw = true;
    }
    REQUIRE(empty_id_threw);
    Compiled<double> f;
    REQUIRE(!f.load_if_cached("absent", dir, "x"));
    REQUIRE(!f.is_valid() && !get_check_mode_ON() && is_load_compiled_enabled());
}

// Neo-Hookean Hex27 element through Compiled<double> on the GPU: E and dE/dx per quadrature
// point, summed over get_integration_rule(Hex27), against the reference's sums (n x 82).
static void nh_hex27(const std::string& dir, const char* in_path, const char* ref_path)
{
    std::ifstream fi(in_path, std::ios::binary), fr(ref_path, std::ios::binary);
    int64_t n = 0;
    fi.read(reinterpret_cast<char*>(&n), sizeof(n));
    std::vector<double> rows(164 * n), ref(82 * n);
    fi.read(reinterpret_cast<char*>(rows.data()), sizeof(double) * rows.size());
    fr.read(reinterpret_cast<char*>(ref.data()), sizeof(double) * ref.size());
    REQUIRE(fi.good() && fr.good() && n > 0);
    Workspace ws;
    std::vector<Vector> x = ws.make_vectors(3, 27), X = ws.make_vectors(3, 27);
    Vector xi = ws.make_vectors(3, 1)[0];
    Scalar mu = ws.make_scalar(), lam = ws.make_scalar();
    Matrix Jx = fem_jacobian(FEM_Element::Hex27, x, xi), JX = fem_jacobian(FEM_Element::Hex27, X, xi);
    Matrix F = Jx * JX.inv();
    Scalar logJ = log(F.det());
    Scalar psi = 0.5 * mu * ((F.transpose() * F).trace() - 3.0) - mu * logJ + 0.5 * lam * logJ.powN(2);
    Compiled<double> c(value_gradient(psi * JX.det(), collect_scalars(x)), "nh_hex27_vg", dir);
    const auto rule = get_integration_rule(FEM_Element::Hex27);
    double scale_e = 0.0, scale_g = 0.0, err_e = 0.0, err_g = 0.0;
    for (int64_t e = 0; e < n; ++e) {
        const double* r = &rows[164 * e];
        for (int v = 0; v < 27; ++v)
            for (int d = 0; d < 3; ++d) {
                c.set(x[v][d], r[3 * v + d]);
                c.set(X[v][d], r[81 + 3 * v + d]);
            }
        c.set(mu, r[162]);
        c.set(lam, r[163]);
        std::vector<double> sum(82, 0.0);
        for (const auto& q : rule) {
            for (int d = 0; d < 3; ++d) c.set(xi[d], q[1 + d]);
            const View<double> o = c.run();
            for (int k = 0; k < 82; ++k) sum[k] += q[0] * o[k];
        }
        scale_e = std::max(scale_e, std::abs(ref[82 * e]));
        err_e = std::max(err_e, std::abs(sum[0] - ref[82 * e]));
        for (int k = 1; k < 82; ++k) {
            scale_g = std::max(scale_g, std::abs(ref[82 * e + k]));
            err_g = std::max(err_g, std::abs(sum[k] - ref[82 * e + k]));
        }
    }
    std::printf("hex27: max |dE| %.3e of %.3e, max |dg| %.3e of %.3e\n", err_e, scale_e, err_g, scale_g);
    REQUIRE(err_e <= 1e-12 * scale_e && err_g <= 1e-12 * scale_g);
}

int main(int argc, char** argv)
{
    if (argc < 3) {
        std::printf("usage: test_compiled nogpu|gpu <folder> [nh_in.bin nh_ref.bin]\n");
        return 2;
    }
    const std::string mode = argv[1], dir = argv[2];
    try {
        if (mode == "nogpu") {
            nogpu(dir);
        } else if (mode == "gpu" && argc == 5) {
            chain(dir);
            multi_expression(dir);
            branches(dir);
            caching(dir);
            threads_and_matrices(dir);
            check_mode(dir);
            batches(dir);
            nh_tet4(dir, argv[3], argv[4]);
        } else if (mode == "hex27" && argc == 5) {
            nh_hex27(dir, argv[3], argv[4]);
        } else {
            std::printf("bad arguments\n");
            return 2;
        }
    } catch (const std::exception& ex) {
        std::printf("FAIL exception: %s\n", ex.what());
        return 1;
    }
    std::printf(fails ? "compiled FAIL (%d)\n" : "compiled PASS\n", fails);
    return fails ? 1 : 0;
}
