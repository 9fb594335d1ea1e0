// The C++ drop-in API on the GPU with user-written potentials, as a user of the reference
// writes them (GlobalPotential::add_potential with MappedWorkspace lambdas, add_dof,
// NewtonsMethod::solve).  The problems are those of the reference harness (oracle/ref_harness.cpp),
// whose outputs are the golden fixtures the Python tests compare against.  Usage:
//   test_gpu_api contact <problem.bin> <scene.bin> <outdir> <precision 0|1>
//       the step problem (Neo-Hookean Tet4, backward-Euler inertia, penalty boundary) plus a
//       conditional ground contact on every vertex and a second DoF set of handles tied to
//       the mesh by springs (examples/dynamic_elasticity_with_contact.cpp:126-139 for the
//       conditional idiom); writes E.bin and grad.bin at the initial state, x_final.bin,
//       h_final.bin and stats.txt of NewtonsMethod::solve
//   test_gpu_api mixed <problem.bin> <lambda.bin> <out.bin>
//       the step problem at its initial state: NewtonsMethod::parameter_gradient of mu and of
//       lambda for the adjoint vector in lambda.bin (n_dofs doubles); writes both (2 * n_elements)
#include <symx>

#include <array>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

using namespace symx;
using Vec3 = std::array<double, 3>;

namespace {

template <typename T>
void read_into(std::ifstream& f, std::vector<T>& v, size_t n)
{
    v.resize(n);
    if (n) f.read(reinterpret_cast<char*>(v.data()), sizeof(T) * n);
    if (!f) {
        std::cerr << "test_gpu_api: short read\n";
        std::exit(2);
    }
}

template <typename T>
void write_raw(const std::string& path, const T* data, size_t n)
{
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(data), sizeof(T) * n);
}

std::vector<Vec3> to_vec3(const std::vector<double>& a)
{
    std::vector<Vec3> out(a.size() / 3);
    for (size_t i = 0; i < out.size(); ++i) out[i] = {a[3 * i], a[3 * i + 1], a[3 * i + 2]};
    return out;
}

// The problem file of tests/golden/problem_io.py (the reference harness reads the same).
struct Problem {
    int64_t nv = 0, ne = 0, nbc = 0, nodes = 0;
    double dt = 0, k_bc = 0;
    Vec3 g{0, 0, 0};
    std::vector<Vec3> X, x0, v0, x, bc_target;
    std::vector<double> mass, mu, lam;
    std::vector<int> conn_numbered;
    LabelledConnectivity<2> bc_conn{{"constraint_idx", "vertex_idx"}};
    std::vector<std::array<int, 1>> vertices;
};

void load_problem(const std::string& path, Problem& p)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        std::cerr << "test_gpu_api: cannot open " << path << "\n";
        std::exit(2);
    }
    int64_t hdr[4];
    f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
    p.nv = hdr[0];
    p.ne = hdr[1];
    p.nbc = hdr[2];
    p.nodes = hdr[3];
    double sc[5];
    f.read(reinterpret_cast<char*>(sc), sizeof(sc));
    p.dt = sc[0];
    p.g = {sc[1], sc[2], sc[3]};
    p.k_bc = sc[4];
    std::vector<double> tmp;
    read_into(f, tmp, p.nv * 3);
    p.X = to_vec3(tmp);
    read_into(f, tmp, p.nv * 3);
    p.x0 = to_vec3(tmp);
    read_into(f, tmp, p.nv * 3);
    p.v0 = to_vec3(tmp);
    read_into(f, tmp, p.nv * 3);
    p.x = to_vec3(tmp);
    read_into(f, p.mass, p.nv);
    std::vector<int32_t> conn;
    read_into(f, conn, p.ne * p.nodes);
    read_into(f, p.mu, p.ne);
    read_into(f, p.lam, p.ne);
    std::vector<int32_t> bc_idx;
    read_into(f, bc_idx, p.nbc);
    read_into(f, tmp, p.nbc * 3);
    p.bc_target = to_vec3(tmp);
    for (int64_t i = 0; i < p.nbc; ++i) p.bc_conn.numbered_push_back({bc_idx[i]});
    for (int64_t e = 0; e < p.ne; ++e) {
        p.conn_numbered.push_back((int)e);
        for (int64_t a = 0; a < p.nodes; ++a) p.conn_numbered.push_back(conn[e * p.nodes + a]);
    }
    p.vertices.resize(p.nv);
    for (int64_t i = 0; i < p.nv; ++i) p.vertices[i] = {(int)i};
}

// Neo-Hookean Tet4 + backward-Euler inertia + penalty boundary: the reference harness's
// build_global_potential written against this library's headers.
spGlobalPotential step_potential(Problem& p)
{
    const int stride = (int)p.nodes + 1;
    spGlobalPotential G = GlobalPotential::create();
    G->add_potential("nh_tet4", p.conn_numbered, stride, [&p, stride](MappedWorkspace<double>& mws, Element& elem) {
        std::vector<Vector> x = mws.make_vectors(p.x, elem.slice(1, stride));
        std::vector<Vector> X = mws.make_vectors(p.X, elem.slice(1, stride));
        Scalar mu = mws.make_scalar(p.mu, elem[0]);
        Scalar lam = mws.make_scalar(p.lam, elem[0]);
        return fem_integrator(mws, FEM_Element::Tet4, [&](Scalar& w, Vector& xi) {
            Matrix F = fem_jacobian(FEM_Element::Tet4, x, xi) * fem_jacobian(FEM_Element::Tet4, X, xi).inv();
            Matrix JX = fem_jacobian(FEM_Element::Tet4, X, xi);
            Scalar logdetF = log(F.det());
            Scalar psi = 0.5 * mu * ((F.transpose() * F).trace() - 3.0) - mu * logdetF + 0.5 * lam * logdetF.powN(2);
            return psi * JX.det() * w;
        });
    });
    G->add_potential("be_inertia", p.vertices, [&p](MappedWorkspace<double>& mws, Element& elem) {
        Vector x1 = mws.make_vector(p.x, elem[0]);
        Vector x0 = mws.make_vector(p.x0, elem[0]);
        Vector v0 = mws.make_vector(p.v0, elem[0]);
        Scalar m = mws.make_scalar(p.mass, elem[0]);
        Vector g = mws.make_vector(p.g);
        Scalar dt = mws.make_scalar(p.dt);
        Vector dev = x1 - (x0 + dt * v0 + dt * dt * g);
        return 0.5 * m * dev.squared_norm() / dt.powN(2);
    });
    if (p.nbc > 0) {
        G->add_potential("boundary_conditions", p.bc_conn, [&p](MappedWorkspace<double>& mws, Element& conn) {
            Vector x = mws.make_vector(p.x, conn["vertex_idx"]);
            Vector target = mws.make_vector(p.bc_target, conn["constraint_idx"]);
            Scalar k = mws.make_scalar(p.k_bc);
            return 0.5 * k * (x - target).squared_norm();
        });
    }
    G->add_dof(p.x);
    return G;
}

void settings(NewtonsMethod& n, int precision)
{
    n.settings.projection_mode = ProjectionToPD::ProjectedNewton;
    n.settings.projection_eps = 1e-10;
    n.settings.project_to_pd_use_mirroring = false;
    n.settings.linear_solver = LinearSolver::BDPCG;
    n.settings.cg_rel_tolerance = 1e-3;
    n.settings.line_search_armijo_beta = 1e-4;
    n.settings.residual_tolerance_abs = 1e-6;
    n.settings.precision = precision ? Precision::Mixed : Precision::FP64;
}

int mode_contact(const std::string& pfile, const std::string& sfile, const std::string& outdir, int precision)
{
    Problem p;
    load_problem(pfile, p);
    std::ifstream f(sfile, std::ios::binary);
    double sc[4];
    f.read(reinterpret_cast<char*>(sc), sizeof(sc));
    int64_t nh = 0;
    f.read(reinterpret_cast<char*>(&nh), sizeof(nh));
    std::vector<int32_t> hv;
    std::vector<double> tmp;
    read_into(f, hv, (size_t)nh);
    read_into(f, tmp, (size_t)nh * 3);
    std::vector<Vec3> handles = to_vec3(tmp);
    read_into(f, tmp, (size_t)nh * 3);
    std::vector<Vec3> targets = to_vec3(tmp);
    const double ground_y = sc[0], k_contact = sc[1], k_spring = sc[2], k_pull = sc[3];
    LabelledConnectivity<2> hconn{{"handle", "vertex"}};
    for (int64_t j = 0; j < nh; ++j) hconn.numbered_push_back({hv[j]});

    spGlobalPotential G = step_potential(p);
    // conditional potential: a vertex contributes only while it is below the ground plane
    G->add_potential("ground_contact", p.vertices, [&](MappedWorkspace<double>& mws, Element& elem) {
        Vector x = mws.make_vector(p.x, elem[0]);
        Scalar k = mws.make_scalar(k_contact);
        Scalar yg = mws.make_scalar(ground_y);
        Scalar pen = yg - x[1];
        Scalar P = k * pen.powN(3) / 3.0;
        Scalar cond = pen > 0.0;
        return std::make_pair(P, cond);
    });
    // a second DoF set, coupled to the first in one potential
    G->add_potential("handle_spring", hconn, [&](MappedWorkspace<double>& mws, Element& conn) {
        Vector x = mws.make_vector(p.x, conn["vertex"]);
        Vector h = mws.make_vector(handles, conn["handle"]);
        Scalar k = mws.make_scalar(k_spring);
        return 0.5 * k * (x - h).squared_norm();
    });
    G->add_potential("handle_pull", hconn, [&](MappedWorkspace<double>& mws, Element& conn) {
        Vector h = mws.make_vector(handles, conn["handle"]);
        Vector t = mws.make_vector(targets, conn["handle"]);
        Scalar k = mws.make_scalar(k_pull);
        return 0.5 * k * (h - t).squared_norm();
    });
    G->add_dof(handles);

    spContext ctx = Context::create();
    NewtonsMethod newton(G, ctx);
    settings(newton, precision);
    const int ndofs = G->get_total_n_dofs();
    std::vector<double> grad((size_t)ndofs);
    newton.upload();
    const double E = newton.evaluate(grad.data());
    write_raw(outdir + "/E.bin", &E, 1);
    write_raw(outdir + "/grad.bin", grad.data(), grad.size());
    const SolverReturn ret = newton.solve();
    std::vector<double> xf, hf;
    for (const Vec3& v : p.x) xf.insert(xf.end(), v.begin(), v.end());
    for (const Vec3& v : handles) hf.insert(hf.end(), v.begin(), v.end());
    write_raw(outdir + "/x_final.bin", xf.data(), xf.size());
    write_raw(outdir + "/h_final.bin", hf.data(), hf.size());
    const SolveStats& st = newton.get_last_solve_stats();
    std::ofstream(outdir + "/stats.txt") << (int)ret << " " << st.newton_iterations << " " << st.cg_iterations << " "
                                        << st.final_residual << "\n";
    return 0;
}

int mode_mixed(const std::string& pfile, const std::string& lfile, const std::string& out)
{
    Problem p;
    load_problem(pfile, p);
    spGlobalPotential G = step_potential(p);
    spContext ctx = Context::create();
    NewtonsMethod newton(G, ctx);
    settings(newton, 0);
    std::ifstream f(lfile, std::ios::binary);
    std::vector<double> lambda;
    read_into(f, lambda, (size_t)G->get_total_n_dofs());
    newton.upload();
    std::vector<double> d_mu = newton.parameter_gradient(p.mu, lambda);
    std::vector<double> d_lam = newton.parameter_gradient(p.lam, lambda);
    d_mu.insert(d_mu.end(), d_lam.begin(), d_lam.end());
    write_raw(out, d_mu.data(), d_mu.size());
    return 0;
}

}  // namespace

int main(int argc, char** argv)
{
    try {
        const std::string mode = argc > 1 ? argv[1] : "";
        if (mode == "contact" && argc >= 6) return mode_contact(argv[2], argv[3], argv[4], std::atoi(argv[5]));
        if (mode == "mixed" && argc >= 5) return mode_mixed(argv[2], argv[3], argv[4]);
    } catch (const std::exception& e) {
        std::cerr << "test_gpu_api: " << e.what() << "\n";
        return 3;
    }
    std::cerr << "usage: test_gpu_api contact <problem> <scene> <outdir> <precision> | mixed <problem> <lambda> <out>\n";
    return 1;
}
