// Test infrastructure, not product code.
//
// Harness that drives the unmodified reference SymX (compiled from its own
// sources by oracle/Makefile.ref into oracle/_ref/) through its PUBLIC API only
// (`#include <symx>
#include <Eigen/Sparse>`), to produce golden vectors for the second-order solve
// path and to time the reference's own OpenMP path.  It never runs on the GPU
// machine (the reference sources are not there); its outputs are committed as
// small fixtures under tests/golden/.
//
// The problem it builds mirrors the reference's own idioms:
//   * Neo-Hookean density: examples/elasticity_potentials.h:7-13
//   * FEM quadrature (Tet4 1-point, Hex8 2x2x2): symx/src/solver/fem_integrators.cpp:52-133
//   * backward-Euler inertia with lumped mass: examples/dynamic_elasticity_with_contact.cpp:86-103
//   * penalty Dirichlet condition: examples/rubber_extrusion.cpp:94-107
//   * NewtonsMethod settings: symx/src/solver/solver_utils.h:272-358
//
// Usage:
//   symx_ref_harness elem    <in.bin> <out.bin>            per-element NH Tet4 [E, g(12), H(144)]
//   symx_ref_harness project <in.bin> <out.bin>            project_to_PD_inplace on n x n matrices
//   symx_ref_harness eval    <problem.bin> <outdir> <thr>  E, grad, element Hessians, BCSR triplets
//   symx_ref_harness solve   <problem.bin> <outdir> <thr> [max_newton] [cg_rel_tol] [projection mode]
//   symx_ref_harness mesh    d|f <type> <nx> <ny> <nz> <sx> <sy> <sz> <out.bin>   generate_cuboid_mesh
//   symx_ref_harness rcm     <in.bin> <out.bin> <reorder_elements 0|1>           reorder_connectivity_RCM
//   symx_ref_harness elem27  <in.bin> <out.bin>            NH Hex27 [E, g(81)] over get_integration_rule(Hex27)
//   symx_ref_harness mixed   <in.bin> <out.bin>            NH Tet4 [dg/dmu (12), dg/dlambda (12)] via gradient()
//   symx_ref_harness contact <problem.bin> <scene.bin> <outdir> <thr>
//                     the step problem plus a conditional ground contact and a second DoF set
//                     (handles): E and gradient at the initial state, NewtonsMethod::solve
#include <symx>
#include <Eigen/Sparse>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

using namespace symx;

namespace {

template <typename T>
void read_into(std::ifstream& f, std::vector<T>& v, size_t n)
{
    v.resize(n);
    if (n) f.read(reinterpret_cast<char*>(v.data()), sizeof(T) * n);
    if (!f) { std::cerr << "harness: short read\n"; std::exit(2); }
}

template <typename T>
void write_raw(const std::string& path, const T* data, size_t n)
{
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(data), sizeof(T) * n);
}

// Problem file written by tests/golden/make_golden.py (little-endian):
//   int64  n_verts, n_elems, n_bc, nodes_per_elem
//   f64    dt, gx, gy, gz, k_bc
//   f64    X[nv*3], x0[nv*3], v0[nv*3], x_init[nv*3], mass[nv]
//   int32  conn[ne*nodes]
//   f64    mu[ne], lambda[ne]
//   int32  bc_vertex[nbc];  f64 bc_target[nbc*3]
struct Problem {
    int64_t nv = 0, ne = 0, nbc = 0, nodes = 0;
    double dt = 0, k_bc = 0;
    std::array<double, 3> g{0, 0, 0};  // held here: data maps keep a pointer to it
    std::vector<Eigen::Vector3d> X, x0, v0, x;
    std::vector<double> mass, mu, lam;
    std::vector<int32_t> conn_flat;
    LabelledConnectivity<2> bc_conn{{"constraint_idx", "vertex_idx"}};
    std::vector<Eigen::Vector3d> bc_target;
    std::vector<std::array<int, 1>> all_vertices;  // one vertex per inertia element
};

std::vector<Eigen::Vector3d> to_vec3(const std::vector<double>& a)
{
    std::vector<Eigen::Vector3d> out(a.size() / 3);
    for (size_t i = 0; i < out.size(); ++i) out[i] = Eigen::Vector3d(a[3 * i], a[3 * i + 1], a[3 * i + 2]);
    return out;
}

Problem load_problem(const std::string& path)
{
    Problem p;
    std::ifstream f(path, std::ios::binary);
    if (!f) { std::cerr << "harness: cannot open " << path << "\n"; std::exit(2); }
    int64_t hdr[4];
    f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
    p.nv = hdr[0]; p.ne = hdr[1]; p.nbc = hdr[2]; p.nodes = hdr[3];
    double sc[5];
    f.read(reinterpret_cast<char*>(sc), sizeof(sc));
    p.dt = sc[0]; p.g[0] = sc[1]; p.g[1] = sc[2]; p.g[2] = sc[3]; p.k_bc = sc[4];
    std::vector<double> tmp;
    read_into(f, tmp, p.nv * 3); p.X = to_vec3(tmp);
    read_into(f, tmp, p.nv * 3); p.x0 = to_vec3(tmp);
    read_into(f, tmp, p.nv * 3); p.v0 = to_vec3(tmp);
    read_into(f, tmp, p.nv * 3); p.x = to_vec3(tmp);
    read_into(f, p.mass, p.nv);
    read_into(f, p.conn_flat, p.ne * p.nodes);
    read_into(f, p.mu, p.ne);
    read_into(f, p.lam, p.ne);
    std::vector<int32_t> bc_idx;
    read_into(f, bc_idx, p.nbc);
    read_into(f, tmp, p.nbc * 3); p.bc_target = to_vec3(tmp);
    for (int64_t i = 0; i < p.nbc; ++i) p.bc_conn.numbered_push_back({bc_idx[i]});
    p.all_vertices.resize(p.nv);
    for (int64_t i = 0; i < p.nv; ++i) p.all_vertices[i] = {(int)i};
    return p;
}

// Connectivity with the element index prepended (mesh_generation.cpp:24-35 `enumerate`).
std::vector<int> numbered_connectivity(const Problem& p)
{
    return symx::enumerate(std::vector<int>(p.conn_flat.begin(), p.conn_flat.end()), (int)p.nodes);
}

spGlobalPotential build_global_potential(Problem& p, std::vector<int>& numbered)
{
    const FEM_Element type = p.nodes == 4 ? FEM_Element::Tet4 : p.nodes == 10 ? FEM_Element::Tet10 : FEM_Element::Hex8;
    const int stride = (int)p.nodes + 1;
    spGlobalPotential G = GlobalPotential::create();

    G->add_potential("nh_" + get_name(type), numbered, stride,
        [&](MappedWorkspace<double>& mws, Element& elem)
        {
            std::vector<Vector> x = mws.make_vectors(p.x, elem.slice(1, stride));
            std::vector<Vector> X = mws.make_vectors(p.X, elem.slice(1, stride));
            Scalar mu = mws.make_scalar(p.mu, elem[0]);
            Scalar lam = mws.make_scalar(p.lam, elem[0]);
            Scalar P = fem_integrator(mws, type,
                [&](Scalar& w, Vector xi)
                {
                    Matrix Jx = fem_jacobian(type, x, xi);
                    Matrix JX = fem_jacobian(type, X, xi);
                    Matrix F = Jx * JX.inv();
                    Matrix C = F.transpose() * F;
                    Scalar Ic = C.trace();
                    Scalar logdetF = log(F.det());
                    Scalar psi = 0.5 * mu * (Ic - 3.0) - mu * logdetF + 0.5 * lam * logdetF.powN(2);
                    return psi * JX.det() * w;
                });
            return P;
        });

    G->add_potential("be_inertia", p.all_vertices,
        [&](MappedWorkspace<double>& mws, Element& elem)
        {
            Vector x1 = mws.make_vector(p.x, elem[0]);
            Vector x0 = mws.make_vector(p.x0, elem[0]);
            Vector v0 = mws.make_vector(p.v0, elem[0]);
            Scalar m = mws.make_scalar(p.mass, elem[0]);
            Vector g = mws.make_vector(p.g);
            Scalar dt = mws.make_scalar(p.dt);
            Vector xhat = x0 + dt * v0 + dt * dt * g;
            Vector dev = x1 - xhat;
            return 0.5 * m * dev.squared_norm() / dt.powN(2);
        });

    if (p.nbc > 0) {
        G->add_potential("boundary_conditions", p.bc_conn,
            [&](MappedWorkspace<double>& mws, Element& conn)
            {
                Vector x = mws.make_vector(p.x, conn["vertex_idx"]);
                Vector target = mws.make_vector(p.bc_target, conn["constraint_idx"]);
                Scalar k = mws.make_scalar(p.k_bc);
                return 0.5 * k * (x - target).squared_norm();
            });
    }
    G->add_dof(p.x);
    return G;
}

spContext make_context(int n_threads, const std::string& outdir)
{
    spContext ctx = Context::create();
    ctx->n_threads = n_threads;
    ctx->compilation_directory = symx::get_codegen_dir();
    ctx->output->set_console_verbosity(Verbosity::Medium);
    (void)outdir;
    return ctx;
}

int mode_elem(const std::string& in, const std::string& out)
{
    // in: int64 n; then n x 26 f64 rows [x0..x3 (12), X0..X3 (12), mu, lambda]
    std::ifstream f(in, std::ios::binary);
    int64_t n = 0;
    f.read(reinterpret_cast<char*>(&n), sizeof(n));
    std::vector<double> rows;
    read_into(f, rows, (size_t)n * 26);

    Workspace ws;
    std::vector<Vector> x = ws.make_vectors(3, 4);
    std::vector<Vector> X = ws.make_vectors(3, 4);
    Scalar mu = ws.make_scalar();
    Scalar lam = ws.make_scalar();
    auto jac = [&](const std::vector<Vector>& v) {
        Matrix J = ws.get_identity_matrix(3);
        J.set_col(0, v[1] - v[0]);
        J.set_col(1, v[2] - v[0]);
        J.set_col(2, v[3] - v[0]);
        return J;
    };
    Matrix Jx = jac(x);
    Matrix JX = jac(X);
    Matrix F = Jx * JX.inv();
    Matrix C = F.transpose() * F;
    Scalar logdetF = log(F.det());
    Scalar psi = 0.5 * mu * (C.trace() - 3.0) - mu * logdetF + 0.5 * lam * logdetF.powN(2);
    Scalar E = psi * JX.det() * (1.0 / 6.0);
    std::vector<Scalar> dofs = collect_scalars(x);
    std::vector<Scalar> vgh = value_gradient_hessian(E, dofs);
    Compiled<double> c(vgh, "ref_harness_nh_tet4_vgh", symx::get_codegen_dir());

    std::vector<double> result((size_t)n * 157);
    for (int64_t e = 0; e < n; ++e) {
        const double* r = rows.data() + 26 * e;
        for (int v = 0; v < 4; ++v) {
            for (int d = 0; d < 3; ++d) {
                c.set(x[v][d], r[3 * v + d]);
                c.set(X[v][d], r[12 + 3 * v + d]);
            }
        }
        c.set(mu, r[24]);
        c.set(lam, r[25]);
        View<double> o = c.run();
        for (int i = 0; i < 157; ++i) result[157 * e + i] = o[i];
    }
    write_raw(out, result.data(), result.size());
    return 0;
}

int mode_project(const std::string& in, const std::string& out)
{
    // in: int64 count, int64 n; count x n*n f64 row-major matrices; eps fixed at the
    // reference default 1e-10 without mirroring (solver_utils.h:323-324).
    std::ifstream f(in, std::ios::binary);
    int64_t hdr[2];
    f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
    std::vector<double> m;
    read_into(f, m, (size_t)(hdr[0] * hdr[1] * hdr[1]));
    std::vector<uint8_t> changed(hdr[0]);
    for (int64_t i = 0; i < hdr[0]; ++i) {
        changed[i] = project_to_PD_inplace(m.data() + i * hdr[1] * hdr[1], (int)hdr[1], 1e-10, false) ? 1 : 0;
    }
    write_raw(out, m.data(), m.size());
    write_raw(out + ".changed", changed.data(), changed.size());
    return 0;
}

int mode_eval(const std::string& pfile, const std::string& outdir, int n_threads)
{
    Problem p = load_problem(pfile);
    std::vector<int> numbered = numbered_connectivity(p);
    spGlobalPotential G = build_global_potential(p, numbered);
    spContext ctx = make_context(n_threads, outdir);
    SecondOrderCompiledGlobal compiled(G, ctx);

    const int ndofs = G->get_total_n_dofs();
    double E = 0.0;
    Eigen::VectorXd grad(ndofs);
    spElementHessians eh = compiled.evaluate_P__dP_du__local_d2P_du2(E, grad);
    write_raw(outdir + "/E.bin", &E, 1);
    write_raw(outdir + "/grad.bin", grad.data(), (size_t)ndofs);

    // Unprojected element Hessians in evaluation order (potentials in definition order,
    // elements in order within each potential when n_threads == 1).
    std::vector<double> hv;
    std::vector<int32_t> hrows, hsize;
    for (const auto& h : eh->hessians) {
        const int n = 3 * h.n_blocks_per_dim;
        hsize.push_back(n);
        hv.insert(hv.end(), h.values, h.values + n * n);
        hrows.insert(hrows.end(), h.block_rows, h.block_rows + h.n_blocks_per_dim);
    }
    write_raw(outdir + "/hess_elem.bin", hv.data(), hv.size());
    write_raw(outdir + "/hess_elem_rows.bin", hrows.data(), hrows.size());
    write_raw(outdir + "/hess_elem_size.bin", hsize.data(), hsize.size());

    eh->project_to_PD_inplace__all(1e-10, false);
    std::vector<double> pv;
    for (const auto& h : eh->hessians) {
        const int n = 3 * h.n_blocks_per_dim;
        pv.insert(pv.end(), h.values, h.values + n * n);
    }
    write_raw(outdir + "/hess_elem_projected.bin", pv.data(), pv.size());

    auto H = eh->assemble_global(n_threads, ndofs);
    std::vector<Eigen::Triplet<double>> trip;
    H->to_triplets(trip);
    std::vector<int32_t> ti; std::vector<double> tv;
    for (const auto& t : trip) { ti.push_back(t.row()); ti.push_back(t.col()); tv.push_back(t.value()); }
    write_raw(outdir + "/bcsr_triplet_idx.bin", ti.data(), ti.size());
    write_raw(outdir + "/bcsr_triplet_val.bin", tv.data(), tv.size());

    double E_only = 0.0;
    compiled.evaluate_P(E_only);
    write_raw(outdir + "/E_only.bin", &E_only, 1);
    return 0;
}

int mode_solve(const std::string& pfile, const std::string& outdir, int n_threads, int max_newton, double cg_rel_tol,
               int projection)
{
    Problem p = load_problem(pfile);
    std::vector<int> numbered = numbered_connectivity(p);
    spGlobalPotential G = build_global_potential(p, numbered);
    spContext ctx = make_context(n_threads, outdir);

    auto t_setup0 = std::chrono::steady_clock::now();
    NewtonsMethod newton(G, ctx);
    auto t_setup1 = std::chrono::steady_clock::now();
    newton.settings.projection_mode = projection == 0   ? ProjectionToPD::Newton
                                      : projection == 2 ? ProjectionToPD::ProjectOnDemand
                                      : projection == 3 ? ProjectionToPD::Progressive
                                                        : ProjectionToPD::ProjectedNewton;
    newton.settings.projection_eps = 1e-10;
    newton.settings.project_to_pd_use_mirroring = false;
    newton.settings.linear_solver = LinearSolver::BDPCG;
    newton.settings.cg_rel_tolerance = cg_rel_tol;
    newton.settings.line_search_armijo_beta = 1e-4;
    newton.settings.residual_tolerance_abs = 1e-6;
    if (max_newton > 0) {
        newton.settings.max_iterations = max_newton;
        newton.settings.max_iterations_as_success = true;
    }

    auto t0 = std::chrono::steady_clock::now();
    SolverReturn ret = newton.solve();
    auto t1 = std::chrono::steady_clock::now();
    const double wall = std::chrono::duration<double>(t1 - t0).count();

    std::vector<double> xf(3 * p.nv);
    for (int64_t i = 0; i < p.nv; ++i) for (int d = 0; d < 3; ++d) xf[3 * i + d] = p.x[i][d];
    write_raw(outdir + "/x_final.bin", xf.data(), xf.size());

    auto& L = *ctx->logger;
    std::ofstream js(outdir + "/stats.json");
    js.precision(17);
    js << "{\n  \"return\": " << (int)ret << ",\n  \"wall_s\": " << wall
       << ",\n  \"setup_s\": " << std::chrono::duration<double>(t_setup1 - t_setup0).count()
       << ",\n  \"n_threads\": " << n_threads
       << ",\n  \"newton_iterations\": " << newton.get_last_solve_stats().newton_iterations
       << ",\n  \"cg_iterations\": " << newton.get_last_solve_stats().cg_iterations
       << ",\n  \"ls_bt_iterations\": " << newton.get_last_solve_stats().ls_bt_iterations
       << ",\n  \"n_hessians\": " << newton.get_last_solve_stats().n_hessians
       << ",\n  \"n_projected_hessians\": " << newton.get_last_solve_stats().n_projected_hessians
       << ",\n  \"timers\": {";
    bool first = true;
    for (const auto& label : L.get_timer_labels()) {
        js << (first ? "" : ",") << "\n    \"" << label << "\": " << L.get_timer_total(label);
        first = false;
    }
    js << "\n  }\n}\n";
    return ret == SolverReturn::Successful ? 0 : 3;
}

// Mixed second derivatives of the NH Tet4 element energy, d(dE/dx)/dmu and d(dE/dx)/dlambda,
// through the reference's own symbolic differentiation (gradient(), symx/src/symbol/diff.h:32-35)
// and Compiled<double>.  in: as mode_elem; out: n x 24.
int mode_mixed(const std::string& in, const std::string& out)
{
    std::ifstream f(in, std::ios::binary);
    int64_t n = 0;
    f.read(reinterpret_cast<char*>(&n), sizeof(n));
    std::vector<double> rows;
    read_into(f, rows, (size_t)n * 26);
    Workspace ws;
    std::vector<Vector> x = ws.make_vectors(3, 4);
    std::vector<Vector> X = ws.make_vectors(3, 4);
    Scalar mu = ws.make_scalar();
    Scalar lam = ws.make_scalar();
    auto jac = [&](const std::vector<Vector>& v) {
        Matrix J = ws.get_identity_matrix(3);
        J.set_col(0, v[1] - v[0]);
        J.set_col(1, v[2] - v[0]);
        J.set_col(2, v[3] - v[0]);
        return J;
    };
    Matrix F = jac(x) * jac(X).inv();
    Scalar logdetF = log(F.det());
    Scalar psi = 0.5 * mu * ((F.transpose() * F).trace() - 3.0) - mu * logdetF + 0.5 * lam * logdetF.powN(2);
    Scalar E = psi * jac(X).det() * (1.0 / 6.0);
    Vector g = gradient(E, collect_scalars(x));
    std::vector<Scalar> outs;
    for (int i = 0; i < 12; ++i) outs.push_back(gradient(g[i], std::vector<Scalar>{mu})[0]);
    for (int i = 0; i < 12; ++i) outs.push_back(gradient(g[i], std::vector<Scalar>{lam})[0]);
    Compiled<double> c(outs, "ref_harness_nh_tet4_mixed", symx::get_codegen_dir());
    std::vector<double> result((size_t)n * 24);
    for (int64_t e = 0; e < n; ++e) {
        const double* r = rows.data() + 26 * e;
        for (int v = 0; v < 4; ++v)
            for (int d = 0; d < 3; ++d) {
                c.set(x[v][d], r[3 * v + d]);
                c.set(X[v][d], r[12 + 3 * v + d]);
            }
        c.set(mu, r[24]);
        c.set(lam, r[25]);
        View<double> o = c.run();
        for (int i = 0; i < 24; ++i) result[24 * e + i] = o[i];
    }
    write_raw(out, result.data(), result.size());
    return 0;
}

// The step problem of mode_solve plus
//   * a cubic ground-contact penalty k p^3 / 3 on every vertex, p = ground_y - y, active only
//     where p > 0 (the conditional-potential idiom of examples/dynamic_elasticity_with_contact.cpp:126-139);
//   * a second DoF set, "handles" h_j, each tied to mesh vertex v_j by a spring
//     k_s / 2 |x_v - h_j|^2 and pulled to a target t_j by k_p / 2 |h_j - t_j|^2.
// scene.bin: f64 ground_y, k_contact, k_spring, k_pull; int64 n_handles; int32 vertex[n];
// f64 handle[n*3], target[n*3].  Writes E.bin and grad.bin (x DoFs, then handle DoFs) at the
// initial state, x_final.bin, h_final.bin and stats.json of NewtonsMethod::solve.
int mode_contact(const std::string& pfile, const std::string& sfile, const std::string& outdir, int n_threads)
{
    Problem p = load_problem(pfile);
    std::ifstream f(sfile, std::ios::binary);
    double sc[4];
    f.read(reinterpret_cast<char*>(sc), sizeof(sc));
    int64_t nh = 0;
    f.read(reinterpret_cast<char*>(&nh), sizeof(nh));
    std::vector<int32_t> hv;
    std::vector<double> tmp;
    read_into(f, hv, (size_t)nh);
    read_into(f, tmp, (size_t)nh * 3);
    std::vector<Eigen::Vector3d> handles = to_vec3(tmp);
    read_into(f, tmp, (size_t)nh * 3);
    std::vector<Eigen::Vector3d> targets = to_vec3(tmp);
    double ground_y = sc[0], k_contact = sc[1], k_spring = sc[2], k_pull = sc[3];
    LabelledConnectivity<2> hconn{{"handle", "vertex"}};
    for (int64_t j = 0; j < nh; ++j) hconn.numbered_push_back({hv[j]});

    std::vector<int> numbered = numbered_connectivity(p);
    spGlobalPotential G = build_global_potential(p, numbered);
    G->add_potential("ground_contact", p.all_vertices,
        [&](MappedWorkspace<double>& mws, Element& elem)
        {
            Vector x = mws.make_vector(p.x, elem[0]);
            Scalar k = mws.make_scalar(k_contact);
            Scalar yg = mws.make_scalar(ground_y);
            Scalar pen = yg - x[1];
            Scalar P = k * pen.powN(3) / 3.0;
            Scalar cond = pen > 0.0;
            return std::make_pair(P, cond);
        });
    G->add_potential("handle_spring", hconn,
        [&](MappedWorkspace<double>& mws, Element& conn)
        {
            Vector x = mws.make_vector(p.x, conn["vertex"]);
            Vector h = mws.make_vector(handles, conn["handle"]);
            Scalar k = mws.make_scalar(k_spring);
            return 0.5 * k * (x - h).squared_norm();
        });
    G->add_potential("handle_pull", hconn,
        [&](MappedWorkspace<double>& mws, Element& conn)
        {
            Vector h = mws.make_vector(handles, conn["handle"]);
            Vector t = mws.make_vector(targets, conn["handle"]);
            Scalar k = mws.make_scalar(k_pull);
            return 0.5 * k * (h - t).squared_norm();
        });
    G->add_dof(handles);
    spContext ctx = make_context(n_threads, outdir);
    {
        SecondOrderCompiledGlobal compiled(G, ctx);
        const int ndofs = G->get_total_n_dofs();
        double E = 0.0;
        Eigen::VectorXd grad(ndofs);
        compiled.evaluate_P__dP_du__local_d2P_du2(E, grad);
        write_raw(outdir + "/E.bin", &E, 1);
        write_raw(outdir + "/grad.bin", grad.data(), (size_t)ndofs);
    }
    NewtonsMethod newton(G, ctx);
    newton.settings.projection_mode = ProjectionToPD::ProjectedNewton;
    newton.settings.projection_eps = 1e-10;
    newton.settings.project_to_pd_use_mirroring = false;
    newton.settings.linear_solver = LinearSolver::BDPCG;
    newton.settings.cg_rel_tolerance = 1e-3;
    newton.settings.line_search_armijo_beta = 1e-4;
    newton.settings.residual_tolerance_abs = 1e-6;
    SolverReturn ret = newton.solve();
    std::vector<double> xf(3 * p.nv), hf(3 * nh);
    for (int64_t i = 0; i < p.nv; ++i) for (int d = 0; d < 3; ++d) xf[3 * i + d] = p.x[i][d];
    for (int64_t i = 0; i < nh; ++i) for (int d = 0; d < 3; ++d) hf[3 * i + d] = handles[i][d];
    write_raw(outdir + "/x_final.bin", xf.data(), xf.size());
    write_raw(outdir + "/h_final.bin", hf.data(), hf.size());
    std::ofstream js(outdir + "/stats.json");
    js << "{\n  \"return\": " << (int)ret
       << ",\n  \"newton_iterations\": " << newton.get_last_solve_stats().newton_iterations
       << ",\n  \"cg_iterations\": " << newton.get_last_solve_stats().cg_iterations
       << ",\n  \"ls_bt_iterations\": " << newton.get_last_solve_stats().ls_bt_iterations << "\n}\n";
    return ret == SolverReturn::Successful ? 0 : 3;
}

}  // namespace

// generate_cuboid_mesh (mesh_generation.cpp:306-327) written as int64 {n_vertices, n_elements,
// stride}, the vertices (FLOAT) and the connectivity (int32).
template <typename FLOAT>
int write_mesh(int type, const std::array<int32_t, 3>& n, const Eigen::Matrix<FLOAT, 3, 1>& size, const char* path)
{
    const FEMMesh<FLOAT> m = generate_cuboid_mesh<FLOAT>(static_cast<FEM_Element>(type), size, n);
    std::ofstream f(path, std::ios::binary);
    const int64_t hdr[3] = {(int64_t)m.vertices.size(), (int64_t)m.n_elements, (int64_t)m.connectivity_stride};
    f.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
    for (const auto& v : m.vertices) f.write(reinterpret_cast<const char*>(v.data()), 3 * sizeof(FLOAT));
    f.write(reinterpret_cast<const char*>(m.connectivity.data()), sizeof(int) * m.connectivity.size());
    return f ? 0 : 1;
}

int mode_mesh(char** a)
{
    const int type = std::atoi(a[1]);
    const std::array<int32_t, 3> n = {std::atoi(a[2]), std::atoi(a[3]), std::atoi(a[4])};
    if (std::string(a[0]) == "f")
        return write_mesh<float>(type, n, Eigen::Vector3f((float)std::atof(a[5]), (float)std::atof(a[6]), (float)std::atof(a[7])), a[8]);
    return write_mesh<double>(type, n, Eigen::Vector3d(std::atof(a[5]), std::atof(a[6]), std::atof(a[7])), a[8]);
}

// Neo-Hookean Hex27 element: E and dE/dx summed over get_integration_rule(Hex27)
// (fem_integrators.cpp:83-113) with fem_jacobian's triquadratic shape functions
// (fem_integrators.h:101-147).  in: int64 n, then n x 164 f64 rows [x (81), X (81), mu, lambda];
// out: n x 82 [E, g(81)].
int mode_elem27(const std::string& in, const std::string& out)
{
    std::ifstream f(in, std::ios::binary);
    int64_t n = 0;
    f.read(reinterpret_cast<char*>(&n), sizeof(n));
    std::vector<double> rows;
    read_into(f, rows, (size_t)n * 164);
    Workspace ws;
    std::vector<Vector> x = ws.make_vectors(3, 27), X = ws.make_vectors(3, 27);
    Vector xi = ws.make_vectors(3, 1)[0];
    Scalar mu = ws.make_scalar(), lam = ws.make_scalar();
    Matrix Jx = fem_jacobian(FEM_Element::Hex27, x, xi);
    Matrix JX = fem_jacobian(FEM_Element::Hex27, X, xi);
    Matrix F = Jx * JX.inv();
    Scalar logdetF = log(F.det());
    Scalar psi = 0.5 * mu * ((F.transpose() * F).trace() - 3.0) - mu * logdetF + 0.5 * lam * logdetF.powN(2);
    Compiled<double> c(value_gradient(psi * JX.det(), collect_scalars(x)), "ref_harness_nh_hex27_vg",
                       symx::get_codegen_dir());
    const std::vector<std::array<double, 4>> rule = get_integration_rule(FEM_Element::Hex27);
    std::vector<double> result((size_t)n * 82, 0.0);
    for (int64_t e = 0; e < n; ++e) {
        const double* r = rows.data() + 164 * e;
        for (int v = 0; v < 27; ++v)
            for (int d = 0; d < 3; ++d) {
                c.set(x[v][d], r[3 * v + d]);
                c.set(X[v][d], r[81 + 3 * v + d]);
            }
        c.set(mu, r[162]);
        c.set(lam, r[163]);
        for (const auto& q : rule) {
            for (int d = 0; d < 3; ++d) c.set(xi[d], q[1 + d]);
            View<double> o = c.run();
            for (int i = 0; i < 82; ++i) result[82 * e + i] += q[0] * o[i];
        }
    }
    write_raw(out, result.data(), result.size());
    return 0;
}

// reorder_connectivity_RCM (mesh_ordering.cpp:231-252) on an arbitrary connectivity.
// in: int64 {stride, n_elements, num_nodes}, int32 conn; out: int32 old_to_new, int32 conn.
int mode_rcm(const char* in, const char* out, bool reorder_elements)
{
    std::ifstream f(in, std::ios::binary);
    int64_t hdr[3];
    f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
    std::vector<int> conn;
    read_into(f, conn, (size_t)(hdr[0] * hdr[1]));
    const ReorderResult r = reorder_connectivity_RCM(conn.data(), (int)hdr[0], (int)hdr[1], (int)hdr[2], reorder_elements);
    std::ofstream o(out, std::ios::binary);
    o.write(reinterpret_cast<const char*>(r.old_to_new.data()), sizeof(int) * r.old_to_new.size());
    o.write(reinterpret_cast<const char*>(conn.data()), sizeof(int) * conn.size());
    return o ? 0 : 1;
}

int main(int argc, char** argv)
{
    if (argc >= 11 && std::string(argv[1]) == "mesh") return mode_mesh(argv + 2);
    if (argc >= 5 && std::string(argv[1]) == "rcm") return mode_rcm(argv[2], argv[3], std::atoi(argv[4]) != 0);
    if (argc < 4) {
        std::cerr << "usage: symx_ref_harness elem|project|eval|solve <in> <out> [threads] [max_newton] [cg_rel_tol]\n";
        return 1;
    }
    symx::suppress_compiler_output(true);
    const std::string mode = argv[1];
    const int n_threads = argc > 4 ? std::atoi(argv[4]) : 1;
    if (mode == "elem") return mode_elem(argv[2], argv[3]);
    if (mode == "elem27") return mode_elem27(argv[2], argv[3]);
    if (mode == "mixed") return mode_mixed(argv[2], argv[3]);
    if (mode == "contact" && argc >= 5)
        return mode_contact(argv[2], argv[3], argv[4], argc > 5 ? std::atoi(argv[5]) : 1);
    if (mode == "project") return mode_project(argv[2], argv[3]);
    if (mode == "eval") return mode_eval(argv[2], argv[3], n_threads);
    if (mode == "solve") {
        const int max_newton = argc > 5 ? std::atoi(argv[5]) : -1;
        const double cg_rel = argc > 6 ? std::atof(argv[6]) : 1e-3;
        const int projection = argc > 7 ? std::atoi(argv[7]) : 1;  // 0 Newton, 1 projected, 2 on demand, 3 progressive
        return mode_solve(argv[2], argv[3], n_threads, max_newton, cg_rel, projection);
    }
    std::cerr << "unknown mode " << mode << "\n";
    return 1;
}
