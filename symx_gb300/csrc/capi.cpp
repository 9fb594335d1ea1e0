// C ABI of symx_gb300 (declared in include/symx_gb300.h).
//
// The elastic-step problem is defined here with the same C++ user API a SymX user writes
// (GlobalPotential::add_potential with MappedWorkspace lambdas, fem_integrator,
// NewtonsMethod), so the C entry points exercise exactly the drop-in path.
#include "../../include/symx_gb300.h"

#include <array>
#include <chrono>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "bcsr_pcg.h"
#include "fem.h"
#include "global_potential.h"
#include "kernels.cuh"
#include "mesh.h"
#include "newton.h"

namespace {

thread_local std::string g_last_error;

template <typename F>
int guarded(F&& f)
{
    try {
        g_last_error.clear();
        return f();
    } catch (const std::invalid_argument& e) {
        g_last_error = e.what();
        return SYMXG_ERR_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return SYMXG_ERR_RUNTIME;
    } catch (...) {
        g_last_error = "unknown error";
        return SYMXG_ERR_RUNTIME;
    }
}

using Vec3 = std::array<double, 3>;

}  // namespace

struct symxg_solver {
    // host data the potentials are bound to (the maps keep pointers to these members)
    std::vector<Vec3> x, x0, v0, X, bc_target;
    std::vector<double> mu, lam, mass;
    std::vector<int32_t> conn_numbered;  // element index + nodes
    std::vector<std::array<int32_t, 1>> vertices;
    symx::LabelledConnectivity<2> bc_conn{{"constraint_idx", "vertex_idx"}};
    double dt = 0.0, k_bc = 0.0;
    Vec3 gravity{0, 0, 0};
    int nodes = 0;
    bool has_inertia = false;
    symx::spGlobalPotential G;
    std::unique_ptr<symx::NewtonsMethod> newton;
    // rollout: (x0, v0) before every checkpoint_every-th step of the last forward rollout
    std::vector<std::vector<Vec3>> ckpt_x0, ckpt_v0;
    int rollout_steps = 0, checkpoint_every = 0;
    // The bound host arrays are page-locked once their size is final (they are only written
    // in place afterwards), so every upload and download copies at full host-device link
    // speed.  A refused registration is skipped (the copies then go through pageable memory).
    std::vector<void*> pinned;
    template <typename V>
    void pin(V& v)
    {
        if (v.empty()) return;
        if (cudaHostRegister(v.data(), sizeof(v[0]) * v.size(), cudaHostRegisterDefault) == cudaSuccess)
            pinned.push_back(v.data());
        else
            cudaGetLastError();
    }
    ~symxg_solver()
    {
        newton.reset();
        for (void* p : pinned) cudaHostUnregister(p);
    }
};

template <typename T>
static int project_impl(T* m, int32_t n, int64_t count, T eps, int32_t mirroring, int32_t* nc, void* stream)
{
    return guarded([&] {
        if (n <= 0 || n % 3 != 0 || n > 30) throw std::invalid_argument("n must be a multiple of 3 up to 30");
        if (count < 0) throw std::invalid_argument("negative count");
        if (count == 0) return SYMXG_OK;
        if (!m || !nc) throw std::invalid_argument("null device pointer");
        symxg::launch_project_pd<T>(m, n, count, eps, mirroring != 0, nc, (cudaStream_t)stream);
        return SYMXG_OK;
    });
}

template <typename T>
static int spmv_impl(int32_t nb, const int32_t* rp, const int32_t* cols, const T* vals, int64_t vs, const T* x, T* y,
                     void* stream)
{
    return guarded([&] {
        if (nb < 0 || vs < 0) throw std::invalid_argument("negative size");
        if (nb > 0 && (!rp || !cols || !vals || !x || !y)) throw std::invalid_argument("null device pointer");
        if (nb > 0) symxg::launch_bcsr_spmv<T>(nb, rp, cols, vals, vs, x, y, (cudaStream_t)stream);
        return SYMXG_OK;
    });
}

template <typename T>
static int pcg_impl(int32_t nb, const int32_t* rp, const int32_t* cols, const T* vals, int64_t vs, const T* b, T* x,
                    double abs_tol, double rel_tol, int32_t max_it, symxg_pcg_info* info, void* stream)
{
    return guarded([&] {
        if (!info) throw std::invalid_argument("null info");
        std::memset(info, 0, sizeof(*info));
        if (nb < 0 || vs < 0 || max_it < 0) throw std::invalid_argument("negative size");
        if (nb > 0 && (!rp || !cols || !vals || !b || !x)) throw std::invalid_argument("null device pointer");
        const unsigned parts = symxg::pcg_max_grid();
        const size_t bytes = symxg::bcsr_pcg_workspace_bytes<T>(nb, parts);
        void* ws = nullptr;
        if (nb > 0) {
            const cudaError_t e = cudaMalloc(&ws, bytes);
            if (e != cudaSuccess) throw std::runtime_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
            symxg::note_device_alloc((int64_t)bytes);
        }
        struct Free {
            void* p;
            size_t bytes;
            ~Free()
            {
                if (p) {
                    cudaFree(p);
                    symxg::note_device_free((int64_t)bytes);
                }
            }
        } guard{ws, bytes};
        const symxg::BcsrPcgResult r = symxg::run_bcsr_pcg<T>(nb, rp, cols, vals, vs, b, x, abs_tol, rel_tol, max_it, ws,
                                                               bytes, parts, (cudaStream_t)stream);
        info->converged = r.converged;
        info->n_iterations = r.iterations;
        info->error = r.error;
        info->found_indefiniteness = r.indefinite;
        info->missing_diagonal = r.missing_diagonal;
        if (r.missing_diagonal) throw std::invalid_argument("block rows without a diagonal block");
        return SYMXG_OK;
    });
}

static void fill_stats(const symx::SolveStats& st, symx::SolverReturn r, symxg_solve_stats* o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->solver_return = (int32_t)r;
    o->newton_iterations = st.newton_iterations;
    o->cg_iterations = st.cg_iterations;
    o->ls_bt_iterations = st.ls_bt_iterations;
    o->final_residual = st.final_residual;
    o->final_energy = st.final_energy;
    o->projection_not_converged = st.projection_not_converged;
    auto get = [&](const char* k) {
        auto it = st.timers.find(k);
        return it == st.timers.end() ? 0.0 : it->second;
    };
    o->t_evaluate_P_grad_hess = get("evaluate_P_grad_hess");
    o->t_project_to_PD = get("project_to_PD");
    o->t_assembly = get("assembly");
    o->t_linear_system_solve = get("linear_system_solve");
    o->t_evaluate_P = get("evaluate_P");
    o->h2d_bytes = st.h2d_bytes;
    for (size_t i = 0; i < st.cg_iterations_per_newton.size() && i < 16; ++i)
        o->cg_iterations_per_newton[i] = st.cg_iterations_per_newton[i];
    o->d2h_bytes = st.d2h_bytes;
    o->n_hessians = (int64_t)st.n_hessians;
    o->n_projected_hessians = (int64_t)st.n_projected_hessians;
    o->cg_residual_replacements = st.cg_residual_replacements;
    for (const auto& kv : st.kernels) {
        if (kv.first.rfind("pcg_spmv", 0) == 0) {
            o->spmv_launches += kv.second.first;
            o->spmv_seconds += kv.second.second;
        } else if (kv.first.rfind("project_pd_12_", 0) == 0) {  // the 12 x 12 (Tet4) launches only
            o->project_launches += kv.second.first;
            o->project_seconds += kv.second.second;
        } else if (kv.first.rfind("pcg_solve", 0) == 0) {
            o->pcg_solve_iterations += kv.second.first;
            o->pcg_solve_seconds += kv.second.second;
        }
    }
}

namespace {

std::vector<double> flat(const std::vector<Vec3>& v)
{
    std::vector<double> out(3 * v.size());
    std::memcpy(out.data(), v.data(), sizeof(double) * out.size());
    return out;
}

// One implicit-Euler step of the handle's problem from (x0, v0): Newton from x = x0, then
// x0 <- x, v0 <- (x - x0_old) / dt.  When the Armijo line search stalls (near the solution the
// energy decrease falls below the rounding of the energy), the step continues from its last
// iterate with full Newton steps, which still converge quadratically there.
void rollout_step(symxg_solver* s, int n, symxg_rollout_info* info)
{
    s->x = s->x0;
    symx::SolverReturn r = s->newton->solve();
    auto count = [&] {
        const auto& st = s->newton->get_last_solve_stats();
        if (info) {
            info->newton_iterations += st.newton_iterations;
            info->cg_iterations += st.cg_iterations;
        }
    };
    count();
    if (r == symx::SolverReturn::TooManyArmijoIterations) {
        symx::NewtonSettings& S = s->newton->settings;
        const symx::NewtonSettings saved = S;
        S.enable_armijo_backtracking = false;
        S.max_iterations = 20;
        try {
            r = s->newton->solve();
        } catch (...) {
            S = saved;
            throw;
        }
        S = saved;
        count();
        if (info) info->armijo_polished_steps += 1;
    }
    if (r != symx::SolverReturn::Successful)
        throw std::runtime_error("rollout step " + std::to_string(n) + " did not converge: " + symx::to_string(r));
    for (size_t i = 0; i < s->x.size(); ++i)
        for (int d = 0; d < 3; ++d) s->v0[i][d] = (s->x[i][d] - s->x0[i][d]) / s->dt;
    s->x0 = s->x;
}

}  // namespace

extern "C" {

const char* symxg_last_error(void) { return g_last_error.c_str(); }
int symxg_abi_version(void) { return SYMXG_ABI_VERSION; }
int64_t symxg_launch_count(void) { return symxg::launch_count(); }
void symxg_set_wait_poll_limit(int64_t polls) { symxg::set_wait_poll_limit((long long)polls); }
void symxg_device_memory(int64_t* current, int64_t* peak, int32_t reset_peak)
{
    if (current) *current = symxg::device_bytes_current();
    const int64_t p = symxg::device_bytes_peak(reset_peak != 0);
    if (peak) *peak = p;
}
int64_t symxg_wait_poll_limit(void) { return (int64_t)symxg::wait_poll_limit(); }

void symxg_default_settings(symxg_newton_settings* s)
{
    const symx::NewtonSettings d;
    s->max_iterations = d.max_iterations;
    s->min_iterations = d.min_iterations;
    s->residual_tolerance_abs = d.residual_tolerance_abs;
    s->residual_tolerance_rel = d.residual_tolerance_rel;
    s->step_tolerance = d.step_tolerance;
    s->max_iterations_as_success = d.max_iterations_as_success ? 1 : 0;
    s->step_cap = d.step_cap;
    s->enable_armijo_backtracking = d.enable_armijo_backtracking ? 1 : 0;
    s->line_search_armijo_beta = d.line_search_armijo_beta;
    s->max_backtracking_armijo_iterations = d.max_backtracking_armijo_iterations;
    s->project_to_pd = 1;
    s->projection_eps = d.projection_eps;
    s->project_to_pd_use_mirroring = d.project_to_pd_use_mirroring ? 1 : 0;
    s->cg_max_iterations = d.cg_max_iterations;
    s->cg_abs_tolerance = d.cg_abs_tolerance;
    s->cg_rel_tolerance = d.cg_rel_tolerance;
    s->bailout_residual = d.bailout_residual;
    s->precision = SYMXG_PRECISION_FP64;
    s->time_kernels = 0;
    s->project_on_demand_countdown = d.project_on_demand_countdown;
    s->ppn_tightening_factor = d.ppn_tightening_factor;
    s->ppn_release_factor = d.ppn_release_factor;
    s->projection_fp64_refinement = d.projection_fp64_refinement ? 1 : 0;
    s->cg_residual_replacement = d.cg_residual_replacement;
    s->cg_fp64_partial_sums = d.cg_fp64_partial_sums ? 1 : 0;
    s->cg_lookahead = d.cg_lookahead ? 1 : 0;
}

int symxg_elastic_create(const symxg_elastic_problem* p, const char* cache_dir, symxg_solver** out)
{
    return guarded([&] {
        if (!p || !out) throw std::invalid_argument("null argument");
        if (p->nodes_per_element != 4 && p->nodes_per_element != 8 && p->nodes_per_element != 10)
            throw std::invalid_argument("nodes_per_element must be 4 (Tet4), 10 (Tet10) or 8 (Hex8)");
        if (p->n_vertices <= 0 || p->n_elements < 0 || !p->connectivity || !p->rest_positions || !p->mu || !p->lambda)
            throw std::invalid_argument("missing mesh or material arrays");
        if (p->n_bc > 0 && (!p->bc_vertices || !p->bc_targets)) throw std::invalid_argument("missing boundary arrays");
        const int nn = p->nodes_per_element;
        for (int64_t i = 0; i < (int64_t)p->n_elements * nn; ++i)
            if (p->connectivity[i] < 0 || p->connectivity[i] >= p->n_vertices)
                throw std::invalid_argument("connectivity references a vertex out of range");
        for (int i = 0; i < p->n_bc; ++i)
            if (p->bc_vertices[i] < 0 || p->bc_vertices[i] >= p->n_vertices)
                throw std::invalid_argument("boundary vertex out of range");
        auto S = std::make_unique<symxg_solver>();
        const int nv = p->n_vertices;
        S->nodes = nn;
        S->X.resize(nv);
        std::memcpy(S->X.data(), p->rest_positions, sizeof(double) * 3 * nv);
        S->x = S->X;
        S->x0 = S->X;
        S->v0.assign(nv, Vec3{0, 0, 0});
        S->mu.assign(p->mu, p->mu + p->n_elements);
        S->lam.assign(p->lambda, p->lambda + p->n_elements);
        S->has_inertia = p->mass != nullptr;
        if (S->has_inertia) S->mass.assign(p->mass, p->mass + nv);
        S->dt = p->dt;
        S->gravity = {p->gravity[0], p->gravity[1], p->gravity[2]};
        S->k_bc = p->bc_stiffness;
        S->conn_numbered.reserve((size_t)p->n_elements * (nn + 1));
        for (int e = 0; e < p->n_elements; ++e) {
            S->conn_numbered.push_back(e);
            for (int a = 0; a < nn; ++a) S->conn_numbered.push_back(p->connectivity[(int64_t)e * nn + a]);
        }
        S->vertices.resize(nv);
        for (int i = 0; i < nv; ++i) S->vertices[i] = {i};
        for (int i = 0; i < p->n_bc; ++i) {
            S->bc_conn.numbered_push_back({p->bc_vertices[i]});
            S->bc_target.push_back({p->bc_targets[3 * i], p->bc_targets[3 * i + 1], p->bc_targets[3 * i + 2]});
        }

        using namespace symx;
        symxg_solver* s = S.get();
        const FEM_Element type = nn == 4 ? FEM_Element::Tet4 : nn == 10 ? FEM_Element::Tet10 : FEM_Element::Hex8;
        S->G = GlobalPotential::create();
        S->G->add_potential("neo_hookean_" + get_name(type), S->conn_numbered, nn + 1,
            [s, type, nn](MappedWorkspace<double>& mws, Element& elem) {
                std::vector<Vector> x = mws.make_vectors(s->x, elem.slice(1, nn + 1));
                std::vector<Vector> X = mws.make_vectors(s->X, elem.slice(1, nn + 1));
                Scalar mu = mws.make_scalar(s->mu, elem[0]);
                Scalar lam = mws.make_scalar(s->lam, elem[0]);
                return fem_integrator(mws, type, [&](Scalar& w, Vector& xi) {
                    Matrix Jx = fem_jacobian(type, x, xi);
                    Matrix JX = fem_jacobian(type, X, xi);
                    Matrix F = Jx * JX.inv();
                    Matrix C = F.transpose() * F;
                    Scalar logdetF = log(F.det());
                    Scalar psi = 0.5 * mu * (C.trace() - 3.0) - mu * logdetF + 0.5 * lam * logdetF.powN(2);
                    return psi * JX.det() * w;
                });
            });
        if (S->has_inertia && S->dt <= 0.0) {  // quasistatic: gravity as the potential -m g.x
            S->G->add_potential("gravity", S->vertices, [s](MappedWorkspace<double>& mws, Element& elem) {
                Vector x = mws.make_vector(s->x, elem[0]);
                Scalar m = mws.make_scalar(s->mass, elem[0]);
                Vector g = mws.make_vector(s->gravity);
                return -m * g.dot(x);
            });
        } else if (S->has_inertia) {
            S->G->add_potential("backward_euler_inertia", S->vertices, [s](MappedWorkspace<double>& mws, Element& elem) {
                Vector x1 = mws.make_vector(s->x, elem[0]);
                Vector x0 = mws.make_vector(s->x0, elem[0]);
                Vector v0 = mws.make_vector(s->v0, elem[0]);
                Scalar m = mws.make_scalar(s->mass, elem[0]);
                Vector g = mws.make_vector(s->gravity);
                Scalar dt = mws.make_scalar(s->dt);
                Vector dev = x1 - (x0 + dt * v0 + dt * dt * g);
                return 0.5 * m * dev.squared_norm() / dt.powN(2);
            });
        }
        if (p->n_bc > 0) {
            S->G->add_potential("boundary_conditions", S->bc_conn, [s](MappedWorkspace<double>& mws, Element& conn) {
                Vector x = mws.make_vector(s->x, conn["vertex_idx"]);
                Vector target = mws.make_vector(s->bc_target, conn["constraint_idx"]);
                Scalar k = mws.make_scalar(s->k_bc);
                return 0.5 * k * (x - target).squared_norm();
            });
        }
        S->G->add_dof(S->x);
        auto ctx = Context::create();
        if (cache_dir) ctx->compilation_directory = cache_dir;
        S->newton = std::make_unique<NewtonsMethod>(S->G, ctx);
        S->pin(S->x);
        S->pin(S->x0);
        S->pin(S->v0);
        S->pin(S->X);
        S->pin(S->bc_target);
        S->pin(S->mu);
        S->pin(S->lam);
        S->pin(S->mass);
        *out = S.release();
        return SYMXG_OK;
    });
}

int symxg_destroy(symxg_solver* s)
{
    return guarded([&] {
        delete s;
        return SYMXG_OK;
    });
}

int symxg_set_settings(symxg_solver* s, const symxg_newton_settings* c)
{
    return guarded([&] {
        if (!s || !c) throw std::invalid_argument("null argument");
        if (c->precision != SYMXG_PRECISION_FP64 && c->precision != SYMXG_PRECISION_MIXED)
            throw std::invalid_argument("unknown precision");
        symx::NewtonSettings& t = s->newton->settings;
        t.max_iterations = c->max_iterations;
        t.min_iterations = c->min_iterations;
        t.residual_tolerance_abs = c->residual_tolerance_abs;
        t.residual_tolerance_rel = c->residual_tolerance_rel;
        t.step_tolerance = c->step_tolerance;
        t.max_iterations_as_success = c->max_iterations_as_success != 0;
        t.step_cap = c->step_cap;
        t.enable_armijo_backtracking = c->enable_armijo_backtracking != 0;
        t.line_search_armijo_beta = c->line_search_armijo_beta;
        t.max_backtracking_armijo_iterations = c->max_backtracking_armijo_iterations;
        if (c->project_to_pd < SYMXG_PROJECTION_NEWTON || c->project_to_pd > SYMXG_PROJECTION_PROGRESSIVE)
            throw std::invalid_argument("unknown projection mode");
        t.projection_mode = static_cast<symx::ProjectionToPD>(c->project_to_pd);
        t.project_on_demand_countdown = c->project_on_demand_countdown;
        t.ppn_tightening_factor = c->ppn_tightening_factor;
        t.ppn_release_factor = c->ppn_release_factor;
        t.projection_eps = c->projection_eps;
        t.project_to_pd_use_mirroring = c->project_to_pd_use_mirroring != 0;
        t.cg_max_iterations = c->cg_max_iterations;
        t.cg_abs_tolerance = c->cg_abs_tolerance;
        t.cg_rel_tolerance = c->cg_rel_tolerance;
        t.bailout_residual = c->bailout_residual;
        t.precision = c->precision == SYMXG_PRECISION_MIXED ? symx::Precision::Mixed : symx::Precision::FP64;
        t.time_kernels = c->time_kernels != 0;
        if (c->cg_residual_replacement < 0) throw std::invalid_argument("negative cg_residual_replacement");
        t.projection_fp64_refinement = c->projection_fp64_refinement != 0;
        t.cg_residual_replacement = c->cg_residual_replacement;
        t.cg_fp64_partial_sums = c->cg_fp64_partial_sums != 0;
        t.cg_lookahead = c->cg_lookahead != 0;
        return SYMXG_OK;
    });
}

int symxg_set_state(symxg_solver* s, const double* x, const double* x0, const double* v0)
{
    return guarded([&] {
        if (!s) throw std::invalid_argument("null solver");
        const size_t n = s->x.size() * 3;
        if (x) std::memcpy(s->x.data(), x, sizeof(double) * n);
        if (x0) std::memcpy(s->x0.data(), x0, sizeof(double) * n);
        if (v0) std::memcpy(s->v0.data(), v0, sizeof(double) * n);
        return SYMXG_OK;
    });
}

int symxg_get_positions(symxg_solver* s, double* x)
{
    return guarded([&] {
        if (!s || !x) throw std::invalid_argument("null argument");
        std::memcpy(x, s->x.data(), sizeof(double) * 3 * s->x.size());
        return SYMXG_OK;
    });
}

int symxg_solve(symxg_solver* s, int32_t* ret, symxg_solve_stats* stats)
{
    return guarded([&] {
        if (!s) throw std::invalid_argument("null solver");
        const symx::SolverReturn r = s->newton->solve();
        if (ret) *ret = (int32_t)r;
        fill_stats(s->newton->get_last_solve_stats(), r, stats);
        return SYMXG_OK;
    });
}

int symxg_upload(symxg_solver* s)
{
    return guarded([&] {
        if (!s) throw std::invalid_argument("null solver");
        s->newton->upload();
        return SYMXG_OK;
    });
}

int symxg_solve_device(symxg_solver* s, int32_t* ret, symxg_solve_stats* stats)
{
    return guarded([&] {
        if (!s) throw std::invalid_argument("null solver");
        const symx::SolverReturn r = s->newton->solve_device();
        if (ret) *ret = (int32_t)r;
        fill_stats(s->newton->get_last_solve_stats(), r, stats);
        return SYMXG_OK;
    });
}

int symxg_download(symxg_solver* s)
{
    return guarded([&] {
        if (!s) throw std::invalid_argument("null solver");
        s->newton->download();
        return SYMXG_OK;
    });
}

int symxg_evaluate(symxg_solver* s, double* energy, double* grad)
{
    return guarded([&] {
        if (!s || !energy) throw std::invalid_argument("null argument");
        s->newton->upload();
        *energy = s->newton->evaluate(grad);
        return SYMXG_OK;
    });
}

int symxg_evaluate_energy(symxg_solver* s, double* energy)
{
    return guarded([&] {
        if (!s || !energy) throw std::invalid_argument("null argument");
        s->newton->upload();
        *energy = s->newton->evaluate_energy();
        return SYMXG_OK;
    });
}

int symxg_assembled_hessian(symxg_solver* s, int32_t project, int32_t* n_blocks, int64_t* nnzb, int32_t* row_ptr,
                            int32_t* cols, double* vals)
{
    return guarded([&] {
        if (!s || !n_blocks || !nnzb) throw std::invalid_argument("null argument");
        if (vals && (!row_ptr || !cols)) throw std::invalid_argument("row_ptr and cols are required with vals");
        if (vals) s->newton->upload();
        s->newton->assembled_hessian(project != 0, n_blocks, nnzb, row_ptr, cols, vals);
        return SYMXG_OK;
    });
}

int symxg_element_outputs(symxg_solver* s, int32_t potential, int32_t project, double* E, double* g, double* H)
{
    return guarded([&] {
        if (!s) throw std::invalid_argument("null solver");
        if (potential < 0 || potential >= s->G->get_n_potentials()) throw std::invalid_argument("no such potential");
        s->newton->upload();
        s->newton->element_outputs(potential, project != 0, E, g, H);
        return SYMXG_OK;
    });
}

int symxg_generate_cuboid_mesh(int32_t type, const double size[3], const int32_t cells[3], int64_t* n_vertices,
                               int64_t* n_elements, int32_t* stride, double* vertices, int32_t* connectivity)
{
    return guarded([&] {
        if (!size || !cells || !n_vertices || !n_elements || !stride) throw std::invalid_argument("null argument");
        if (type < 0 || type > 3) throw std::invalid_argument("element_type must be 0 (Tet4), 1 (Tet10), 2 (Hex8) or 3 (Hex27)");
        const symx::FEMMesh<double> m = symx::generate_cuboid_mesh<double>(
            static_cast<symx::FEM_Element>(type), Vec3{size[0], size[1], size[2]}, {cells[0], cells[1], cells[2]});
        const int64_t nv = (int64_t)m.vertices.size(), ne = m.n_elements;
        if (vertices && connectivity) {
            if (*n_vertices < nv || *n_elements < ne) throw std::invalid_argument("mesh buffers too small");
            for (int64_t i = 0; i < nv; ++i)
                for (int k = 0; k < 3; ++k) vertices[3 * i + k] = m.vertices[i][k];
            std::copy(m.connectivity.begin(), m.connectivity.end(), connectivity);
        }
        *n_vertices = nv;
        *n_elements = ne;
        *stride = m.connectivity_stride;
        return SYMXG_OK;
    });
}

int symxg_op_counts(symxg_solver* s, int32_t potential, int64_t counts[3])
{
    return guarded([&] {
        if (!s || !counts) throw std::invalid_argument("null argument");
        if (potential < 0 || potential >= s->G->get_n_potentials()) throw std::invalid_argument("no such potential");
        const auto c = s->newton->op_counts(potential);
        for (int i = 0; i < 3; ++i) counts[i] = c[i];
        return SYMXG_OK;
    });
}

int symxg_project_pd_f32(float* m, int32_t n, int64_t count, float eps, int32_t mirroring, int32_t* nc, void* stream)
{
    return project_impl<float>(m, n, count, eps, mirroring, nc, stream);
}
int symxg_project_pd_f64(double* m, int32_t n, int64_t count, double eps, int32_t mirroring, int32_t* nc, void* stream)
{
    return project_impl<double>(m, n, count, eps, mirroring, nc, stream);
}

int symxg_bcsr_spmv_f32(int32_t nb, const int32_t* rp, const int32_t* cols, const float* vals, int64_t vs, const float* x,
                        float* y, void* stream)
{
    return spmv_impl<float>(nb, rp, cols, vals, vs, x, y, stream);
}
int symxg_bcsr_spmv_f64(int32_t nb, const int32_t* rp, const int32_t* cols, const double* vals, int64_t vs,
                        const double* x, double* y, void* stream)
{
    return spmv_impl<double>(nb, rp, cols, vals, vs, x, y, stream);
}

int symxg_bcsr_pcg_f32(int32_t nb, const int32_t* rp, const int32_t* cols, const float* vals, int64_t vs, const float* b,
                       float* x, double abs_tol, double rel_tol, int32_t max_it, symxg_pcg_info* info, void* stream)
{
    return pcg_impl<float>(nb, rp, cols, vals, vs, b, x, abs_tol, rel_tol, max_it, info, stream);
}
int symxg_bcsr_pcg_f64(int32_t nb, const int32_t* rp, const int32_t* cols, const double* vals, int64_t vs,
                       const double* b, double* x, double abs_tol, double rel_tol, int32_t max_it, symxg_pcg_info* info,
                       void* stream)
{
    return pcg_impl<double>(nb, rp, cols, vals, vs, b, x, abs_tol, rel_tol, max_it, info, stream);
}

int symxg_bcsr_pcg_f32_noalloc(int32_t nb, const int32_t* rp, const int32_t* cols, const float* vals, int64_t vs,
                               const float* b, float* x, double abs_tol, double rel_tol, int32_t max_it,
                               symxg_pcg_info* info, void* stream)
{
    return guarded([&] {
        if (!info) throw std::invalid_argument("null info");
        std::memset(info, 0, sizeof(*info));
        if (nb < 0 || vs < 0 || max_it < 0) throw std::invalid_argument("negative size");
        if (nb > 0 && (!rp || !cols || !vals || !b || !x)) throw std::invalid_argument("null device pointer");
        if (symxg::bcsr_pcg_noalloc_max_blocks() != SYMXG_PCG_NOALLOC_MAX_BLOCKS) throw std::logic_error("limit mismatch");
        const symxg::BcsrPcgResult r = symxg::run_bcsr_pcg_noalloc_f32(nb, rp, cols, vals, vs, b, x, abs_tol, rel_tol,
                                                                       max_it, (cudaStream_t)stream);
        info->converged = r.converged;
        info->n_iterations = r.iterations;
        info->error = r.error;
        info->found_indefiniteness = r.indefinite;
        info->missing_diagonal = r.missing_diagonal;
        if (r.missing_diagonal) throw std::invalid_argument("block rows without a diagonal block");
        return SYMXG_OK;
    });
}

int symxg_adjoint(symxg_solver* s, const double* dLdx, double rel_tol, int32_t max_iterations, double* lambda,
                  double* dLdmu, double* dLdlambda, double* dLdx0, double* dLdv0, symxg_adjoint_info* info)
{
    return guarded([&] {
        if (!s || !dLdx) throw std::invalid_argument("null argument");
        if (!(rel_tol > 0.0) || max_iterations <= 0) throw std::invalid_argument("rel_tol and max_iterations must be positive");
        const size_t nd = 3 * s->x.size();
        std::vector<double> lam(nd);
        const symx::AdjointInfo ai = s->newton->adjoint_solve(dLdx, lam.data(), rel_tol, max_iterations);
        if (info) {
            info->converged = ai.converged ? 1 : 0;
            info->iterations = ai.iterations;
            info->error = ai.error;
        }
        if (lambda) std::memcpy(lambda, lam.data(), sizeof(double) * nd);
        if (dLdmu) s->newton->parameter_gradient(reinterpret_cast<std::uintptr_t>(&s->mu), lam.data(), dLdmu, (int64_t)s->mu.size());
        if (dLdlambda)
            s->newton->parameter_gradient(reinterpret_cast<std::uintptr_t>(&s->lam), lam.data(), dLdlambda, (int64_t)s->lam.size());
        const bool inertia = s->has_inertia && s->dt > 0.0;
        if (dLdx0) {
            if (inertia) s->newton->parameter_gradient(reinterpret_cast<std::uintptr_t>(&s->x0), lam.data(), dLdx0, (int64_t)nd);
            else std::fill(dLdx0, dLdx0 + nd, 0.0);
        }
        if (dLdv0) {
            if (inertia) s->newton->parameter_gradient(reinterpret_cast<std::uintptr_t>(&s->v0), lam.data(), dLdv0, (int64_t)nd);
            else std::fill(dLdv0, dLdv0 + nd, 0.0);
        }
        if (!ai.converged) throw std::runtime_error("adjoint PCG did not converge (" + std::to_string(ai.iterations) + " iterations)");
        return SYMXG_OK;
    });
}

int symxg_rollout_forward(symxg_solver* s, int32_t n_steps, int32_t checkpoint_every, symxg_rollout_info* info)
{
    return guarded([&] {
        if (!s) throw std::invalid_argument("null argument");
        if (n_steps <= 0 || checkpoint_every <= 0) throw std::invalid_argument("n_steps and checkpoint_every must be positive");
        if (!(s->has_inertia && s->dt > 0.0)) throw std::invalid_argument("a rollout needs masses and dt > 0");
        if (info) std::memset(info, 0, sizeof(*info));
        const auto t0 = std::chrono::steady_clock::now();
        s->ckpt_x0.clear();
        s->ckpt_v0.clear();
        for (int n = 0; n < n_steps; ++n) {
            if (n % checkpoint_every == 0) {
                s->ckpt_x0.push_back(s->x0);
                s->ckpt_v0.push_back(s->v0);
            }
            rollout_step(s, n, info);
        }
        s->rollout_steps = n_steps;
        s->checkpoint_every = checkpoint_every;
        if (info) {
            info->steps = n_steps;
            info->checkpoints = (int32_t)s->ckpt_x0.size();
            info->seconds_forward = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
        return SYMXG_OK;
    });
}

int symxg_rollout_backward(symxg_solver* s, const double* dLdx_final, const double* dLdv_final, double rel_tol,
                           int32_t max_iterations, double* dLdx_init, double* dLdv_init, double* dLdmu,
                           double* dLdlambda, symxg_rollout_info* info)
{
    return guarded([&] {
        if (!s || !dLdx_final) throw std::invalid_argument("null argument");
        if (s->rollout_steps <= 0) throw std::invalid_argument("no forward rollout to differentiate");
        if (!(rel_tol > 0.0) || max_iterations <= 0) throw std::invalid_argument("rel_tol and max_iterations must be positive");
        const auto t0 = std::chrono::steady_clock::now();
        const size_t nv = s->x.size(), nd = 3 * nv, ne = s->mu.size();
        const double dt = s->dt;
        std::vector<double> ax(dLdx_final, dLdx_final + nd), av(nd, 0.0), a(nd), lam(nd), gx(nd), gv(nd);
        if (dLdv_final) av.assign(dLdv_final, dLdv_final + nd);
        std::vector<double> dmu(ne, 0.0), dlam(ne, 0.0), tmu(ne), tlam(ne);
        const int N = s->rollout_steps, K = s->checkpoint_every;
        const std::vector<Vec3> x_final = s->x, x0_final = s->x0, v0_final = s->v0;
        for (int seg = (int)s->ckpt_x0.size() - 1; seg >= 0; --seg) {
            const int start = seg * K, end = std::min(start + K, N);
            // recompute the segment's states from its checkpoint
            std::vector<std::vector<Vec3>> xs{s->ckpt_x0[seg]}, vs{s->ckpt_v0[seg]};
            s->x0 = s->ckpt_x0[seg];
            s->v0 = s->ckpt_v0[seg];
            for (int n = start; n < end; ++n) {
                rollout_step(s, n, info);
                xs.push_back(s->x0);
                vs.push_back(s->v0);
                if (info) info->recomputed_steps += 1;
            }
            for (int n = end - 1; n >= start; --n) {
                const int k = n - start;
                s->x = xs[k + 1];
                s->x0 = xs[k];
                s->v0 = vs[k];
                s->newton->upload();
                for (size_t i = 0; i < nd; ++i) a[i] = ax[i] + av[i] / dt;
                const symx::AdjointInfo ai = s->newton->adjoint_solve(a.data(), lam.data(), rel_tol, max_iterations);
                if (info) info->adjoint_iterations += ai.iterations;
                if (!ai.converged)
                    throw std::runtime_error("adjoint PCG of rollout step " + std::to_string(n) + " did not converge");
                s->newton->parameter_gradient(reinterpret_cast<std::uintptr_t>(&s->x0), lam.data(), gx.data(), (int64_t)nd);
                s->newton->parameter_gradient(reinterpret_cast<std::uintptr_t>(&s->v0), lam.data(), gv.data(), (int64_t)nd);
                if (dLdmu) {
                    s->newton->parameter_gradient(reinterpret_cast<std::uintptr_t>(&s->mu), lam.data(), tmu.data(), (int64_t)ne);
                    for (size_t e = 0; e < ne; ++e) dmu[e] += tmu[e];
                }
                if (dLdlambda) {
                    s->newton->parameter_gradient(reinterpret_cast<std::uintptr_t>(&s->lam), lam.data(), tlam.data(), (int64_t)ne);
                    for (size_t e = 0; e < ne; ++e) dlam[e] += tlam[e];
                }
                for (size_t i = 0; i < nd; ++i) {
                    ax[i] = gx[i] - av[i] / dt;
                    av[i] = gv[i];
                }
            }
        }
        // leave the handle at the end of the rollout
        s->x = x_final;
        s->x0 = x0_final;
        s->v0 = v0_final;
        if (dLdx_init) std::memcpy(dLdx_init, ax.data(), sizeof(double) * nd);
        if (dLdv_init) std::memcpy(dLdv_init, av.data(), sizeof(double) * nd);
        if (dLdmu) std::memcpy(dLdmu, dmu.data(), sizeof(double) * ne);
        if (dLdlambda) std::memcpy(dLdlambda, dlam.data(), sizeof(double) * ne);
        if (info) info->seconds_backward = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return SYMXG_OK;
    });
}

}  // extern "C"
