// Projected Newton's method on one GPU (reference: symx/src/solver/NewtonsMethod.{h,cpp},
// settings and return codes symx/src/solver/solver_utils.h:15-26, 272-358).
//
// Construction differentiates every potential with respect to its DoF symbols, generates
// CUDA element kernels (energy + gradient in FP64, Hessian in the storage precision),
// compiles them with NVRTC and builds the BCSR sparsity and the fixed-order assembly maps.
// solve() uploads the user's arrays, runs the whole Newton loop on the device (element
// evaluation, PD projection, assembly, block-Jacobi PCG, Armijo line search) with only
// scalars crossing to the host, and writes the converged DoFs back into the user's arrays.
#pragma once

#include <array>
#include <cstdint>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "global_potential.h"

namespace symx {

enum class SolverReturn {
    Successful,
    Running,
    InvalidInitialState,
    TooManyIterations,
    TooManyArmijoIterations,
    LinearSystemSolveFailure,
    TooManyInvalidIntermediateIterations,
    StepDoesNotDescend,
    InvalidConvergedState,
};

enum class ProjectionToPD { Newton, ProjectedNewton, ProjectOnDemand, Progressive };
enum class LinearSolver { DirectLLT, BDPCG };

// Arithmetic of the Hessian path.  FP64: everything in double.  Mixed: element energy and
// gradient, line-search energy, residual and dot-product accumulation in double; element
// Hessians, their projection, the BCSR matrix and the PCG vectors in float.
enum class Precision { FP64 = 0, Mixed = 1 };

struct NewtonSettings {
    int max_iterations = std::numeric_limits<int>::max();
    int min_iterations = 0;
    double residual_tolerance_abs = 1e-6;
    double residual_tolerance_rel = 0.0;
    double step_tolerance = 0.0;
    bool max_iterations_as_success = false;
    double step_cap = std::numeric_limits<double>::infinity();
    bool enable_armijo_backtracking = true;
    double line_search_armijo_beta = 1e-4;
    int max_backtracking_armijo_iterations = 20;
    int max_backtracking_invalid_state_iterations = 8;
    ProjectionToPD projection_mode = ProjectionToPD::ProjectedNewton;
    double projection_eps = 1e-10;
    bool project_to_pd_use_mirroring = false;
    int project_on_demand_countdown = 4;   // ProjectOnDemand: Newton iterations projected after a failure
    double ppn_tightening_factor = 0.5;    // Progressive: threshold factor after a failed direction
    double ppn_release_factor = 2.0;       // Progressive: threshold factor after a successful one
    LinearSolver linear_solver = LinearSolver::BDPCG;
    int cg_max_iterations = 10000;
    double cg_abs_tolerance = 1e-12;
    double cg_rel_tolerance = 1e-4;
    bool cg_stop_on_indefiniteness = true;
    double bailout_residual = 1e-10;
    Precision precision = Precision::FP64;
    // Record CUDA events around every PCG SpMV and PD-projection launch (SolveStats::kernels).
    bool time_kernels = false;
    // 12 x 12 element projections (Tet4) with FP64-accurate arithmetic in either precision: an
    // FP32 Jacobi refined by one FP64 Ogita-Aishima step, the clamping applied as an FP64
    // correction (the reference's projection is FP64 Eigen, project_to_PD.cpp:12-32).  Mixed
    // precision keeps the FP32 element Hessians and BCSR matrix; only the projection's
    // arithmetic changes.  Other element sizes are projected as without it.
    bool projection_fp64_refinement = false;
    // One-launch FP32 PCG (Mixed): every this many iterations the recursive residual is
    // replaced by the true residual b - A x accumulated in FP64 and the convergence test
    // is made on it (0: never; the FP64 PCG never replaces).
    int cg_residual_replacement = 0;
    // One-launch FP32 PCG (Mixed): the chunk and block partials of its dot products (p.Ap,
    // r.r, r.z) are accumulated in FP64 in a fixed order; false (default): in float-float.
    // Products and the per-thread and per-warp sums are float-float (exact products) in both.
    // Every block forms the sums itself, so FP64 costs FP64-pipe time in every block
    // (GB300's FP64 rate is 1/64 of FP32): about 8 us per iteration on the 64^3 Tet4 step.
    bool cg_fp64_partial_sums = false;
    // One-launch FP32 PCG (Mixed): one grid barrier per iteration, the update of x, r and z folded
    // into the next product pass (k_pcg_solve_la); false: the two-barrier form (product pass,
    // barrier, update, barrier).  Same iterates up to rounding.
    bool cg_lookahead = false;
};

struct Context {
    int n_threads = 1;                   // kept for API compatibility; the GPU path ignores it
    std::string compilation_directory;   // NVRTC kernel cache ("" = default)
    int verbosity = 0;                   // 0 silent, 1 per-iteration lines
    static std::shared_ptr<Context> create() { return std::make_shared<Context>(); }
};
using spContext = std::shared_ptr<Context>;

struct SolveStats {
    int newton_iterations = 0;
    int cg_iterations = 0;
    int ls_cap_iterations = 0;
    int ls_max_iterations = 0;
    int ls_inv_iterations = 0;
    int ls_bt_iterations = 0;
    uint64_t n_hessians = 0;
    uint64_t n_projected_hessians = 0;
    double projected_hessians_ratio = 0.0;
    double final_residual = 0.0;
    double final_energy = 0.0;
    int projection_not_converged = 0;
    int64_t h2d_bytes = 0;  // host->device bytes of the last upload()
    int64_t d2h_bytes = 0;  // device->host bytes of the last download()
    // Device time per stage in seconds (CUDA events), with the reference's timer labels.
    std::map<std::string, double> timers;
    // With time_kernels: per kernel name, {launches that did work, total seconds}.
    std::map<std::string, std::pair<int64_t, double>> kernels;
    // PCG iterations of each Newton iteration's linear solve, in order.
    std::vector<int> cg_iterations_per_newton;
    // residual replacements made by the FP32 PCG (cg_residual_replacement)
    int cg_residual_replacements = 0;
};

struct SolverImpl;

struct AdjointInfo {
    int iterations = 0;
    bool converged = false;
    double error = 0.0;  // sqrt(r.r / b.b) at exit
};

class NewtonsMethod {
public:
    NewtonsMethod(spGlobalPotential global_potential, spContext context);
    ~NewtonsMethod();
    static std::shared_ptr<NewtonsMethod> create(spGlobalPotential g, spContext c)
    {
        return std::make_shared<NewtonsMethod>(g, c);
    }

    SolverReturn solve();
    const SolveStats& get_last_solve_stats() const { return stats; }

    NewtonSettings settings;

    // ---- device-resident entry points used by the C ABI, tests and benchmarks
    // Upload every bound array and the DoFs from the user's containers.
    void upload();
    // Copy the device DoFs back into the user's containers.
    void download();
    // Run the Newton loop on the data already on the device (no host transfers).
    SolverReturn solve_device();
    // Energy and gradient (host output, may be null) at the device DoFs.
    double evaluate(double* grad_host);
    // Energy only at the device DoFs.
    double evaluate_energy();
    // Assemble the (optionally projected) Hessian at the device DoFs in the current
    // precision and copy it out: row_ptr (n_blocks+1), cols (nnzb), vals (nnzb*9, row-major
    // blocks, as double).  Pass null outputs to query the sizes.
    void assembled_hessian(bool project, int32_t* n_blocks, int64_t* nnzb, int32_t* row_ptr, int32_t* cols, double* vals);
    // Element outputs of potential `p` at the device DoFs: E (n), g (n*nd), H (n*nd*nd, row-major,
    // optionally projected), as double.
    void element_outputs(int p, bool project, double* E, double* g, double* H);
    int n_dof_blocks() const;
    int64_t n_hessian_blocks() const;
    // Device pointers (for tests that exercise single kernels): DoFs (double, 3 per block).
    double* device_dofs();
    // Op counts of the generated code of potential p: [E+g, H, E-only].
    std::array<int64_t, 3> op_counts(int p) const;
    std::string generated_source(int p) const;

    // ---- adjoint (an addition of this library; the reference has no adjoint)
    // Solve H lambda = rhs with block-Jacobi PCG, H the Hessian of the total energy at the
    // device DoFs (true Hessian, or projected with `project`), assembled in the current
    // precision.  rhs and lambda are host arrays of n_dofs doubles.  Stops at
    // sqrt(r.r / b.b) < rel_tol (or after max_iterations).
    AdjointInfo adjoint_solve(const double* rhs, double* lambda, double rel_tol, int max_iterations,
                              bool project = false);
    // out = -sum over elements of lambda_e . d g_e / d p for the data container `param`
    // (identified by its address, bound in the potentials with make_scalar / make_vector(s)):
    // the contribution of an implicit state x(p) with g(x(p), p) = 0 to dL/dp when
    // H lambda = dL/dx.  The mixed derivatives d g / d p are differentiated symbolically from
    // the potentials and compiled on first use.  Evaluated in FP64 at the device DoFs and
    // uploaded data; `out` (host) holds n_out doubles, the container's size.
    void parameter_gradient(std::uintptr_t param, const double* lambda, double* out, int64_t n_out);
    template <typename C>
    std::vector<double> parameter_gradient(const C& param, const std::vector<double>& lambda)
    {
        const int64_t n = (int64_t)(param.size() * (sizeof(typename C::value_type) / sizeof(double)));
        std::vector<double> out((size_t)n);
        parameter_gradient(reinterpret_cast<std::uintptr_t>(&param), lambda.data(), out.data(), n);
        return out;
    }

private:
    spGlobalPotential global_potential;
    spContext context;
    SolveStats stats;
    int64_t h2d_bytes_ = 0, d2h_bytes_ = 0;
    std::unique_ptr<SolverImpl> impl;
};
using spNewtonsMethod = std::shared_ptr<NewtonsMethod>;

std::string to_string(SolverReturn r);
// CUDA source of the element kernels NewtonsMethod would generate for each potential
// (differentiation + code generation only; no GPU or compiler involved).
std::vector<std::string> generate_element_kernel_sources(const GlobalPotential& gp);
// CUDA source of the mixed-derivative kernels parameter_gradient would generate for the data
// container with address `param`, one per (potential, binding).
std::vector<std::string> generate_mixed_kernel_sources(const GlobalPotential& gp, std::uintptr_t param);

}  // namespace symx
