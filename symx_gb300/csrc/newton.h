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
    LinearSolver linear_solver = LinearSolver::BDPCG;
    int cg_max_iterations = 10000;
    double cg_abs_tolerance = 1e-12;
    double cg_rel_tolerance = 1e-4;
    bool cg_stop_on_indefiniteness = true;
    double bailout_residual = 1e-10;
    Precision precision = Precision::FP64;
    // Record CUDA events around every PCG SpMV and PD-projection launch (SolveStats::kernels).
    bool time_kernels = false;
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
};

struct SolverImpl;

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

}  // namespace symx
