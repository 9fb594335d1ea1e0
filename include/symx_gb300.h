/*
 * symx_gb300 C ABI: the GPU second-order solve path of SymX behind plain C types.
 *
 * The reference (InteractiveComputerGraphics/SymX) is a C++ library whose solve path is
 * reached through GlobalPotential::add_potential + NewtonsMethod::solve
 * (symx/src/solver/GlobalPotential.h:37-76, symx/src/solver/NewtonsMethod.h:83-87) and whose
 * generated kernels sit behind a dlopen'ed plugin ABI `void f(T* in, T* out)` with
 * get_n_inputs/get_n_outputs (symx/src/compile/Compilation.cpp:292-323).  This header is
 * the C boundary of the GPU implementation: opaque handles, host or device pointers and
 * sizes, int status codes (0 = success), never exit() or a trap.  The C++ API
 * (include/symx) is the drop-in for C++ users; this ABI is what an FFI binds.
 *
 * Threading: one handle must not be used from two threads at once; separate handles are
 * independent.  All work of a handle runs on its own CUDA stream on the current device.
 */
#ifndef SYMX_GB300_H
#define SYMX_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SYMXG_ABI_VERSION 5

/* status codes */
#define SYMXG_OK 0
#define SYMXG_ERR_INVALID_ARGUMENT 1
#define SYMXG_ERR_RUNTIME 2 /* CUDA, NVRTC or internal failure; see symxg_last_error() */

/* arithmetic of the Hessian path */
/* projection modes (symx::ProjectionToPD): no projection, every element Hessian, all of them
 * for a few iterations after a failed direction, or those near large gradients */
#define SYMXG_PROJECTION_NEWTON 0
#define SYMXG_PROJECTION_PROJECTED_NEWTON 1
#define SYMXG_PROJECTION_ON_DEMAND 2
#define SYMXG_PROJECTION_PROGRESSIVE 3
#define SYMXG_PRECISION_FP64 0
#define SYMXG_PRECISION_MIXED 1 /* FP32 element Hessians, projection, BCSR and PCG vectors;
                                   FP64 energy, gradient, residual, line search, dot sums */

/* solver return codes: same values and meaning as symx::SolverReturn
   (symx/src/solver/solver_utils.h:15-26) */
#define SYMXG_SOLVER_SUCCESSFUL 0
#define SYMXG_SOLVER_TOO_MANY_ITERATIONS 3
#define SYMXG_SOLVER_TOO_MANY_ARMIJO_ITERATIONS 4
#define SYMXG_SOLVER_LINEAR_SYSTEM_SOLVE_FAILURE 5
#define SYMXG_SOLVER_STEP_DOES_NOT_DESCEND 7

typedef struct symxg_solver symxg_solver;

/* One implicit-Euler step (or a quasistatic solve when mass == NULL) of a clamped
 * Neo-Hookean solid, written with the reference's own idioms: classic Neo-Hookean density
 * (examples/elasticity_potentials.h:7-13) integrated with the FEM rule of the element type
 * (symx/src/solver/fem_integrators.cpp:52-133), backward-Euler inertia
 * 1/2 m |x - (x0 + dt v0 + dt^2 g)|^2 / dt^2 (examples/dynamic_elasticity_with_contact.cpp:86-103)
 * and penalty Dirichlet 1/2 k |x - target|^2 (examples/rubber_extrusion.cpp:94-107).
 * With mass given and dt <= 0 the solve is quasistatic: gravity enters as the potential
 * -m g.x instead of the inertia term.  All arrays are copied at creation. */
typedef struct symxg_elastic_problem {
    int32_t n_vertices;
    int32_t n_elements;
    int32_t nodes_per_element;     /* 4 (Tet4), 10 (Tet10) or 8 (Hex8) */
    const int32_t* connectivity;   /* n_elements * nodes_per_element */
    const double* rest_positions;  /* n_vertices * 3 */
    const double* mu;              /* n_elements Lame mu */
    const double* lambda;          /* n_elements Lame lambda */
    const double* mass;            /* n_vertices lumped masses, or NULL (no inertia term) */
    double dt;
    double gravity[3];
    int32_t n_bc;
    const int32_t* bc_vertices;    /* n_bc */
    const double* bc_targets;      /* n_bc * 3 */
    double bc_stiffness;
} symxg_elastic_problem;

/* Mirror of symx::NewtonSettings (symx/src/solver/solver_utils.h:272-358) for the fields
 * the GPU path implements, plus the precision. */
typedef struct symxg_newton_settings {
    int32_t max_iterations;
    int32_t min_iterations;
    double residual_tolerance_abs;
    double residual_tolerance_rel;
    double step_tolerance;
    int32_t max_iterations_as_success;
    double step_cap;
    int32_t enable_armijo_backtracking;
    double line_search_armijo_beta;
    int32_t max_backtracking_armijo_iterations;
    int32_t project_to_pd;           /* SYMXG_PROJECTION_*: symx::ProjectionToPD (solver_utils.h:137-142) */
    double projection_eps;
    int32_t project_to_pd_use_mirroring;
    int32_t cg_max_iterations;
    double cg_abs_tolerance;
    double cg_rel_tolerance;
    double bailout_residual;
    int32_t precision;               /* SYMXG_PRECISION_* */
    int32_t time_kernels;            /* 1: record CUDA events around PCG SpMV and projection launches */
    int32_t project_on_demand_countdown; /* ProjectOnDemand: iterations projected after a failure (4) */
    double ppn_tightening_factor;    /* Progressive: threshold factor after a failed direction (0.5) */
    double ppn_release_factor;       /* Progressive: threshold factor after a successful one (2.0) */
    int32_t projection_fp64_refinement; /* 1: 12x12 projections FP64-accurate (FP32 Jacobi + one FP64
                                           refinement step, FP64 clamping correction), either precision */
    int32_t cg_residual_replacement; /* Mixed: every k PCG iterations replace the residual by b - A x
                                        accumulated in FP64 (0: never) */
    int32_t cg_fp64_partial_sums;    /* Mixed: dot-product partials of the PCG summed in FP64 (1) or
                                        float-float (0, default; faster) */
    int32_t cg_lookahead;            /* Mixed: 1: the one-launch PCG with one grid barrier per
                                        iteration (update folded into the next product pass); 0 (default): two */
} symxg_newton_settings;

typedef struct symxg_solve_stats {
    int32_t solver_return;
    int32_t newton_iterations;
    int32_t cg_iterations;
    int32_t ls_bt_iterations;
    double final_residual;           /* max |grad| at the last evaluation */
    double final_energy;
    int32_t projection_not_converged;
    double t_evaluate_P_grad_hess;   /* device seconds per stage (CUDA events) */
    double t_project_to_PD;
    double t_assembly;
    double t_linear_system_solve;
    double t_evaluate_P;
    int64_t h2d_bytes;               /* host->device bytes of the last upload */
    int64_t d2h_bytes;               /* device->host bytes of the last download */
    int64_t spmv_launches;           /* with time_kernels: PCG SpMV launches that did work ... */
    double spmv_seconds;             /* ... and their summed device time */
    int64_t project_launches;        /* with time_kernels: 12x12 projection launches ... */
    double project_seconds;          /* ... and their summed device time */
    int64_t pcg_solve_iterations;    /* with time_kernels: PCG iterations run by the one-launch PCG ... */
    double pcg_solve_seconds;        /* ... and the device time of those launches */
    int32_t cg_iterations_per_newton[16]; /* PCG iterations of the first 16 linear solves (0 after) */
    int64_t n_hessians;              /* element Hessians of the Newton iterations that found a direction */
    int64_t n_projected_hessians;    /* ... and how many of them were projected */
    int32_t cg_residual_replacements; /* residual replacements made by the FP32 PCG */
    int32_t pad;
} symxg_solve_stats;

/* message of the last failing call on this thread ("" if none) */
const char* symxg_last_error(void);
int symxg_abi_version(void);
void symxg_default_settings(symxg_newton_settings* settings);

/* Build the potentials, differentiate, generate and compile (NVRTC, cached in cache_dir or
 * the default cache when NULL) the element kernels, and build the BCSR sparsity. */
int symxg_elastic_create(const symxg_elastic_problem* problem, const char* cache_dir, symxg_solver** out);
int symxg_destroy(symxg_solver* solver);
int symxg_set_settings(symxg_solver* solver, const symxg_newton_settings* settings);

/* Host state: positions x (the DoFs, also the Newton initial guess), previous positions
 * x0 and velocities v0 (each n_vertices*3; x0/v0 may be NULL to keep the current ones). */
int symxg_set_state(symxg_solver* solver, const double* x, const double* x0, const double* v0);
int symxg_get_positions(symxg_solver* solver, double* x);

/* NewtonsMethod::solve(): upload the host state, run the Newton loop on the device,
 * download the positions.  solver_return receives a SYMXG_SOLVER_* code. */
int symxg_solve(symxg_solver* solver, int32_t* solver_return, symxg_solve_stats* stats);

/* Device-resident pieces of symxg_solve for callers that keep the state on the GPU. */
int symxg_upload(symxg_solver* solver);
int symxg_solve_device(symxg_solver* solver, int32_t* solver_return, symxg_solve_stats* stats);
int symxg_download(symxg_solver* solver);

/* Energy and gradient (n_vertices*3, may be NULL) at the host state. */
int symxg_evaluate(symxg_solver* solver, double* energy, double* grad);
/* Energy only, at the host state (line-search kernel). */
int symxg_evaluate_energy(symxg_solver* solver, double* energy);
/* Assembled Hessian at the host state in the current precision, projected or not.
 * Call with vals == NULL to get n_blocks and nnzb; then row_ptr (n_blocks+1), cols (nnzb)
 * and vals (nnzb*9, row-major 3x3 blocks, as double). */
int symxg_assembled_hessian(symxg_solver* solver, int32_t project, int32_t* n_blocks, int64_t* nnzb,
                            int32_t* row_ptr, int32_t* cols, double* vals);
/* Element outputs of potential `potential` (0 elastic, 1 inertia, 2 boundary) at the host
 * state: E (n), g (n*m), H (n*m*m row-major, optionally projected), m = 3 * nodes. */
int symxg_element_outputs(symxg_solver* solver, int32_t potential, int32_t project, double* E, double* g, double* H);
/* Number of scalar operations in the generated code of a potential: E+g, H, E-only. */
int symxg_op_counts(symxg_solver* solver, int32_t potential, int64_t counts[3]);

/* Structured box mesh as the reference's generate_cuboid_mesh builds it
 * (symx/src/solver/mesh_generation.cpp:306-327, mesh_ordering.cpp:231-252): a box of `size`
 * centred at the origin with `cells` per axis, element_type 0 Tet4 (6 per cell), 1 Tet10,
 * 2 Hex8, 3 Hex27, nodes renumbered by reverse Cuthill-McKee, elements in the reference's
 * order.  Host only.  With vertices or connectivity NULL: writes the sizes.  Otherwise
 * *n_vertices and *n_elements hold the buffers' capacities (vertices: 3 doubles each,
 * connectivity: *stride int32 each) and are set to the sizes written. */
int symxg_generate_cuboid_mesh(int32_t element_type, const double size[3], const int32_t cells[3], int64_t* n_vertices,
                               int64_t* n_elements, int32_t* stride, double* vertices, int32_t* connectivity);

/* Number of CUDA kernels this library has launched since it was loaded (all handles). */
int64_t symxg_launch_count(void);

/* Device memory held by this library's own buffers (solver handles, Compiled<T> batches,
 * stand-alone PCG workspaces; not the CUDA context, the loaded kernel images or the driver's
 * local-memory reservation), and its high-water mark since the last reset (reset_peak != 0
 * sets it to the current value after reading it).  Either pointer may be NULL. */
void symxg_device_memory(int64_t* current, int64_t* peak, int32_t reset_peak);

/* Bound on the waits inside the staged PCG kernels (no counterpart in the reference, whose
 * CPU solver never waits on another processor).  Every wait of those kernels on a
 * shared-memory stage or on the other blocks of the launch polls at most this many times;
 * when one gives up, the kernel stops its work, waits (with the default bound) for its own
 * copies in flight, flags the solve and returns, and the call fails with SYMXG_ERR_RUNTIME
 * ("a bounded wait in the PCG kernels gave up").  The context stays usable.  Process-wide,
 * read at each launch; polls < 0 restores the default (2^22).  A small value (0: give up
 * without polling) makes the waits run out on purpose, to test a caller's error path. */
void symxg_set_wait_poll_limit(int64_t polls);
int64_t symxg_wait_poll_limit(void);

/* ---- stand-alone kernels on caller-owned DEVICE memory (stream: a cudaStream_t or NULL) ---- */

/* Project `count` symmetric n x n matrices (n = 3k <= 30), stored block-major (3x3 block
 * (a,b) at offset (a*k+b)*9, row-major inside), in place.  not_converged: device int set
 * to 1 if a Jacobi sweep cap was hit.  Replaces project_to_PD_inplace
 * (symx/src/solver/second_order/project_to_PD.cpp:12-81).  n = 3..12 run one matrix per
 * thread in registers, n = 18, 24, 30 one matrix per warp in shared memory.  n = 15, 21, 27
 * run one matrix per thread with the matrix and its eigenvectors in local memory: the first
 * such call makes the driver reserve local memory for every thread the device can hold
 * (several GB in f64), which the context keeps until it is destroyed. */
int symxg_project_pd_f32(float* matrices, int32_t n, int64_t count, float eps, int32_t mirroring,
                         int32_t* not_converged, void* stream);
int symxg_project_pd_f64(double* matrices, int32_t n, int64_t count, double eps, int32_t mirroring,
                         int32_t* not_converged, void* stream);
/* y = A x for a 3x3-block CSR matrix: row_ptr (n_blocks+1), cols (nnzb) and values stored
 * component-major, i.e. component m (row-major inside the 3x3 block) of block k at
 * vals[m * vals_stride + k], vals_stride >= nnzb (the layout the solver's PCG uses).
 * The SpMV runs asynchronously and cannot read row_ptr[n_blocks] back, so vals_stride >= nnzb
 * is the caller's to ensure (the PCG calls below check it).
 * Replaces BlockedSparseMatrix::spmxv_from_ptr (BlockedSparseMatrix.h:986-1138). */
int symxg_bcsr_spmv_f32(int32_t n_blocks, const int32_t* row_ptr, const int32_t* cols, const float* vals,
                        int64_t vals_stride, const float* x, float* y, void* stream);
int symxg_bcsr_spmv_f64(int32_t n_blocks, const int32_t* row_ptr, const int32_t* cols, const double* vals,
                        int64_t vals_stride, const double* x, double* y, void* stream);

/* Outcome of a PCG solve: the fields of bsm::PCGInfo (solve_pcg.h:21-27), plus the number of
 * block rows without a diagonal block (nonzero: the solve did not run, call fails). */
typedef struct symxg_pcg_info {
    int32_t converged;
    int32_t n_iterations;
    double error;                  /* sqrt(r.r / b.b) at exit */
    int32_t found_indefiniteness;  /* p.Ap <= 0 met (the solve stops there) */
    int32_t missing_diagonal;
} symxg_pcg_info;

/* Solve A x = b with block-Jacobi PCG on the device: A as for symxg_bcsr_spmv_*, b and x
 * (3 * n_blocks) device arrays, x starting at zero.  Stops when sqrt(r.r/b.b) < abs_tol, when
 * it falls below rel_tol times its initial value, on p.Ap <= 0, or after max_iterations.
 * Every row must hold its diagonal block; vals_stride below row_ptr[n_blocks] fails with
 * SYMXG_ERR_INVALID_ARGUMENT before any kernel runs.  Allocates its workspace (about 150 bytes per block
 * row in f32, 300 in f64) on each call and returns with `stream` synchronized.  Replaces
 * BlockedSparseMatrix::prepare_preconditioning (BlockedSparseMatrix.h:1147) followed by
 * bsm::solve_pcg (solve_pcg.h:83-232), as NewtonsMethod.cpp:427-446 calls them. */
int symxg_bcsr_pcg_f32(int32_t n_blocks, const int32_t* row_ptr, const int32_t* cols, const float* vals,
                       int64_t vals_stride, const float* b, float* x, double abs_tol, double rel_tol,
                       int32_t max_iterations, symxg_pcg_info* info, void* stream);
int symxg_bcsr_pcg_f64(int32_t n_blocks, const int32_t* row_ptr, const int32_t* cols, const double* vals,
                       int64_t vals_stride, const double* b, double* x, double abs_tol, double rel_tol,
                       int32_t max_iterations, symxg_pcg_info* info, void* stream);

/* Allocation-free variant of symxg_bcsr_pcg_f32; it has no counterpart in the reference.  Same
 * arguments and results, but the workspace is a static device array sized for
 * SYMXG_PCG_NOALLOC_MAX_BLOCKS block rows (about 9.5 MB per device), so the call allocates no
 * device memory.  It is meant for callers that cannot allocate while they run: all device
 * memory reserved up front by a caching allocator or a fixed budget, or no room for the
 * device-wide wait that cudaFree implies.  Larger systems fail with SYMXG_ERR_INVALID_ARGUMENT
 * before any launch.  The array is shared by all calls on a device: overlapping calls (two
 * threads or two streams at once) race on it, so issue them one after another.  The first
 * call on a device (with that device current) looks up the array's address; if that call is
 * part of a program's set-up, it must come before any stream capture.  Each call clears the
 * reduction tickets and counters it needs zeroed, on its stream, before its first kernel,
 * and returns with `stream` synchronized. */
#define SYMXG_PCG_NOALLOC_MAX_BLOCKS 65536
int symxg_bcsr_pcg_f32_noalloc(int32_t n_blocks, const int32_t* row_ptr, const int32_t* cols, const float* vals,
                               int64_t vals_stride, const float* b, float* x, double abs_tol, double rel_tol,
                               int32_t max_iterations, symxg_pcg_info* info, void* stream);

/* ---- adjoint (no counterpart in the reference; an addition of this library) ----
 *
 * The state x of a step solves g(x; mu, lambda, x0, v0) = 0 (g the gradient of the step's
 * energy).  For a loss L(x), with H lambda_adj = dL/dx (H the true Hessian at x), the
 * gradient of L with respect to any input q of the energy is -lambda_adj . dg/dq; the
 * mixed derivatives dg/dq are differentiated symbolically from the same potentials. */
typedef struct symxg_adjoint_info {
    int32_t converged;
    int32_t iterations;   /* PCG iterations of the adjoint solve */
    double error;         /* sqrt(r.r / b.b) at exit */
} symxg_adjoint_info;

/* At the current device state (after symxg_solve / symxg_solve_device): solve
 * H lambda = dLdx (n_vertices*3) in the handle's precision (PCG to rel_tol), then
 * dLdmu[e] = -lambda . dg/dmu_e, dLdlambda[e] = -lambda . dg/dlambda_e (n_elements each),
 * dLdx0 = -lambda . dg/dx0 and dLdv0 = -lambda . dg/dv0 (n_vertices*3; zero without inertia).
 * Every output may be NULL.  For E-scaled parameters p_e = ln E_e (mu, lambda proportional
 * to E_e): dL/dp_e = mu_e dLdmu[e] + lambda_e dLdlambda[e]. */
int symxg_adjoint(symxg_solver* solver, const double* dLdx, double rel_tol, int32_t max_iterations, double* lambda,
                  double* dLdmu, double* dLdlambda, double* dLdx0, double* dLdv0, symxg_adjoint_info* info);

typedef struct symxg_rollout_info {
    int32_t steps;
    int32_t checkpoints;
    int32_t newton_iterations;   /* forward solves, including the recomputed ones */
    int32_t cg_iterations;
    int32_t recomputed_steps;
    int32_t adjoint_iterations;  /* PCG iterations of all adjoint solves */
    int32_t armijo_polished_steps; /* steps finished with full Newton steps after an Armijo stall */
    int32_t pad;
    double seconds_forward;
    double seconds_backward;
} symxg_rollout_info;

/* n_steps implicit-Euler steps from the handle's state (x0, v0 as set by symxg_set_state):
 * each step runs Newton from x = x0, then x0 <- x, v0 <- (x - x0_old) / dt.  The state before
 * every checkpoint_every-th step is kept (host memory) for symxg_rollout_backward.  On
 * return symxg_get_positions gives the final positions. */
int symxg_rollout_forward(symxg_solver* solver, int32_t n_steps, int32_t checkpoint_every, symxg_rollout_info* info);
/* Reverse-time adjoint of the last forward rollout for a loss of the final state
 * (dLdx_final, dLdv_final (may be NULL) with respect to x_N and v_N): recomputes each segment
 * from its checkpoint, then per step solves H lambda = dL/dx_{n+1} + dL/dv_{n+1} / dt and
 * propagates through the mixed derivatives to (x_n, v_n) and the material.  Outputs (each
 * may be NULL): dL/dx_0, dL/dv_0 (n_vertices*3), dL/dmu, dL/dlambda (n_elements). */
int symxg_rollout_backward(symxg_solver* solver, const double* dLdx_final, const double* dLdv_final, double rel_tol,
                           int32_t max_iterations, double* dLdx_init, double* dLdv_init, double* dLdmu,
                           double* dLdlambda, symxg_rollout_info* info);

#ifdef __cplusplus
}
#endif

#endif /* SYMX_GB300_H */
