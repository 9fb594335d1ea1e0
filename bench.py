"""Benchmark: Newton step time of SymX's second-order solve path on one GB300.

Workload (the metric's configuration): one implicit-Euler step of a clamped Neo-Hookean
Tet4 cube, 64^3 cells = 274,625 vertices and 1,572,864 tets, dt = 1/60, E = 1e5 Pa,
nu = 0.3, seeded 5%-of-spacing perturbation of the initial positions, solved by projected
Newton (eps 1e-10, block-Jacobi PCG to relative 1e-3, Armijo c = 1e-4) to
max |grad E| < 1e-6.  Synthetic, seeded inputs (symx_gb300.problems, "tet4_64").

A bench step is one complete implicit-Euler step solve from the same initial state.
`value` is the Newton step time: device ms of that solve divided by its Newton
iterations, in mixed precision; the all-FP64 GPU form of the same solve is timed in the
same run (`fp64`).  Inputs stay resident in HBM for `value`; `e2e` times the same solve
through the C ABI with host arrays (state upload + solve + position download each step).

    python bench.py [--steps K] [--warmup W] [--impl ours|reference] [--config tet4_64]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Newton step time at 1.57M tets: mixed-precision vs FP64 GPU, 1e-6 rel residual"
UNIT = "ms"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while a region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


ELEMENT_KINDS = {4: "Tet4", 10: "Tet10 (4 quadrature points)", 8: "Hex8 (2x2x2 Gauss points)"}


def element_kind(p):
    nodes = p["conn"].shape[1]
    if nodes not in ELEMENT_KINDS:
        raise ValueError(f"no bench description for elements with {nodes} nodes")
    return nodes


def workload_name(name, p):
    cfg = __import__("symx_gb300.problems", fromlist=["CONFIGS"]).CONFIGS.get(name, {})
    kind = ELEMENT_KINDS[element_kind(p)]
    cells = "x".join(str(c) for c in cfg.get("cells", ())) or "custom"
    return (f"Neo-Hookean {kind} implicit-Euler step, {cells} cells ({p['X'].shape[0]:,} vertices, "
            f"{p['conn'].shape[0]:,} elements)")


def projection_kernel(p):
    return {4: "k_project_pd_sort<float,12> + k_project_pd_deflated_listed<float,12> + k_project_pd_listed<float,12>",
            10: "k_project_pd_pairs<float,30> (one warp per matrix, pair-block parallel Jacobi)",
            8: "k_project_pd_pairs<float,24> (one warp per matrix, pair-block parallel Jacobi)"}[element_kind(p)]


def working_set(p):
    """Device bytes of the element Hessians (f32) and the BCSR values the timed solve streams."""
    m = 3 * p["conn"].shape[1]
    h_bytes = p["conn"].shape[0] * m * m * 4
    return f"working set > L2 (element Hessians {h_bytes / 1e9:.2f} GB f32, plus the BCSR matrix)"


def spmv_roofline(solver, torch, sg, n_rep=30):
    """Time the BCSR SpMV kernel (the PCG's dominant HBM-bound kernel) on the assembled
    mixed-precision Hessian of the workload, with CUDA events on its stream."""
    rp, cols, vals = solver.assembled_hessian(project=True)
    dev = torch.device("cuda")
    rp_t = torch.tensor(rp, device=dev)
    cols_t = torch.tensor(cols, device=dev)
    vals_t = sg.component_major(torch.tensor(vals, dtype=torch.float32, device=dev))
    n = 3 * (rp.size - 1)
    x = torch.randn(n, dtype=torch.float32, device=dev)
    y = torch.zeros_like(x)
    stream = torch.cuda.current_stream()
    for _ in range(3):
        sg.bcsr_spmv(rp_t, cols_t, vals_t, x, y)  # warm-up
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2
    times = []
    for _ in range(n_rep):
        flush.fill_(1.0)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        sg.bcsr_spmv(rp_t, cols_t, vals_t, x, y)
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b) * 1e-3)
    nnzb, nb = cols.size, rp.size - 1  # vals_t is (9, nnzb): component-major
    algo_bytes = nnzb * (9 * 4 + 4) + (nb + 1) * 4 + n * 4 + n * 4
    t = statistics.median(times)
    return {"nnzb": int(nnzb), "n_block_rows": int(nb), "algorithmic_bytes": int(algo_bytes), "seconds": t}


def run_ours(args):
    import torch

    import symx_gb300 as sg
    from symx_gb300 import problems

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    p = problems.step_problem(args.config)
    solver = sg.ElasticSolver(p)
    # time_kernels: CUDA events around every PCG SpMV / projection launch (roofline, live)
    solver.set_settings(cg_rel_tolerance=1e-3, precision="mixed", time_kernels=1)

    def device_solve(precision, **kw):
        solver.set_settings(precision=precision, **{"projection_fp64_refinement": 0, "cg_residual_replacement": 0,
                                                    "cg_fp64_partial_sums": 0, **kw})
        solver.set_state(p["x_init"], p["x0"], p["v0"])
        solver.upload()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        st = solver.solve_device()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b), st

    # warm-up (also compiles / loads the generated kernels)
    for _ in range(args.warmup):
        device_solve("mixed")
    lc0 = sg.load().symxg_launch_count()
    ms, stats = [], []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            t, st = device_solve("mixed")
            ms.append(t)
            stats.append(st)
    lc1 = sg.load().symxg_launch_count()
    st = stats[-1]
    assert st["solver_return"] == 0 and st["final_residual"] < 1e-6, st
    solver.download()
    x_mixed = solver.get_positions()
    newton_its = st["newton_iterations"]
    ms_step = statistics.mean(ms)

    # all-FP64 GPU form of the same solve
    fp64_ms, fp64_st = [], None
    for i in range(max(1, args.fp64_steps) + 1):
        t, s64 = device_solve("fp64")
        if i > 0:
            fp64_ms.append(t)
        fp64_st = s64
    solver.download()
    x_fp64 = solver.get_positions()

    # the split that keeps the projection's arithmetic, the PCG's residual and its dot-product
    # accumulation in FP64: FP32 Jacobi refined by one FP64 step (12 x 12 element Hessians),
    # FP64 residual replacement every 50 PCG iterations, FP64 sums of the dot partials; and the
    # FP64 form with the same refined projection
    variants = {"mixed_fp64_projection_residual_and_sums": ("mixed", dict(projection_fp64_refinement=1,
                                                                          cg_residual_replacement=50,
                                                                          cg_fp64_partial_sums=1)),
                "fp64_refined_projection": ("fp64", dict(projection_fp64_refinement=1))}
    variant_out, variant_x = {}, {}
    for name, (prec, kw) in variants.items():
        if args.no_variants:
            break
        vms, vst = [], None
        for i in range(max(1, args.fp64_steps) + 1):
            t, vst = device_solve(prec, **kw)
            if i > 0:
                vms.append(t)
        assert vst["solver_return"] == 0 and vst["final_residual"] < 1e-6, vst
        solver.download()
        variant_x[name] = (solver.get_positions(), vst)
        variant_out[name] = {
            "precision": prec, **kw, "ms_per_step": round(statistics.mean(vms), 3),
            "ms_per_newton_step": round(statistics.mean(vms) / vst["newton_iterations"], 4),
            "newton_iterations": vst["newton_iterations"], "cg_iterations": vst["cg_iterations"],
            "cg_residual_replacements": vst["cg_residual_replacements"], "final_residual": vst["final_residual"],
            "stage_seconds": {k: round(vst[k], 6) for k in vst if k.startswith("t_")},
            "vs_fp64_step_speedup": round(statistics.mean(fp64_ms) / statistics.mean(vms), 3)}

    # end to end through the C ABI with host arrays, with the headline's settings (the variants
    # above changed the projection, residual and partial-sum settings)
    solver.set_settings(precision="mixed", projection_fp64_refinement=0, cg_residual_replacement=0,
                        cg_fp64_partial_sums=0)
    e2e_ms, e2e_st = [], None
    for i in range(args.steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        solver.set_state(p["x_init"], p["x0"], p["v0"])
        e2e_st = solver.solve()
        x_host = solver.get_positions()
        t1 = time.perf_counter()
        if i > 0:
            e2e_ms.append((t1 - t0) * 1e3)

    # max over ranks (replicas)
    if world > 1:
        import torch.distributed as dist

        tt = torch.tensor([ms_step], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms_step = float(tt.item())
    if rank != 0:
        return None

    peak, peak_kind = measured_peaks()
    rf = spmv_roofline(solver, torch, sg)
    achieved_standalone = rf["algorithmic_bytes"] / rf["seconds"] / 1e9
    # live PCG SpMV launches of the timed solves: p = z + beta p_old fused, so z and p_old are
    # read and p_new and q written (4 vectors) besides the matrix
    n3 = 3 * rf["n_block_rows"]
    spmv_bytes = rf["nnzb"] * (9 * 4 + 4) + (rf["n_block_rows"] + 1) * 4 + 4 * n3 * 4
    n_spmv = sum(x["spmv_launches"] for x in stats)
    t_spmv = sum(x["spmv_seconds"] for x in stats) / max(1, n_spmv)
    # the one-launch PCG (k_pcg_solve_staged): per iteration the product pass (matrix; z, p_old
    # and q_old read, p and q written: 5 vectors, as it forms q = A z + beta q_old) plus the
    # update's (read x, r, p, q: 4 x 16 B and Dinv 48 B, write x, r, z: 3 x 16 B per row)
    n_pcg_it = sum(x["pcg_solve_iterations"] for x in stats)
    t_pcg_it = sum(x["pcg_solve_seconds"] for x in stats) / max(1, n_pcg_it)
    pcg_it_bytes = spmv_bytes + n3 * 4 + 160 * rf["n_block_rows"]
    if n_pcg_it:
        kernel_name = "k_pcg_solve_staged (all PCG iterations in one cooperative launch; unit = one iteration)"
        roof_bytes, roof_t, roof_n, traffic_key = pcg_it_bytes, t_pcg_it, n_pcg_it, "k_pcg_solve_staged per iteration"
    else:
        kernel_name = "k_pcg_spmv_staged (PCG SpMV with fused direction update, live in the timed solves)"
        roof_bytes, roof_t, roof_n, traffic_key = spmv_bytes, t_spmv, n_spmv, "k_pcg_spmv<float>"
    achieved = roof_bytes / roof_t / 1e9 if roof_n else achieved_standalone
    n_proj = sum(x["project_launches"] for x in stats)
    t_proj = sum(x["project_seconds"] for x in stats) / max(1, n_proj)
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as f:
            traffic = json.load(f).get(traffic_key, {}).get(args.config)
    except (OSError, ValueError):
        traffic = None
    rel_vs_fp64 = float(np.linalg.norm(x_mixed - x_fp64) / np.linalg.norm(x_fp64))
    out = {
        "metric": METRIC,
        "value": round(ms_step / newton_its, 4),
        "unit": UNIT + " per Newton step",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_step, 3),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 Hessian/PCG, f64 energy/gradient/line search",
        "data": f"synthetic (seeded {args.config})",
        "config": {"workload": workload_name(args.config, p),
                   "name": args.config, "precision": "mixed", "newton_iterations": newton_its,
                   "cg_iterations": st["cg_iterations"], "final_residual": st["final_residual"],
                   "l2": working_set(p),
                   "parallelism": "replicas only" if world > 1 else "single GPU"},
        "stage_seconds": {k: round(st[k], 6) for k in st if k.startswith("t_")},
        "fp64": {"ms_per_step": round(statistics.mean(fp64_ms), 3),
                 "ms_per_newton_step": round(statistics.mean(fp64_ms) / fp64_st["newton_iterations"], 4),
                 "newton_iterations": fp64_st["newton_iterations"], "cg_iterations": fp64_st["cg_iterations"],
                 "stage_seconds": {k: round(fp64_st[k], 6) for k in fp64_st if k.startswith("t_")}},
        "mixed_vs_fp64_step_speedup": round(statistics.mean(fp64_ms) / ms_step, 3),
        "variants": variant_out,
        "mixed_vs_fp64_position_rel_err": rel_vs_fp64,
        "e2e": {"value": round(statistics.mean(e2e_ms) / e2e_st["newton_iterations"], 4),
                "unit": UNIT + " per Newton step", "ms_per_step": round(statistics.mean(e2e_ms), 3),
                "h2d_bytes_per_step": int(e2e_st["h2d_bytes"]), "d2h_bytes_per_step": int(e2e_st["d2h_bytes"])},
        "gpu_launches": int((lc1 - lc0) / max(1, args.steps)),
        "gpu_launches_total": int(lc1 - lc0),
        "roofline": {"kernel": kernel_name,
                     "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "algorithmic_bytes": int(roof_bytes), "launch_seconds": roof_t, "launches": int(roof_n),
                     "traffic": traffic},
        "spmv_standalone": {"kernel": "k_bcsr_spmv<float>", "algorithmic_bytes": rf["algorithmic_bytes"],
                            "launch_seconds": rf["seconds"], "achieved_gbs": round(achieved_standalone, 1),
                            "frac": round(achieved_standalone / peak, 4)},
        "projection": {"kernel": projection_kernel(p), "launch_seconds": t_proj, "launches": int(n_proj),
                       "matrices_per_launch": int(p["conn"].shape[0]),
                       "ns_per_matrix": round(t_proj / p["conn"].shape[0] * 1e9, 3) if n_proj else None},
        "clocks": clocks.summary(),
    }
    if args.cpu_baseline:
        out["cpu_baseline"], x_oracle, oracle_stats = cpu_baseline(p, args)
        if x_oracle is not None:
            out["oracle_parity"] = oracle_parity(p, x_oracle, oracle_stats,
                                                 {"mixed": (x_mixed, st), "fp64": (x_fp64, fp64_st), **variant_x})
    return out


def oracle_parity(p, x_oracle, oracle_stats, runs):
    """Final positions of the GPU solves against the oracle's complete FP64 solve of the same
    inputs: relative to |x_oracle| and to the step's displacement |x_oracle - x0|."""
    disp = float(np.linalg.norm(x_oracle - p["x0"]))
    nrm = float(np.linalg.norm(x_oracle))
    out = {"oracle": "FP64 CPU restatement of the reference's solve (complete solve, same inputs)",
           "oracle_newton_iterations": int(oracle_stats["newton_iterations"]),
           "oracle_cg_iterations": int(oracle_stats["cg_iterations"]),
           "oracle_final_residual": float(oracle_stats["final_residual"])}
    for name, (x, st) in runs.items():
        d = float(np.linalg.norm(x - x_oracle))
        out[name] = {"rel_err": d / nrm, "rel_err_displacement": d / disp,
                     "max_abs_err_m": float(np.max(np.abs(x - x_oracle))),
                     "newton_iterations": int(st["newton_iterations"]), "cg_iterations": int(st["cg_iterations"])}
    return out


def oracle_settings(O, n_newton):
    kw = dict(cg_rel_tolerance=1e-3)
    if n_newton > 0:
        kw.update(max_iterations=n_newton, max_iterations_as_success=1)
    return O.default_settings(**kw)


def cpu_baseline(p, args):
    """The oracle restatement of the reference's CPU path on this host's cores, on the same
    solve (all Newton iterations unless --cpu-newton-iterations bounds it)."""
    from oracle import oracle as O

    n = args.cpu_newton_iterations
    P = O.Problem(p, 0)
    threads = O.lib().oracle_num_threads()
    P.set_x(p["x_init"])
    st = P.solve(oracle_settings(O, n))
    its = max(1, st["newton_iterations"])
    what = "the complete" if n <= 0 else f"the first {its} Newton iterations of the"
    x = P.get_x() if n <= 0 and st["solver_return"] == 0 else None
    return {"value": round(st["t_total"] * 1e3 / its, 3), "unit": UNIT + " per Newton step", "cores": threads,
            "kind": "port",
            "sample": f"{what} {args.config} solve (oracle port, OpenMP): {its} Newton / {st['cg_iterations']} CG "
                      f"iterations in {st['t_total']:.1f} s",
            "stage_seconds": {k: round(st[k], 3) for k in ("t_eval", "t_project", "t_assembly", "t_linear_solve",
                                                            "t_line_search")}}, x, st


def run_profile(args):
    """Setup + one warm-up and one timed solve of the workload in one precision (the command
    the ncu captures wrap).  Prints the stage times of the timed solve."""
    import torch

    import symx_gb300 as sg
    from symx_gb300 import problems

    p = problems.step_problem(args.config)
    solver = sg.ElasticSolver(p)
    solver.set_settings(cg_rel_tolerance=1e-3, precision=args.profile_solve)
    if args.profile_split:  # FP64-accurate projection, FP64 residual replacement and partial sums
        solver.set_settings(projection_fp64_refinement=1, cg_residual_replacement=50, cg_fp64_partial_sums=1)
    if args.pcg_two_barrier:
        solver.set_settings(cg_lookahead=0)
    out = None
    for i in range(2):
        solver.set_state(p["x_init"], p["x0"], p["v0"])
        solver.upload()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = solver.solve_device()
        torch.cuda.synchronize()
        out = {"profile_solve": args.profile_solve, "config": args.config, "wall_ms": (time.perf_counter() - t0) * 1e3,
               **{k: st[k] for k in st}}
    print(json.dumps(out))
    return None


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return None
    from oracle import oracle as O
    from symx_gb300 import problems

    p = problems.step_problem(args.config)
    P = O.Problem(p, 0)
    threads = O.lib().oracle_num_threads()
    n = args.cpu_newton_iterations
    per_step, per_solve, its = [], [], 1
    for i in range(args.warmup + args.steps):
        P.set_x(p["x_init"])
        # warm-up steps run a single Newton iteration (they only touch the memory)
        st = P.solve(oracle_settings(O, 1 if i < args.warmup else n))
        if i >= args.warmup:
            its = max(1, st["newton_iterations"])
            per_step.append(st["t_total"] * 1e3 / its)
            per_solve.append(st["t_total"] * 1e3)
    v = statistics.mean(per_step)
    return {
        "impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": UNIT + " per Newton step",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(statistics.mean(per_solve), 3),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic (seeded {args.config})",
        "config": {"workload": workload_name(args.config, p),
                   "name": args.config},
        "cpu_baseline": {"value": round(v, 3), "unit": UNIT + " per Newton step", "cores": threads, "kind": "port",
                         "sample": ("each step: the complete solve" if n <= 0 else f"each step: the first {n} Newton "
                                    f"iterations of the solve") + f" from the same state ({its} Newton iterations)"},
        "e2e": {"value": round(v, 3), "unit": UNIT + " per Newton step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def measure_adjoint(args):
    """Quasistatic adjoint (config 3 sizes by default: tet4_32): forward solve and adjoint in
    FP64 and mixed precision, dL/d(ln E) against the oracle's FP64 adjoint at the FP64 state and
    against central differences (h = 1e-6) of GPU FP64 solves on 16 seeded elements."""
    import torch

    import symx_gb300 as sg
    from oracle import oracle as O
    from symx_gb300 import problems

    cfg = args.config if args.config != "tet4_64" else "tet4_32"
    p = problems.adjoint_problem(cfg)
    # The configuration's stopping rule is |grad E|_inf < 1e-6; near that point the Armijo test
    # stalls on the rounding of the energy, so states used for differences are polished with
    # full Newton steps (no line search) to 1e-8 (the floor is ~3e-9: the 1e8 boundary penalty
    # times the rounding of x).
    settings = dict(residual_tolerance_abs=1e-6, cg_rel_tolerance=1e-3, max_iterations=100)
    polish = dict(residual_tolerance_abs=1e-8, cg_rel_tolerance=1e-10, max_iterations=30,
                  enable_armijo_backtracking=0)

    def solve(q, precision="fp64", x_init=None, polished=True):
        s = sg.ElasticSolver(q)
        s.set_settings(precision=precision, **settings)
        s.set_state(q["x_init"] if x_init is None else x_init, q["x0"], q["v0"])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = s.solve() if x_init is None else {"solver_return": 0, "newton_iterations": 0}
        t = time.perf_counter() - t0
        if st["solver_return"] != 0:
            raise RuntimeError(f"solve failed: {st}")
        if polished:
            s.set_settings(precision=precision, **polish)
            s.set_state(s.get_positions() if x_init is None else x_init, q["x0"], q["v0"])
            st2 = s.solve()
            if st2["solver_return"] != 0:
                raise RuntimeError(f"polish failed: {st2}")
        return s, st, t

    x_star = solve(dict(p, mu=p["mu_target"], lam=p["lam_target"]))[0].get_positions()
    out = {"measure": "adjoint", "config": cfg, "n_vertices": int(p["X"].shape[0]),
           "n_elements": int(p["conn"].shape[0]), "loss": "0.5 |x(p) - x*|^2, p_e = ln E_e"}
    grads = {}
    for precision in ("fp64", "mixed"):
        solve(p, precision, polished=False)  # warm: compiled kernels
        s, st, t_fwd = solve(p, precision, polished=False)  # timed: the configuration's own tolerance
        if precision == "fp64":
            s, _, _ = solve(p, precision)  # polished state for the gradient checks
        x = s.get_positions()
        rel_tol = 1e-12 if precision == "fp64" else 1e-10  # mixed: FP32 PCG inside FP64 defect correction
        s.adjoint((x - x_star).ravel(), rel_tol=rel_tol)  # warm-up (compiles the mixed-derivative kernels)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        a = s.adjoint((x - x_star).ravel(), rel_tol=rel_tol)
        t_adj = time.perf_counter() - t0
        grads[precision] = p["mu"] * a["dLdmu"] + p["lam"] * a["dLdlam"]
        out[precision] = {"forward_s": round(t_fwd, 4), "newton_iterations": st["newton_iterations"],
                          "adjoint_s": round(t_adj, 4), "adjoint_pcg_iterations": a["info"]["iterations"],
                          "adjoint_error": a["info"]["error"]}
        if precision == "fp64":
            x64 = x
    P = O.Problem(p, 0)
    P.set_x(x64)
    ref = O.adjoint(P, p, (x64 - x_star).ravel(), solver="pcg")
    g_ref = p["mu"] * ref["dLdmu"] + p["lam"] * ref["dLdlam"]
    scale = np.max(np.abs(g_ref))
    for precision in ("fp64", "mixed"):
        out[precision]["rel_err_vs_oracle_fp64"] = float(np.max(np.abs(grads[precision] - g_ref)) / scale)
    # central differences of FP64 GPU solves on 16 seeded elements
    h = 1e-6
    elems = problems.splitmix64(31, 16) % p["conn"].shape[0]
    fd = []
    for e in elems:
        vals = []
        for sgn in (1.0, -1.0):
            logE = p["logE"].copy()
            logE[e] += sgn * h
            mu, lam = problems.lame(np.exp(logE), 0.3)
            xx = solve(dict(p, mu=mu, lam=lam), x_init=x64)[0].get_positions()
            vals.append(0.5 * float(np.sum((xx - x_star) ** 2)))
        fd.append((vals[0] - vals[1]) / (2 * h))
    fd = np.array(fd)
    fd_scale = np.max(np.abs(fd))
    for precision in ("fp64", "mixed"):
        out[precision]["max_rel_err_vs_central_differences_16"] = float(
            np.max(np.abs(grads[precision][elems] - fd)) / fd_scale)
    out["central_differences"] = {"h": h, "elements": [int(e) for e in elems], "max_abs_fd": float(fd_scale)}
    # directional central differences over all elements: ln E + t d, d_e = 1 + 0.3 N(0, 1); the
    # summed derivative is large enough that h = 1e-3 resolves it far above the solve floor;
    # Richardson's combination of h and h/2 removes the O(h^2) truncation
    d = 1.0 + 0.3 * problems.normal(32, p["logE"].size)

    def fd_dir(hd):
        vals = []
        for sgn in (1.0, -1.0):
            mu, lam = problems.lame(np.exp(p["logE"] + sgn * hd * d), 0.3)
            xx = solve(dict(p, mu=mu, lam=lam), x_init=x64)[0].get_positions()
            vals.append(0.5 * float(np.sum((xx - x_star) ** 2)))
        return (vals[0] - vals[1]) / (2 * hd)

    hd = 1e-3
    f1, f2 = fd_dir(hd), fd_dir(hd / 2)
    fr = (4.0 * f2 - f1) / 3.0
    out["directional_central_difference"] = {
        "h": [hd, hd / 2], "direction": "d_e = 1 + 0.3 N(0,1), all elements", "fd": [f1, f2], "richardson": fr,
        **{f"rel_err_{pr}_h": float(abs(grads[pr] @ d - f1) / abs(f1)) for pr in ("fp64", "mixed")},
        **{f"rel_err_{pr}_richardson": float(abs(grads[pr] @ d - fr) / abs(fr)) for pr in ("fp64", "mixed")}}
    return out


def measure_rollout(args):
    """Differentiable rollout (config 4 sizes by default: tet4_40, 50 steps, checkpoint every
    10): forward and reverse-time adjoint in FP64 and mixed precision, device memory held by
    the solver, and the gradients along seeded directions of v0 and ln E against central
    differences of FP64 GPU rollouts."""
    import torch

    import symx_gb300 as sg
    from symx_gb300 import problems

    cfg = args.config if args.config != "tet4_64" else "tet4_40"
    n_steps, every = args.rollout_steps, 10
    p = problems.rollout_problem(cfg)
    settings = dict(residual_tolerance_abs=1e-8, cg_rel_tolerance=1e-3, max_iterations=100)

    def forward(q, precision="fp64"):
        s = sg.ElasticSolver(q)
        s.set_settings(precision=precision, **settings)
        s.set_state(q["x_init"], q["x0"], q["v0"])
        info = s.rollout_forward(n_steps, every)
        xN = s.get_positions()
        d = xN.mean(axis=0) - q["target"]
        return s, info, xN, 0.5 * float(d @ d)

    out = {"measure": "rollout", "config": cfg, "n_vertices": int(p["X"].shape[0]),
           "n_elements": int(p["conn"].shape[0]), "steps": n_steps, "checkpoint_every": every,
           "loss": "0.5 |centroid(x_N) - target|^2; gradients wrt v0 and ln E"}
    grads = {}
    lib = sg.load()
    cur, peak = __import__("ctypes").c_int64(), __import__("ctypes").c_int64()
    for precision in ("fp64", "mixed"):
        free0, total = torch.cuda.mem_get_info()
        lib.symxg_device_memory(None, None, 1)  # high-water mark from here
        s, info_f, xN, L = forward(p, precision)
        d = xN.mean(axis=0) - p["target"]
        dLdx = np.tile(d / xN.shape[0], (xN.shape[0], 1))
        g = s.rollout_backward(dLdx, rel_tol=1e-10)  # mixed: FP32 PCG inside FP64 defect correction
        free1, _ = torch.cuda.mem_get_info()
        lib.symxg_device_memory(__import__("ctypes").byref(cur), __import__("ctypes").byref(peak), 0)
        grads[precision] = (g["dLdv0"], p["mu"] * g["dLdmu"] + p["lam"] * g["dLdlam"])
        out[precision] = {"forward_s": round(info_f["seconds_forward"], 3),
                          "backward_s": round(g["info"]["seconds_backward"], 3),
                          "newton_iterations_forward": info_f["newton_iterations"],
                          "recomputed_steps": g["info"]["recomputed_steps"],
                          "armijo_polished_steps": info_f["armijo_polished_steps"] + g["info"]["armijo_polished_steps"],
                          "adjoint_pcg_iterations": g["info"]["adjoint_iterations"],
                          "device_memory_peak_mb": round(peak.value / 2**20, 1),
                          "device_memory_peak_note": "high-water mark of the library's device buffers over the "
                                                     "forward and backward rollout (symxg_device_memory)",
                          "device_memory_held_after_mb": round((free0 - free1) / 2**20, 1), "loss": L}
        del s
    h = 1e-4
    dv = np.tile([1.0, 0.5, -0.3], (p["v0"].shape[0], 1)) + 0.1 * problems.normal(41, p["v0"].size).reshape(-1, 3)
    dp = 1.0 + 0.3 * problems.normal(42, p["logE"].size)

    def fd_v(hh):
        return (forward(dict(p, v0=p["v0"] + hh * dv))[3] - forward(dict(p, v0=p["v0"] - hh * dv))[3]) / (2 * hh)

    def fd_p(hh):
        vals = []
        for sgn in (1.0, -1.0):
            mu, lam = problems.lame(np.exp(p["logE"] + sgn * hh * dp), 0.3)
            vals.append(forward(dict(p, mu=mu, lam=lam))[3])
        return (vals[0] - vals[1]) / (2 * hh)

    # central differences at h and h/2; Richardson's (4 f(h/2) - f(h)) / 3 removes their O(h^2)
    # truncation error
    fv = [fd_v(h), fd_v(h / 2)]
    fp = [fd_p(h), fd_p(h / 2)]
    rv, rp = (4 * fv[1] - fv[0]) / 3, (4 * fp[1] - fp[0]) / 3
    for precision in ("fp64", "mixed"):
        gv, gp = grads[precision]
        out[precision]["rel_err_dv0_direction"] = float(abs(gv @ dv.ravel() - fv[0]) / abs(fv[0]))
        out[precision]["rel_err_dlnE_direction"] = float(abs(gp @ dp - fp[0]) / abs(fp[0]))
        out[precision]["rel_err_dv0_direction_richardson"] = float(abs(gv @ dv.ravel() - rv) / abs(rv))
        out[precision]["rel_err_dlnE_direction_richardson"] = float(abs(gp @ dp - rp) / abs(rp))
    out["central_differences"] = {"h": [h, h / 2], "d_v0": fv, "d_lnE": fp, "d_v0_richardson": rv,
                                  "d_lnE_richardson": rp}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="tet4_64")
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--cpu-newton-iterations", type=int, default=0, help="0: the complete solve")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-variants", action="store_true", help="skip the FP64-projection / residual-replacement runs")
    ap.add_argument("--profile-solve", choices=["mixed", "fp64"], default=None)
    ap.add_argument("--pcg-two-barrier", action="store_true",
                    help="with --profile-solve: the two-barrier one-launch PCG instead of the look-ahead form")
    ap.add_argument("--profile-split", action="store_true",
                    help="with --profile-solve: the FP64 projection / residual / partial-sum settings")
    ap.add_argument("--measure", choices=["adjoint", "rollout"], default=None,
                    help="instead of the bench line: the adjoint (quasistatic) or rollout measurement")
    ap.add_argument("--rollout-steps", type=int, default=50)
    args = ap.parse_args()
    if args.measure:
        out = measure_adjoint(args) if args.measure == "adjoint" else measure_rollout(args)
        print(json.dumps(out))
        return
    rank, world, _ = dist_env()
    if world > 1 and args.impl == "ours":
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(dist_env()[2])
        dist.init_process_group("nccl")
    if args.profile_solve:
        run_profile(args)
        return
    if args.impl == "reference":
        out = run_reference(args)
    else:
        if world > 1 and rank != 0:
            args.cpu_baseline = False
        out = run_ours(args)
    if out is not None and rank == 0:
        print(json.dumps(out))
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
