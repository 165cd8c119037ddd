"""Benchmark: one CheFSI iteration (filter + Rayleigh-Ritz + residuals) on one GB300.

Workload (default, the mixed-precision configuration): periodic cube L = 30 bohr, 20^3 cells,
FE degree 6 (1,728,000 dofs), 64 seeded Gaussian wells with 8 Gaussian projectors each,
1024 wavefunctions, Chebyshev degree 30, filter HX on the tensor cores with FP16-split
operands, FP64 Cholesky and projected eigensolve. Synthetic seeded inputs (the reference
publishes no input decks for this path). A "step" is one CheFSI iteration (chefsi_solve).

Prints one JSON line. With --impl reference it times the CPU oracle (the FP64 restatement
of the reference's CPU CheFSI) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
METRIC = "CheFSI iter time & HX GFLOP/s on 1 GB300: mixed vs FP64 at <=1e-6 Ha Ritz error"


def peaks():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i, v in enumerate(r[5:9])
                          if v.strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


# dram__bytes_read.sum + dram__bytes_write.sum per launch of the filter's tensor-core kernel
# (ncu captures summarised in profiles/): the separate-pass HX kernel on the full workload, and
# the fused step's kernel (None until captured)
TC_TRAFFIC_BYTES = {("mixed", "separate"): 20.33e9 + 8.20e9,
                    # mixed_small captures scaled by 8000 / 512 cells: the shifted step with
                    # FP32 input (1.310 + 0.479 GB), the unshifted kernel (1.302 + 0.470 GB)
                    ("mixed", "folded"): (1.310375e9 + 0.478750e9) * 8000 / 512,
                    ("mixed", "axpby"): (1.302e9 + 0.470e9) * 8000 / 512}


def hx_algorithmic(pr, B, s_h=4, s_x=4, fused=False):
    """Bytes and flops of one filter HX over B vectors (reference formulation):
    flops = 2 n_c n_e^2 B + 4 n_nlc-rows P B; bytes = s_H n_c n_e^2 + 2 s_X M B + 4 n_c n_e.
    A filter step that finishes the recurrence in the same launch (the fused step; the shifted
    default, which reduces a (A - c) x_{k-1} into the buffer of x_{k-2}) also reads x_{k-2}:
    + s_X M B."""
    nc, ne = pr.mesh.n_cells, pr.mesh.nodes_per_cell
    nl_rows = 0 if pr.nonlocal_ is None else int(pr.nonlocal_.ptr[-1])
    P = 0 if pr.nonlocal_ is None else pr.nonlocal_.n_proj
    flops = 2.0 * nc * ne * ne * B + 4.0 * nl_rows * P * B
    bytes_ = s_h * nc * ne * ne + (3.0 if fused else 2.0) * s_x * pr.n_dofs * B + 4.0 * nc * ne
    return flops, bytes_


def build_workload(name, seed):
    from dftfe_gb300 import problems
    return problems.workload(name, seed=seed)


def first_bounds(chefsi, op, n_wfc):
    """First-call bounds of the reference (chefsi.initial_bounds). Its bLow = a0 + (b - a0) N/M
    200 passes b when N/M > 1/200 (small meshes with many wavefunctions); there it is capped at
    the midpoint of [a0, b]. The large workloads (N/M < 1/200) are unchanged."""
    lo, blow, up = chefsi.initial_bounds(op, n_wfc)
    return lo, min(blow, lo + 0.5 * (up - lo)), up


CPU_SAMPLE_VECTORS = 8


class OracleIterations:
    """Real CheFSI iterations of the CPU oracle (the FP64 restatement of the reference's CPU
    solve: filter, RR-GEP, residual norms, bounds update) on a bounded sample of the workload:
    the workload's operator (same mesh, cell matrices and projectors) with n_s of its N
    vectors. The first-call bounds use the workload's N, so the filter polynomial is the one
    the full problem would get."""

    def __init__(self, pr, m, n_s=CPU_SAMPLE_VECTORS):
        from oracle import oracle as orc
        self.orc = orc
        self.pr, self.m, self.n_s = pr, m, min(n_s, pr.n_wfc)
        self.op = orc.OracleOperator(pr.cell_map, pr.cell_mats, pr.inv_sqrt_mass, pr.n_dofs,
                                     projectors=pr.nonlocal_)
        self.threads = orc.lib().oracle_num_threads()
        v0 = np.random.default_rng(0).uniform(0.0, 1.0, pr.n_dofs)
        lo, up = orc.lanczos_bounds(self.op, v0, 20)
        blow = lo + (up - lo) / pr.n_dofs * pr.n_wfc * 200.0
        self.state = orc.SolverState(a0=lo, b_low=min(blow, lo + 0.5 * (up - lo)), b_up=up)
        self.X = np.ascontiguousarray(pr.initial_vectors(self.n_s))
        self.steps = []

    def step(self):
        t0 = time.perf_counter()
        ev, res, self.X = self.orc.solve(self.op, self.X, self.state, m=self.m)
        dt = time.perf_counter() - t0
        self.steps.append(dt)
        return dt

    def extrapolated(self, t_step):
        """Scale a sample iteration to all N vectors: the filter and the HX are linear in N;
        the dense Rayleigh-Ritz products (X^T X, X^T H X, X W: 3 x 2 M N^2 flops) are timed as
        one numpy (M x 128 x 128) product and scaled by (N/128)^2 (labelled as an estimate)."""
        pr, N = self.pr, self.pr.n_wfc
        ns = min(N, 128)
        Xs = np.random.default_rng(1).standard_normal((pr.n_dofs, ns))
        t0 = time.perf_counter()
        S = Xs.T @ Xs
        _ = Xs @ S
        t_gemm = (time.perf_counter() - t0) / 2.0
        return {"value": t_step * N / self.n_s + 3 * t_gemm * (N / ns) ** 2, "unit": "s/iter",
                "kind": "extrapolated",
                "how": f"sample iteration x N/{self.n_s} + 3 dense (M x N x N) products from a "
                       f"timed {pr.n_dofs}x{ns}x{ns} numpy GEMM x (N/{ns})^2"}

    def describe(self):
        return (f"real oracle CheFSI iterations (Chebyshev filter degree {self.m}, RR-GEP, "
                f"residual norms, bounds update) on the workload's operator "
                f"({self.pr.n_dofs} dofs) with {self.n_s} of its {self.pr.n_wfc} vectors")


def cpu_baseline_line(pr, m):
    """cpu_baseline of the bench line: two real oracle iterations on the bounded sample (the
    second timed), and the labelled extrapolation to the full workload."""
    it = OracleIterations(pr, m)
    it.step()
    t = it.step()
    return {"value": t, "unit": "s/iter", "cores": it.threads, "kind": "port",
            "sample": it.describe(), "n_wfc_sample": it.n_s, "steps_run": 2,
            "extrapolated_full_n": it.extrapolated(t)}


def run_reference(args):
    """The reference arm: the reference's CPU CheFSI (the oracle port of it; the reference
    itself cannot be built here) timed on the machine's host cores. Every step is one real
    iteration on the bounded sample; nothing in `value` is scaled."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    pr = build_workload(args.workload, args.seed)
    m = pr.cheb_degree
    it = OracleIterations(pr, m)
    for _ in range(args.warmup):
        it.step()
    t0 = time.perf_counter()
    vals = [it.step() for _ in range(args.steps)]
    wall = time.perf_counter() - t0
    v = float(np.mean(vals))
    line = {"metric": METRIC, "value": v, "unit": "s/iter", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "n_dofs": pr.n_dofs, "n_wfc": pr.n_wfc,
                       "n_wfc_sample": it.n_s, "cheb_degree": m},
            "steps_run": args.warmup + args.steps, "timed_wall_s": wall,
            "cpu_baseline": {"value": v, "unit": "s/iter", "cores": it.threads, "kind": "port",
                             "sample": it.describe()},
            "extrapolated_full_n": it.extrapolated(v),
            "e2e": {"value": v, "unit": "s/iter", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def e2e_pipeline(step, X, n_steps):
    """The iteration end to end through the public API with host buffers: every step copies
    its input block from pinned host memory to the device, runs chefsi_solve (through the
    Python mirror) and copies the rotated block back to pinned host memory. Two device
    buffers and two copy streams pipeline the copies: the upload of step i+1 and the download
    of step i-1 run on the copy engines while step i solves. Also measured: each copy alone
    (the host link's rates)."""
    import torch
    M, N = X.shape
    host_in = torch.empty((M, N), dtype=torch.float64, pin_memory=True)
    host_in.copy_(X)
    host_out = torch.empty((M, N), dtype=torch.float64, pin_memory=True)
    bufs = [torch.empty_like(X), torch.empty_like(X)]
    comp = torch.cuda.current_stream()
    up_s, down_s = torch.cuda.Stream(), torch.cuda.Stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)
    # the copies alone
    a, b, c = ev(), ev(), ev()
    torch.cuda.synchronize()
    a.record(comp)
    bufs[0].copy_(host_in, non_blocking=True)
    b.record(comp)
    host_out.copy_(bufs[0], non_blocking=True)
    c.record(comp)
    torch.cuda.synchronize()
    h2d_ms, d2h_ms = a.elapsed_time(b), b.elapsed_time(c)
    uploaded = [ev() for _ in range(n_steps)]
    solved = [ev() for _ in range(n_steps)]
    downloaded = [None, None]
    torch.cuda.synchronize()
    t0, t1 = ev(), ev()
    t0.record(comp)
    up_s.wait_stream(comp)
    with torch.cuda.stream(up_s):
        bufs[0].copy_(host_in, non_blocking=True)
        uploaded[0].record(up_s)
    for i in range(n_steps):
        if i + 1 < n_steps:
            nb = (i + 1) % 2
            if downloaded[nb] is not None:
                up_s.wait_event(downloaded[nb])
            with torch.cuda.stream(up_s):
                bufs[nb].copy_(host_in, non_blocking=True)
                uploaded[i + 1].record(up_s)
        comp.wait_event(uploaded[i])
        step(bufs[i % 2])
        solved[i].record(comp)
        down_s.wait_event(solved[i])
        with torch.cuda.stream(down_s):
            host_out.copy_(bufs[i % 2], non_blocking=True)
            d = ev()
            d.record(down_s)
        downloaded[i % 2] = d
    comp.wait_stream(down_s)
    t1.record(comp)
    torch.cuda.synchronize()
    e2e_ms = t0.elapsed_time(t1) / n_steps
    return {"value": e2e_ms / 1e3, "unit": "s/iter", "h2d_bytes_per_step": M * N * 8,
            "d2h_bytes_per_step": M * N * 8 + 2 * N * 8, "steps": n_steps,
            "pipeline": "2 device buffers; upload of step i+1 and download of step i-1 overlap "
                        "the solve of step i (copy streams)",
            "h2d_ms_alone": h2d_ms, "d2h_ms_alone": d2h_ms,
            "h2d_gbs": M * N * 8 / (h2d_ms * 1e-3) / 1e9, "d2h_gbs": M * N * 8 / (d2h_ms * 1e-3) / 1e9}


def fp64_leg(pr, op, X, solver, params, up):
    """The FP64 leg of the headline: from the bench's current block and bounds, one CheFSI
    iteration of the project's FP64 GPU path and one mixed iteration, each timed with CUDA
    events (not estimated); the mixed Ritz values against the FP64 ones (occupied and all),
    the largest principal angle between the occupied Ritz subspaces and the largest occupied
    residual norms."""
    import torch
    from dftfe_gb300 import chefsi
    N, nocc = pr.n_wfc, pr.n_occupied
    a0, bl, bu, _ = solver_bounds(solver)
    out, occ = {}, {}
    torch.cuda.empty_cache()
    for mode in ("fp64", "mixed"):
        # the FP64 iteration on a solver of its own (freed after it), the mixed one on the
        # bench's solver (its workspaces exist already)
        sv = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(params) if mode == "fp64" else solver
        sv.reinitSpectrumBounds(a0, bl, bu)
        Xc = X.clone()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        e, r = sv.solve(op, Xc, useMixedPrec=(mode == "mixed"))
        e1.record()
        torch.cuda.synchronize()
        out[mode] = (e.copy(), r.copy(), e0.elapsed_time(e1) / 1e3, sv.timings(mode == "mixed"))
        occ[mode] = Xc[:, :nocc].contiguous()
        del Xc, sv
        torch.cuda.empty_cache()
    # largest principal angle: arcsin of || Qm - Qf (Qf^T Qm) ||_2 (accurate for small angles)
    Qf, Qm = occ["fp64"], occ["mixed"]
    r = Qm - Qf @ (Qf.T @ Qm)
    angle = float(np.arcsin(min(1.0, float(torch.linalg.matrix_norm(r, ord=2)))))
    del occ
    d = np.abs(out["mixed"][0] - out["fp64"][0])
    return {"fp64_s_per_iter": out["fp64"][2], "mixed_s_per_iter_same_block": out["mixed"][2],
            "speedup_mixed_vs_fp64": out["fp64"][2] / out["mixed"][2],
            "ritz_err_vs_fp64_Ha": {"occupied": float(d[:nocc].max()), "all": float(d.max()),
                                    "occupied_states": nocc},
            "subspace_angle_rad": angle,
            "res_occ_max": {"mixed": float(out["mixed"][1][:nocc].max()),
                            "fp64": float(out["fp64"][1][:nocc].max())},
            "fp64_phases_ms": out["fp64"][3],
            "fp64_leg": "one FP64 and one mixed CheFSI iteration from the bench's final block and "
                        "bounds (CUDA events); Ritz errors against the FP64 iteration"}


def fp64_leg_reduced(pr, op, args, up, n_r=512, n_pre=8):
    """The FP64 leg where the full block does not fit twice (the large workload): on the
    workload's operator with n_r vectors (blocks of 256, the workload's degree), n_pre mixed
    iterations from a seeded block (bLow the reference's first-call value for n_r vectors, kept:
    moved to the block's highest Ritz value, the filtered block's overlap outgrows what the
    mixed Gram resolves), then one FP64 and one mixed iteration from the same block and bounds;
    Ritz errors of the mixed iteration against the FP64 one (as for the other workloads, from
    a block the iteration has brought towards convergence)."""
    import torch
    from dftfe_gb300 import chefsi
    N, m, M = pr.n_wfc, pr.cheb_degree, pr.n_dofs
    nocc = n_r // 2
    prm = chefsi.SolverParams(chebyshevOrder=m, chebyWfcBlockSize=256, wfcBlockSize=256,
                              mixed_precision="mixed", rr_precision=args.rr_precision,
                              filter_variant=args.filter)
    lo, blow, up0 = first_bounds(chefsi, op, n_r)
    sv = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(prm)
    sv.reinitSpectrumBounds(lo, blow, up)
    g = torch.Generator(device="cuda")
    g.manual_seed(args.seed + 2)
    X = torch.rand((M, n_r), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
    for _ in range(n_pre):
        ev, _ = sv.solve(op, X, useMixedPrec=True)
        sv.reinitSpectrumBounds(ev[0], blow, up)
    out, occ = {}, {}
    for mode in ("fp64", "mixed"):
        s2 = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(prm)
        s2.reinitSpectrumBounds(ev[0], blow, up)
        Xc = X.clone()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        e, r = s2.solve(op, Xc, useMixedPrec=(mode == "mixed"))
        e1.record()
        torch.cuda.synchronize()
        out[mode] = (e.copy(), r.copy(), e0.elapsed_time(e1) / 1e3)
        occ[mode] = Xc[:, :nocc].contiguous()
        del Xc, s2
        torch.cuda.empty_cache()
    Qf, Qm = occ["fp64"], occ["mixed"]
    angle = float(np.arcsin(min(1.0, float(torch.linalg.matrix_norm(Qm - Qf @ (Qf.T @ Qm), ord=2)))))
    d = np.abs(out["mixed"][0] - out["fp64"][0])
    return {"fp64_leg_reduced": {
        "n_wfc": n_r, "fp64_s_per_iter": out["fp64"][2], "mixed_s_per_iter": out["mixed"][2],
        "ritz_err_vs_fp64_Ha": {"occupied": float(d[:nocc].max()), "all": float(d.max()),
                                "occupied_states": nocc},
        "subspace_angle_rad": angle,
        "res_occ_max": {"mixed": float(out["mixed"][1][:nocc].max()),
                        "fp64": float(out["fp64"][1][:nocc].max())},
        "pre_iterations": n_pre,
        "note": "the workload's operator with 512 of its 4096 vectors: X (134 GB) cannot be held "
                "twice for an FP64 iteration of the full block"}}


def solver_bounds(solver):
    import ctypes
    from dftfe_gb300 import _lib
    lib = _lib.load()
    a0, bl, bu, d = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int32()
    _lib.check(lib.chefsi_solver_get_bounds(solver._handle(True), ctypes.byref(a0), ctypes.byref(bl),
                                            ctypes.byref(bu), ctypes.byref(d)))
    return a0.value, bl.value, bu.value, d.value


def run_ours(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from dftfe_gb300 import build, chefsi
    build.build()
    pr = build_workload(args.workload, args.seed + rank)   # independent replica per rank
    N, m, M = pr.n_wfc, pr.cheb_degree, pr.n_dofs
    op = chefsi.KohnShamOperator.from_problem(pr)
    lo, blow, up = first_bounds(chefsi, op, N)
    # the large workload (4096 vectors) is filtered in blocks of 256, the others in one block
    blk = 256 if args.workload == "large" else N
    # the fused step and the shifted default each finish the recurrence in the HX launch (it
    # reads x_{j-2} as well)
    fused = args.filter in ("fused", "folded")
    params = chefsi.SolverParams(chebyshevOrder=m, chebyWfcBlockSize=blk, wfcBlockSize=blk,
                                 mixed_precision="mixed", rr_precision=args.rr_precision,
                                 filter_variant=args.filter)
    solver = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(params)
    solver.reinitSpectrumBounds(lo, blow, up)
    solver.set_profiling(True, mixed=True)
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed + 1)
    # filled in place: X of the large workload is 134 GB, and temporaries of its size would stay
    # in torch's cache, out of the library's reach
    X = torch.empty((M, N), device=dev, dtype=torch.float64).uniform_(-1.0, 1.0, generator=g)
    torch.cuda.empty_cache()

    large = args.workload == "large"

    def step(Xd):
        ev, res = solver.solve(op, Xd, useMixedPrec=True)
        # the large workload keeps its first-call bounds: 4096 vectors filtered from random ones
        # with bLow at their largest Ritz value (some 28,000 states below it) leave an overlap
        # with condition ~1e10, beyond the 22 bits of the mixed Gram; the cost of an iteration
        # does not depend on the bounds
        if not large:
            solver.reinitSpectrumBounds(ev[0], ev[-1], up)
        return ev, res

    for _ in range(args.warmup):
        step(X)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    hx_n, hx_ms = 0, 0.0
    lib = __import__("dftfe_gb300._lib", fromlist=["load"]).load()
    launches0 = lib.chefsi_launch_count()
    with ClockSampler(local) as clk:
        torch.cuda.nvtx.range_push("timed")
        start.record()
        for _ in range(args.steps):
            ev, res = step(X)
            n_, t_ = solver.hx_stats(True)
            hx_n += n_
            hx_ms += t_
        end.record()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    launches = lib.chefsi_launch_count() - launches0
    if world > 1:
        dist.barrier()
    t_ms = start.elapsed_time(end) / args.steps
    if world > 1:
        from dftfe_gb300 import pools
        t_ms = pools.max_over_ranks(t_ms)
    phases = solver.timings(True)

    # the large workload's X (134 GB) leaves no room for the pipelined copies' device buffers
    # the pipeline's fill (first upload) and drain (last download) are in the timed region; at
    # least 4 steps so that they weigh as in a longer run of iterations
    e2e = None if large else e2e_pipeline(step, X, max(4, min(args.steps, 8)))
    torch.cuda.empty_cache()
    free_b, total_b = torch.cuda.mem_get_info()

    # one filter HX launch covers one column block of blk vectors
    hx_flops, hx_bytes = hx_algorithmic(pr, blk, fused=fused)
    hbm, bf16, src = peaks()
    avg_hx_ms = hx_ms / max(hx_n, 1)
    achieved = hx_bytes / (avg_hx_ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": t_ms / 1e3, "unit": "s/iter", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f16split/f64",
        "data": "synthetic (seeded wells/projectors, X0 ~ U(-1,1)); inputs larger than L2",
        "config": {"workload": args.workload, "n_dofs": M, "n_cells": pr.mesh.n_cells,
                   "fe_degree": pr.mesh.p, "n_wfc": N, "cheb_degree": m,
                   "wells": int(pr.info["n_wells"]),
                   "projectors_per_well": 0 if pr.nonlocal_ is None else pr.nonlocal_.n_proj,
                   "precision": "mixed", "filter_block": blk,
                   "rr_hx_precision": args.rr_precision,
                   "l2": f"inputs > L2 (X is {M * N * 8 / 1e9:.1f} GB)",
                   "filter": args.filter,
                   "parallelism": f"replicas{world}"},
        "hx_gflops": hx_flops / (avg_hx_ms * 1e-3) / 1e9,
        "hx_ms": avg_hx_ms, "hx_launches_timed": hx_n,
        "phases_ms": phases,
        "ritz_sample": [float(ev[0]), float(ev[N // 2]), float(ev[-1])],
        "gpu_launches": None,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm,
                     "traffic": TC_TRAFFIC_BYTES.get((args.workload, args.filter)), "peak_source": src,
                     "traffic_scope": "the filter step's tensor-core kernel launch alone, dram "
                                      "read + write, ncu (profiles/)",
                     "kernel": {"fused": "cell_hx_tc_kernel<FUSED> + nonlocal projection: one "
                                         "filter step (HX, nonlocal, recurrence)",
                                "folded": "cell_hx_tc_kernel with the shift on the tiles' "
                                          "diagonals and the nonlocal apply as extra K columns "
                                          "+ nonlocal projection: one filter step x_j = a (A - c) "
                                          "x_{j-1} + b x_{j-2} reduced into x_{j-2}'s buffer, "
                                          "the FP32 input split by the launch's producer warps",
                                "axpby": "cell_hx_tc_kernel with the nonlocal apply as extra K "
                                         "columns + nonlocal projection (filter HX; recurrence "
                                         "pass not included)",
                                "separate": "cell_hx_tc_kernel + nonlocal kernels (filter HX; "
                                            "recurrence pass not included)"}[args.filter],
                     "algorithmic_bytes_per_launch": hx_bytes},
        "e2e": e2e,
        "device_memory_used_gb": (total_b - free_b) / 1e9,
        "clocks": clk.summary(),
    }
    line["gpu_launches"] = int(launches)
    if not args.no_fp64_leg and world == 1:
        if large:
            # the timed block and its solver's workspaces make room for the reduced leg
            del X, solver
            import gc
            gc.collect()
            torch.cuda.empty_cache()
            line.update(fp64_leg_reduced(pr, op, args, up))
        else:
            line.update(fp64_leg(pr, op, X, solver, params, up))
    if rank == 0 and not args.no_cpu_baseline and world == 1 and not large:
        line["cpu_baseline"] = cpu_baseline_line(pr, m)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_hx_only(args):
    """K launches of the mixed filter HX (tensor-core cell kernel + nonlocal) on FP32 blocks."""
    import torch
    from dftfe_gb300 import build, chefsi
    build.build()
    dev = torch.device("cuda", 0)
    pr = build_workload(args.workload, args.seed)
    N, M = pr.n_wfc, pr.n_dofs
    op = chefsi.KohnShamOperator.from_problem(pr)
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed + 1)
    X = torch.rand((M, N), generator=g, device=dev, dtype=torch.float32) * 2 - 1
    Y = torch.empty_like(X)
    for _ in range(args.warmup):
        op.HX(X, Y, precision="mixed")
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed")
    s.record()
    for _ in range(args.steps):
        op.HX(X, Y, precision="mixed")
    e.record()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / args.steps
    fl, by = hx_algorithmic(pr, N)
    hbm, bf16, src = peaks()
    print(json.dumps({"metric": "filter HX (mixed) time", "value": ms, "unit": "ms",
                      "workload": args.workload, "n_dofs": M, "n_wfc": N,
                      "hx_gflops": fl / (ms * 1e-3) / 1e9,
                      "achieved_gbs": by / (ms * 1e-3) / 1e9, "hbm_peak_gbs": hbm,
                      "algorithmic_bytes": by, "algorithmic_flops": fl}))
    return 0


def run_ritz_check(args):
    """Mixed vs FP64 on the same subspace: after three mixed iterations from X0, one CheFSI
    iteration in FP64 and one in mixed precision start from the same block and bounds; the
    Ritz values are compared (the FP64 ones are the reference) and both iterations timed."""
    import torch
    from dftfe_gb300 import build, chefsi
    build.build()
    pr = build_workload(args.workload, args.seed)
    N, m, M = pr.n_wfc, pr.cheb_degree, pr.n_dofs
    op = chefsi.KohnShamOperator.from_problem(pr)
    lo, blow, up = first_bounds(chefsi, op, N)
    mk = lambda: chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(chefsi.SolverParams(
        chebyshevOrder=m, chebyWfcBlockSize=N, wfcBlockSize=min(N, 512), mixed_precision="mixed",
        rr_precision=args.rr_precision))
    s = mk()
    s.reinitSpectrumBounds(lo, blow, up)
    g = torch.Generator(device="cuda")
    g.manual_seed(args.seed + 1)
    X = torch.rand((M, N), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
    for _ in range(3):
        ev, _ = s.solve(op, X, useMixedPrec=True)
        s.reinitSpectrumBounds(ev[0], ev[-1], up)
    bounds = (ev[0], ev[-1], up)
    out = {}
    nocc = pr.n_occupied
    occ = {}
    for mode in ("fp64", "mixed"):
        sv = mk()
        sv.reinitSpectrumBounds(*bounds)
        Xc = X.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e, r = sv.solve(op, Xc, useMixedPrec=(mode == "mixed"))
        torch.cuda.synchronize()
        out[mode] = (e.copy(), r.copy(), time.perf_counter() - t0, sv.timings(mode == "mixed"))
        occ[mode] = Xc[:, :nocc].contiguous()
        del Xc
    # largest principal angle between the occupied Ritz subspaces (both blocks orthonormal)
    sv_q = np.linalg.svd((occ["fp64"].T @ occ["mixed"]).cpu().numpy(), compute_uv=False)
    angle = float(np.arccos(np.clip(sv_q.min(), -1.0, 1.0)))
    del occ
    e64, e32 = out["fp64"][0], out["mixed"][0]
    d = np.abs(e32 - e64)
    print(json.dumps({
        "metric": "mixed vs FP64 Ritz error (one iteration from the same block)",
        "workload": args.workload, "n_dofs": M, "n_wfc": N, "occupied": nocc,
        "max_abs_err_occupied_Ha": float(d[:nocc].max()), "max_abs_err_all_Ha": float(d.max()),
        "fp64_iter_s": out["fp64"][2], "mixed_iter_s": out["mixed"][2],
        "speedup_mixed_vs_fp64": out["fp64"][2] / out["mixed"][2],
        "fp64_phases_ms": out["fp64"][3], "mixed_phases_ms": out["mixed"][3],
        "res_occ_max_fp64": float(out["fp64"][1][:nocc].max()),
        "res_occ_max_mixed": float(out["mixed"][1][:nocc].max()),
        "subspace_angle_occupied_rad": angle}))
    return 0


def run_spectrum_split_check(args):
    """Spectrum-split Rayleigh-Ritz (rayleighRitzGEPSpectrumSplitDirect) on the workload, with
    the core-state count of DFT-FE's FAST mode on a device (0.8 of the occupied states, floored
    to a multiple of the 128-vector block). After three mixed iterations from X0, (1) one mixed
    CheFSI iteration with the full and with the spectrum-split RR from the same block and
    bounds, phases timed; (2) the RR step alone in FP64 and in mixed precision (fractional
    block FP64, and reduced) on the same filtered block: fractional Ritz values compared with
    the FP64 ones, XFrac spans compared."""
    import torch
    from dftfe_gb300 import build, chefsi
    build.build()
    pr = build_workload(args.workload, args.seed)
    N, m, M = pr.n_wfc, pr.cheb_degree, pr.n_dofs
    blk = 128
    n_core = int(0.8 * pr.n_occupied) // blk * blk
    op = chefsi.KohnShamOperator.from_problem(pr)
    lo, blow, up = first_bounds(chefsi, op, N)
    mk = lambda reduced=False: chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(
        chefsi.SolverParams(chebyshevOrder=m, chebyWfcBlockSize=N, wfcBlockSize=blk,
                            mixed_precision="mixed", rr_precision=args.rr_precision,
                            spectrum_split_frac_reduced=reduced))
    s = mk()
    s.reinitSpectrumBounds(lo, blow, up)
    g = torch.Generator(device="cuda")
    g.manual_seed(args.seed + 1)
    X = torch.rand((M, N), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
    for _ in range(3):
        ev, _ = s.solve(op, X, useMixedPrec=True)
        s.reinitSpectrumBounds(ev[0], ev[-1], up)
    bounds = (ev[0], ev[-1], up)
    it = {}
    for mode in ("full", "split_frac_fp64", "split_frac_reduced"):
        sv = mk(mode == "split_frac_reduced")
        sv.reinitSpectrumBounds(*bounds)
        Xc = X.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if mode == "full":
            e, r = sv.solve(op, Xc, useMixedPrec=True)
        else:
            e, r, XF = sv.solveSpectrumSplit(op, Xc, n_core, useMixedPrec=True)
            del XF
        torch.cuda.synchronize()
        it[mode] = {"iter_s": time.perf_counter() - t0, "phases_ms": sv.timings(True),
                    "res_max_fractional": float(r[-(N - n_core):].max())}
        del Xc
    Xf = X.clone()
    chefsi.chebyshevFilter(op, Xf, m, bounds[1], bounds[2], bounds[0], precision="mixed")
    rr = {}
    spans = {}
    for key, prec, reduced in (("fp64", "fp64", False), ("mixed_frac_fp64", "mixed", False),
                               ("mixed_frac_reduced", "mixed", True)):
        Xc = Xf.clone()
        XF = torch.empty((M, N - n_core), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e = chefsi.rayleighRitzGEPSpectrumSplitDirect(op, Xc, XF, n_core, precision=prec,
                                                      frac_reduced=reduced)
        torch.cuda.synchronize()
        rr[key] = {"ev": e, "s": time.perf_counter() - t0}
        spans[key] = XF
        del Xc
    out = {}
    for key in ("mixed_frac_fp64", "mixed_frac_reduced"):
        d = np.abs(rr[key]["ev"] - rr["fp64"]["ev"])
        sv_q = np.linalg.svd((spans["fp64"].T @ spans[key]).cpu().numpy(), compute_uv=False)
        out[key] = {"rr_s": rr[key]["s"], "max_abs_err_Ha": float(d.max()),
                    "subspace_angle_rad": float(np.arccos(np.clip(sv_q.min(), -1.0, 1.0)))}
    print(json.dumps({
        "metric": "spectrum-split Rayleigh-Ritz: iteration time and fractional Ritz error",
        "workload": args.workload, "n_dofs": M, "n_wfc": N, "occupied": pr.n_occupied,
        "core_states": n_core, "fractional_states": N - n_core,
        "iteration_full_rr": it["full"], "iteration_split_frac_fp64": it["split_frac_fp64"],
        "iteration_split_frac_reduced": it["split_frac_reduced"],
        "rr_fp64_s": rr["fp64"]["s"], "rr_mixed": out}))
    return 0


def run_dm_response_check(args):
    """First-order density-matrix response (densityMatrixEigenBasisFirstOrderResponse) on the
    workload: the Ritz vectors of three mixed CheFSI iterations from X0, their Ritz values, the
    Fermi energy between the occupied states and the next, T = 500 K. H' applies dense cell
    matrices of the workload's shape (the workload's own local cell matrices, without the
    nonlocal part: the cost of a first-order potential operator). FP64 and mixed timed with
    CUDA events (one warm-up call each); the mixed X P' is compared with the FP64 one."""
    import torch
    from dftfe_gb300 import build, chefsi
    build.build()
    pr = build_workload(args.workload, args.seed)
    N, m, M = pr.n_wfc, pr.cheb_degree, pr.n_dofs
    op = chefsi.KohnShamOperator.from_problem(pr)
    op_prime = chefsi.KohnShamOperator(pr.cell_map, pr.cell_mats, pr.sqrt_mass,
                                       pr.inv_sqrt_mass, pr.n_dofs)
    lo, blow, up = first_bounds(chefsi, op, N)
    s = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(chefsi.SolverParams(
        chebyshevOrder=m, chebyWfcBlockSize=N, wfcBlockSize=min(N, 512), mixed_precision="mixed",
        rr_precision=args.rr_precision))
    s.reinitSpectrumBounds(lo, blow, up)
    g = torch.Generator(device="cuda")
    g.manual_seed(args.seed + 1)
    X = torch.rand((M, N), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
    for _ in range(3):
        ev, _ = s.solve(op, X, useMixedPrec=True)
        s.reinitSpectrumBounds(ev[0], ev[-1], up)
    nocc = pr.n_occupied
    mu = 0.5 * (ev[nocc - 1] + ev[nocc])
    res = {}
    for prec in ("fp64", "mixed"):
        Xc = X.clone()
        chefsi.densityMatrixEigenBasisFirstOrderResponse(op_prime, Xc, ev, mu, 500.0,
                                                         precision=prec)
        Xc.copy_(X)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        dmu = chefsi.densityMatrixEigenBasisFirstOrderResponse(op_prime, Xc, ev, mu, 500.0,
                                                               precision=prec)
        e1.record()
        torch.cuda.synchronize()
        res[prec] = (Xc, e0.elapsed_time(e1), dmu)
    err = float((res["mixed"][0] - res["fp64"][0]).abs().max() / res["fp64"][0].abs().max())
    print(json.dumps({
        "metric": "first-order density-matrix response (X^T H' X, recursive Fermi-operator "
                  "expansion, X <- X P')", "workload": args.workload, "n_dofs": M, "n_wfc": N,
        "fermi_energy": mu, "temperature_K": 500.0, "fp64_ms": res["fp64"][1],
        "mixed_ms": res["mixed"][1], "speedup_mixed_vs_fp64": res["fp64"][1] / res["mixed"][1],
        "mixed_max_rel_err_vs_fp64": err,
        "dmu_max_rel_diff": float(np.abs(res["mixed"][2] - res["fp64"][2]).max()
                                  / np.abs(res["fp64"][2]).max())}))
    return 0


def run_density_check(args):
    """Density of the Ritz vectors at the quadrature points (chefsi_density, densityCalculator)
    on the mixed workload: 1024 vectors with occupations 2 for the lowest 512, the (p+3)^3 Gauss
    points of every cell. FP64. Timed with CUDA events; checked against a direct
    interpolate-square-sum (numpy) on 16 seeded cells."""
    import torch
    from dftfe_gb300 import build, chefsi, fe
    build.build()
    pr = build_workload(args.workload, args.seed)
    N, M, mesh = pr.n_wfc, pr.n_dofs, pr.mesh
    op = chefsi.KohnShamOperator.from_problem(pr)
    nq1 = mesh.p + 3
    xq, _ = fe.gauss_nodes_weights(nq1)
    phi, _ = mesh.shape_1d(xq)
    q = np.arange(nq1 ** 3)
    qx, qy, qz = q % nq1, (q // nq1) % nq1, q // (nq1 * nq1)
    i = np.arange(mesh.nodes_per_cell)
    p1 = mesh.p + 1
    shape = phi[qx][:, i % p1] * phi[qy][:, (i // p1) % p1] * phi[qz][:, i // (p1 * p1)]
    _, w3 = mesh.quadrature(nq1)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
    g = torch.Generator(device="cuda")
    g.manual_seed(args.seed + 1)
    X = torch.rand((M, N), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
    occ = np.where(np.arange(N) < N // 2, 2.0, 0.0)
    occ_d, shape_d = t(occ), t(shape)
    jxw_d = t(np.broadcast_to(w3, (mesh.n_cells, len(w3))))
    def timed(prec):
        for _ in range(max(1, args.warmup)):
            r = chefsi.density(op, X, occ_d, shape_d, jxw_d, precision=prec)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(args.steps):
            r = chefsi.density(op, X, occ_d, shape_d, jxw_d, precision=prec)
        e.record()
        torch.cuda.synchronize()
        return r, s.elapsed_time(e) / args.steps

    rho_m, ms_m = timed("mixed")
    rho, ms = timed("fp64")
    mixed_err = float((rho_m - rho).abs().max() / rho.abs().max())
    # direct interpolate-square-sum on 16 seeded cells (FP64 numpy)
    cells = np.random.default_rng(args.seed).choice(mesh.n_cells, 16, replace=False)
    ref = np.empty((16, len(w3)))
    for k, c in enumerate(cells):
        dofs = pr.cell_map[c]
        nodal = pr.inv_sqrt_mass[dofs][:, None] * X[torch.from_numpy(dofs).cuda()].cpu().numpy()
        psi = shape @ nodal
        ref[k] = ((psi * psi) @ occ) * w3
    got = rho[torch.from_numpy(cells).cuda()].cpu().numpy()
    ne, nq, nc = mesh.nodes_per_cell, len(w3), mesh.n_cells
    flops = 2.0 * nc * ne * ne * N + 2.0 * nc * nq * ne * ne
    print(json.dumps({"metric": "density at the quadrature points (FP64)", "value": ms, "unit": "ms",
                      "workload": args.workload, "n_dofs": M, "n_wfc": N, "n_q": nq,
                      "gflops": flops / (ms * 1e-3) / 1e9,
                      "mixed_ms": ms_m, "mixed_max_rel_err_vs_fp64": mixed_err,
                      "mixed_interp_tflops": 2.0 * nc * nq * ne * N / (ms_m * 1e-3) / 1e12,
                      "max_rel_err_vs_direct_16_cells": float(np.abs(got - ref).max() / np.abs(ref).max())}))
    return 0


def run_adjoint_check(args):
    """Adjoint workload: 10^3 cells, degree 4, 256 wavefunctions, loss = sum of the lowest 128
    Ritz values after 5 CheFSI iterations (degree 24, checkpoints every 6); the gradient w.r.t.
    V at every quadrature point against central differences (h = 1e-5, frozen bounds) at 64
    seeded random points and against the density of the 128 states."""
    import torch
    from dftfe_gb300 import adjoint, build
    build.build()
    pr = build_workload("adjoint", args.seed)
    s = adjoint.AdjointSetup.from_problem(pr, n_iter=5, n_sum=128, degree=24, checkpoint=6)
    w3 = pr.mesh.quadrature()[1]
    v0 = torch.from_numpy(pr.info["vjxw"] / w3[None, :]).cuda().contiguous()
    v = v0.clone().requires_grad_(True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L = adjoint.ritz_sum(v, s)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    L.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    g = v.grad.detach()
    _, ev, X, tape = adjoint.run_forward(s, v0)
    rho = adjoint.density_term(s, X)
    s.bounds_per_iter = [t[2] for t in tape]
    rng = np.random.default_rng(args.seed + 7)
    h = 1e-5
    errs, vals = [], []
    gh = g.cpu().numpy()
    for _ in range(64):
        c, q = int(rng.integers(v0.shape[0])), int(rng.integers(v0.shape[1]))
        vp, vm = v0.clone(), v0.clone()
        vp[c, q] += h
        vm[c, q] -= h
        fd = (adjoint.run_forward(s, vp)[0] - adjoint.run_forward(s, vm)[0]) / (2 * h)
        errs.append(abs(fd - gh[c, q]))
        vals.append(abs(fd))
    scale = max(vals)
    out = {"metric": "adjoint check", "workload": "adjoint", "n_dofs": pr.n_dofs, "n_wfc": pr.n_wfc,
           "n_sum": 128, "iterations": 5, "degree": 24, "checkpoint": 6, "loss": float(L),
           "forward_s": t1 - t0, "backward_s": t2 - t1,
           "fd_points": 64, "fd_h": h, "fd_max_abs_err": float(max(errs)),
           "fd_max_rel_err": float(max(errs) / scale), "grad_max_abs": float(scale),
           "grad_vs_density_rel": float(((g - rho).abs().max() / rho.abs().max()).item())}
    print(json.dumps(out))
    return 0


def run_bloch(args):
    """Batched Bloch workload: 32 independent complex Hamiltonians (6^3..14^3 cells at FE
    degree 4, 64..512 wavefunctions, 4..16 wells, k uniform in the first Brillouin zone).
    A step is one CheFSI iteration of every Hamiltonian through chefsi_solve_batched
    (mixed precision: the Bloch filters on the real form of the operators, grouped into one
    recurrence launch and one persistent tensor-core HX launch per degree, replayed as a CUDA
    graph; tensor-core Gram products and rotation; FP64 complex Cholesky and Hermitian
    eigensolve on the worker streams). Also timed: the same batch without grouping on one
    stream and on the worker streams. The batched call is synchronous, so it is timed on the host
    (the library's worker streams are not ordered with a caller event)."""
    import torch
    from dftfe_gb300 import build, chefsi, problems
    build.build()
    dev = torch.device("cuda", 0)
    prs = problems.bloch_set(args.batch, seed=args.seed)
    ops = [chefsi.KohnShamOperator.from_problem(p) for p in prs]
    X0 = [torch.from_numpy(p.initial_vectors()).to(dev) for p in prs]
    bounds = [first_bounds(chefsi, op, p.n_wfc) for op, p in zip(ops, prs)]

    # one filter block per Hamiltonian (chebyWfcBlockSize >= the largest N), so every filter
    # can join the grouped launches
    nmax = max(p.n_wfc for p in prs)

    def fresh():
        solvers = []
        for b in bounds:
            sv = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(
                chefsi.SolverParams(rr_precision=args.rr_precision, chebyWfcBlockSize=nmax,
                                    wfcBlockSize=nmax))
            sv.reinitSpectrumBounds(*b)
            solvers.append(sv)
        return solvers, [x.clone() for x in X0]

    def iterate(solvers, Xs, n_streams, group, count):
        times = []
        for _ in range(count):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            evs, _ = chefsi.solve_batched(solvers, ops, Xs, useMixedPrec=True, n_streams=n_streams,
                                          group=group)
            times.append(time.perf_counter() - t0)
            for sv, ev, b in zip(solvers, evs, bounds):
                sv.reinitSpectrumBounds(ev[0], ev[-1], b[2])
        return times, evs

    results = {}
    for key in [(1, False), (args.streams, False), (args.streams, True)]:
        solvers, Xs = fresh()
        iterate(solvers, Xs, key[0], key[1], args.warmup)
        with ClockSampler() as clk:
            times, evs = iterate(solvers, Xs, key[0], key[1], args.steps)
        results[key] = (float(np.mean(times)), clk.summary(), evs)
    best = results[(args.streams, True)]
    line = {
        "metric": "batched Bloch CheFSI iteration time (32 complex Hamiltonians, mixed)",
        "value": best[0], "unit": "s/iter", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": best[0] * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f16split/f64 complex",
        "data": "synthetic seeded Bloch Hamiltonians",
        "config": {"workload": "bloch", "hamiltonians": len(prs),
                   "meshes": [p.mesh.n for p in prs], "n_wfc": [p.n_wfc for p in prs],
                   "n_dofs_total": int(sum(p.n_dofs for p in prs)), "streams": args.streams},
        "one_stream_ungrouped_s": results[(1, False)][0],
        "streams_ungrouped_s": results[(args.streams, False)][0],
        "batching_speedup": results[(1, False)][0] / best[0],
        "hamiltonian_iters_per_s": len(prs) / best[0],
        "clocks": best[1],
        "ritz_sample": [float(best[2][0][0]), float(best[2][-1][0])],
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="mixed",
                    choices=["mixed", "small", "large", "mixed_small", "bloch"])
    ap.add_argument("--batch", type=int, default=32, help="Hamiltonians in the bloch workload")
    ap.add_argument("--streams", type=int, default=8, help="streams of the batched bloch solve")
    ap.add_argument("--ritz-check", action="store_true",
                    help="one FP64 and one mixed iteration from the same block: Ritz error, times")
    ap.add_argument("--adjoint-check", action="store_true",
                    help="adjoint workload: gradient vs central differences at 64 points")
    ap.add_argument("--hx-only", action="store_true",
                    help="time only the tensor-core filter HX (K launches after W warm-up)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--rr-precision", default="fp32tc", choices=["fp64", "fp32", "fp32tc", "mixed"])
    ap.add_argument("--filter", default="folded", choices=["folded", "fused", "separate", "axpby"],
                    help="mixed filter variant: one tensor-core launch per degree with the "
                         "Chebyshev shift on the tiles' diagonals and the nonlocal apply as extra "
                         "K columns (folded, default), a recurrence pass + that launch without "
                         "the shift (axpby), the recurrence in the HX launch (fused), or "
                         "separate nonlocal kernels (separate)")
    ap.add_argument("--no-fp64-leg", action="store_true",
                    help="skip the FP64 iteration and the Ritz-error comparison after the timed steps")
    ap.add_argument("--density-check", action="store_true",
                    help="time chefsi_density on the workload and check 16 cells against a direct sum")
    ap.add_argument("--spectrum-split-check", action="store_true",
                    help="full vs spectrum-split RR iteration; split RR in FP64 vs mixed")
    ap.add_argument("--dm-response-check", action="store_true",
                    help="time the first-order density-matrix response in FP64 and mixed")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "bloch":
        return run_bloch(args)
    if args.hx_only:
        return run_hx_only(args)
    if args.adjoint_check:
        return run_adjoint_check(args)
    if args.density_check:
        return run_density_check(args)
    if args.spectrum_split_check:
        return run_spectrum_split_check(args)
    if args.dm_response_check:
        return run_dm_response_check(args)
    if args.ritz_check:
        return run_ritz_check(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
