"""Benchmark of the FAS multigrid hot path on GB300.

Workload (one step): solve the 3-D adaptive Poisson problem
poisson3d_nc8_gauss4_seed2 -- 8^3-cell boxes, Dirichlet 0, four seeded
Gaussians, 1.564e7 leaf cells -- from phi = 0 to a relative residual of 1e-8
(max |f - L phi| / max |f| over leaf cells), with FP32 V-cycles inside FP64
defect correction. The metric is V-cycle unknowns/s: leaf cells x V-cycles /
solve time. The same solve with FP64 V-cycles is timed beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU oracle (the C++/OpenMP restatement of the
reference's solver, oracle/) on all host cores, FP64 V-cycles on the same
tree, one solve to 1e-8 per step. Under torchrun each rank solves its own replica
(one tree does not shard; there is no data-path collective).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

TOL = 1e-8
METRIC = "V-cycle unknowns/s, solve to 1e-8 relative residual"
os.environ.setdefault("OMP_PROC_BIND", "close")


def config_of(spec, cells, boxes):
    return {"workload": spec["name"], "leaf_cells": int(cells), "boxes": int(boxes), "tol": TOL,
            "step": "one solve from phi = 0", "l2": "inputs larger than L2 (no flush)"}


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if os.environ.get("AFV_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce(x, world, op):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x, world):
    import torch.distributed as dist
    return _reduce(x, world, dist.ReduceOp.MAX) if world > 1 else x


def sum_over_ranks(x, world):
    import torch.distributed as dist
    return _reduce(x, world, dist.ReduceOp.SUM) if world > 1 else x


class Clocks:
    """nvidia-smi samples of SM clocks and throttle reasons during a region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p is not None:
            time.sleep(0.3)
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                self.out = ""

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def vcycle_bytes(trees, w=4):
    """Algorithmic bytes of one FAS V(2,2) cycle over a set of trees, per
    operator of the reference's schedule (src/m_aX_mg.f90:208-255), each
    input read once and each output written once over its interior, ghost
    fills 2w per face-ghost cell (no edges or corners). On level l above the
    coarsest, with N_l interior cells and G_l face-ghost cells of all its
    boxes: 8 half-sweeps 24 N_l w, their fills 16 G_l w, residual 3 N_l w,
    restriction (2 + 2/2^D) N_l w, fills after restriction and correction
    2 (G_{l-1} + G_l) w, coarse rhs 4 N_l/2^D w, parent difference
    3 N_l/2^D w, correction (2 + 1/2^D) N_l w; the coarsest level's 4
    half-sweeps and fills (12 N + 8 G) w."""
    total = 0.0
    for t in trees:
        inf = t.info()
        D, nc, l0, top = inf["dim"], inf["n_cell"], inf["min_lvl"], inf["highest_lvl"]
        N, G = {}, {}
        for l in range(l0, top + 1):
            ncl = nc if l >= 1 else nc >> (1 - l)
            nb = len(t.level(l)[0])
            N[l], G[l] = nb * ncl ** D, nb * 2 * D * ncl ** (D - 1)
        f = 1.0 / (1 << D)
        total += (12 * N[l0] + 8 * G[l0]) * w
        for l in range(l0 + 1, top + 1):
            total += ((24 + 3 + (2 + 2 * f) + 4 * f + 3 * f + (2 + f)) * N[l] + 16 * G[l]
                      + 2 * (G[l - 1] + G[l])) * w
    return total


def solve_roofline(trees, leaf_cells, cycles, ms, peak, peak_kind):
    """Whole-solve roofline of a mixed solve: per outer iteration the FP32
    V-cycle's algorithmic bytes plus the FP64 defect and accumulate (read u,
    f, write r; read e, read and write u: 48 B per leaf cell), over the
    solve's time."""
    per_iter = vcycle_bytes(trees) + 48.0 * leaf_cells
    total = per_iter * cycles
    achieved = total / (ms / 1e3) / 1e9
    return {"bound": "hbm", "algorithmic_bytes_per_iteration": per_iter, "iterations": cycles,
            "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "counts": "FP32 V(2,2) cycle by operator (vcycle_bytes) + 48 B per leaf cell of FP64 "
                      "defect and accumulate, per iteration; the solve's own CUDA-event time"}


def cpu_model():
    """The host CPU's model name and architecture (lscpu, else /proc/cpuinfo)."""
    import platform
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                name = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not name:
        try:
            with open("/proc/cpuinfo") as f:
                for line in f:
                    if line.lower().startswith(("model name", "cpu model")):
                        name = line.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return "%s (%s)" % (name or "unknown", platform.machine())


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    p = os.path.join(ROOT, "profiles", "roofline_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


def build_workload(spec):
    from afivo_gb300 import workloads as W
    t0 = time.time()
    tree = W.build_tree(spec)
    return tree, time.time() - t0


class OracleSolver:
    """The CPU oracle (C++/OpenMP restatement of the reference solver) on the
    same tree and source: FP64 V-cycles from phi = 0 until the leaf residual
    max |f - L phi| <= TOL * max |f|, the reference's own loop
    (examples/poisson_basic_2d.f90:84-92)."""

    def __init__(self, spec, threads, rhs_interior=None):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle as O
        from helpers import interior_to_ghosted, oracle_tree
        O.build()
        O.set_threads(threads)
        self.O = O
        self.ot = oracle_tree(spec)
        if rhs_interior is None:
            self.ot.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
        else:  # a host-layout interior-only right-hand side
            g = interior_to_ghosted(rhs_interior, self.ot, spec["n_cell"], spec["dim"])
            off = 0
            for lvl in range(self.ot.min_lvl, self.ot.highest_lvl + 1):
                a = self.ot.get_level(lvl, O.I_RHS, spec["n_cell"])
                self.ot.set_level(lvl, O.I_RHS, g[off:off + a.size].reshape(a.shape))
                off += a.size
        self.ot.mg_init()
        self.spec = spec
        self.fmax = self.ot.max_abs(O.I_RHS)
        nc, D = spec["n_cell"], spec["dim"]
        self.leaves = sum(len(self.ot.level(l)[1]) for l in range(self.ot.min_lvl, self.ot.highest_lvl + 1))
        self.boxes = sum(len(self.ot.level(l)[0]) for l in range(self.ot.min_lvl, self.ot.highest_lvl + 1))
        self.cells = self.leaves * nc ** D

    def phi(self):
        """The oracle's phi in the host layout (ghosted)."""
        from helpers import oracle_var
        return oracle_var(self.ot, self.O.I_PHI, self.spec["n_cell"])

    def error_of(self, gpu_phi):
        """max |gpu - oracle| over leaf interiors / max |oracle phi| there, for
        a ghosted host-layout GPU solution."""
        from helpers import leaf_error
        return leaf_error(gpu_phi, self.phi(), self.ot, self.spec["n_cell"], self.spec["dim"])

    def solve(self, max_cycles=60):
        """One solve; returns (V-cycles, seconds, relative residual)."""
        O, ot = self.O, self.ot
        ot.zero(O.I_PHI)
        t0 = time.perf_counter()
        for k in range(1, max_cycles + 1):
            ot.vcycle(set_residual=True)
            rel = ot.max_abs_residual() / self.fmax
            if rel <= TOL:
                break
        return k, time.perf_counter() - t0, rel


def cpu_baseline_sample(spec, threads, seconds=10.0):
    """Oracle solves on the host cores for about `seconds`, after one warm-up
    solve; value = median over solves of leaf cells x V-cycles / solve time."""
    s = OracleSolver(spec, threads)
    s.solve()
    rates, total, n = [], 0.0, 0
    while total < seconds or n < 5:
        c, dt, _ = s.solve()
        rates.append(s.cells * c / dt)
        total += dt
        n += 1
    return statistics.median(rates), total, n, s


def run_reference(args, spec):
    rank, world, local = dist_setup(args.gpus)
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    s = OracleSolver(spec, cores)
    for _ in range(args.warmup):
        s.solve()
    cycles, secs, rels = [], [], []
    for _ in range(args.steps):
        c, dt, rel = s.solve()
        cycles.append(c)
        secs.append(dt)
        rels.append(rel)
    total = sum(secs)
    value = s.cells * sum(cycles) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "unknowns/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(spec, s.cells, s.boxes),
        "solve": {"cycles": cycles, "rel_res": max(rels),
                  "ms_p50": float(np.percentile(secs, 50)) * 1e3,
                  "ms_p99": float(np.percentile(secs, 99)) * 1e3},
        "cpu_baseline": {"value": value, "unit": "unknowns/s", "cores": cores, "kind": "port",
                         "cpu": cpu_model(),
                         "sample": f"{args.steps} FP64 solves of the full tree to {TOL:g} "
                                   f"(oracle: C++/OpenMP restatement of the reference solver, "
                                   f"{cores} threads)"},
        "e2e": {"value": value, "unit": "unknowns/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def _batched_solve_roofline(trees, mine, forest, cyc, ms):
    """solve_roofline of a batch: trees converge after their own number of
    iterations (the solve stops a tree's work when it converges), so each
    tree's bytes count for its own cycles."""
    peak, peak_kind = load_peaks()
    total = 0.0
    for k, i in enumerate(mine):
        t = trees[i]
        total += (vcycle_bytes([t]) + 48.0 * t.leaf_cells()) * int(cyc[k])
    achieved = total / (ms / 1e3) / 1e9
    return {"bound": "hbm", "algorithmic_bytes": total, "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "counts": "per tree: FP32 V(2,2) cycle by operator (vcycle_bytes) + 48 B per leaf cell of FP64 "
                      "defect and accumulate, times the tree's iterations; the batch solve's CUDA-event time",
            "gap": "below 0.6: the 8x8 boxes' half-sweep is bound by the warp's per-box work (about 291 "
                   "warp instructions per box for 32 updated cells, 56-64 % issue active; "
                   "profiles/k_sweep_warp_random2d_c4.md) and by the per-launch latency of levels that give "
                   "each resident warp two boxes; the FP64 defect (520 us per launch, 4 cells per thread) is "
                   "bound by instruction issue too"}


def run_batched(afv, W, local, rank, world, n_trees=256, check_errors=False):
    """Batched 2-D solves: 256 independent random quadtrees in one forest per
    GPU (trees placed over the ranks), one launch per level and operator for
    all of them, autotuned sweep kernel, mixed-precision solve to 1e-8."""
    import torch
    from afivo_gb300 import placement
    specs = W.c4_random_2d(n_trees)
    t0 = time.time()
    trees = [W.build_tree(s) for s in specs]
    t_build = time.time() - t0
    work = [float(t.leaf_cells()) for t in trees]
    mine = placement.shard(list(range(n_trees)), work, rank, world)
    forest = afv.Forest([trees[i] for i in mine], device=local, mixed=True)
    for k, i in enumerate(mine):
        forest.set_source(k, specs[i]["gauss"], lpl=True)
    choice, tune_ms = forest.autotune_all()
    ext = torch.cuda.ExternalStream(forest.stream())

    def solve():
        forest.zero(afv.AFV_PHI)
        cyc, rel, rc = forest.solve(afv.AFV_PREC_MIXED, tol=TOL, max_cycles=60, check=False)
        if rc != 0:
            raise RuntimeError(f"batched solve failed: rc={rc}")
        return cyc, rel

    solve()
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    cyc, rel = solve()
    e1.record(ext)
    e1.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1), world)
    cells = forest.info()["leaf_cells"]
    unknowns = sum(float(t.leaf_cells()) * c for t, c in zip([trees[i] for i in mine], cyc))
    unknowns = sum_over_ranks(unknowns, world)
    total_cells = sum_over_ranks(float(cells), world)
    # per-kernel bandwidth of one profiled solve (kernel by kernel, each
    # iteration behind a 5 ms device-side wait so that the events time the
    # kernels), and the sweep's roofline
    forest.set_option(afv.AFV_OPT_PROFILE_LEAD_US, 5000)
    forest.profile((1 << len(afv.KERNEL_KINDS)) - 1)
    forest.zero(afv.AFV_PHI)
    forest.solve(afv.AFV_PREC_MIXED, tol=TOL, max_cycles=60, check=False)
    kern = {}
    for k, kname in enumerate(afv.KERNEL_KINDS):
        n, kms, kb = forest.profile_read(k)
        if n and kms > 0:
            kern[kname] = {"launches": int(n), "ms": round(kms, 4), "GB/s": round(kb / (kms / 1e3) / 1e9, 1)}
    forest.profile(0)
    forest.set_option(afv.AFV_OPT_PROFILE_LEAD_US, 0)
    peak, peak_kind = load_peaks()
    sw = kern.get("sweep")
    roof = None
    if sw:
        roof = {"kernel": "sweep (chosen variant %d)" % choice["sweep_kernel"], "achieved": sw["GB/s"],
                "peak": peak, "unit": "GB/s", "frac": sw["GB/s"] / peak,
                "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                "gap": "below 0.6: the half-sweep is latency-bound, not bandwidth-bound; each 8x8 box "
                       "(400 B of FP32 cells) needs its descriptor, its cells and 32 scattered ghost "
                       "sources from its neighbours, a chain of dependent L2 round trips, and the level "
                       "stays in L2 between half-sweeps so DRAM moves a fraction of the algorithmic bytes"}
    errors = None
    if check_errors:
        errors = batched_errors(afv, forest, specs, mine)
    out = {"workload": "random2d_256trees_seed4", "trees": n_trees, "leaf_cells": int(total_cells),
           "boxes": int(sum_over_ranks(float(forest.info()["n_boxes"]), world)),
           "ms_per_solve": ms, "unknowns_per_s": unknowns / (ms / 1e3),
           "cycles_min": int(min(cyc)), "cycles_max": int(max(cyc)), "rel_res_max": float(max(rel)),
           "autotune_choice": choice, "autotune_ms_per_vcycle": {k: round(v, 3) for k, v in tune_ms.items()},
           "kernels_mixed_solve": kern, "roofline": roof,
           "solve_roofline": _batched_solve_roofline(trees, mine, forest, cyc, ms),
           "tree_build_s": round(t_build, 2), "err_vs_fp64_oracle": errors}
    forest.close()
    return out


def batched_errors(afv, forest, specs, mine):
    """Per tree, the mixed solution in the forest against the oracle's FP64
    solve of the same tree to the same tolerance (max over leaf interiors,
    relative to max |phi|)."""
    cores = os.cpu_count() or 1
    errs = []
    for k, i in enumerate(mine):
        s = OracleSolver(specs[i], cores)
        s.solve()
        errs.append(s.error_of(forest.get_var(k, afv.AFV_PHI)))
    worst = int(np.argmax(errs))
    return {"max": float(max(errs)), "median": float(np.median(errs)), "worst_tree": mine[worst],
            "per_tree": [float("%.3g" % e) for e in errs],
            "note": "mixed solution vs the oracle's FP64 solve to the same tolerance, max over "
                    "leaf interiors / max |phi|"}


def _leaf_cells(spec):
    """Leaf cells of a uniform request tree (8^3 boxes to level lvl_max)."""
    side = spec["n_cell"] * 2 ** (spec["lvl_max"] - 1)
    return float(side ** spec["dim"])


def run_serving(afv, W, local, rank, world, n_requests=500, keep_ids=()):
    """Served 3-D requests (Poisson arrivals, mean 200/s; uniform octrees of
    8^3 boxes from 32^3 to 256^3 cells): resident per-shape forests under an
    HBM budget, continuous batching, mixed and FP64. Each rate's run follows
    one run that warms the resident forests; p50/p99 latency with its
    queueing and service parts, solves/s; then the same stream at half the
    served rate (below capacity)."""
    from afivo_gb300 import placement, serving
    reqs = W.c5_requests(n=n_requests)
    work = [_leaf_cells(r) for r in reqs]
    mine = placement.shard(list(range(len(reqs))), work, rank, world)
    mreqs = [reqs[i] for i in mine]
    out = {"workload": "poisson3d_requests_seed5", "requests": len(reqs),
           "shapes": len({serving.shape_key(r) for r in reqs})}
    kept = {}
    for name, prec in (("mixed", afv.AFV_PREC_MIXED), ("fp64", afv.AFV_PREC_FP64)):
        keep = {k for k, i in enumerate(mine) if i in keep_ids}
        srv = serving.Server(device=local, budget_bytes=32 << 30, slots=4, max_batch=8, precision=prec,
                             keep_phi=keep)
        srv.serve(mreqs, realtime=False)  # builds the resident forests (a server that has been running)
        res = srv.serve(mreqs, realtime=True)
        summ = serving.summary(res)
        rate = float(len(mreqs) / (mreqs[-1]["arrival"] - mreqs[0]["arrival"]))
        low = 0.5 * min(summ["solves_per_s"], rate)
        slow = [dict(r, arrival=r["arrival"] * rate / low) for r in mreqs]
        res_low = srv.serve(slow, realtime=True)
        summ_low = serving.summary(res_low)
        for sm in (summ, summ_low):
            sm["p99_ms"] = max_over_ranks(sm["p99_ms"], world)
            sm["solves_per_s"] = sum_over_ranks(sm["solves_per_s"], world)
            sm["unknowns_per_s"] = sum_over_ranks(sm["unknowns_per_s"], world)
        summ["offered_per_s"] = rate
        summ_low["offered_per_s"] = low
        summ["peak_device_bytes"] = srv.last_peak_bytes
        f6 = lambda v: float("%.6g" % v) if isinstance(v, float) else v  # noqa: E731
        out[name] = {k: f6(v) for k, v in summ.items()}
        out[name]["below_capacity"] = {k: f6(v) for k, v in summ_low.items()}
        if name == "mixed":
            kept = {mine[k]: res[k].phi for k in keep}
        srv.close()
    return out, reqs, kept


def run_uniform(afv, W, local, rank, world, check_errors=False):
    """2-D uniform periodic case: 16x16 boxes, 4096^2 cells, white-noise
    source with zero mean (seed 3); FMG followed by V-cycles to 1e-8, FP64
    and mixed, with the per-kernel bandwidth of one mixed solve. The
    periodic problem is singular; its source has zero mean, so the residual
    converges without subtracting the mean of phi."""
    import torch
    spec = W.c3_uniform_2d()
    tree = W.build_tree(spec)
    forest = afv.Forest([tree], device=local, mixed=True)
    info = forest.info()
    nc = spec["n_cell"]
    rng = np.random.default_rng(3)
    parts = []
    for lvl in range(tree.min_lvl, tree.highest_lvl + 1):
        n = len(tree.level(lvl)[0]) * tree.n_cell_at(lvl) ** 2
        parts.append(rng.standard_normal(n) if lvl == tree.highest_lvl else np.zeros(n))
    top = parts[-1]
    top -= top.mean()
    rhs_int = np.concatenate(parts)
    forest.set_var(0, afv.AFV_RHS, rhs_int, interior_only=True)
    ext = torch.cuda.ExternalStream(forest.stream())
    out = {"workload": spec["name"], "leaf_cells": info["leaf_cells"], "boxes": info["n_boxes"]}
    solutions = {}
    for name, prec in (("mixed", afv.AFV_PREC_MIXED), ("fp64", afv.AFV_PREC_FP64)):
        def run():
            forest.zero(afv.AFV_PHI)
            forest.fmg(set_residual=False, have_guess=False)
            cyc, rel, rc = forest.solve(prec, tol=TOL, max_cycles=60, check=False)
            return int(cyc[0]), float(rel[0]), rc
        run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        cyc, rel, rc = run()
        e1.record(ext)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        out[name] = {"fmg_then_cycles": cyc, "rel_res": rel, "status": rc, "ms": round(ms, 3),
                     "unknowns_per_s": info["leaf_cells"] * (cyc + 1) / (ms / 1e3)}
        if check_errors:
            solutions[name] = forest.get_var(0, afv.AFV_PHI)
    if check_errors:
        # the oracle's FP64 FMG followed by V-cycles to the same tolerance
        s = OracleSolver(spec, os.cpu_count() or 1, rhs_interior=rhs_int)
        s.ot.fmg(set_residual=True, have_guess=False)
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from helpers import oracle_solve
        n = oracle_solve(s.ot, TOL)
        for name, phi in solutions.items():
            out[name]["err_vs_fp64_oracle"] = s.error_of(phi)
        out["oracle_fmg_then_cycles"] = n
    forest.profile((1 << len(afv.KERNEL_KINDS)) - 1)
    forest.zero(afv.AFV_PHI)
    forest.solve(afv.AFV_PREC_MIXED, tol=TOL, max_cycles=60, check=False)
    kern = {}
    for k, kname in enumerate(afv.KERNEL_KINDS):
        n, kms, kb = forest.profile_read(k)
        if n and kms > 0:
            kern[kname] = {"launches": int(n), "ms": round(kms, 4), "GB/s": round(kb / (kms / 1e3) / 1e9, 1)}
    forest.profile(0)
    out["kernels_mixed_solve"] = kern
    forest.close()
    return out


def serving_picks(n_requests, n=8):
    return list(range(0, n_requests, max(1, n_requests // n)))[:n]


def run_next_rows(afv, W, local, threads):
    """The rows beyond the solver, each on a full-size tree with the oracle
    (the C++/OpenMP restatement, on `threads` host cores) timed beside it as
    that row's CPU baseline, and the GPU result compared with the oracle's:
    the device tree build (C2's tree refined on the device), the operator
    variants (one FP64 V-cycle of lpld, auto and lpllsf on the C2 tree, clpl
    on a cylindrical 2-D tree), the ghost-cell and transfer utilities on the
    C2 tree, and the VTK writer (C1's leaves). GPU times include the call's
    host side and a synchronisation."""
    import shutil
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle as O
    from helpers import (bval_field, compare_var, cyl_spec, fill_from_centres, lsf_sphere, oracle_tree,
                         oracle_var)
    O.build()
    O.set_threads(threads)
    out = {"cores": threads}

    def timed(fn, sync, reps=1):
        fn()
        sync()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        sync()
        return 1e3 * (time.perf_counter() - t0) / reps

    def once(fn):
        t0 = time.perf_counter()
        fn()
        return 1e3 * (time.perf_counter() - t0)

    spec = W.c2_poisson_3d()
    nc, D = spec["n_cell"], spec["dim"]

    # device tree build: the C2 refinement from the base box
    box = {}
    t_host = once(lambda: box.__setitem__("host", W.build_tree(spec)))
    base = afv.Tree(D, nc, spec["dr"], coarsen_to=spec["coarsen_to"]).set_base(spec["ix"], spec["nb"])
    dt = afv.DeviceTree(base, device=local)
    t_dev = once(lambda: dt.refine_builtin(spec["crit"], spec["lvl_max"], thr=spec["thr"], gauss=spec["gauss"],
                                          lpl=spec["lpl"]))
    n_dev = dt.info()["n_boxes"]
    dt.close()
    t_orc = once(lambda: box.__setitem__("oracle", oracle_tree(spec)))
    ot = box["oracle"]
    n_host = box["host"].info()["n_boxes"]
    out["device_tree_build"] = {"workload": spec["name"], "boxes": n_dev, "same_box_count": n_dev == n_host,
                                "device_ms": round(t_dev, 2), "host_ms": round(t_host, 2),
                                "oracle_ms": round(t_orc, 2)}

    # operator variants: one FP64 V-cycle from the same state on GPU and oracle
    ops = {}
    ot.fill_gauss(O.I_RHS, spec["gauss"], lpl=True)
    ot.mg_init()
    ot.add_vars(3, 0)
    eps = fill_from_centres(ot, 3, lambda r: np.where(r[..., 0] > 0.53, 100.0, 1.0), nc)
    lsf = fill_from_centres(ot, 4, lsf_sphere, nc)
    bval = fill_from_centres(ot, 5, bval_field, nc)
    rhs = oracle_var(ot, O.I_RHS, nc)
    f = afv.Forest([box["host"]], device=local)
    f.add_vars(3, 0)
    for iv, a in ((3, eps), (4, lsf), (5, bval), (afv.AFV_RHS, rhs)):
        f.set_var(0, iv, a)
    cells = f.info()["leaf_cells"]
    all_cells = f.info()["n_boxes"] * nc ** D
    for name, op, args in (("lpld", 1, (3, -1, -1)), ("auto_eps", 2, (3, -1, -1)), ("lpllsf", 5, (-1, 4, 5))):
        f.zero(afv.AFV_PHI)
        ot.zero(O.I_PHI)
        f.set_operator(op, *args)
        assert ot.set_operator(op, *args)
        g_ms = timed(lambda: f.vcycle(set_residual=False), f.sync, reps=1)  # two cycles run
        o_ms = once(lambda: ot.vcycle(set_residual=False))
        ot.vcycle(set_residual=False)
        err = compare_var(f.get_var(0, afv.AFV_PHI), oracle_var(ot, O.I_PHI, nc), ot, nc, D, False)
        ops[name] = {"gpu_ms_per_vcycle": round(g_ms, 3), "oracle_ms_per_vcycle": round(o_ms, 1),
                     "speedup": round(o_ms / g_ms, 1), "max_rel_diff_vs_oracle": err}
    f.set_operator(0)
    f.close()
    cs = cyl_spec(lvl_max=10)
    cot = oracle_tree(cs)
    cot.fill_gauss(O.I_RHS, cs["gauss"], lpl=True)
    cot.mg_init()
    cf = afv.Forest([W.build_tree(cs)], device=local)
    cf.set_var(0, afv.AFV_RHS, oracle_var(cot, O.I_RHS, cs["n_cell"]))
    cf.set_operator(3)
    assert cot.set_operator(3)
    g_ms = timed(lambda: cf.vcycle(set_residual=False), cf.sync, reps=1)
    o_ms = once(lambda: cot.vcycle(set_residual=False))
    cot.vcycle(set_residual=False)
    err = compare_var(cf.get_var(0, afv.AFV_PHI), oracle_var(cot, O.I_PHI, cs["n_cell"]), cot, cs["n_cell"], 2,
                      False)
    ops["clpl_cylindrical_2d"] = {"leaf_cells": cf.info()["leaf_cells"], "gpu_ms_per_vcycle": round(g_ms, 3),
                                  "oracle_ms_per_vcycle": round(o_ms, 1), "speedup": round(o_ms / g_ms, 1),
                                  "max_rel_diff_vs_oracle": err}
    cf.close()
    out["operators"] = {"workload": spec["name"], "leaf_cells": cells, "cells_all_levels": all_cells, **ops}

    # ghost cells, transfers and fluxes on the C2 tree, random data
    rng = np.random.default_rng(12)
    ot.add_vars(1, 1)  # cell variable 6, face variable 0
    g = afv.Forest([box["host"]], device=local)
    g.add_vars(4, 1)
    for iv in (3, 6):
        parts = []
        for lvl in range(ot.min_lvl, ot.highest_lvl + 1):
            a = rng.standard_normal(ot.get_level(lvl, iv, nc).shape)
            ot.set_level(lvl, iv, a)
            parts.append(a.ravel())
        g.set_var(0, iv, np.concatenate(parts))
    fcv = rng.standard_normal(g.fc_count(0))
    ot.set_fc(0, fcv)
    g.set_fc(0, 0, fcv)
    top = ot.highest_lvl
    ghost_vals = f_cells = 0
    for lvl in range(ot.min_lvl, top + 1):
        nb = len(ot.level(lvl)[0])
        ncl = ot.n_cell_at(lvl, nc)
        ghost_vals += nb * 2 * D * ncl ** (D - 1)
        f_cells += nb * ncl ** D
    tr = {}
    steps = (
        ("gc_tree_interp", lambda: g.gc_tree_var(3, rb=afv.AFV_RB_INTERP, bc=afv.AFV_BCM_DIRICHLET_ZERO),
         lambda: ot.gc_tree_var(3, rb=2, bc=-1), 3, 2 * 8 * ghost_vals),
        ("prolong2_finest", lambda: g.prolong(top - 1, 6, 6, order=2),
         lambda: ot.prolong(top - 1, 6, 6, order=2), 6, None),
        ("restrict_tree", lambda: g.restrict_tree(3, 6), lambda: ot.restrict_tree(3, 6), 6, None),
        ("consistent_fluxes", lambda: g.consistent_fluxes([0]), lambda: ot.consistent_fluxes([0]), None, None),
    )
    for name, gf, of, iv, nbytes in steps:
        g_ms = timed(gf, g.sync, reps=1)
        o_ms = once(of)
        of()  # the GPU ran it twice; so does the oracle
        if iv is not None:
            same = bool(np.array_equal(g.get_var(0, iv), oracle_var(ot, iv, nc)))
        else:
            same = bool(np.array_equal(g.get_fc(0, 0), ot.get_fc(0)))
        tr[name] = {"gpu_ms": round(g_ms, 3), "oracle_ms": round(o_ms, 1), "speedup": round(o_ms / g_ms, 1),
                    "bit_identical": same}
        if nbytes:
            tr[name]["GB/s"] = round(nbytes / (g_ms / 1e3) / 1e9, 1)
    g.close()
    out["transfer"] = {"workload": spec["name"], "cells_all_levels": f_cells, **tr}

    # VTK output of C1's leaves (phi holding the source)
    s1 = W.c1_poisson_2d()
    vot = oracle_tree(s1)
    vot.fill_gauss(O.I_PHI, s1["gauss"], lpl=True)
    vf = afv.Forest([W.build_tree(s1)], device=local)
    vf.set_var(0, afv.AFV_PHI, oracle_var(vot, O.I_PHI, s1["n_cell"]))
    d = tempfile.mkdtemp(prefix="afv_vtk_")
    try:
        g_ms = timed(lambda: vf.write_vtk(0, os.path.join(d, "gpu"), [afv.AFV_PHI], ["phi"]), lambda: None)
        o_ms = once(lambda: vot.write_vtk(os.path.join(d, "orc.vtu"), [O.I_PHI], ["phi"]))
        a = open(os.path.join(d, "gpu.vtu"), "rb").read()
        b = open(os.path.join(d, "orc.vtu"), "rb").read()
        out["vtk"] = {"workload": s1["name"], "bytes": len(a), "gpu_ms": round(g_ms, 2), "oracle_ms": round(o_ms, 2),
                      "byte_identical": a == b}
    finally:
        shutil.rmtree(d, ignore_errors=True)
    vf.close()
    return out


def cpu_serving_sample(reqs, threads, picks, served_phi):
    """The oracle's FP64 solve of a sample of the requests on the host cores
    (one after another, as a CPU server would): its time per request, and the
    served mixed-precision solution's error against it (max over leaf
    interiors / max |phi|)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import interior_to_ghosted
    times, cells, errs = [], [], []
    for i in picks:
        s = OracleSolver(reqs[i], threads)
        c, dt, _ = s.solve()
        times.append(dt * 1e3)
        cells.append(s.cells * c)
        if served_phi.get(i) is not None:
            errs.append(s.error_of(interior_to_ghosted(served_phi[i], s.ot, 8, 3)))
    return {"sample": f"requests {picks}, solved one at a time on {threads} threads",
            "ms_p50": float(np.percentile(times, 50)), "ms_max": float(max(times)),
            "solves_per_s": len(times) / (sum(times) / 1e3),
            "unknowns_per_s": sum(cells) / (sum(times) / 1e3),
            "err_vs_fp64_oracle": {"max": float(max(errs)) if errs else None,
                                   "per_request": [float("%.3g" % e) for e in errs]}}


def profile_solves(spec, n):
    """n mixed solves of the workload with nothing timed: the command the
    kernel profiles are taken on (few launches before the first V-cycle)."""
    from afivo_gb300 import build as B
    B.build()
    import afivo_gb300 as afv
    tree, _ = build_workload(spec)
    forest = afv.Forest([tree], mixed=True)
    forest.set_source(0, spec["gauss"], lpl=True)
    # stream launches, not the graph: a profiler does not see kernel nodes of
    # a graph with a conditional node
    forest.set_option(afv.AFV_OPT_GRAPHS, 0)
    for _ in range(n):
        forest.zero(afv.AFV_PHI)
        l0 = forest.launches()
        cyc, rel, rc = forest.solve(afv.AFV_PREC_MIXED, tol=TOL, max_cycles=60, check=False)
        print(f"solve: rc {rc}, cycles {int(cyc[0])}, rel {float(rel[0]):.3e}, "
              f"launches {forest.launches() - l0}", flush=True)
        if rc != 0:
            raise SystemExit(1)


def profile_batched(n_trees, sweep_kernel=4):
    """One mixed solve of the first n_trees trees of the 256-tree batch in one
    forest, with the sweep variant the tuning pass picks for that batch (12
    warps x 3 stages) and stream launches: the command the 2-D kernel
    profiles are taken on."""
    from afivo_gb300 import build as B
    B.build()
    import afivo_gb300 as afv
    from afivo_gb300 import workloads as W
    specs = W.c4_random_2d(256)[:n_trees]
    forest = afv.Forest([W.build_tree(s) for s in specs], mixed=True)
    for t, s in enumerate(specs):
        forest.set_source(t, s["gauss"], lpl=True)
    forest.set_option(afv.AFV_OPT_SWEEP_KERNEL, sweep_kernel)
    forest.set_option(afv.AFV_OPT_GRAPHS, 0)
    cyc, rel, rc = forest.solve(afv.AFV_PREC_MIXED, tol=TOL, max_cycles=60, check=False)
    info = forest.info()
    print(f"batch of {n_trees}: rc {rc}, leaf cells {info['leaf_cells']}, boxes {info['n_boxes']}, "
          f"cycles {int(min(cyc))}..{int(max(cyc))}", flush=True)
    if rc != 0:
        raise SystemExit(1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--small", action="store_true", help="smaller tree (quick checks)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 256-tree batched solve")
    ap.add_argument("--no-serving", action="store_true", help="skip the served request stream")
    ap.add_argument("--no-uniform", action="store_true", help="skip the 4096^2 periodic case")
    ap.add_argument("--no-next-rows", action="store_true",
                    help="skip the device tree build, operator, transfer and VTK measurements")
    ap.add_argument("--profile-solves", type=int, default=0,
                    help="only run this many mixed solves, untimed (a short command to profile)")
    ap.add_argument("--profile-batched", type=int, default=0,
                    help="only run one mixed solve of this many trees of the batch, untimed")
    args = ap.parse_args()
    from afivo_gb300 import workloads as W
    spec = W.c2_poisson_3d(thr=3e-3, lvl_max=7) if args.small else W.c2_poisson_3d()
    if args.small:
        spec["name"] += "_thr3e-3_lvl7"
    if args.impl == "reference":
        return run_reference(args, spec)
    if args.profile_solves:
        return profile_solves(spec, args.profile_solves)
    if args.profile_batched:
        return profile_batched(args.profile_batched)

    rank, world, local = dist_setup(args.gpus)
    import torch
    torch.cuda.set_device(local)
    from afivo_gb300 import build as B
    B.build()
    import afivo_gb300 as afv

    tree, t_build = build_workload(spec)
    forest = afv.Forest([tree], device=local, mixed=True)
    info = forest.info()
    cells = info["leaf_cells"]
    forest.set_source(0, spec["gauss"], lpl=True)
    ext = torch.cuda.ExternalStream(forest.stream())

    def solve(prec):
        forest.zero(afv.AFV_PHI)
        cyc, rel, rc = forest.solve(prec, tol=TOL, max_cycles=60, check=False)
        if rc != 0:
            raise RuntimeError(f"solve did not converge: rc={rc} rel={rel[0]:.3e}")
        return int(cyc[0]), float(rel[0])

    def timed(prec, steps, mask=0):
        """`steps` solves between events on the forest's stream; mask != 0
        turns on per-launch CUDA events of those kernel kinds (and so runs
        the solve without graphs)."""
        forest.profile(mask)
        cycles, rels, per = [], [], []
        barrier(world)
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        l0 = forest.launches()
        ev0.record(ext)
        for _ in range(steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            c, r = solve(prec)
            e1.record(ext)
            e1.synchronize()
            per.append(e0.elapsed_time(e1))
            cycles.append(c)
            rels.append(r)
        ev1.record(ext)
        torch.cuda.synchronize()
        barrier(world)
        ms = ev0.elapsed_time(ev1)
        return ms, cycles, rels, per, forest.launches() - l0

    for _ in range(args.warmup):
        solve(afv.AFV_PREC_MIXED)
        solve(afv.AFV_PREC_FP64)

    # headline: mixed solves, graphs on, nothing profiled (the clock sampler
    # starts first, so that its start-up does not fall into the timed region)
    with Clocks(local) as clk:
        time.sleep(0.5)
        solve(afv.AFV_PREC_MIXED)
        ms, cyc, rels, per, launches = timed(afv.AFV_PREC_MIXED, args.steps)
    ms = max_over_ranks(ms, world)
    value = cells * sum_over_ranks(float(sum(cyc)), world) / (ms / 1e3)

    ms64, cyc64, rels64, per64, _ = timed(afv.AFV_PREC_FP64, args.steps)
    ms64 = max_over_ranks(ms64, world)
    value64 = cells * sum_over_ranks(float(sum(cyc64)), world) / (ms64 / 1e3)

    # roofline: one mixed solve with CUDA events around the sweeps (one pair
    # per run of consecutive half-sweeps of a level). Profiled solves launch
    # kernel by kernel; each iteration is queued behind a 5 ms device-side
    # wait so that the host is ahead and the events time the kernels.
    forest.set_option(afv.AFV_OPT_PROFILE_LEAD_US, 5000)
    timed(afv.AFV_PREC_MIXED, 1, mask=1 << 0)
    sweep_n, sweep_ms, sweep_bytes = forest.profile_read(0)
    pe = forest.profile_entries()
    by_level = {}
    for k, lv, t_ms, b, c in zip(pe["kind"], pe["level"], pe["ms"], pe["bytes"], pe["launches"]):
        if k != 0 or c == 0:
            continue
        a = by_level.setdefault(int(lv), [0, 0.0, 0.0])
        a[0] += int(c)
        a[1] += float(t_ms)
        a[2] += float(b)
    sweep_levels = {str(lv): {"launches": a[0], "us_per_launch": round(1e3 * a[1] / a[0], 2),
                              "GB/s": round(a[2] / (a[1] / 1e3) / 1e9, 1)}
                    for lv, a in sorted(by_level.items())}
    # per-kernel breakdown: one mixed solve, every kind profiled
    timed(afv.AFV_PREC_MIXED, 1, mask=(1 << len(afv.KERNEL_KINDS)) - 1)
    breakdown = {}
    pe = forest.profile_entries()
    for k, name in enumerate(afv.KERNEL_KINDS):
        n, kms, kb = forest.profile_read(k)
        if n:
            lv_ms = {}
            for kk, lv, t_ms in zip(pe["kind"], pe["level"], pe["ms"]):
                if kk == k:
                    lv_ms[str(int(lv))] = lv_ms.get(str(int(lv)), 0.0) + float(t_ms)
            breakdown[name] = {"launches": n, "ms": round(kms, 4),
                               "GB/s": round(kb / (kms / 1e3) / 1e9, 1) if kms > 0 else None,
                               "us_by_level": {lv: round(1e3 * t, 1) for lv, t in lv_ms.items()}}
    forest.profile(0)
    forest.set_option(afv.AFV_OPT_PROFILE_LEAD_US, 0)

    # end to end through the C ABI: every step copies its rhs in from pinned
    # host memory, solves, and copies the solution out. Serial: one forest,
    # step after step. Pipelined (the reported e2e): two forests of the same
    # tree, each driven by its own host thread (the second starting once the
    # first step's rhs is in), so that one step's copies run beside the other
    # forest's solve (the C calls release the interpreter lock); every step
    # still does all of its copies inside the timed region. (Making the
    # solves take turns on the GPU was slower: the copies' gather and scatter
    # kernels then hold SMs the running solve needs.)
    n_in = forest._n_values(0, True)
    host_rhs = torch.empty(n_in, dtype=torch.float64, pin_memory=True)
    forest.get_var(0, afv.AFV_RHS, interior_only=True, out=host_rhs.numpy())
    twin = afv.Forest([tree], device=local, mixed=True)
    for opt in range(len(afv.OPTION_NAMES)):
        twin.set_option(opt, forest.get_option(opt))
    pair = (forest, twin)
    zero_copy = forest.get_option(afv.AFV_OPT_ZERO_COPY)
    host_phi = [torch.empty(n_in, dtype=torch.float64, pin_memory=True) for _ in pair]

    import threading
    first_in = threading.Event()  # the second thread starts once the first step's rhs is in

    def e2e_step(k):
        f = pair[k]
        f.set_var(0, afv.AFV_RHS, host_rhs.numpy(), interior_only=True)
        first_in.set()
        f.zero(afv.AFV_PHI)
        cyc_, rel_, rc_ = f.solve(afv.AFV_PREC_MIXED, tol=TOL, max_cycles=60, check=False)
        if rc_ != 0:
            raise RuntimeError(f"solve did not converge: rc={rc_}")
        f.get_var(0, afv.AFV_PHI, interior_only=True, out=host_phi[k].numpy())
        return int(cyc_[0])

    for k in (0, 1):  # warm the twin (graph capture) and the pair
        e2e_step(k)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_cycles = sum(e2e_step(0) for _ in range(args.steps))
    torch.cuda.synchronize()
    e2e_serial_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e_serial = cells * sum_over_ranks(float(e2e_cycles), world) / e2e_serial_s

    done = [0, 0]
    errors = []

    def worker(k, n):
        try:
            if k == 1:
                first_in.wait(timeout=60)
            for _ in range(n):
                done[k] += e2e_step(k)
        except Exception as exc:  # reported after the join
            errors.append(exc)

    # through the staging buffer, so that the copies leave the SMs to the
    # other forest's solve (kernel loads over the host link would hold them)
    for f in pair:
        f.set_option(afv.AFV_OPT_ZERO_COPY, 0)
    for k in (0, 1):  # the staging buffers
        e2e_step(k)

    def pipelined():
        """One timed run of `steps` steps over the two threads; its rate."""
        done[0] = done[1] = 0
        barrier(world)
        torch.cuda.synchronize()
        first_in.clear()
        t0 = time.perf_counter()
        threads = [threading.Thread(target=worker, args=(k, (args.steps + 1 - k) // 2)) for k in (0, 1)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        torch.cuda.synchronize()
        if errors:
            raise errors[0]
        secs = max_over_ranks(time.perf_counter() - t0, world)
        return cells * sum_over_ranks(float(sum(done)), world) / secs

    # three timed runs, the median reported: a run of a few steps over two
    # host threads is exposed to the host's scheduling
    e2e_runs = [pipelined() for _ in range(3)]
    e2e_value = float(np.median(e2e_runs))
    e2e_same = bool(np.array_equal(host_phi[0].numpy(), host_phi[1].numpy()))
    forest.set_option(afv.AFV_OPT_ZERO_COPY, zero_copy)
    twin.close()

    # The solutions are checked against the oracle's FP64 solves on the host
    # cores (rank 0 of a single-GPU run, beside the CPU baseline).
    check = rank == 0 and world == 1 and not args.no_cpu_baseline
    batched = None if args.no_batched else run_batched(afv, W, local, rank, world, check_errors=check)
    picks = serving_picks(500)
    served, reqs, served_phi = (None, None, {}) if args.no_serving else run_serving(
        afv, W, local, rank, world, keep_ids=set(picks) if check else ())
    uniform = None if args.no_uniform else run_uniform(afv, W, local, rank, world, check_errors=check)
    next_rows = None
    if check and not args.no_next_rows:
        next_rows = run_next_rows(afv, W, local, os.cpu_count() or 1)

    peak, peak_kind = load_peaks()
    achieved = sweep_bytes / (sweep_ms / 1e3) / 1e9 if sweep_ms > 0 else None
    traffic = load_traffic()
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        v, dt, n, osolve = cpu_baseline_sample(spec, cores)
        cpu = {"value": v, "unit": "unknowns/s", "cores": cores, "kind": "port", "cpu": cpu_model(),
               "sample": f"{n} FP64 solves of the full tree to {TOL:g} on the oracle "
                         f"({dt:.1f} s, {cores} threads; median rate)"}
        # the headline's solution (the last end-to-end mixed solve) and a GPU
        # FP64 solve against the oracle's FP64 solution of the same tree
        err_mixed = osolve.error_of(forest.get_var(0, afv.AFV_PHI))
        solve(afv.AFV_PREC_FP64)
        err_fp64 = osolve.error_of(forest.get_var(0, afv.AFV_PHI))
        if served is not None:
            served["cpu_oracle"] = cpu_serving_sample(reqs, cores, picks, served_phi)
    if rank != 0:
        return
    errs = {} if cpu is None else {"err_vs_fp64_oracle": err_mixed}
    errs64 = {} if cpu is None else {"err_vs_oracle": err_fp64}
    line = {
        "metric": METRIC, "value": value, "unit": "unknowns/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic",
        "config": config_of(spec, cells, info["n_boxes"]),
        "method": "mixed: FP32 FAS V(2,2) cycles inside FP64 defect correction; CUDA graphs",
        "solve": {"cycles": cyc, "rel_res": max(rels), "ms_p50": float(np.percentile(per, 50)),
                  "ms_p99": float(np.percentile(per, 99)), "ms_each": [round(x, 3) for x in per],
                  **errs},
        "fp64": {"value": value64, "unit": "unknowns/s", "cycles": cyc64, "rel_res": max(rels64),
                 "ms_per_solve": ms64 / len(cyc64), **errs64},
        "mixed_vs_fp64_solve_speedup": (ms64 / len(cyc64)) / (ms / args.steps),
        "solve_roofline": solve_roofline([tree], cells, max(cyc), ms / args.steps, peak, peak_kind),
        "roofline": {"bound": "hbm", "kernel": "k_sweep_warp<3,8,float>",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                     "algorithmic_bytes": "12 B per cell of the swept level per half-sweep "
                                          "(read phi, rhs; write phi; FP32)",
                     "timed": "CUDA events around each run of consecutive half-sweeps of a level "
                              "(4 launches), one profiled mixed solve, each iteration queued "
                              "behind a 5 ms device-side wait (host ahead of the device)",
                     "per_level": sweep_levels,
                     "gap": "below 0.6 because of the coarse levels: levels 2-5 (under 3 % of the "
                            "bytes) take about a quarter of the sweep time at 4-5 us per launch, the "
                            "chain of dependent L2 round trips of a half-sweep; the finest levels run "
                            "at 0.62-0.67. A cluster-barrier kernel and an unstaged sweep for the small "
                            "levels were bit-identical but not faster",
                     "launches": sweep_n, "ms": sweep_ms,
                     "traffic": traffic.get("dram_bytes_per_launch") if traffic else None,
                     "traffic_note": traffic.get("note") if traffic else None},
        "kernels": breakdown,
        "batched": batched,
        "serving": served,
        "uniform_periodic": uniform,
        "next_rows": next_rows,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "unknowns/s", "h2d_bytes_per_step": n_in * 8,
                "d2h_bytes_per_step": n_in * 8,
                "pipeline": "two forests of the tree, one host thread each: a step's copies (copy "
                            "engines, through a staging buffer) overlap the other forest's solve; every "
                            "step copies rhs in and phi out",
                "solutions_identical": e2e_same,
                "runs": [round(v, 1) for v in e2e_runs], "of_runs": "median of three timed runs",
                "note": "with two solves in flight each fills the other's idle gaps on the coarse "
                        "levels, so the pipelined rate can exceed the single-solve device rate",
                "serial": {"value": e2e_serial, "ms_per_step": 1e3 * e2e_serial_s / args.steps}},
        "clocks": clk.summary(),
        "gpu_launches": launches,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
