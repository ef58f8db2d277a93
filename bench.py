"""Benchmark: block-parallel IDA* on one GB300 (replicas across GPUs).

Workload (one step = solving the whole batch, every threshold iteration):
  15-puzzle, 100 uniformly random solvable permutations (seeded Fisher-Yates,
  parity-fixed), additive 5-5-5 PDB (max of regular and reflected partition),
  root set ~2048 subproblems per instance, static re-split + in-kernel
  donation, the library's default threshold loop (small iterations in one
  persistent launch, large ones in the host round loop).  Rank r solves its
  own batch (seed + r): weak scaling, no data collective.

Prints one JSON line (rank 0).  `value` = generated nodes per second with
the instances already in device memory (sp_solve_batch_device); `e2e` = the
same through sp_solve_batch with host buffers.  `--impl reference` times the
reference's serial IDA* restated in C (the oracle) on the host cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sliding-puzzle_gb300"))

import numpy as np  # noqa: E402

METRIC = "nodes/sec & instances/sec (optimal, exact); learned-LB vs plain LB, 1 GB300"
UNIT = "nodes/s"
BYTES_PER_NODE = 64  # 2 table lookups (1 regular + 1 reflected pattern) x 32-byte sector


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
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
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for name, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def job_max_sum(max_vals, sum_vals, world, device):
    """Whole-job figures: the max over ranks of each of `max_vals` (times)
    and the sum over ranks of each of `sum_vals` (work).  One rank: as is."""
    if world <= 1:
        return [float(x) for x in max_vals], [float(x) for x in sum_vals]
    import torch
    import torch.distributed as dist
    tm = torch.tensor([float(x) for x in max_vals], dtype=torch.float64, device=device)
    ts = torch.tensor([float(x) for x in sum_vals], dtype=torch.float64, device=device)
    dist.all_reduce(tm, op=dist.ReduceOp.MAX)
    dist.all_reduce(ts, op=dist.ReduceOp.SUM)
    return tm.tolist(), ts.tolist()


def workload(rank, n=100):
    import instances
    return 4, instances.random_permutations(4, n, seed=0x15B + rank)


def cpu_sample(w, states, budget_s, threads):
    """Oracle on a bounded sample: instances in order, each capped by a node
    budget, until about budget_s seconds of wall time."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    tabs = oracle.tables(w)
    # calibrate nodes/s on a short probe, then size the budget
    t0 = time.perf_counter()
    probe = oracle.solve(w, states[:threads], oracle.PDB, tabs, threads=threads, node_budget=2_000_000)
    dt = time.perf_counter() - t0
    rate = sum(r["nodes_total"] for r in probe) / max(dt, 1e-6)
    per_inst = max(1_000_000, int(rate * budget_s / max(1, min(len(states), 4 * threads))))
    sample = states[: min(len(states), 4 * threads)]
    t0 = time.perf_counter()
    res = oracle.solve(w, sample, oracle.PDB, tabs, threads=threads, node_budget=per_inst)
    dt = time.perf_counter() - t0
    nodes = sum(r["nodes_total"] for r in res)
    done = sum(1 for r in res if r["status"] == 0)
    return {"value": nodes / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d instances of the workload, node budget %d each (%d solved), %.1f s" %
                      (len(sample), per_inst, done, dt),
            "seconds": dt, "nodes": nodes}


def run_reference(args):
    _, rank, _ = dist_setup()
    if rank != 0:
        return
    w, states = workload(0)
    threads = os.cpu_count() or 1
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_sample(w, states, budget_s=args.ref_seconds, threads=threads)
        if i >= args.warmup:
            vals.append(r)
    v = sum(x["nodes"] for x in vals) / sum(x["seconds"] for x in vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * sum(x["seconds"] for x in vals) / len(vals), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded)",
            "config": {"workload": "15puzzle_random100_pdb555", "instances": len(states),
                       "solver": "oracle/ida_oracle.c: serial IDA*, one instance per host thread"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": vals[-1]["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_probe(args):
    """Steady-state kernel probes, one threshold round each.  balanced: one
    root replicated `--roots` times (identical subtrees: no load imbalance,
    every lane reads the same table entries).  mixed: `--roots` distinct walk
    endpoints (100-220 moves for the 24-puzzle, 40-80 for the 15-puzzle),
    each given the depth that puts it `--probe-slack`/2 threshold steps below
    one common limit, so the table reads scatter as in a real search."""
    import torch
    import instances
    import slide
    import train_lb
    torch.cuda.set_device(0)
    width = 4 if args.probe_width == 4 else 5
    s = slide.Solver(width, args.probe_heuristic)
    if args.probe_heuristic == "pdb":
        s.build_pdb()
    n = args.roots
    pre = -np.ones(n, np.int32)
    if args.probe == "balanced":
        root = instances.random_walks(width, 1, 50, seed=5)
        h0 = int(s.heuristic_values(root)[0])
        roots = np.repeat(root, n, axis=0)
        depth = np.zeros(n, np.int32)
        limit = h0 + args.probe_slack
    else:
        lo, hi = (100, 220) if width == 5 else (40, 80)
        roots = train_lb.vector_walks(width, n, lo, hi, seed=7)
        h = s.heuristic_values(roots).astype(np.int64)
        limit = int(h.max()) + args.probe_slack
        depth = (limit - args.probe_slack - h).astype(np.int32)
    s.dfs_round(roots[:1024], depth[:1024], pre[:1024], limit)  # warm-up
    nodes, _ = s.dfs_round(roots, depth, pre, limit)
    x = s.stats()
    d = {"probe": args.probe, "width": width, "heuristic": args.probe_heuristic, "roots": n,
         "nodes_per_root": float(nodes.mean()), "kernel_ms": x["kernel_ms"],
         "nodes_per_s": float(nodes.sum()) / (x["kernel_ms"] / 1000.0),
         "lane_step_fraction": x["dev_lane_steps"] / max(1, x["dev_lane_slots"]),
         "idle_fraction": x["dev_idle_cycles"] / max(1, x["dev_warp_cycles"])}
    if args.probe_heuristic == "manhattan":
        d["roofline"] = _int_roofline(float(nodes.sum()), x["kernel_ms"], slide.probe_int_issue()[0])
    print(json.dumps(d), flush=True)


def _timed_solve(solver, states, reps=1):
    """Best wall time of `reps` host-buffer solves (after one warm-up)."""
    import torch
    solver.solve_raw(states)
    best, res, st = None, None, None
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = solver.solve_raw(states)
        dt = time.perf_counter() - t0
        if best is None or dt < best:
            best, res, st = dt, r, solver.stats()
    n = states.shape[0]
    for i in range(n):
        if res[i].status != 0:
            raise RuntimeError("instance %d failed with status %d" % (i, res[i].status))
    return best, [res[i] for i in range(n)], st


def _summary(label, dt, res, st, extra=None):
    nodes = sum(r.nodes_total for r in res)
    lens = sorted(r.len for r in res)
    lat = sorted(r.seconds for r in res)

    def q(a, f):
        return a[min(len(a) - 1, int(f * len(a)))]
    d = {"workload": label, "instances": len(res), "seconds": dt, "nodes": nodes, "nodes_per_s": nodes / dt,
         "instances_per_s": len(res) / dt, "kernel_ms": st["kernel_ms"], "rounds": st["rounds"],
         "kernel_launches": st["kernel_launches"], "tasks_donated": st["tasks_donated"],
         "frontier_ms": st["frontier_ms"],
         "lane_step_fraction": st["dev_lane_steps"] / max(1, st["dev_lane_slots"]),
         "optimal_len": {"min": lens[0], "p50": q(lens, 0.5), "max": lens[-1]},
         "latency_s": {"p50": q(lat, 0.5), "p99": q(lat, 0.99), "max": lat[-1]}}
    if extra:
        d.update(extra)
    return d


def _int_roofline(nodes, kernel_ms, peak_ops):
    """Integer-issue roofline of a Manhattan-heuristic search: the algorithmic
    integer operations of its generated nodes over its kernel time, against
    the integer rate sp_probe_int_issue measured in the same process."""
    import slide
    achieved = nodes * slide.MD_OPS_PER_NODE / (kernel_ms / 1000.0) / 1e9
    peak = peak_ops / 1e9
    return {"bound": "int-issue", "achieved": achieved, "peak": peak, "unit": "G int32 op/s",
            "frac": achieved / peak, "ops_per_node": slide.MD_OPS_PER_NODE,
            "peak_source": "sp_probe_int_issue, measured in this run"}


def run_workload(args):
    """Secondary workloads (the other configurations of the benchmark plan),
    one JSON line each; the headline line is the default mode."""
    import torch
    import instances
    import slide
    torch.cuda.set_device(0)
    out = []
    modes = [("round", dict(persistent=0)), ("persistent", dict(persistent=1, handback_nodes=0)),
             ("hybrid", dict(persistent=1, handback_nodes=600000))]
    if args.workload == "15_md_walk60":
        w, states = instances.config_instances("15_md_walk60")
        peak_ops, _ = slide.probe_int_issue()
        for name, pers in modes:
            s = slide.Solver(w, "manhattan", lb_mode="static", **pers)
            dt, res, st = _timed_solve(s, states, reps=3)
            d = _summary("15_md_walk60/" + name, dt, res, st, {"heuristic": "manhattan"})
            d["roofline"] = _int_roofline(d["nodes"], st["kernel_ms"], peak_ops)
            out.append(d)
            s.close()
    elif args.workload == "15_mixed4096":
        w, states = instances.config_instances("15_mixed4096")
        for name, pers in modes:
            s = slide.Solver(w, "pdb", lb_mode="static", frontier_target=args.frontier, **pers)
            s.build_pdb()
            dt, res, st = _timed_solve(s, states, reps=2)
            out.append(_summary("15_mixed4096/" + name, dt, res, st,
                                {"heuristic": "pdb555", "frontier_target": args.frontier}))
            s.close()
    elif args.workload == "24_bins":
        s = slide.Solver(5, "pdb", lb_mode="static", frontier_target=args.frontier)
        t0 = time.perf_counter()
        s.build_pdb()
        pdb_s = time.perf_counter() - t0
        for m in (120, 160, 200):
            _, states = instances.config_instances("24_walk%d" % m)
            dt, res, st = _timed_solve(s, states)
            out.append(_summary("24_walk%d" % m, dt, res, st,
                                {"heuristic": "pdb6666", "pdb_build_s": pdb_s, "frontier_target": args.frontier}))
    elif args.workload == "lb_ab":
        import train_lb

        def log(m):
            print("[lb_ab %.1fs] %s" % (time.perf_counter() - t_start, m), file=sys.stderr, flush=True)
        t_start = time.perf_counter()
        # round mode: the learned model stands in for the loads of roots that
        # the previous round did not measure, which only the round loop plans
        s = slide.Solver(5, "pdb", frontier_target=8192, persistent=0)
        s.build_pdb()
        t0 = time.perf_counter()
        tiles, slack, target, mean = train_lb.make_dataset(s, args.tuples, 7, 0x1B, log=log)
        data_s = time.perf_counter() - t0
        s.lbm_init(0x1B)
        metrics = train_lb.train(s, tiles, slack, target, epochs=args.epochs, log=log)
        log("model %s" % metrics)
        _, states = instances.config_instances("24_walk%d" % args.ab_bin)
        rows = {}
        for lb in ("static", "learned"):
            s.set_config(lb_mode=lb, frontier_target=8192)
            dt, res, st = _timed_solve(s, states)
            log("%s solve %.2f s" % (lb, dt))
            rows[lb] = _summary("24_walk%d/%s" % (args.ab_bin, lb), dt, res, st)
            rows[lb]["round_kernel_ms"] = [round(x, 2) for x in st["round_kernel_ms"]]
        out.append({"workload": "lb_ab", "bin": "24_walk%d" % args.ab_bin, "frontier_target": 8192,
                    "tuples": int(len(target)), "slack_mean_nodes": [float(x) for x in mean],
                    "data_s": data_s, "model": metrics,
                    "static_s": rows["static"]["seconds"], "learned_s": rows["learned"]["seconds"],
                    "speedup_learned": rows["static"]["seconds"] / rows["learned"]["seconds"],
                    "static": rows["static"], "learned": rows["learned"]})
    for d in out:
        print(json.dumps(d), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--probe", choices=["balanced", "mixed"], default=None)
    ap.add_argument("--workload", choices=["15_md_walk60", "15_mixed4096", "24_bins", "lb_ab"], default=None)
    ap.add_argument("--tuples", type=int, default=1_000_000)
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--ab-bin", type=int, default=200)
    ap.add_argument("--probe-heuristic", default="pdb", choices=["manhattan", "pdb"])
    ap.add_argument("--probe-width", type=int, default=4)
    ap.add_argument("--probe-slack", type=int, default=8)
    ap.add_argument("--roots", type=int, default=100000)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--instances", type=int, default=100)
    ap.add_argument("--frontier", type=int, default=2048)
    ap.add_argument("--lb", default="static")
    ap.add_argument("--persistent", type=int, default=None, choices=[0, 1],
                    help="threshold loop on the device (default: the library's, 1)")
    ap.add_argument("--handback", type=int, default=None,
                    help="persistent mode: nodes per instance iteration from which the host round loop takes over "
                         "(default: the library's, 600000; 0 = never)")
    ap.add_argument("--autotune", action="store_true",
                    help="pick block size, poll interval, persistence and donation reserve first "
                         "(the root-set size stays the configured one)")
    ap.add_argument("--ref-seconds", type=float, default=8.0)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.probe:
        return run_probe(args)
    if args.workload:
        return run_workload(args)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import slide

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w, states = workload(rank, args.instances)
    n = states.shape[0]
    opts = dict(frontier_target=args.frontier, lb_mode=args.lb)
    if args.persistent is not None:
        opts["persistent"] = args.persistent
    if args.handback is not None:
        opts["handback_nodes"] = args.handback
    solver = slide.Solver(w, "pdb", **opts)
    t0 = time.perf_counter()
    solver.build_pdb()
    pdb_ms = 1000 * (time.perf_counter() - t0)
    tuned = None
    if args.autotune:
        space = tuple(p for p in slide.AUTOTUNE_SPACE if p[0] != "frontier_target")
        tuned, _ = slide.autotune(solver, states, space=space, reps=2)
    d_tiles = torch.from_numpy(states.copy()).to("cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    def check(res):
        lens = []
        for i in range(n):
            if res[i].status != 0:
                raise RuntimeError("instance %d failed with status %d" % (i, res[i].status))
            lens.append(res[i].len)
        return lens

    ref_lens = None
    for _ in range(args.warmup):
        lens = check(solver.solve_device_raw(d_tiles.data_ptr(), n))
        ref_lens = ref_lens or lens

    # timed region: device-resident inputs
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    step_ms, kern_ms, nodes, launches, rounds, donated = [], [], 0, 0, 0, 0
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.fill_(k & 0xFF)
            torch.cuda.synchronize()
            l0 = slide.kernel_launch_count()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            res = solver.solve_device_raw(d_tiles.data_ptr(), n)
            e1.record()
            torch.cuda.synchronize()
            launches += slide.kernel_launch_count() - l0
            step_ms.append(e0.elapsed_time(e1))
            st = solver.stats()
            kern_ms.append(st["kernel_ms"])
            rounds += st["rounds"]
            donated += st["tasks_donated"]
            if check(res) != ref_lens:
                raise RuntimeError("lengths changed between steps")
            nodes += sum(res[i].nodes_total for i in range(n))
    total_ms = sum(step_ms)
    (total_ms,), (all_nodes,) = job_max_sum([total_ms], [nodes], world, "cuda")
    value = all_nodes / (total_ms / 1000.0)

    # e2e: host buffers through sp_solve_batch (H2D/D2H inside)
    e2e_ms, h2d, d2h = [], 0, 0
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        res = solver.solve_raw(states)
        e1.record()
        torch.cuda.synchronize()
        e2e_ms.append(e0.elapsed_time(e1))
        st = solver.stats()
        h2d += st["h2d_bytes"] + states.nbytes
        d2h += st["d2h_bytes"]
        if [res[i].len for i in range(n)] != ref_lens:
            raise RuntimeError("e2e lengths differ")
    e2e_total = sum(e2e_ms)
    (e2e_total,), _ = job_max_sum([e2e_total], [], world, "cuda")
    e2e_value = all_nodes / (e2e_total / 1000.0)

    peak, peak_kind = load_peaks()
    kms = sum(kern_ms)
    achieved = nodes * BYTES_PER_NODE / (kms / 1000.0) / 1e9 if kms > 0 else 0.0
    traffic = None  # DRAM bytes per search launch, from the committed ncu summary
    hybrid = solver.config.persistent and solver.config.handback_nodes
    prof = os.path.join(ROOT, "profiles", "search_hybrid_pdb15_random100.md" if hybrid
                        else "search_round_pdb15_random100.md")
    if os.path.exists(prof):
        for line in open(prof):
            if line.startswith("traffic_bytes_per_launch:"):
                traffic = float(line.split(":")[1])
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_sample(w, states, budget_s=args.cpu_seconds, threads=os.cpu_count() or 1)
        cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded)",
            "config": {"workload": "15puzzle_random100_pdb555", "instances_per_gpu": n,
                       "heuristic": "additive 5-5-5 PDB, max(regular, reflected)",
                       "frontier_target": args.frontier, "lb": args.lb + "+donation",
                       "threshold_loop": (("device, handing iterations predicted at >= %d nodes per "
                                           "instance to the host round loop" % solver.config.handback_nodes
                                           if solver.config.handback_nodes else "device (one launch)")
                                          if solver.config.persistent else "host (one launch per round)"),
                       "autotuned": {k: tuned[k] for k in ("threads_per_block", "steps_per_poll", "persistent",
                                                           "handback_nodes", "donate_reserve")} if tuned else None,
                       "parallelism": "replicas" if world > 1 else "1 GPU",
                       "l2": "512 MB buffer written between timed steps",
                       "pdb_build_ms": round(pdb_ms, 2)},
            "instances_per_s": world * n / (total_ms / 1000.0),
            "nodes_per_step": all_nodes / args.steps,
            "rounds_per_step": rounds / args.steps,
            "tasks_donated_per_step": donated / args.steps,
            "kernel_ms_per_step": kms / args.steps,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d // args.steps,
                    "d2h_bytes_per_step": d2h // args.steps, "ms_per_step": e2e_total / args.steps},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "search_round_kernel<4,pdb>", "peak_kind": peak_kind,
                         "bytes_per_node": BYTES_PER_NODE},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
