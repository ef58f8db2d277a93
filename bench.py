"""Benchmark: block-parallel IDA* on one GB300 (replicas across GPUs).

Headline (one step = solving the whole batch, every threshold iteration):
  15-puzzle, 100 uniformly random solvable permutations (seeded Fisher-Yates,
  parity-fixed), additive 5-5-5 PDB (max of regular and reflected partition),
  static re-split + in-kernel donation, the library's default threshold loop
  (small iterations in one persistent launch, large ones in the host round
  loop), launch and balance settings from the autotuner (cached per GPU,
  puzzle, heuristic and batch size; every candidate must return identical
  answers).  Rank r solves its own batch (seed + r): weak scaling, no data
  collective.

Prints one JSON line (rank 0).  `value` = generated nodes per second with
the instances already in device memory (sp_solve_batch_device); `e2e` = the
same through sp_solve_batch with host buffers.  `roofline` holds the search
kernel against the measured rate of random one-byte table reads from a 3 MB
working set (its tables stay in L2), with the integer-issue and HBM figures
beside it.  `cpu_baseline` = the oracle (the reference's serial IDA*
restated in C) on all host cores solving the same 100 instances
completely.  `secondary` = the reference's own 24-puzzle set
(yama24_50_hard_new, 6-6-6-6 PDB) beside the thesis's published totals, the
three 24-puzzle bins, the learned-versus-static balancer A/B, the
4096-instance batch and the Manhattan walks.  `--impl reference` times the
oracle alone on all host cores, each timed step the complete workload.
"""
import argparse
import hashlib
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
SECTOR_BYTES = 32
HEADLINE = "15puzzle_random100_pdb555"
# The reference's published totals over yama24_50_hard_new with the 6-6-6-6
# PDB (thesis main.tex:858-863; GRID K520 GPU, Xeon E5-2670 single thread).
THESIS_PDB24 = {"bpida_global_gpu_s": 6.45871, "bpida_gpu_s": 16.2875, "ida_cpu_1thread_s": 34.1312,
                "source": "main.tex:858-863", "hardware": "NVIDIA GRID K520 / Intel Xeon E5-2670"}


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


def oracle_module():
    """The CPU oracle (test infrastructure; here only as the CPU baseline)."""
    p = os.path.join(ROOT, "oracle")
    if p not in sys.path:
        sys.path.insert(0, p)
    import oracle
    return oracle


def cpu_full(w, states, heuristic, tabs, threads):
    """The oracle solving every instance completely (no node budget), all
    host threads on one instance at a time (orc_solve_batch_split: the serial
    search's counts and lengths).  Returns the rate and the answers."""
    oracle = oracle_module()
    t0 = time.perf_counter()
    res = oracle.solve(w, states, heuristic, tabs, threads=threads, split=True)
    dt = time.perf_counter() - t0
    bad = [i for i, r in enumerate(res) if r["status"] != 0]
    if bad:
        raise RuntimeError("oracle failed on instances %s" % bad[:8])
    nodes = sum(r["nodes_total"] for r in res)
    return {"value": nodes / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "instances_per_s": len(res) / dt, "seconds": dt, "nodes": nodes,
            "sample": "all %d instances solved completely (every threshold iteration), all %d host threads "
                      "on one instance at a time; %.1f s" % (len(res), threads, dt),
            "answers": [(r["len"], r["nodes_total"]) for r in res]}


def cpu_budget(w, states, heuristic, tabs, threads, budget_s):
    """The oracle on a bounded sample: up to 2 instances per thread, one per
    thread at a time, each cut at a node budget sized for about budget_s
    seconds of wall time."""
    oracle = oracle_module()
    sample = states[: min(len(states), 2 * threads)]
    t0 = time.perf_counter()
    probe = oracle.solve(w, sample[:threads], heuristic, tabs, threads=threads, node_budget=1_000_000)
    dt = time.perf_counter() - t0
    rate = sum(r["nodes_total"] for r in probe) / max(dt, 1e-6)
    per_inst = max(1_000_000, int(rate * budget_s / max(1, len(sample))))
    t0 = time.perf_counter()
    res = oracle.solve(w, sample, heuristic, tabs, threads=threads, node_budget=per_inst)
    dt = time.perf_counter() - t0
    nodes = sum(r["nodes_total"] for r in res)
    done = sum(1 for r in res if r["status"] == 0)
    return {"value": nodes / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d instances, node budget %d each (%d solved), %.1f s" % (len(sample), per_inst, done, dt)}


def host_threads():
    return os.cpu_count() or 1


def run_reference(args):
    """The reference arm: the oracle (the reference's serial IDA* restated in
    C; the reference's own binaries are x86 builds of this container and its
    checkout is not on the GPU machine) on all host cores.  Each timed step solves
    the complete headline workload; warm-up steps solve its first 8
    instances (a CPU needs no more warming)."""
    _, rank, _ = dist_setup()
    if rank != 0:
        return
    # the table build's OpenMP threads must not spin on the cores the timed
    # search runs on (set before the oracle library loads the runtime)
    os.environ.setdefault("OMP_WAIT_POLICY", "PASSIVE")
    oracle = oracle_module()
    w, states = workload(0)
    tabs = oracle.tables(w)
    threads = host_threads()
    for _ in range(args.warmup):
        cpu_full(w, states[:8], oracle.PDB, tabs, threads)
    vals = [cpu_full(w, states, oracle.PDB, tabs, threads) for _ in range(args.steps)]
    secs = sum(x["seconds"] for x in vals)
    v = sum(x["nodes"] for x in vals) / secs
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * secs / len(vals),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded)",
            "config": {"workload": HEADLINE, "instances_per_gpu": len(states),
                       "heuristic": "additive 5-5-5 PDB, max(regular, reflected)",
                       "solver": "oracle/ida_oracle.c: serial IDA* restated (64-bit counters), all host threads on "
                                 "one instance at a time (frontier split per iteration)",
                       "warmup_sample": "first 8 instances"},
            "instances_per_s": len(states) * len(vals) / secs,
            "nodes_per_step": vals[-1]["nodes"],
            "step_seconds": [round(x["seconds"], 3) for x in vals],
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": vals[-1]["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_sector_probe(args):
    """The roofline denominators alone: random one-byte reads over the
    15-puzzle's and the 24-puzzle's table sizes, and the integer issue rate."""
    import torch
    torch.cuda.set_device(0)
    print(json.dumps({"probe": "sectors", **measure_peaks()}), flush=True)


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


def _timed_solve(solver, states, reps=1, warm=True):
    """Best wall time of `reps` host-buffer solves (after one warm-up solve
    unless warm is False)."""
    import torch
    if warm:
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
         "idle_fraction": st["dev_idle_cycles"] / max(1, st["dev_warp_cycles"]),
         "optimal_len": {"min": lens[0], "p50": q(lens, 0.5), "max": lens[-1]},
         "latency_s": {"p50": q(lat, 0.5), "p99": q(lat, 0.99), "max": lat[-1]}}
    if extra:
        d.update(extra)
    return d


def _int_roofline(nodes, kernel_ms, peak_ops):
    """Integer-issue roofline of a search: the algorithmic integer operations
    of its generated nodes over its kernel time, against the integer rate
    sp_probe_int_issue measured in the same process."""
    import slide
    achieved = nodes * slide.MD_OPS_PER_NODE / (kernel_ms / 1000.0) / 1e9
    peak = peak_ops / 1e9
    return {"bound": "int-issue", "achieved": achieved, "peak": peak, "unit": "G int32 op/s",
            "frac": achieved / peak, "ops_per_node": slide.MD_OPS_PER_NODE,
            "peak_source": "sp_probe_int_issue, measured in this run"}


def _sector_roofline(nodes, kernel_ms, reads_per_s, bound, working_set):
    """Random-read roofline of a PDB search: its algorithmic table bytes (one
    regular and one reflected lookup per generated node, a 32-byte sector
    each) over its kernel time, against the random one-byte read rate that
    sp_probe_random_sectors measured in the same process on a buffer of the
    tables' size (times the 32-byte sector each read costs)."""
    achieved = nodes * BYTES_PER_NODE / (kernel_ms / 1000.0) / 1e9
    peak = reads_per_s * SECTOR_BYTES / 1e9
    return {"bound": bound, "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "bytes_per_node": BYTES_PER_NODE, "lookups_per_s": 2.0 * nodes / (kernel_ms / 1000.0),
            "peak_reads_per_s": reads_per_s,
            "peak_source": "sp_probe_random_sectors over %d bytes, measured in this run" % working_set}


def measure_peaks():
    """Roofline denominators measured in this process: random one-byte reads
    over the 15-puzzle's 3 MB of tables (L2) and the 24-puzzle's 488 MB (mostly
    DRAM), and the 32-bit integer issue rate."""
    import slide
    l2, _ = slide.probe_random_sectors(slide.pdb_table_bytes(4), 256, 3)
    hbm, _ = slide.probe_random_sectors(slide.pdb_table_bytes(5), 64, 3)
    ops, _ = slide.probe_int_issue()
    return {"l2_random_reads_per_s": l2, "hbm_random_reads_per_s": hbm, "int_ops_per_s": ops}


def _pdb_rooflines(nodes, kernel_ms, peaks, width):
    import slide
    return {"l2_random": _sector_roofline(nodes, kernel_ms, peaks["l2_random_reads_per_s"], "l2-random",
                                          slide.pdb_table_bytes(4)),
            "hbm_random": _sector_roofline(nodes, kernel_ms, peaks["hbm_random_reads_per_s"], "hbm-random",
                                           slide.pdb_table_bytes(5)),
            "tables_bytes": slide.pdb_table_bytes(width)}


def _tables_checked(solver):
    """The solver's GPU-built tables in the reference's byte order, checked
    against the oracle's fingerprints before the CPU legs search with them."""
    fp = json.load(open(os.path.join(ROOT, "tests", "golden", "pdb_fingerprints.json")))["tables"]
    tabs = []
    for t in range(solver.num_tables()):
        a = solver.export_pdb(t)
        if hashlib.sha256(a.tobytes()).hexdigest() != fp["%d_%d" % (solver.width, t)]["sha256"]:
            raise RuntimeError("GPU table %d of width %d differs from the oracle's" % (t, solver.width))
        tabs.append(a)
    return tabs


def _hist(vals):
    h = {}
    for v in vals:
        h[str(v)] = h.get(str(v), 0) + 1
    return dict(sorted(h.items(), key=lambda kv: int(kv[0])))


def sec_yama24(s5, tabs5, peaks, threads):
    """The reference's own 24-puzzle set (yama24_50_hard_new, 6-6-6-6 PDB):
    every row checked against its golden (length, nodes), timed beside the
    oracle solving the same 50 instances on all host cores and the thesis's
    published totals."""
    oracle = oracle_module()
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "yama24_hard_new.json")))["instances"]
    states = np.array([x["tiles"] for x in g], dtype=np.uint8)
    dt, res, st = _timed_solve(s5, states, reps=3)
    match = sum(1 for x, r in zip(g, res) if (r.len, r.nodes_total) == tuple(x["pdb"]))
    if match != len(g):
        raise RuntimeError("yama24_50_hard_new: %d of %d golden rows reproduced" % (match, len(g)))
    d = _summary("yama24_50_hard_new", dt, res, st,
                 {"heuristic": "pdb6666", "frontier_target": int(s5.config.frontier_target),
                  "golden_rows_match": "%d/%d" % (match, len(g))})
    d["roofline"] = _pdb_rooflines(d["nodes"], st["kernel_ms"], peaks, 5)
    cpu = cpu_full(5, states, oracle.PDB, tabs5, threads)
    d["cpu_oracle"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "instances_per_s", "seconds", "sample")}
    d["cpu_same_answers"] = cpu["answers"] == [(r.len, r.nodes_total) for r in res]
    d["published"] = THESIS_PDB24
    d["x_vs_published_gpu"] = THESIS_PDB24["bpida_global_gpu_s"] / dt
    d["x_vs_published_cpu"] = THESIS_PDB24["ida_cpu_1thread_s"] / dt
    d["x_vs_cpu_oracle_here"] = cpu["seconds"] / dt
    return d


def sec_bins(s5, tabs5, peaks, threads, cpu_s, frontier):
    """The three 24-puzzle bins (50 seeded walks of 120 / 160 / 200 moves),
    one timed pass each (the bins' instances are too hard for warm-up
    repeats), with a bounded CPU-oracle sample beside each."""
    import instances
    oracle = oracle_module()
    out = []
    s5.set_config(frontier_target=frontier)
    for m in (120, 160, 200):
        _, states = instances.config_instances("24_walk%d" % m)
        dt, res, st = _timed_solve(s5, states, warm=False)
        d = _summary("24_walk%d" % m, dt, res, st, {"heuristic": "pdb6666", "frontier_target": frontier})
        d["length_hist"] = _hist(r.len for r in res)
        d["roofline"] = _pdb_rooflines(d["nodes"], st["kernel_ms"], peaks, 5)
        d["cpu_oracle"] = cpu_budget(5, states, oracle.PDB, tabs5, threads, cpu_s)
        out.append(d)
    return out


def sec_lb_ab(s5, tuples, epochs, ab_bin, frontier, log, persistent=None):
    """Learned balancer against the static one on a 24-puzzle bin.  A model
    is trained on GPU-labelled tuples (walk ends, slack 0..7, label log2(1 +
    subtree nodes)); then the bin is solved with the static balancer (each
    root's next load = its measured load x the instance's growth) and with
    the learned one (every root's load predicted by the model: measured load
    x its own predicted growth, or the model's size estimate), same answers
    required."""
    import instances
    import train_lb
    t0 = time.perf_counter()
    tiles, slack, target, mean = train_lb.make_dataset(s5, tuples, 7, 0x1B, log=log)
    data_s = time.perf_counter() - t0
    s5.lbm_init(0x1B)
    t0 = time.perf_counter()
    metrics = train_lb.train(s5, tiles, slack, target, epochs=epochs, log=log)
    train_s = time.perf_counter() - t0
    _, states = instances.config_instances("24_walk%d" % ab_bin)
    rows, answers = {}, {}
    extra = {} if persistent is None else {"persistent": persistent}
    for lb in ("static", "learned"):
        s5.set_config(lb_mode=lb, frontier_target=frontier, **extra)
        dt, res, st = _timed_solve(s5, states, warm=False)
        log("%s solve %.2f s" % (lb, dt))
        rows[lb] = _summary("24_walk%d/%s" % (ab_bin, lb), dt, res, st)
        rows[lb]["round_kernel_ms"] = [round(x, 2) for x in st["round_kernel_ms"]]
        answers[lb] = [(r.len, r.nodes_total) for r in res]
    s5.set_config(lb_mode="static")
    if answers["static"] != answers["learned"]:
        raise RuntimeError("lb_ab: the learned balancer changed answers")
    return {"workload": "lb_ab", "bin": "24_walk%d" % ab_bin, "frontier_target": frontier,
            "threshold_loop": "round" if persistent == 0 else "default (hybrid)",
            "tuples": int(len(target)), "slack_mean_nodes": [float(x) for x in mean], "data_s": data_s,
            "train_s": train_s, "model": metrics,
            "static_s": rows["static"]["seconds"], "learned_s": rows["learned"]["seconds"],
            "speedup_learned": rows["static"]["seconds"] / rows["learned"]["seconds"],
            "same_answers": True, "static": rows["static"], "learned": rows["learned"]}


def sec_batch4096(peaks):
    """The 4096-instance 15-puzzle batch (2048 walks of 40-80 moves + 2048
    random states, 5-5-5 PDB), default threshold loop."""
    import instances
    import slide
    w, states = instances.config_instances("15_mixed4096")
    with slide.Solver(w, "pdb") as s:
        s.build_pdb()
        dt, res, st = _timed_solve(s, states, reps=2)
    d = _summary("15_mixed4096", dt, res, st, {"heuristic": "pdb555"})
    d["roofline"] = _pdb_rooflines(d["nodes"], st["kernel_ms"], peaks, 4)
    return d


def sec_md_walk60(peaks):
    """100 seeded 60-move walks, 15-puzzle, Manhattan distance."""
    import instances
    import slide
    w, states = instances.config_instances("15_md_walk60")
    with slide.Solver(w, "manhattan") as s:
        dt, res, st = _timed_solve(s, states, reps=3)
    d = _summary("15_md_walk60", dt, res, st, {"heuristic": "manhattan"})
    d["roofline"] = _int_roofline(d["nodes"], st["kernel_ms"], peaks["int_ops_per_s"])
    return d


def secondary(args, peaks, threads, log):
    """The other configurations of the benchmark plan, one pass each."""
    import slide
    out = {}
    with slide.Solver(5, "pdb") as s5:
        t0 = time.perf_counter()
        s5.build_pdb()
        pdb_s = time.perf_counter() - t0
        tabs5 = _tables_checked(s5)
        out["pdb24_build_s"] = pdb_s
        log("24-puzzle tables built in %.2f s" % pdb_s)
        out["yama24_50_hard_new"] = sec_yama24(s5, tabs5, peaks, threads)
        log("yama24_50_hard_new done")
        out["24_bins"] = sec_bins(s5, tabs5, peaks, threads, args.cpu_bin_seconds, args.frontier24)
        log("24-puzzle bins done")
        if args.tuples > 0:
            out["lb_ab"] = sec_lb_ab(s5, args.tuples, args.epochs, args.ab_bin, args.frontier24, log)
            log("lb_ab done")
    out["15_mixed4096"] = sec_batch4096(peaks)
    out["15_md_walk60"] = sec_md_walk60(peaks)
    return out


def run_workload(args):
    """One secondary configuration on its own (a JSON line each)."""
    import torch
    import slide
    torch.cuda.set_device(0)

    def log(m):
        print("[%s] %s" % (args.workload, m), file=sys.stderr, flush=True)
    peaks = measure_peaks()
    threads = host_threads()
    out = []
    if args.workload == "15_md_walk60":
        out.append(sec_md_walk60(peaks))
    elif args.workload == "15_mixed4096":
        out.append(sec_batch4096(peaks))
    else:
        with slide.Solver(5, "pdb") as s5:
            s5.build_pdb()
            tabs5 = _tables_checked(s5)
            if args.workload == "24_bins":
                out.extend(sec_bins(s5, tabs5, peaks, threads, args.cpu_bin_seconds, args.frontier24))
            elif args.workload == "yama24":
                out.append(sec_yama24(s5, tabs5, peaks, threads))
            elif args.workload == "lb_ab":
                out.append(sec_lb_ab(s5, args.tuples, args.epochs, args.ab_bin, args.frontier24, log,
                                     persistent=args.persistent))
    for d in out:
        print(json.dumps(d), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--probe", choices=["balanced", "mixed", "sectors"], default=None)
    ap.add_argument("--workload", choices=["15_md_walk60", "15_mixed4096", "24_bins", "yama24", "lb_ab"],
                    default=None)
    ap.add_argument("--tuples", type=int, default=1_000_000,
                    help="training tuples of the learned-balancer A/B (0 skips it)")
    ap.add_argument("--epochs", type=int, default=3)
    ap.add_argument("--ab-bin", type=int, default=200)
    ap.add_argument("--frontier24", type=int, default=8192, help="root set per 24-puzzle instance")
    ap.add_argument("--probe-heuristic", default="pdb", choices=["manhattan", "pdb"])
    ap.add_argument("--probe-width", type=int, default=4)
    ap.add_argument("--probe-slack", type=int, default=8)
    ap.add_argument("--roots", type=int, default=100000)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--instances", type=int, default=100)
    ap.add_argument("--frontier", type=int, default=3072)
    ap.add_argument("--lb", default="static")
    ap.add_argument("--persistent", type=int, default=None, choices=[0, 1],
                    help="threshold loop on the device (default: the library's, 1)")
    ap.add_argument("--handback", type=int, default=None,
                    help="persistent mode: nodes per instance iteration from which the host round loop takes over "
                         "(default: the library's, 600000; 0 = never)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the configured settings instead of the autotuner's (cached per GPU, puzzle, "
                         "heuristic and batch size)")
    ap.add_argument("--cpu-bin-seconds", type=float, default=3.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
    args = ap.parse_args()
    if args.probe == "sectors":
        return run_sector_probe(args)
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

    def log(m):
        if rank == 0:
            print("[bench %.1fs] %s" % (time.perf_counter() - t_start, m), file=sys.stderr, flush=True)
    t_start = time.perf_counter()
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
    peaks = measure_peaks()
    log("peaks %s" % peaks)
    tuned, tuned_hit = None, None
    if not args.no_autotune:
        tuned, tuned_hit = slide.autotune_cached(solver, states, torch.cuda.get_device_name(local), reps=2)
        log("autotuned %s (cache hit %s)" % (tuned, tuned_hit))
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
    lane_steps, lane_slots = 0, 0
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
            round_ms = [round(x, 3) for x in st["round_kernel_ms"]]
            rounds += st["rounds"]
            donated += st["tasks_donated"]
            lane_steps += st["dev_lane_steps"]
            lane_slots += st["dev_lane_slots"]
            if check(res) != ref_lens:
                raise RuntimeError("lengths changed between steps")
            nodes += sum(res[i].nodes_total for i in range(n))
        answers = [(res[i].len, res[i].nodes_total) for i in range(n)]

        # e2e: host buffers through sp_solve_batch (H2D/D2H inside); the
        # clocks are sampled over both timed loops
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
    total_ms = sum(step_ms)
    (total_ms,), (all_nodes,) = job_max_sum([total_ms], [nodes], world, "cuda")
    value = all_nodes / (total_ms / 1000.0)
    e2e_total = sum(e2e_ms)
    (e2e_total,), _ = job_max_sum([e2e_total], [], world, "cuda")
    e2e_value = all_nodes / (e2e_total / 1000.0)
    log("headline %.3g nodes/s, e2e %.3g" % (value, e2e_value))

    hbm_peak, hbm_kind = load_peaks()
    kms = sum(kern_ms)
    traffic = None  # DRAM bytes per search launch, from the committed ncu summary
    prof = os.path.join(ROOT, "profiles", "search_hybrid_pdb15_random100.md")
    if os.path.exists(prof):
        for line in open(prof):
            if line.startswith("traffic_bytes_per_launch:"):
                traffic = float(line.split(":")[1])
    roofline = _sector_roofline(nodes, kms, peaks["l2_random_reads_per_s"], "l2-random", slide.pdb_table_bytes(4))
    roofline.update({
        "traffic": traffic, "kernel": "search_round_kernel<4,pdb> (+ split pre-pass and pool set-up)",
        "int_issue": _int_roofline(nodes, kms, peaks["int_ops_per_s"]),
        "hbm_copy": {"peak": hbm_peak, "peak_kind": hbm_kind, "unit": "GB/s",
                     "frac_if_every_lookup_went_to_dram": nodes * BYTES_PER_NODE / (kms / 1000.0) / 1e9 / hbm_peak,
                     "note": "the 3 MB of tables stay in L2: DRAM bytes per launch are `traffic`"}})
    cpu, sec = None, None
    if rank == 0 and not args.no_cpu_baseline:
        oracle = oracle_module()
        c = cpu_full(w, states, oracle.PDB, _tables_checked(solver), host_threads())
        cpu = {k: c[k] for k in ("value", "unit", "cores", "kind", "sample", "instances_per_s", "seconds")}
        cpu["same_answers"] = c["answers"] == answers
        log("cpu baseline %.3g nodes/s" % c["value"])
    if rank == 0 and not args.no_secondary:
        sec = secondary(args, peaks, host_threads(), log)
    if rank == 0:
        cfg = solver.config
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded)",
            "config": {"workload": HEADLINE, "instances_per_gpu": n,
                       "heuristic": "additive 5-5-5 PDB, max(regular, reflected)",
                       "frontier_target": int(cfg.frontier_target), "lb": args.lb + "+donation",
                       "threshold_loop": (("device, handing iterations predicted at >= %d nodes per "
                                           "instance to the host round loop" % cfg.handback_nodes
                                           if cfg.handback_nodes else "device (one launch)")
                                          if cfg.persistent else "host (one launch per round)"),
                       "autotuned": dict(tuned, cache_hit=tuned_hit) if tuned else None,
                       "parallelism": "replicas" if world > 1 else "1 GPU",
                       "l2": "512 MB buffer written between timed steps",
                       "pdb_build_ms": round(pdb_ms, 2)},
            "instances_per_s": world * n * args.steps / (total_ms / 1000.0),
            "nodes_per_step": all_nodes / args.steps,
            "rounds_per_step": rounds / args.steps,
            "tasks_donated_per_step": donated / args.steps,
            "kernel_ms_per_step": kms / args.steps,
            "step_ms": [round(x, 3) for x in step_ms],
            "last_step_round_kernel_ms": round_ms,
            "lane_step_fraction": lane_steps / max(1, lane_slots),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d // args.steps,
                    "d2h_bytes_per_step": d2h // args.steps, "ms_per_step": e2e_total / args.steps,
                    "instances_per_s": world * n * args.steps / (e2e_total / 1000.0)},
            "gpu_launches": launches,
            "roofline": roofline,
            "peaks_measured": peaks,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "secondary": sec,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
