"""Python binding of libslide (include/slide.h) over ctypes.

Mirrors the reference's solver interface -- state in, optimal move sequence
and per-iteration node counts out (src/24puzzle_expand.cc:146-164 prints
`len node_num`; src/24puzzle_block_parallel_with_pdb.cu:756-922 solves one
instance per call) -- for batches of instances on one GPU.  There is no CPU
search path: loading fails loudly when libslide.so is missing, and creating
a solver fails when no GPU is usable.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libslide.so")

SP_MAX_ITERS = 96
SP_PLAN_STRIDE = 252
SP_MAX_MOVES = 240
HEUR = {"manhattan": 0, "md": 0, "pdb": 1}
LB = {"steal": 0, "static": 1, "static_steal": 1, "none": 2, "learned": 3}
MOVE_NAMES = "URLD"  # blank moves: 0 up, 1 right, 2 left, 3 down


class SlideError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


class SpConfig(ctypes.Structure):
    _fields_ = [("frontier_target", ctypes.c_int32), ("threads_per_block", ctypes.c_int32),
                ("blocks_per_sm", ctypes.c_int32), ("lb_mode", ctypes.c_int32),
                ("donate_min_slack", ctypes.c_int32), ("steps_per_poll", ctypes.c_int32),
                ("timeout_ms", ctypes.c_int32), ("static_split_cap", ctypes.c_int32),
                ("donate_reserve", ctypes.c_int32), ("persistent", ctypes.c_int32),
                ("handback_nodes", ctypes.c_int32)]


class SpResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("len", ctypes.c_int32), ("n_iter", ctypes.c_int32),
                ("n_moves", ctypes.c_int32), ("nodes_total", ctypes.c_uint64),
                ("f_limit", ctypes.c_int32 * SP_MAX_ITERS), ("nodes", ctypes.c_uint64 * SP_MAX_ITERS),
                ("moves", ctypes.c_uint8 * SP_MAX_MOVES), ("seconds", ctypes.c_double)]


SP_MAX_ROUNDS = 96


class SpStats(ctypes.Structure):
    _fields_ = [("frontier_ms", ctypes.c_double), ("kernel_ms", ctypes.c_double), ("wall_ms", ctypes.c_double),
                ("rounds", ctypes.c_int32), ("kernel_launches", ctypes.c_int32),
                ("tasks_initial", ctypes.c_uint64), ("tasks_donated", ctypes.c_uint64),
                ("nodes", ctypes.c_uint64), ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
                ("round_instances", ctypes.c_int32 * SP_MAX_ROUNDS), ("round_tasks", ctypes.c_int32 * SP_MAX_ROUNDS),
                ("round_kernel_ms", ctypes.c_float * SP_MAX_ROUNDS),
                ("round_host_ms", ctypes.c_float * SP_MAX_ROUNDS),
                ("round_nodes", ctypes.c_uint64 * SP_MAX_ROUNDS), ("round_donated", ctypes.c_uint64 * SP_MAX_ROUNDS),
                ("dev_lane_steps", ctypes.c_uint64), ("dev_lane_slots", ctypes.c_uint64),
                ("dev_idle_cycles", ctypes.c_uint64), ("dev_warp_cycles", ctypes.c_uint64),
                ("dev_donate_tries", ctypes.c_uint64), ("dev_donate_notfree", ctypes.c_uint64),
                ("dev_donate_nowait", ctypes.c_uint64), ("dev_tasks_done", ctypes.c_uint64)]


_lib = None


def load(build=True):
    """Load libslide.so (building it first when `build` and sources changed)."""
    global _lib
    if _lib is not None:
        return _lib
    if build:
        import importlib.util
        spec = importlib.util.spec_from_file_location("slide_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    if not os.path.exists(LIB_PATH):
        raise OSError("libslide.so not built: %s" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    P, I32, U64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint64
    sig = {
        "sp_config_default": (None, [ctypes.POINTER(SpConfig)]),
        "sp_create": (I32, [I32, I32, ctypes.POINTER(SpConfig), ctypes.POINTER(P)]),
        "sp_destroy": (None, [P]),
        "sp_set_config": (I32, [P, ctypes.POINTER(SpConfig)]),
        "sp_pdb_build": (I32, [P]),
        "sp_pdb_table_size": (U64, [I32]),
        "sp_pdb_num_tables": (I32, [I32]),
        "sp_pdb_export": (I32, [P, I32, P, U64]),
        "sp_pdb_import": (I32, [P, I32, P, U64]),
        "sp_heuristic": (I32, [P, P, I32, P]),
        "sp_solve_batch": (I32, [P, P, I32, ctypes.POINTER(SpResult)]),
        "sp_solve_batch_device": (I32, [P, P, I32, ctypes.POINTER(SpResult)]),
        "sp_dfs_round": (I32, [P, P, P, P, I32, I32, P, P]),
        "sp_last_stats": (I32, [P, ctypes.POINTER(SpStats)]),
        "sp_status_string": (ctypes.c_char_p, [I32]),
        "sp_last_error": (ctypes.c_char_p, [P]),
        "sp_kernel_launch_count": (U64, []),
        "sp_lbm_num_params": (U64, [I32]),
        "sp_lbm_init": (I32, [P, U64]),
        "sp_lbm_import": (I32, [P, P, U64]),
        "sp_lbm_export": (I32, [P, P, U64]),
        "sp_lbm_predict": (I32, [P, P, P, I32, P]),
        "sp_lbm_train_step": (I32, [P, P, P, P, I32, ctypes.c_float, P]),
        "sp_lbm_gradients": (I32, [P, P, P, P, I32, P, P]),
        "sp_gemm_bf16_nt": (I32, [P, P, P, I32, I32, I32]),
        "sp_selftest_stall": (I32, [P, I32, P]),
        "sp_selftest_gemm_stall": (I32, [I32, I32, P]),
        "sp_probe_int_issue": (I32, [I32, I32, P, P]),
        "sp_probe_random_sectors": (I32, [U64, I32, I32, P, P]),
        "sp_dfs_round_md_noalloc": (I32, [I32, P, P, P, I32, I32, P, P, P]),
        "sp_idas_parallel": (I32, [P, I32, P, I32, P, P, P]),
        "sp_root_set_template": (I32, [I32, I32, I32, P, ctypes.c_uint32, P, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def root_set_template(width, blank, target, cap=0):
    """The root-set template of a blank cell (host only, no GPU): (nodes,
    depth, leaves, paths) with paths the first `cap` nodes in breadth-first
    order as 2-bit move sequences from the root, first move lowest."""
    lib = load()
    paths = np.zeros(max(cap, 1), dtype=np.uint64)
    n, d, nl = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
    st = lib.sp_root_set_template(int(width), int(blank), int(target), paths.ctypes.data, int(cap),
                                  ctypes.byref(n), ctypes.byref(d), ctypes.byref(nl))
    if st != 0:
        raise SlideError(st, "sp_root_set_template: %s" % lib.sp_status_string(st).decode())
    return n.value, d.value, nl.value, paths[: min(cap, n.value)]


def default_config(**overrides):
    lib = load()
    cfg = SpConfig()
    lib.sp_config_default(ctypes.byref(cfg))
    for k, v in overrides.items():
        if k == "lb_mode" and isinstance(v, str):
            v = LB[v]
        setattr(cfg, k, int(v))
    return cfg


def _as_tiles(tiles, width):
    a = np.ascontiguousarray(np.asarray(tiles, dtype=np.uint8))
    if a.ndim == 1:
        a = a.reshape(1, -1)
    if a.ndim != 2 or a.shape[1] != width * width:
        raise ValueError("tiles must have shape (n, %d)" % (width * width))
    return a


class Solver:
    """One GPU solver (one CUDA stream, device memory owned by the handle)."""

    def __init__(self, width, heuristic="manhattan", config=None, **overrides):
        self.lib = load()
        self.width = int(width)
        self.heuristic = heuristic
        cfg = config if config is not None else default_config(**overrides)
        h = ctypes.c_void_p()
        st = self.lib.sp_create(self.width, HEUR[heuristic], ctypes.byref(cfg), ctypes.byref(h))
        if st != 0:
            raise SlideError(st, "sp_create failed: %s" % self.lib.sp_status_string(st).decode())
        self.h = h
        self.config = cfg

    def _check(self, st, what):
        if st != 0:
            msg = self.lib.sp_last_error(self.h).decode() or self.lib.sp_status_string(st).decode()
            raise SlideError(st, "%s: %s" % (what, msg))

    def close(self):
        if getattr(self, "h", None):
            self.lib.sp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_config(self, **overrides):
        cfg = SpConfig.from_buffer_copy(self.config)
        for k, v in overrides.items():
            if k == "lb_mode" and isinstance(v, str):
                v = LB[v]
            setattr(cfg, k, int(v))
        self._check(self.lib.sp_set_config(self.h, ctypes.byref(cfg)), "sp_set_config")
        self.config = cfg

    # --- pattern databases ---
    def build_pdb(self):
        self._check(self.lib.sp_pdb_build(self.h), "sp_pdb_build")

    def table_size(self):
        return int(self.lib.sp_pdb_table_size(self.width))

    def num_tables(self):
        return int(self.lib.sp_pdb_num_tables(self.width))

    def export_pdb(self, table):
        out = np.empty(self.table_size(), dtype=np.uint8)
        self._check(self.lib.sp_pdb_export(self.h, table, out.ctypes.data, out.size), "sp_pdb_export")
        return out

    def import_pdb(self, table, data):
        a = np.ascontiguousarray(np.asarray(data, dtype=np.uint8))
        self._check(self.lib.sp_pdb_import(self.h, table, a.ctypes.data, a.size), "sp_pdb_import")

    # --- search ---
    def heuristic_values(self, tiles):
        a = _as_tiles(tiles, self.width)
        out = np.empty(a.shape[0], dtype=np.int32)
        self._check(self.lib.sp_heuristic(self.h, a.ctypes.data, a.shape[0], out.ctypes.data), "sp_heuristic")
        return out

    def solve_raw(self, tiles):
        a = _as_tiles(tiles, self.width)
        res = (SpResult * max(1, a.shape[0]))()
        self._check(self.lib.sp_solve_batch(self.h, a.ctypes.data, a.shape[0], res), "sp_solve_batch")
        return res

    def solve(self, tiles):
        """Solve a batch; returns one dict per instance."""
        return [result_dict(r) for r in self.solve_raw(tiles)[: _as_tiles(tiles, self.width).shape[0]]]

    def solve_device_raw(self, dev_ptr, n):
        res = (SpResult * max(1, n))()
        self._check(self.lib.sp_solve_batch_device(self.h, ctypes.c_void_p(dev_ptr), n, res),
                    "sp_solve_batch_device")
        return res

    def dfs_round(self, roots, depth, pre, limit):
        """One threshold round over a root set (the reference's dfs_kernel)."""
        a = _as_tiles(roots, self.width)
        n = a.shape[0]
        d = np.ascontiguousarray(np.asarray(depth, dtype=np.int32).reshape(n))
        p = np.ascontiguousarray(np.asarray(pre, dtype=np.int32).reshape(n))
        nodes = np.zeros(n, dtype=np.uint64)
        found = ctypes.c_int32(-1)
        self._check(self.lib.sp_dfs_round(self.h, a.ctypes.data, d.ctypes.data, p.ctypes.data, n, int(limit),
                                          nodes.ctypes.data, ctypes.byref(found)), "sp_dfs_round")
        return nodes, int(found.value)

    def selftest_stall(self, timeout_ms=200):
        """Device status of a search launch whose only task never arrives
        (SP_ERR_TIMEOUT = -8 when the bounded waits work)."""
        st = ctypes.c_int32(0)
        self._check(self.lib.sp_selftest_stall(self.h, int(timeout_ms), ctypes.byref(st)), "sp_selftest_stall")
        return int(st.value)

    # --- learned load balancer ---
    def lbm_num_params(self):
        return int(self.lib.sp_lbm_num_params(self.width))

    def lbm_init(self, seed=1):
        self._check(self.lib.sp_lbm_init(self.h, int(seed)), "sp_lbm_init")

    def lbm_import(self, params):
        a = np.ascontiguousarray(np.asarray(params, dtype=np.float32))
        self._check(self.lib.sp_lbm_import(self.h, a.ctypes.data, a.size), "sp_lbm_import")

    def lbm_export(self):
        out = np.empty(self.lbm_num_params(), dtype=np.float32)
        self._check(self.lib.sp_lbm_export(self.h, out.ctypes.data, out.size), "sp_lbm_export")
        return out

    def _lbm_rows(self, tiles, slack):
        a = _as_tiles(tiles, self.width)
        s = np.ascontiguousarray(np.asarray(slack, dtype=np.int32).reshape(a.shape[0]))
        return a, s

    def lbm_predict(self, tiles, slack):
        a, s = self._lbm_rows(tiles, slack)
        out = np.empty(a.shape[0], dtype=np.float32)
        self._check(self.lib.sp_lbm_predict(self.h, a.ctypes.data, s.ctypes.data, a.shape[0], out.ctypes.data),
                    "sp_lbm_predict")
        return out

    def lbm_train_step(self, tiles, slack, target, lr):
        a, s = self._lbm_rows(tiles, slack)
        t = np.ascontiguousarray(np.asarray(target, dtype=np.float32).reshape(a.shape[0]))
        loss = ctypes.c_float(0)
        self._check(self.lib.sp_lbm_train_step(self.h, a.ctypes.data, s.ctypes.data, t.ctypes.data, a.shape[0],
                                               float(lr), ctypes.byref(loss)), "sp_lbm_train_step")
        return float(loss.value)

    def lbm_gradients(self, tiles, slack, target):
        a, s = self._lbm_rows(tiles, slack)
        t = np.ascontiguousarray(np.asarray(target, dtype=np.float32).reshape(a.shape[0]))
        g = np.empty(self.lbm_num_params(), dtype=np.float32)
        loss = ctypes.c_float(0)
        self._check(self.lib.sp_lbm_gradients(self.h, a.ctypes.data, s.ctypes.data, t.ctypes.data, a.shape[0],
                                              g.ctypes.data, ctypes.byref(loss)), "sp_lbm_gradients")
        return float(loss.value), g

    def stats(self):
        s = SpStats()
        self._check(self.lib.sp_last_stats(self.h, ctypes.byref(s)), "sp_last_stats")
        out = {}
        for f, _ in SpStats._fields_:
            v = getattr(s, f)
            out[f] = list(v)[: s.rounds] if f.startswith("round_") else v
        return out


def result_dict(r):
    n = r.n_iter
    return {
        "status": int(r.status),
        "len": int(r.len),
        "n_iter": int(n),
        "f_limit": [int(x) for x in r.f_limit[:n]],
        "nodes": [int(x) for x in r.nodes[:n]],
        "nodes_total": int(r.nodes_total),
        "moves": bytes(r.moves[: r.n_moves]),
        "seconds": float(r.seconds),
    }


AUTOTUNE_SPACE = (
    ("threads_per_block", (256, 128)),
    ("steps_per_poll", (32, 16, 64)),
    ("persistent", (1, 0)),
    ("handback_nodes", (600000, 300000, 1200000, 0, 3000000)),
    ("donate_reserve", (0, -1, 30000)),
    ("donate_min_slack", (6, 4, 8, 10)),
    ("frontier_target", (3072, 2048, 1024, 4096, 8192, 16384)),
)


def autotune(solver, tiles, space=AUTOTUNE_SPACE, reps=2, clock=None, log=None):
    """Pick the fastest launch and balance settings for a workload.

    Coordinate descent over `space` (parameter, candidate values), starting
    from the solver's current settings; each candidate is timed as the best
    of `reps` host-buffer solves after one untimed solve.  These settings
    change only speed: every candidate must return the same lengths and
    per-iteration node counts, and a candidate that does not raises.  The
    solver is left with the best settings; returns (best settings dict,
    [(settings, seconds), ...]).
    """
    import time
    clock = clock or time.perf_counter
    a = _as_tiles(tiles, solver.width)
    cur = {f: int(getattr(solver.config, f)) for f, _ in SpConfig._fields_}
    want = None
    tried = {}

    def measure(cfg):
        key = tuple(sorted(cfg.items()))
        if key in tried:
            return tried[key]
        solver.set_config(**cfg)
        solver.solve_raw(a)
        best, got = None, None
        for _ in range(max(1, reps)):
            t0 = clock()
            res = solver.solve_raw(a)
            dt = clock() - t0
            if best is None or dt < best:
                best = dt
            got = [(int(r.status), int(r.len), tuple(int(x) for x in r.nodes[:r.n_iter])) for r in res[:a.shape[0]]]
        nonlocal want
        if want is None:
            want = got
        elif got != want:
            raise RuntimeError("autotune: results changed under %s" % (cfg,))
        tried[key] = best
        if log:
            log("%s: %.2f ms" % (cfg, best * 1e3))
        return best

    best_t = measure(dict(cur))
    for name, values in space:
        for v in values:
            if v == cur[name]:
                continue
            cand = dict(cur, **{name: v})
            t = measure(cand)
            if t < best_t:
                best_t, cur = t, cand
    solver.set_config(**cur)
    history = [(dict(k), t) for k, t in tried.items()]
    return cur, history


def autotune_cache_path():
    """Where autotune_cached keeps its results: $SLIDE_AUTOTUNE_CACHE, else
    ~/.cache/slide/autotune.json."""
    return os.environ.get("SLIDE_AUTOTUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "slide",
                                                                    "autotune.json")


def autotune_key(device, solver, tiles):
    """Cache key: the GPU, the puzzle, the heuristic and the batch size
    (rounded down to a power of two: the best root-set size and loop shape
    depend on how many instances share the GPU)."""
    n = max(1, _as_tiles(tiles, solver.width).shape[0])
    return "%s|w%d|%s|n%d" % (device, solver.width, solver.heuristic, 1 << (n.bit_length() - 1))


def autotune_cached(solver, tiles, device, path=None, **kw):
    """autotune() with a per-(GPU, puzzle, heuristic, batch size) cache of the
    winning settings in a JSON file: a hit applies the stored settings
    without timing anything.  Returns (settings, hit)."""
    import json
    path = path or autotune_cache_path()
    key = autotune_key(device, solver, tiles)
    cache = {}
    if os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    if key in cache:
        cfg = {k: int(v) for k, v in cache[key].items() if k in dict(SpConfig._fields_)}
        solver.set_config(**cfg)
        return cfg, True
    best, _ = autotune(solver, tiles, **kw)
    cache[key] = best
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".%d.tmp" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)
    return best, False


def gemm_bf16_nt(a_bits, b_bits):
    """C = A . B^T on the tensor cores; A [m][k], B [256][k] as bf16 bit patterns (uint16)."""
    lib = load()
    a = np.ascontiguousarray(np.asarray(a_bits, dtype=np.uint16))
    b = np.ascontiguousarray(np.asarray(b_bits, dtype=np.uint16))
    m, k = a.shape
    n = b.shape[0]
    c = np.empty((m, n), dtype=np.float32)
    st = lib.sp_gemm_bf16_nt(a.ctypes.data, b.ctypes.data, c.ctypes.data, m, n, k)
    if st != 0:
        raise SlideError(st, "sp_gemm_bf16_nt failed: %s" % lib.sp_status_string(st).decode())
    return c


def idas_parallel(d_input, n, d_plan, f_limit, d_h_diff_table=None, d_movable_table=None, stream=None):
    """Horie's idas_parallel_main on device pointers (sp_idas_parallel):
    every root searched on its own to f_limit, its first goal path in
    depth-first order into its SP_PLAN_STRIDE-byte plan row.  Asynchronous
    on `stream` (an int handle or None)."""
    lib = load()
    st = lib.sp_idas_parallel(ctypes.c_void_p(d_input), int(n), ctypes.c_void_p(d_plan), int(f_limit),
                              ctypes.c_void_p(d_h_diff_table) if d_h_diff_table else None,
                              ctypes.c_void_p(d_movable_table) if d_movable_table else None,
                              ctypes.c_void_p(stream) if stream else None)
    if st != 0:
        raise SlideError(st, "sp_idas_parallel failed: %s" % lib.sp_status_string(st).decode())


def selftest_gemm_stall(starve_chunk=1, timeout_ms=50):
    """Device status of a tensor-core GEMM one of whose K chunks is never
    copied in (SP_ERR_TIMEOUT = -8 when its bounded waits work)."""
    lib = load()
    st = ctypes.c_int32(0)
    rc = lib.sp_selftest_gemm_stall(int(starve_chunk), int(timeout_ms), ctypes.byref(st))
    if rc != 0:
        raise SlideError(rc, "sp_selftest_gemm_stall failed: %s" % lib.sp_status_string(rc).decode())
    return int(st.value)


def kernel_launch_count():
    return int(load().sp_kernel_launch_count())


# Integer operations per generated node that the Manhattan search's
# roofline charges, counted on the serial reference search
# (src/24puzzle_expand.cc:111-143) plus the path push that returning a
# solution needs: move legality 1, reverse-move test 1, node count 1, tile
# read 1, blank swap 2, heuristic update 4 (two table reads, a subtraction,
# an addition), goal test 1, f = g + h and its limit test 2, path push 1,
# undo 2.
MD_OPS_PER_NODE = 16


def probe_int_issue(iters=1 << 16, reps=3):
    """(lane operations per second, best launch ms) of the current device:
    the integer-issue roofline denominator (sp_probe_int_issue)."""
    lib = load()
    rate, ms = ctypes.c_double(), ctypes.c_double()
    st = lib.sp_probe_int_issue(int(iters), int(reps), ctypes.byref(rate), ctypes.byref(ms))
    if st != 0:
        raise SlideError(st, "sp_probe_int_issue failed: %s" % lib.sp_status_string(st).decode())
    return rate.value, ms.value


# Bytes a generated node of the PDB search reads, as the roofline charges
# them: one regular and one reflected table entry, each its own 32-byte
# sector (the pattern indices of different lanes never share a sector).
PDB_BYTES_PER_NODE = 64
SECTOR_BYTES = 32


def probe_random_sectors(working_set_bytes, iters=256, reps=3):
    """(random one-byte reads per second, best launch ms) from a device
    buffer of `working_set_bytes`: the PDB search's roofline denominator
    (sp_probe_random_sectors); x 32 bytes = sector bandwidth."""
    lib = load()
    rate, ms = ctypes.c_double(), ctypes.c_double()
    st = lib.sp_probe_random_sectors(int(working_set_bytes), int(iters), int(reps), ctypes.byref(rate),
                                     ctypes.byref(ms))
    if st != 0:
        raise SlideError(st, "sp_probe_random_sectors failed: %s" % lib.sp_status_string(st).decode())
    return rate.value, ms.value


def pdb_table_bytes(width):
    """Bytes of the device lookup tables the PDB search reads (width 4: three
    16^5-byte tables; width 5: two 25^6-byte tables)."""
    return 3 * 16 ** 5 if width == 4 else 2 * 25 ** 6


def replay(tiles, moves, width):
    """Apply blank moves to a state; returns the final state (numpy)."""
    b = np.array(tiles, dtype=np.uint8).reshape(-1).copy()
    blank = int(np.flatnonzero(b == 0)[0])
    delta = (-width, 1, -1, width)
    for m in moves:
        r, c = divmod(blank, width)
        ok = (m == 0 and r > 0) or (m == 1 and c < width - 1) or (m == 2 and c > 0) or (m == 3 and r < width - 1)
        if not ok:
            raise ValueError("illegal move %d at blank %d" % (m, blank))
        src = blank + delta[m]
        b[blank], b[src] = b[src], 0
        blank = src
    return b


def is_solution(tiles, moves, width):
    return bool(np.array_equal(replay(tiles, moves, width), np.arange(width * width, dtype=np.uint8)))
