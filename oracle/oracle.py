"""ctypes wrapper of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module; the product (libslide) never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
CACHE = os.path.join(HERE, "_cache")
MAX_ITERS = 96
MAX_MOVES = 240
MD, PDB = 0, 1
ALL, FIRST = 0, 1
BLANK_FREE, BLANK_ANY, BLANK_HOME = 0, 1, 2


class OrcResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("len", ctypes.c_int32), ("n_iter", ctypes.c_int32),
                ("n_moves", ctypes.c_int32), ("nodes_total", ctypes.c_uint64),
                ("f_limit", ctypes.c_int32 * MAX_ITERS), ("nodes", ctypes.c_uint64 * MAX_ITERS),
                ("moves", ctypes.c_uint8 * MAX_MOVES), ("seconds", ctypes.c_double)]


class OrcHeur(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("heuristic", ctypes.c_int), ("tables", ctypes.c_void_p * 4)]


_lib = None


def build():
    r = subprocess.run(["make", "-s", "-C", HERE, "liboracle.so", "oracle_cli"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        lib.orc_solve_batch.argtypes = [ctypes.POINTER(OrcHeur), ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(OrcResult)]
        lib.orc_solve_batch.restype = ctypes.c_int
        lib.orc_solve_batch_split.argtypes = [ctypes.POINTER(OrcHeur), ctypes.c_void_p, ctypes.c_int,
                                              ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(OrcResult)]
        lib.orc_solve_batch_split.restype = ctypes.c_int
        lib.orc_first_path.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p]
        lib.orc_first_path.restype = ctypes.c_int
        lib.orc_heuristic.argtypes = [ctypes.POINTER(OrcHeur), ctypes.c_void_p]
        lib.orc_heuristic.restype = ctypes.c_int
        lib.orc_pdb_build.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        lib.orc_pdb_build.restype = ctypes.c_int
        lib.orc_table_size.argtypes = [ctypes.c_int]
        lib.orc_table_size.restype = ctypes.c_uint64
        lib.orc_num_tables.argtypes = [ctypes.c_int]
        lib.orc_num_tables.restype = ctypes.c_int
        _lib = lib
    return _lib


def table_size(width):
    return int(load().orc_table_size(width))


def num_tables(width):
    return int(load().orc_num_tables(width))


def build_table(width, table_id, semantics=BLANK_HOME, threads=0):
    out = np.empty(table_size(width), dtype=np.uint8)
    st = load().orc_pdb_build(width, table_id, semantics, threads, out.ctypes.data)
    if st != 0:
        raise RuntimeError("orc_pdb_build failed: %d" % st)
    return out


def tables(width, semantics=BLANK_HOME, cache=True):
    """All tables of a width, cached on disk under oracle/_cache."""
    out = []
    for t in range(num_tables(width)):
        path = os.path.join(CACHE, "pdb%d_%d_s%d.bin" % (width, t, semantics))
        if cache and os.path.exists(path) and os.path.getsize(path) == table_size(width):
            out.append(np.fromfile(path, dtype=np.uint8))
            continue
        arr = build_table(width, t, semantics)
        if cache:
            os.makedirs(CACHE, exist_ok=True)
            arr.tofile(path + ".tmp")
            os.replace(path + ".tmp", path)
        out.append(arr)
    return out


def _heur(width, heuristic, tabs):
    h = OrcHeur()
    h.width = width
    h.heuristic = heuristic
    for i, t in enumerate(tabs or []):
        h.tables[i] = t.ctypes.data
    return h


def solve(width, tiles, heuristic=MD, tabs=None, mode=ALL, threads=None, node_budget=0, split=False):
    """Solve a batch.  One instance per thread at a time; with split=True all
    threads work on one instance at a time (orc_solve_batch_split: same
    lengths and counts, ALL mode only, budget checked between iterations)."""
    a = np.ascontiguousarray(np.asarray(tiles, dtype=np.uint8)).reshape(-1, width * width)
    n = a.shape[0]
    res = (OrcResult * max(1, n))()
    h = _heur(width, heuristic, tabs)
    threads = threads or os.cpu_count() or 1
    if split:
        if mode != ALL:
            raise ValueError("split solves support the all-solutions mode only")
        st = load().orc_solve_batch_split(ctypes.byref(h), a.ctypes.data, n, node_budget, threads, res)
    else:
        st = load().orc_solve_batch(ctypes.byref(h), a.ctypes.data, n, mode, node_budget, threads, res)
    if st != 0:
        raise RuntimeError("orc_solve_batch failed: %d" % st)
    out = []
    for i in range(n):
        r = res[i]
        k = r.n_iter
        out.append({"status": r.status, "len": r.len, "n_iter": k, "f_limit": list(r.f_limit[:k]),
                    "nodes": [int(x) for x in r.nodes[:k]], "nodes_total": int(r.nodes_total),
                    "moves": bytes(r.moves[: r.n_moves]), "seconds": r.seconds})
    return out


def heuristic(width, tiles, heuristic=MD, tabs=None):
    a = np.ascontiguousarray(np.asarray(tiles, dtype=np.uint8)).reshape(-1, width * width)
    h = _heur(width, heuristic, tabs)
    return np.array([load().orc_heuristic(ctypes.byref(h), a[i].ctypes.data) for i in range(a.shape[0])])


PLAN_STRIDE = 252


def first_paths(tiles, f_limit, h_diff=None, movable=None):
    """Horie's per-root search on the CPU: one plan row per 15-puzzle root,
    [len, moves...] or [-1] (orc_first_path)."""
    a = np.ascontiguousarray(np.asarray(tiles, dtype=np.uint8)).reshape(-1, 16)
    out = np.zeros((a.shape[0], PLAN_STRIDE), dtype=np.int8)
    hd = None if h_diff is None else np.ascontiguousarray(np.asarray(h_diff, dtype=np.int8).reshape(-1))
    mv = None if movable is None else np.ascontiguousarray(np.asarray(movable, dtype=np.uint8).reshape(-1))
    for i in range(a.shape[0]):
        st = load().orc_first_path(a[i].ctypes.data, int(f_limit), None if hd is None else hd.ctypes.data,
                                   None if mv is None else mv.ctypes.data, out[i].ctypes.data)
        if st != 0:
            raise RuntimeError("orc_first_path failed: %d" % st)
    return out
