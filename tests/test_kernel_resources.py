"""Resource budget of the search kernel, read from ptxas's report (no GPU).

The search launches 768 threads per SM (three 256-thread blocks), which
leaves 65536 / 768 = 85 registers per thread; the kernels are built for 80.
The host round loop's kernels must not spill (the 15-puzzle ones and the
Manhattan 24-puzzle one) or barely (16 bytes for the 24-puzzle PDB one); the
persistent (multi-iteration) kernels keep a small stack for the out-of-line
call that publishes an iteration (an earlier build that inlined it used 126
registers and ran 1.4-1.7x slower).  Three
blocks per SM must also fit the shared memory of one SM (228 KB)."""
import os
import re
import subprocess

import pytest

from conftest import REPO

PKG = os.path.join(REPO, "sliding-puzzle_gb300")


def _build_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("slide_build", os.path.join(PKG, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _ptxas_report():
    build = _build_module()
    out = os.path.join(build.BUILD, "search_ptxas.o")
    os.makedirs(build.BUILD, exist_ok=True)
    cmd = [build.nvcc(), *build.ARCH, *build.FLAGS, "-Xptxas", "-v", "-c",
           os.path.join(build.CSRC, "search.cu"), "-o", out]
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    except FileNotFoundError:
        pytest.skip("nvcc not found")
    assert r.returncode == 0, r.stderr
    kernels, cur = {}, None
    for line in r.stderr.splitlines():
        m = re.search(r"(?:Compiling entry function|Function properties for) '?([\w$]+)'?", line)
        if m:
            cur = m.group(1)
            continue
        if cur is None:
            continue
        k = kernels.setdefault(cur, {})
        m = re.search(r"(\d+) bytes spill stores, (\d+) bytes spill loads", line)
        if m:
            k["spill"] = int(m.group(1)) + int(m.group(2))
        m = re.search(r"Used (\d+) registers.*?(\d+) bytes smem", line)
        if m:
            k["regs"], k["smem"] = int(m.group(1)), int(m.group(2))
    return kernels


def _args(mangled):
    """Template arguments of sp::search_round_kernel<W, PDB, BLOCK, WORDS, MULTI>."""
    d = subprocess.run(["c++filt", mangled], capture_output=True, text=True).stdout.strip()
    m = re.search(r"search_round_kernel<(\d+), (true|false), (\d+), (\d+), (true|false)>", d)
    return None if not m else (int(m.group(1)), m.group(2) == "true", int(m.group(3)), m.group(5) == "true")


def test_search_kernel_registers_spills_and_shared_memory():
    kernels = _ptxas_report()
    seen = 0
    for name, k in kernels.items():
        a = _args(name) if "search_round_kernel" in name else None
        if a is None:
            continue
        w, pdb, block, multi = a
        seen += 1
        assert k["regs"] <= 80, (a, k)
        assert (768 // block) * (k["smem"] + 1024) <= 228 * 1024, (a, k)
        if not multi and (w == 4 or not pdb):
            assert k["spill"] == 0, (a, k)
        else:
            assert k["spill"] <= 1024, (a, k)
    assert seen == 16
