"""libslide's C ABI without a GPU: the library builds, loads, exports every
symbol include/slide.h declares, its structs match the ctypes mirror, and it
refuses to run without a GPU instead of falling back to the CPU."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "slide.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sp_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    import slide
    lib = slide.load()
    names = declared_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
    # exported as C symbols (no C++ mangling)
    out = subprocess.run(["nm", "-D", "--defined-only", slide.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    for name in names:
        assert name in exported, name


def test_struct_layouts_match_header(tmp_path):
    import slide
    prog = tmp_path / "sizes.c"
    prog.write_text('#include "slide.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                    'int main(void){printf("%zu %zu %zu %zu %zu\\n", sizeof(sp_config), sizeof(sp_result),'
                    ' sizeof(sp_stats), offsetof(sp_result, moves), offsetof(sp_result, seconds));return 0;}\n')
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(prog), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    want = [ctypes.sizeof(slide.SpConfig), ctypes.sizeof(slide.SpResult), ctypes.sizeof(slide.SpStats),
            slide.SpResult.moves.offset, slide.SpResult.seconds.offset]
    assert got == want


def test_status_strings_and_config_default():
    import slide
    lib = slide.load()
    for st in range(0, -11, -1):
        s = lib.sp_status_string(st).decode()
        assert s and s != "unknown status", st
    cfg = slide.default_config()
    assert cfg.frontier_target == 3072 and cfg.threads_per_block in (128, 256)
    assert lib.sp_pdb_table_size(4) == 16 * 15 * 14 * 13 * 12
    assert lib.sp_pdb_table_size(5) == 25 * 24 * 23 * 22 * 21 * 20
    assert lib.sp_pdb_num_tables(4) == 3 and lib.sp_pdb_num_tables(5) == 2
    assert lib.sp_pdb_table_size(6) == 0


def test_rejects_bad_arguments_without_gpu():
    import slide
    lib = slide.load()
    h = ctypes.c_void_p()
    assert lib.sp_create(6, 0, None, ctypes.byref(h)) == -1
    assert lib.sp_create(4, 7, None, ctypes.byref(h)) == -1
    assert lib.sp_solve_batch(None, None, 0, None) == -1
    st = ctypes.c_int32(0)
    assert lib.sp_selftest_stall(None, 200, ctypes.byref(st)) == -1
    assert lib.sp_lbm_num_params(6) == 0 and lib.sp_lbm_num_params(5) > lib.sp_lbm_num_params(4)
    rate = ctypes.c_double(1.0)
    assert lib.sp_probe_int_issue(1 << 16, 3, None, None) == -1
    assert lib.sp_probe_int_issue(0, 3, ctypes.byref(rate), None) == -1
    assert lib.sp_probe_int_issue((1 << 24) + 1, 3, ctypes.byref(rate), None) == -1
    assert lib.sp_probe_int_issue(1 << 16, 0, ctypes.byref(rate), None) == -1
    assert lib.sp_probe_random_sectors(3 << 20, 64, 3, None, None) == -1
    assert lib.sp_probe_random_sectors(1024, 64, 3, ctypes.byref(rate), None) == -1
    assert lib.sp_probe_random_sectors(1 << 32, 64, 3, ctypes.byref(rate), None) == -1
    assert lib.sp_probe_random_sectors(3 << 20, 0, 3, ctypes.byref(rate), None) == -1
    assert lib.sp_probe_random_sectors(3 << 20, 64, 101, ctypes.byref(rate), None) == -1
    assert lib.sp_selftest_gemm_stall(4, 50, ctypes.byref(st)) == -1
    assert lib.sp_selftest_gemm_stall(0, 5, ctypes.byref(st)) == -1
    assert lib.sp_selftest_gemm_stall(0, 50, None) == -1
    # the allocation-free round checks its arguments before touching the GPU
    assert lib.sp_dfs_round_md_noalloc(6, None, None, None, 0, 10, None, None, None) == -1
    assert lib.sp_dfs_round_md_noalloc(4, None, None, None, -1, 10, None, None, None) == -1


def test_no_cpu_fallback_when_no_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import slide
    with pytest.raises(slide.SlideError) as e:
        slide.Solver(4, "manhattan")
    assert e.value.status == -5  # SP_ERR_CUDA
    with pytest.raises(slide.SlideError) as e:
        slide.probe_int_issue(1 << 10, 1)
    assert e.value.status == -5
    with pytest.raises(slide.SlideError) as e:
        slide.probe_random_sectors(3 << 20, 4, 1)
    assert e.value.status == -5
