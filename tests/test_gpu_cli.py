"""The command line front end on the GPU: instance files in the reference's
format give the reference's golden `len nodes` lines."""
import numpy as np
import pytest

import slide_cli
from conftest import load_golden

pytestmark = pytest.mark.gpu


def test_cli_lines_equal_the_golden_rows(gpu_solver, tmp_path):
    g = load_golden("yama24_hard_new.json")["instances"][:8]
    paths = []
    for x in g:
        p = tmp_path / x["name"]
        p.write_text(" ".join(str(v) for v in x["tiles"]) + " \n")
        paths.append(str(p))
    lines, secs = slide_cli.run(gpu_solver(5, "pdb"), paths)
    assert lines == ["%s %d %d" % (x["name"], x["pdb"][0], x["pdb"][1]) for x in g]
    assert len(secs) == 8 and all(s > 0 for s in secs)
