"""The integer-issue probe (sp_probe_int_issue), the roofline denominator of
the Manhattan search: its rate is plausible for a GB300 (152 SMs x 128
integer lanes near 2 GHz is about 4e13 lane operations per second) and its
time grows with the work, so the compiler kept the chains."""
import pytest

pytestmark = pytest.mark.gpu


def test_int_issue_rate_is_plausible_and_scales():
    import torch
    import slide
    torch.cuda.set_device(0)
    slide.probe_int_issue(1 << 16, 1)  # lets the SM clock settle
    before = slide.kernel_launch_count()
    r1, ms1 = slide.probe_int_issue(1 << 15, 3)
    r2, ms2 = slide.probe_int_issue(1 << 16, 3)
    assert slide.kernel_launch_count() - before == 8
    for r in (r1, r2):
        assert 5e12 < r < 1e14, r
    # twice the steps take about twice as long (a loop the compiler had
    # removed would give about 1)
    assert 1.4 < ms2 / ms1 < 2.8, (ms1, ms2)
