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


def test_random_sector_rates_are_plausible():
    """The PDB search's roofline denominator (sp_probe_random_sectors): a
    3 MB working set (the 15-puzzle tables) is served by L2, faster than the
    24-puzzle's 488 MB, which mostly misses L2; time grows with the work; and
    neither sector rate exceeds what the memory system can deliver (HBM
    about 8 TB/s, L2 well under 100 TB/s)."""
    import torch
    import slide
    torch.cuda.set_device(0)
    before = slide.kernel_launch_count()
    l2, ms_a = slide.probe_random_sectors(slide.pdb_table_bytes(4), 128, 2)
    _, ms_b = slide.probe_random_sectors(slide.pdb_table_bytes(4), 256, 2)
    hbm, _ = slide.probe_random_sectors(slide.pdb_table_bytes(5), 64, 2)
    assert slide.kernel_launch_count() - before == 9
    assert 1.4 < ms_b / ms_a < 2.8, (ms_a, ms_b)
    assert hbm < l2, (hbm, l2)
    assert 1e9 < hbm * slide.SECTOR_BYTES < 12e12, hbm
    assert 1e11 < l2 * slide.SECTOR_BYTES < 1e14, l2
