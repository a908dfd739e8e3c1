"""bench.py pieces that need no GPU: the roofline's DRAM traffic comes from
the committed ncu summary of the headline kernel, and it is consistent with
the kernel's compulsory bytes."""
import bench

SITES = 32 * 32 * 32 * 64 // 2  # output sites of one 32^3x64 application


def test_headline_traffic_comes_from_the_committed_profile():
    t = bench.profiled_traffic("wilson_dslash_4d_32x32x32x64_f32_recon18")
    compulsory_reads = SITES * (96 + 8 * 72)  # source spinors and links, each once
    algorithmic = SITES * 768  # plus the output spinor
    assert isinstance(t, int)
    # every link and source spinor leaves DRAM at least once; a kernel that
    # re-read them would show well above the algorithmic bytes
    assert compulsory_reads <= t <= 1.1 * algorithmic


def test_missing_profile_gives_no_traffic():
    assert bench.profiled_traffic("no_such_workload") is None
