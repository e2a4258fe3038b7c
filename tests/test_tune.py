"""The autotuner's candidate launch shapes (no GPU): every field is one the C
ABI's ltpg_launch has, the values are in the ranges ltpg_set_launch accepts,
and YCSB offers every late-read setting."""
from ltpg_gb300 import abi, tune


def test_candidates_are_valid_launch_shapes():
    fields = {name for name, _ in abi.LaunchC._fields_}
    for wl in ("ycsb", "tpcc"):
        for staging in (False, True):
            cands = tune.candidates(wl, staging)
            assert cands
            for c in cands:
                assert set(c) == fields, (wl, c)
                assert c["block_threads"] % 32 == 0 and 32 <= c["block_threads"] <= 512
                assert c["ops_per_thread"] in (1, 2, 4, 8)
                assert 1 <= c["stage_ways"] <= 8
                assert c["late_reads"] in (0, 1, 2, 3)
                if wl == "tpcc":
                    assert c["late_reads"] == 0
    late = {c["late_reads"] for c in tune.candidates("ycsb")}
    assert late == {0, 1, 2, 3}
