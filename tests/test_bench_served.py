"""The served bench's trace check (host logic, no GPU): a chain's -log L
trace is compared served against plain up to the point where the traces
part; exact kinds must show identical steps, parting chains are counted."""
import math

import bench


def test_trace_check_counts_identical_steps_and_parting_chains():
    served = {1: ("tt2d", [10.0, 9.5, 9.0]), 2: ("body", [5.0, 4.0000001, 3.0]), 3: ("body", [7.0, 6.0, 1.0]),
              4: ("surface", [2.0, math.inf])}
    plain = {1: ("tt2d", [10.0, 9.5, 9.0, 8.0]), 2: ("body", [5.0, 4.0, 3.0]), 3: ("body", [7.0, 6.5, 2.0]),
             4: ("surface", [2.0, math.inf])}
    out = bench.served_trace_check({"served": served, "plain": plain})
    assert out["tt2d"] == {"chains_compared": 1, "steps_compared": 3, "identical_steps": 3, "max_rel_diff": 0.0,
                           "chains_parted": 0, "identical_frac": 1.0}
    b = out["body"]
    assert b["chains_compared"] == 2 and b["chains_parted"] == 1
    # chain 2: three steps, one differing by 2.5e-8 relative; chain 3: one step before parting
    assert b["steps_compared"] == 4 and b["identical_steps"] == 3
    assert 2e-8 < b["max_rel_diff"] < 3e-8
    assert out["surface"]["identical_steps"] == 2


def test_trace_check_skips_chains_missing_from_one_leg():
    out = bench.served_trace_check({"served": {1: ("tt2d", [1.0])}, "plain": {}})
    assert out == {}
