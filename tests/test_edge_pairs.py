"""The near-edge pairs without a GPU: each constructed pair's FP64 value sits
on the side of its boundary that its step says, and the oracle bins the
pairs exactly as FCFC's rules do from those values (so the oracle, the
checker of the GPU near-edge test, is right at the edges too)."""
import numpy as np
import pytest

import edge_pairs as ep

CFGS = ep.configs()


@pytest.mark.parametrize("cfg", CFGS, ids=[c[0] for c in CFGS])
def test_edge_pairs_oracle(cfg):
    x, B, ob, bins = ep.build(cfg)
    survey = cfg[1]
    assert len(B.a) >= 7 * 8
    # every boundary got pairs on both sides
    sides = {}
    for tag, s in B.tag:
        sides.setdefault(tag, set()).add(np.sign(s) if s else 1)
    assert all(v == {-1, 1} or v == {1} for v in sides.values())
    assert sum(v == {-1, 1} for v in sides.values()) >= len(sides) - 2
    # steps >= 0 sit at or above their edge, the others below it
    for v, edge, step in ep.pair_values(B, bins, survey):
        assert (v >= edge) == (step >= 0), (v, edge, step)
    got = ob.count(x)
    want = ep.expected_counts(B, bins, ob.ntot, survey)
    np.testing.assert_array_equal(got, want)
