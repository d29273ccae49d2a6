"""GPU collider (radix-sorted sweep + grid cull) against the reference collider's pair set, computed by
the oracle's InsertionSortCollider restatement on identical boxes: bit-exact set equality."""
import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi

from test_oracle_collider import brute_pairs, random_boxes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [0, 1, 2])
@pytest.mark.parametrize("walls", [True, False])
def test_pairs_equal_reference_sweep(wdem_lib, seed, walls):
    mins, maxs, mask = random_boxes(2000, seed, walls=walls)
    h = abi.Handle(len(mins))
    got = h.collide_boxes(mins, maxs, mask, 2)
    exp = bridge.collide_boxes(mins, maxs, mask, 2)
    assert len(exp) > 0
    assert np.array_equal(got, exp)


def test_pairs_with_touching_boxes_and_masks(wdem_lib):
    """Closed intervals: boxes that only touch (max == min) are a pair; loneMask and mask=0 excluded."""
    mins = np.array([[0, 0, 0], [1, 0, 0], [2.0000001, 0, 0], [0.5, 0.5, 0.5], [0.5, 0.5, 0.5]], float)
    maxs = mins + 1.0
    mask = np.array([1, 1, 1, 2, 0], np.uint32)
    h = abi.Handle(len(mins))
    got = h.collide_boxes(mins, maxs, mask, 2)
    exp = brute_pairs(mins, maxs, mask, 2)
    assert np.array_equal(got, exp)
    assert [0, 1] in got.tolist() and [1, 2] not in got.tolist()


def test_large_cloud_pairs_match_definition(wdem_lib):
    """100k boxes in a long domain (the sweep axis is the longest one): the GPU set equals the
    oracle's initial sort + sweep."""
    rng = np.random.default_rng(5)
    n = 100_000
    c = rng.uniform(0, 1, (n, 3)) * np.array([0.3, 0.3, 3.0])
    h_ = rng.uniform(0.002, 0.006, (n, 1))
    mins, maxs = c - h_, c + h_
    mask = np.full(n, 5, np.uint32)
    h = abi.Handle(n)
    got = h.collide_boxes(mins, maxs, mask, 2)
    exp = bridge.collide_boxes(mins, maxs, mask, 2, sort_axis=2)
    assert len(exp) > n / 10
    assert np.array_equal(got, exp)
