"""The oracle's InsertionSortCollider restatement against the pair-set definition it implements:
closed-interval box overlap on all three axes (spatialOverlap) + mayCollide masks."""
import numpy as np

from oracle import bridge


def brute_pairs(mins, maxs, mask, lone):
    n = len(mins)
    ov = np.ones((n, n), bool)
    for k in range(3):
        ov &= (mins[:, None, k] <= maxs[None, :, k]) & (maxs[:, None, k] >= mins[None, :, k])
    m = mask[:, None] & mask[None, :]
    ov &= (m != 0) & ((m & lone) == 0)
    i, j = np.nonzero(np.triu(ov, 1))
    return np.stack([i, j], 1).astype(np.int32)


def random_boxes(n, seed, walls=True):
    rng = np.random.default_rng(seed)
    c = rng.uniform(0, 1, (n, 3))
    h = rng.uniform(0.005, 0.04, (n, 1))
    mins, maxs = c - h, c + h
    mask = np.full(n, 5, np.uint32)
    if walls:
        inf = np.inf
        for k, ax in enumerate((0, 2)):
            mins[k] = -inf; maxs[k] = inf
            mins[k, ax] = maxs[k, ax] = 0.02 if k == 0 else 0.98
            mask[k] = 3
    return mins, maxs, mask


def test_initial_sweep_matches_definition():
    for seed in range(3):
        mins, maxs, mask = random_boxes(400, seed)
        got = bridge.collide_boxes(mins, maxs, mask, 2)
        exp = brute_pairs(mins, maxs, mask, 2)
        assert np.array_equal(got, exp)


def test_sort_axis_does_not_change_the_set():
    mins, maxs, mask = random_boxes(300, 7)
    sets = [bridge.collide_boxes(mins, maxs, mask, 2, sort_axis=a) for a in range(3)]
    assert all(np.array_equal(sets[0], s) for s in sets[1:])


def test_incremental_insertion_sort_matches_definition():
    """Boxes move between frames; inversions create and delete potential contacts so that after every
    frame the set equals the overlap set (no real contacts here)."""
    rng = np.random.default_rng(11)
    n, frames = 300, 6
    mins, maxs, mask = random_boxes(n, 11, walls=False)
    allmin, allmax = [mins], [maxs]
    for f in range(1, frames):
        d = rng.normal(0, 0.01, (n, 3))
        allmin.append(allmin[-1] + d); allmax.append(allmax[-1] + d)
    got = bridge.collide_frames(np.array(allmin), np.array(allmax), mask, 2)
    exp = brute_pairs(allmin[-1], allmax[-1], mask, 2)
    assert np.array_equal(got, exp)
