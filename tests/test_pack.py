"""woo_gb300.pack.SpherePack: Woo's packing text format (SpherePack::fromFile / toFile,
src/supp/sphere-pack/SpherePack.cpp:73-130) and SpherePack.toDem (py/pack.py).  The rotated periodic cell
is checked against the reference's own documented output (the doctest of SpherePack_toDem: cellSize 5,
rotation pi/4 about z gives hSize Matrix3(3.5355339059327373,-3.5355339059327378,0, ...))."""
import math

import numpy as np
import pytest

from woo_gb300 import dem, pack, scenes
from woo_gb300.core import Scene


def test_round_trip_and_woo_formatting(tmp_path):
    sp = pack.SpherePack([((0.1, 0.2, 0.3), 0.05), ((1.0 / 3, 2e-5, -4), 0.123456789)])
    sp.cellSize = np.array([2.0, 2.0, 2.5])
    sp.userData = "seed=7"
    f = tmp_path / "p.txt"
    sp.save(f)
    text = f.read_text().splitlines()
    # what a C++ ostream writes with its default precision
    assert text == ["##PERIODIC:: 2 2 2.5", "##USER-DATA:: seed=7", "0.1 0.2 0.3 0.05", "0.333333 2e-05 -4 0.123457"]
    q = pack.SpherePack()
    q.load(f)
    assert q.periodic and np.array_equal(q.cellSize, [2, 2, 2.5]) and q.userData == "seed=7"
    assert len(q) == 2 and q.toList()[1][1] == 0.123457
    sp.save(f, precision=17)
    q.load(f)
    assert all(np.array_equal(a[0], b[0]) and a[1] == b[1] for a, b in zip(sp.toList(), q.toList()))


def test_reading_rules(tmp_path):
    f = tmp_path / "a.txt"
    f.write_text("\n0 0 0 1\t\n 1 1 1 .5 \n\n2e0 2 2abc 0.25\n")
    sp = pack.SpherePack()
    sp.load(f)
    assert [r for _, r in sp] == [1, .5, .25] and np.array_equal(sp.toList()[2][0], [2, 2, 2])
    assert not sp.periodic and not sp.hasClumps()
    f.write_text("0 0 0 1 3\n1 1 1 1 3\n")
    sp.load(f)
    assert sp.hasClumps()
    for bad, msg in (("0 0 0 1\n1 1 1 1 2\n", "same number of columns"), ("0 0 0\n", "must be 4 or 5"),
                     ("##PERIODIC:: 1 2\n", "malformed"), ("0 0 x 1\n", "error parsing number")):
        f.write_text(bad)
        with pytest.raises(RuntimeError, match=msg):
            sp.load(f)
    with pytest.raises(ValueError, match="doesn't exist"):
        sp.load(tmp_path / "missing.txt")


def test_to_dem_rotated_periodic_cell():
    sp = pack.SpherePack([((1, 0, 0), 0.5), ((0, 2, 1), 0.4)])
    sp.cellSize = np.array([5.0, 5.0, 5.0])
    S = Scene(fields=[dem.DemField()])
    assert not S.periodic
    ids = sp.toDem(S, S.dem, rot=scenes.quat_from_axis_angle((0, 0, 1), math.pi / 4))
    assert ids == [0, 1] and S.periodic
    h = S.cell.hSize
    assert h[0, 0] == 3.5355339059327373 and h[0, 1] == -3.5355339059327378 and h[0, 2] == 0
    assert h[1, 0] == 3.5355339059327378 and h[1, 1] == 3.5355339059327373 and h[1, 2] == 0
    assert h[2, 2] == 5 and np.array_equal(S.cell.trsf, np.eye(3))
    assert np.allclose(S.dem.par[0].pos, (math.sqrt(.5), math.sqrt(.5), 0)) and S.dem.par[1].shape.radius == 0.4


def test_clumps_refused():
    sp = pack.SpherePack()
    sp.pack = [(np.zeros(3), 1.0, 0), (np.ones(3), 1.0, 0)]
    S = Scene(fields=[dem.DemField()])
    with pytest.raises(RuntimeError, match="clumps"):
        sp.toSimulation(S)


def test_make_cloud():
    sp = pack.SpherePack()
    n = sp.makeCloud((0, 0, 0), (1, 1, 1), rMean=0.05, rRelFuzz=0.3, num=200, seed=3)
    assert n == len(sp) > 150 and not sp.periodic
    c = np.array([p for p, _ in sp])
    r = np.array([q for _, q in sp])
    d = np.linalg.norm(c[:, None] - c[None], axis=-1) - (r[:, None] + r[None])
    assert (d + np.eye(n) * 10).min() >= 0 and r.min() >= 0.035 and r.max() <= 0.065
    sp.makeCloud((0, 0, 0), (1, 1, 1), rMean=0.05, num=50, periodic=True, seed=4)
    assert sp.periodic and np.array_equal(sp.cellSize, [1, 1, 1])
