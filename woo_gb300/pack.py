"""woo.pack.SpherePack for this engine: Woo's sphere-packing container and its text file format, the usual
way packings reach a DEM scene (SpherePack.load, then toSimulation/toDem).

The file format is the reference's SpherePack::toFile / fromFile (src/supp/sphere-pack/SpherePack.cpp:73-130):
one sphere per line as "x y z r" (or "x y z r clumpId"; all lines the same width), an optional
"##PERIODIC:: sx sy sz" line giving the periodic cell size, an optional "##USER-DATA:: text" line, blank
lines ignored, fields separated by spaces or tabs; numbers are read as C's strtod reads them (the longest
number at the start of the field) and written as C++ streams write doubles by default (6 significant
digits, %g), so a file saved here is the file Woo would save for the same packing.  toDem /
toSimulation restate py/pack.py:SpherePack_toDem: the spheres are added to the field, rotated by `rot`, and
a periodic packing makes the scene periodic with hSize = rot · diag(cellSize) and trsf = identity.
Clumps (5-column files) are read and written, but not simulated: the engine has no clumps.
"""
import re

import numpy as np

_STRTOD = re.compile(r"\s*[+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan)", re.IGNORECASE)


def _stod(tok):
    """std::stod: the longest prefix that is a number (ValueError when there is none)."""
    m = _STRTOD.match(tok)
    if not m:
        raise ValueError(tok)
    return float(m.group(0))


def _stoi(tok):
    m = re.match(r"\s*[+-]?\d+", tok)
    if not m:
        raise ValueError(tok)
    return int(m.group(0))


def quat_to_matrix(q):
    """Quaternion::toRotationMatrix for (w, x, y, z), Eigen's formula."""
    w, x, y, z = (float(v) for v in q)
    tx, ty, tz = 2 * x, 2 * y, 2 * z
    twx, twy, twz = tx * w, ty * w, tz * w
    txx, txy, txz = tx * x, ty * x, tz * x
    tyy, tyz, tzz = ty * y, tz * y, tz * z
    return np.array([[1 - (tyy + tzz), txy - twz, txz + twy],
                     [txy + twz, 1 - (txx + tzz), tyz - twx],
                     [txz - twy, tyz + twx, 1 - (txx + tyy)]])


def _mat3_mul(a, b):
    """3x3 product with Eigen's lazy-product order per coefficient: (a_i0 b_0j + a_i1 b_1j) + a_i2 b_2j."""
    r = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            r[i, j] = (a[i, 0] * b[0, j] + a[i, 1] * b[1, j]) + a[i, 2] * b[2, j]
    return r


def _mat3_vec(a, v):
    return np.array([(a[i, 0] * v[0] + a[i, 1] * v[1]) + a[i, 2] * v[2] for i in range(3)])


class SpherePack:
    """Spheres (centre, radius, clumpId -1 when not clumped), cellSize (zero: aperiodic) and userData."""

    def __init__(self, spheres=()):
        self.pack = []
        self.cellSize = np.zeros(3)
        self.userData = ""
        if spheres:
            self.fromList(spheres)

    # ---- contents
    def fromList(self, spheres):
        """SpherePack::fromList: (centre, radius) pairs; the cell becomes aperiodic."""
        self.pack = [(np.asarray(c, np.float64).copy(), float(r), -1) for c, r in spheres]
        self.cellSize = np.zeros(3)

    def toList(self):
        return [(c.copy(), r) for c, r, _ in self.pack]

    def add(self, c, r):
        self.pack.append((np.asarray(c, np.float64).copy(), float(r), -1))

    def hasClumps(self):
        return any(k >= 0 for _, _, k in self.pack)

    def __len__(self):
        return len(self.pack)

    def __iter__(self):
        return iter(self.toList())

    @property
    def periodic(self):
        return bool(np.any(self.cellSize != 0))

    # ---- the text format
    def load(self, fname):
        """SpherePack::fromFile (SpherePack.cpp:73-117)."""
        import os
        if not os.path.exists(fname):
            raise ValueError(f"File with spheres `{fname}' doesn't exist.")
        self.pack = []
        self.cellSize = np.zeros(3)
        ncols = 0
        with open(fname) as f:
            for lineNo, line in enumerate(f, 1):
                line = line.rstrip("\r\n")
                if line.startswith("##USER-DATA:: "):
                    self.userData = line[14:]
                    continue
                toks = [t for t in re.split(r"[ \t]", line) if t]
                if not toks:
                    continue
                try:
                    if toks[0] == "##PERIODIC::":
                        if len(toks) != 4:
                            raise RuntimeError(f"Spheres file {fname}:{lineNo} contains ##PERIODIC::, but the line is malformed.")
                        self.cellSize = np.array([_stod(t) for t in toks[1:4]])
                        continue
                    if len(toks) not in (4, 5):
                        raise RuntimeError(f"{fname}:{lineNo}: line has {len(toks)} columns (must be 4 or 5).")
                    if ncols == 0:
                        ncols = len(toks)
                    if ncols != len(toks):
                        raise RuntimeError(f"{fname}:{lineNo}: all line must have the same number of columns "
                                           f"(previous had {ncols}, this one has {len(toks)})")
                    c = np.array([_stod(t) for t in toks[:3]])
                    r = _stod(toks[3])
                    k = _stoi(toks[4]) if len(toks) == 5 else -1
                except ValueError:
                    raise RuntimeError(f"{fname}:{lineNo}: error parsing number.") from None
                self.pack.append((c, r, k))

    def save(self, fname, precision=6):
        """SpherePack::toFile (SpherePack.cpp:119-130); precision 6 writes what Woo writes, 17 is lossless."""
        fmt = f"%.{int(precision)}g"
        with open(fname, "w") as f:
            if self.periodic:
                f.write("##PERIODIC:: " + " ".join(fmt % v for v in self.cellSize) + "\n")
            if self.userData:
                if "\n" in self.userData:
                    raise RuntimeError("SpherePack.userData must not contain newline.")
                f.write("##USER-DATA:: " + self.userData + "\n")
            clumps = self.hasClumps()
            for c, r, k in self.pack:
                f.write(" ".join(fmt % v for v in (c[0], c[1], c[2], r)) + (f" {k}" if clumps else "") + "\n")

    # ---- generation and transfer to a scene
    def makeCloud(self, minCorner, maxCorner, rMean, rRelFuzz=0.0, num=-1, periodic=False, seed=0, max_attempts=200):
        """Random sequential addition of non-overlapping spheres (SpherePack::makeCloud, uniform radii in
        rMean (1 +- rRelFuzz)), through the engine's packing generator; returns the number placed."""
        from . import abi
        lo, hi = np.asarray(minCorner, np.float64), np.asarray(maxCorner, np.float64)
        if num < 0:
            raise ValueError("SpherePack.makeCloud: give num (the generator places a fixed count)")
        rmin, rmax = rMean * (1 - rRelFuzz), rMean * (1 + rRelFuzz)
        if periodic:
            radii = np.random.default_rng(seed).uniform(rmin, rmax, num)
            centers, radii = abi.make_cloud_radii(lo, hi, radii, seed, periodic=True, max_attempts=max_attempts)
        else:
            centers, radii = abi.make_cloud(lo, hi, rmin, rmax, num, seed, max_attempts=max_attempts)
        self.pack = [(c.copy(), float(r), -1) for c, r in zip(centers, radii)]
        self.cellSize = (hi - lo) if periodic else np.zeros(3)
        return len(self.pack)

    def toDem(self, scene, dem=None, rot=None, **kw):
        """py/pack.py:SpherePack_toDem: add the spheres (rotated by rot, a (w, x, y, z) quaternion or a 3x3
        matrix) with Sphere.make(**kw); a periodic packing sets scene.periodic, cell.hSize = rot · diag(cellSize)
        and cell.trsf = identity.  Returns the new ids."""
        from . import dem as D
        dem = dem if dem is not None else scene.dem
        if rot is None:
            R = np.eye(3)
        else:
            rot = np.asarray(rot, np.float64)
            R = quat_to_matrix(rot) if rot.shape == (4,) else rot
        if self.periodic:
            scene.periodic = True
            scene.cell.hSize = _mat3_mul(R, np.diag(self.cellSize))
            scene.cell.trsf = np.eye(3)
        if self.hasClumps():
            raise RuntimeError("SpherePack.toDem: clumps are not supported by the GPU engine")
        kw.setdefault("mat", D.defaultMaterial())
        return dem.par.add([D.Sphere.make(_mat3_vec(R, c), r, **kw) for c, r, _ in self.pack])

    def toSimulation(self, scene, rot=None, **kw):
        """py/pack.py:SpherePack_toSimulation: toDem on scene.dem."""
        return self.toDem(scene, scene.dem, rot=rot, **kw)

