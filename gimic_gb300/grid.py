"""Grids and the magnetic field direction, as built by the Fortran driver.

Follows src/fgimic/grid.f90:50-138 (new_grid), :140-163 (std/base),
:165-276 (bond plane), :291-349 (gauss/lobatto axes), :351-373 (even axes),
:403-431 (orthogonalisation), :543-576 (file grid), :697-769 (rotation) and
src/fgimic/magnet.f90:11-86.  All arithmetic is fp64 in the reference's
operation order so that grid points match the reference bit for bit.
A grid point is origin + x1_i basv[:,0] + x2_j basv[:,1] + x3_k basv[:,2].
"""
import math

import numpy as np

from . import api

DPTOL = 1.0e-10


def nint(x):
    """Fortran NINT: round half away from zero."""
    return int(math.floor(x + 0.5)) if x >= 0 else int(math.ceil(x - 0.5))


def _norm(v):
    v = np.asarray(v, dtype=np.float64)
    return v / math.sqrt(float(np.sum(v ** 2)))


def _cross(a, b):
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]])


class Grid:
    def __init__(self):
        self.mode = "std"
        self.gtype = "even"
        self.basv = np.zeros((3, 3))   # basv[:, d] is axis d
        self.l = np.zeros(3)
        self.origin = np.zeros(3)
        self.ortho = np.zeros(3)
        self.step = np.ones(3)
        self.npts = [1, 1, 1]
        self.pts = [np.zeros(1)] * 3
        self.wgt = [np.ones(1)] * 3
        self.gauss = False
        self.radius = 1e10
        self.points_file = None  # (N, 3) for file grids
        self.gauss_order = 0

    # -------------------------------------------------------------------
    def gridpoint(self, i, j, k):
        if self.gtype == "file":
            return self.points_file[i].copy()
        return (self.origin + self.pts[0][i] * self.basv[:, 0] + self.pts[1][j] * self.basv[:, 1]
                + self.pts[2][k] * self.basv[:, 2])

    def points(self):
        """All grid points, i fastest then j then k, as an (N, 3) array with
        the same fp64 expression order as gridpoint()."""
        if self.gtype == "file":
            return self.points_file.copy()
        x1 = self.pts[0][None, None, :, None] * self.basv[:, 0]
        x2 = self.pts[1][None, :, None, None] * self.basv[:, 1]
        x3 = self.pts[2][:, None, None, None] * self.basv[:, 2]
        p = ((self.origin + x1) + x2) + x3
        return p.reshape(-1, 3)

    def size(self):
        return tuple(self.npts)

    def normal(self):
        return self.basv[:, 2].copy()

    def center(self):
        """grid_center (grid.f90:529-541)."""
        v1 = self.gridpoint(self.npts[0] - 1, 0, 0)
        v2 = self.gridpoint(0, self.npts[1] - 1, 0)
        return (v1 + v2) * 0.5

    def is_3d(self):
        return all(n > 1 for n in self.npts)

    def axes(self):
        return [(self.pts[d], self.wgt[d]) for d in range(3)]


def _setup_std(g, inp):
    g.origin = np.array(inp.get("Grid.origin"), dtype=np.float64)
    g.basv[:, 0] = inp.get("Grid.ivec")
    g.basv[:, 1] = inp.get("Grid.jvec")
    g.l = np.array(inp.get("Grid.lengths"), dtype=np.float64)
    if inp.is_set("Grid.spacing"):
        g.step = np.array(inp.get("Grid.spacing"), dtype=np.float64)
    else:
        g.npts = [int(v) for v in inp.get("Grid.grid_points")]
        with np.errstate(divide="ignore", invalid="ignore"):
            g.step = g.l / (np.array(g.npts, dtype=np.float64) - 1)
    g.basv[:, 2] = _cross(g.basv[:, 0], g.basv[:, 1])
    g.ortho = _norm(g.basv[:, 2])


def _setup_bond(g, inp, atoms):
    if inp.is_set("Grid.bond"):
        a1, a2 = inp.get("Grid.bond")
        g.basv[:, 0] = atoms[a1 - 1]
        g.basv[:, 1] = atoms[a2 - 1]
    else:
        g.basv[:, 0] = inp.get("Grid.coord1")
        g.basv[:, 1] = inp.get("Grid.coord2")
    if inp.is_set("Grid.fixpoint"):
        g.origin = np.array(atoms[inp.get("Grid.fixpoint") - 1], dtype=np.float64)
    else:
        g.origin = np.array(inp.get("Grid.fixcoord"), dtype=np.float64)
    g.radius = 1e10
    if inp.is_set("Grid.radius"):
        g.radius = float(inp.get("Grid.radius"))
    l3 = float(inp.get("Grid.distance"))
    if inp.is_set("Grid.height"):
        hgt = list(inp.get("Grid.height"))
        wdt = list(inp.get("Grid.width"))
        hgt[0] = -hgt[0]
        wdt[0] = -wdt[0]
    else:
        wdt = [float(inp.get("Grid.in", -1.0)), float(inp.get("Grid.out", -1.0))]
        hgt = [float(inp.get("Grid.up", -1.0)), float(inp.get("Grid.down", -1.0))]
    g.l = np.array([hgt[0] + hgt[1], wdt[0] + wdt[1], 0.0])
    if wdt[0] + wdt[1] < 0.0:
        raise ValueError("Grid width < 0!")
    if hgt[0] + hgt[1] < 0.0:
        raise ValueError("Grid height < 0!")
    v1 = g.basv[:, 0] - g.origin
    v2 = g.basv[:, 1] - g.origin
    g.ortho = _cross(v1, v2)
    if np.all(g.ortho == 0.0):
        raise ValueError("Basis vectors are linearly dependent, field direction undefined!")
    g.ortho = _norm(g.ortho)
    v3 = _norm(v2 - v1)
    v1 = -g.ortho
    v2 = _norm(_cross(v3, v1))
    oo = g.basv[:, 0] + l3 * v3
    g.origin = oo - wdt[1] * v2 - hgt[1] * v1
    g.basv[:, 0] = v1
    g.basv[:, 1] = v2
    g.basv[:, 2] = v3
    g.bond_center = oo
    if inp.is_set("magnet"):
        g.ortho = _norm(inp.get("magnet"))


def _normalise(basv):
    for i in range(3):
        n = math.sqrt(float(np.sum(basv[:, i] ** 2)))
        if n > 0.0:
            basv[:, i] = basv[:, i] / n


def _ortho_coordsys(g):
    dpr = float(np.dot(g.basv[:, 0], g.basv[:, 1]))
    if abs(dpr) > DPTOL:
        t = _cross(g.basv[:, 0], g.basv[:, 2])
        g.basv[:, 1] = t / math.sqrt(float(np.sum(t ** 2)))
        _normalise(g.basv)


def rotate(g, angle, reference):
    """grid.f90:697-769: right-handed rotations about z, y, then x."""
    rad = np.asarray(angle, dtype=np.float64) / 180.0 * 3.141592653589793
    rot = np.zeros((3, 3))
    euler = np.zeros((3, 3))
    x = rad[2]
    rot[0, 0] = math.cos(x)
    rot[1, 1] = math.cos(x)
    rot[2, 2] = 1.0
    rot[0, 1] = math.sin(x)
    rot[1, 0] = -math.sin(x)
    x = rad[1]
    euler[0, 0] = math.cos(x)
    euler[1, 1] = 1.0
    euler[2, 2] = math.cos(x)
    euler[0, 2] = -math.sin(x)
    euler[2, 0] = math.sin(x)
    euler = euler @ rot
    x = rad[0]
    rot = np.zeros((3, 3))
    rot[0, 0] = 1.0
    rot[1, 1] = math.cos(x)
    rot[2, 2] = math.cos(x)
    rot[1, 2] = math.sin(x)
    rot[2, 1] = -math.sin(x)
    euler = rot @ euler
    g.origin = g.origin - reference
    g.basv = euler @ g.basv
    g.origin = euler @ g.origin
    g.origin = g.origin + reference


def _setup_even(g):
    g.gauss = False
    g.npts = [nint(g.l[0] / g.step[0]) + 1, nint(g.l[1] / g.step[1]) + 1, 1]
    tiny = np.finfo(np.float64).tiny
    if not (abs(g.l[2]) < tiny or abs(g.step[2]) < tiny):
        g.npts[2] = nint(g.l[2] / g.step[2]) + 1
    g.pts = [np.arange(n, dtype=np.float64) * g.step[d] for d, n in enumerate(g.npts)]
    g.wgt = [np.ones(n) for n in g.npts]


def _setup_gauss(g, inp, quadrature):
    order = int(inp.get("Grid.gauss_order"))
    g.gauss_order = order
    if inp.is_set("Grid.grid_points"):
        npts = [int(v) for v in inp.get("Grid.grid_points")]
    else:
        spc = inp.get("Grid.spacing")
        npts = [0 if (abs(spc[i]) < 1e-10 or spc[i] < 0.0) else nint(g.l[i] / spc[i]) for i in range(3)]
    adjusted = False
    for i in range(3):
        if not npts[i] > 1:
            npts[i] = 0
        rem = npts[i] % order
        if rem != 0:
            npts[i] = npts[i] - rem + order
            adjusted = True
    g.adjusted = adjusted
    g.gauss = True
    # the Newton iteration for the Lobatto nodes is unreliable above 13
    # points per panel; like lobattomy (src/libgimic/gaussint.f90:68-75) the
    # grid is kept and a warning is issued
    g.warnings = []
    if quadrature == "lobatto" and order > 13:
        g.warnings = ["lobattomy(): Warning, too many Gauss points:%4d" % order,
                      "lobattomy(): using this many points is not stable."]
    g.pts, g.wgt = [], []
    for i in range(3):
        if npts[i] > 0:
            p, w = api.gauss_data(0.0, g.l[i], order, npts[i], quadrature)
        else:
            npts[i] = 1
            p, w = np.zeros(1), np.ones(1)
        g.pts.append(p)
        g.wgt.append(w)
    g.npts = npts


def _read_grid_file(path):
    vals = np.array(open(path).read().replace("D", "E").replace("d", "e").split(), dtype=np.float64)
    nlines = sum(1 for _ in open(path))
    return vals[: 3 * nlines].reshape(nlines, 3)


def new_grid(inp, atoms, workdir="."):
    """Build the grid of an ``Input`` (see gimic_gb300.inp) for a molecule
    with atom coordinates ``atoms`` (natoms, 3) in Bohr."""
    import os

    g = Grid()
    g.mode = inp.grid_arg
    if g.mode == "file":
        path = inp.get("Grid.file") if inp.is_set("Grid.file") else "GRIDDATA"
        g.points_file = _read_grid_file(os.path.join(workdir, path))
        g.gtype = "file"
        g.npts = [len(g.points_file), 1, 1]
        g.pts = [np.zeros(g.npts[0]), np.zeros(1), np.zeros(1)]
        g.wgt = [np.ones(g.npts[0]), np.ones(1), np.ones(1)]
        return g
    if g.mode in ("std", "base"):
        _setup_std(g, inp)
    elif g.mode == "bond":
        _setup_bond(g, inp, np.asarray(atoms, dtype=np.float64))
    else:
        raise ValueError("Unknown grid type: " + g.mode)
    _normalise(g.basv)
    _ortho_coordsys(g)
    if inp.is_set("Grid.rotation"):
        angle = np.array(inp.get("Grid.rotation"), dtype=np.float64)
        if inp.is_set("Grid.rotation_origin"):
            ref = np.array(inp.get("Grid.rotation_origin"), dtype=np.float64)
        else:
            if inp.is_set("Grid.height"):
                down, out = inp.get("Grid.height")[1], inp.get("Grid.width")[1]
            else:
                out, down = inp.get("Grid.out"), inp.get("Grid.down")
            ref = g.origin + out * g.basv[:, 1] + down * g.basv[:, 0]
        rotate(g, angle, ref)
    g.gtype = inp.get("Grid.type")
    if g.gtype == "even":
        _setup_even(g)
    elif g.gtype in ("gauss", "lobatto"):
        _setup_gauss(g, inp, g.gtype)
    else:
        raise ValueError("Unknown grid type: " + g.gtype)
    return g


def get_magnet(g, inp):
    """Magnetic field direction (src/fgimic/magnet.f90:11-86).  Returns
    (b, flipped) where flipped tells that check_field reversed it."""
    axis = inp.get("magnet_axis") if inp.is_set("magnet_axis") else ""
    ortho = False
    mag = np.zeros(3)
    if axis:
        d = 1.0
        a = axis
        if a[0] == "-":
            d = -1.0
            a = a[1:]
        c = a[:1]
        if c in ("i", "j", "k"):
            mag = g.basv[:, "ijk".index(c)] * d
        elif c in ("x", "y", "z"):
            mag = np.eye(3)[ "xyz".index(c)] * d
        elif c == "X":
            ortho = True
            mag = g.ortho * d
        else:
            raise ValueError("Invalid axis specifier: " + axis)
    else:
        mag = np.array(inp.get("magnet"), dtype=np.float64)
    if np.all(mag == 0.0):
        raise ValueError("Magnetic field is zero, not wasting more CPU.")
    flipped = False
    if not ortho:
        x = float(np.dot(g.basv[:, 2], mag))
        if x > 0.0:
            mag = -mag
            flipped = True
    return np.asarray(mag, dtype=np.float64), flipped
