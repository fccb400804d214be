"""Bond-current profile scans.

The reference's job scripts (jobscripts/src/current-profile-header:112-146)
run GIMIC once per slice: the integration plane through a bond is cut into
strips of width ``delta`` along the in-plane width direction, from ``start``
to ``out``, each integrated separately, which gives the current profile
dI/dx across the bond.  Here all strips are built with the same bond-plane
geometry as src/fgimic/grid.f90:165-276 and integrated in one device pass
(gg_plane_integrals).
"""
import numpy as np

from . import grid as ggrid
from . import inp as ginp


def first_cc_bond(symbols, coords, cutoff=3.0):
    """1-based atoms of the first carbon and its nearest carbon (a bond when
    closer than ``cutoff`` Bohr)."""
    c = np.asarray(coords, dtype=np.float64)
    ci = [i for i, s in enumerate(symbols) if s.upper() == "C"]
    a = ci[0]
    d = [np.linalg.norm(c[j] - c[a]) if j != a else np.inf for j in ci]
    b = ci[int(np.argmin(d))]
    if d[int(np.argmin(d))] > cutoff:
        raise ValueError("no C-C bond shorter than %g Bohr" % cutoff)
    return a + 1, b + 1


def plane_fixcoord(coords, bond):
    """A fixcoord for a bond plane: the molecule's centroid, or, when the
    centroid lies on the bond's line (the bond grid then has no "up"
    direction, src/fgimic/grid.f90:236-241), the point 2 Bohr from the bond
    midpoint in the molecular plane, perpendicular to the bond."""
    c = np.asarray(coords, dtype=np.float64)
    a1, a2 = c[bond[0] - 1], c[bond[1] - 1]
    cen = c.mean(axis=0)
    if np.linalg.norm(np.cross(a1 - cen, a2 - cen)) > 1e-3 * max(1.0, np.linalg.norm(a2 - a1) ** 2):
        return cen
    _, _, vt = np.linalg.svd(c - cen)
    nrm = vt[-1]
    perp = np.cross(nrm, a2 - a1)
    return 0.5 * (a1 + a2) + 2.0 * perp / np.linalg.norm(perp)


def strip_inputs(bond, start, out, nstrips, up=8.0, down=8.0, npts=(60, 60), order=10, quadrature="lobatto",
                 magnet_axis="z", fixpoint=None, fixcoord=(0.0, 0.0, 0.0), distance=None, coords=None):
    """gimic.inp texts for the strips of one profile (1-based atom numbers in
    ``bond``; ``distance`` defaults to half the bond length)."""
    if distance is None:
        a1, a2 = bond
        distance = 0.5 * float(np.linalg.norm(np.asarray(coords[a2 - 1]) - np.asarray(coords[a1 - 1])))
    fix = (("fixpoint=%d" % fixpoint) if fixpoint is not None
           else ("fixcoord=[%r, %r, %r]" % tuple(float(v) for v in fixcoord)))
    distance, up, down, start, out = (float(v) for v in (distance, up, down, start, out))
    delta = (out - start) / float(nstrips)
    texts = []
    for k in range(nstrips):
        w0, w1 = start + k * delta, start + (k + 1) * delta
        texts.append("calc=integral\nmagnet_axis=%s\nGrid(bond) {\n type=%s\n bond=[%d,%d]\n %s\n distance=%r\n"
                     " height=[%r, %r]\n width=[%r, %r]\n grid_points=[%d, %d, 0]\n gauss_order=%d\n}\n"
                     % (magnet_axis, quadrature, bond[0], bond[1], fix, distance, -down, up, w0, w1,
                        npts[0], npts[1], order))
    return texts


def profile_planes(coords, **kw):
    """Grids and magnetic field of every strip of a profile."""
    planes, bb = [], None
    for text in strip_inputs(coords=coords, **kw):
        i = ginp.read(text, is_text=True)
        g = ggrid.new_grid(i, coords)
        b, _ = ggrid.get_magnet(g, i)
        bb = b if bb is None else bb
        planes.append((g.origin, g.basv, g.axes(), g.radius))
    return planes, bb


def run_profile(gimic, coords, **kw):
    """Integrate all strips in one pass; returns (strip centres along the
    width axis in Bohr, current per strip in au, list of result dicts)."""
    planes, bb = profile_planes(coords, **kw)
    gimic.set_magnet(bb)
    res = gimic.plane_integrals(planes)
    start, out, n = kw["start"], kw["out"], kw["nstrips"]
    delta = (out - start) / float(n)
    centres = start + delta * (np.arange(n) + 0.5)
    return centres, np.array([r["current"][0] for r in res]), res
