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


def strip_inputs(bond, start, out, nstrips, up=8.0, down=8.0, npts=(60, 60), order=10, quadrature="lobatto",
                 magnet_axis="z", fixpoint=None, fixcoord=(0.0, 0.0, 0.0), distance=None, coords=None):
    """gimic.inp texts for the strips of one profile (1-based atom numbers in
    ``bond``; ``distance`` defaults to half the bond length)."""
    if distance is None:
        a1, a2 = bond
        distance = 0.5 * float(np.linalg.norm(np.asarray(coords[a2 - 1]) - np.asarray(coords[a1 - 1])))
    fix = ("fixpoint=%d" % fixpoint) if fixpoint is not None else ("fixcoord=[%r, %r, %r]" % tuple(fixcoord))
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
