"""Pins the FP64 CPU oracle (and the host-side grid/magnet builders) to the
reference's own committed outputs: test/c4h4/integration, test/c4h4/read-grid,
test/open-shell/integration and test/open-shell/3d."""
import json
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from gimic_gb300 import grid as ggrid
from gimic_gb300 import inp as ginp

GOLD = json.load(open(os.path.join(GOLDEN, "golden.json")))


def _load(golden_dir, case, inpname, uhf):
    i = ginp.read(str(golden_dir / case / inpname))
    thr = i.get("Advanced.screening_thrs") if i.get("Advanced.screening") else -1.0
    o = oracle.Oracle(str(golden_dir / case / "MOL"), str(golden_dir / case / "XDENS"), uhf=uhf, screening=thr)
    return i, o


def _check_block(out, blk):
    # the reference prints f13.6: compare to half a unit of the last digit
    for got, want in zip(out, (blk["au"], blk["pos"], blk["neg"])):
        assert abs(got - want) <= 5.1e-7, (got, want, blk)
    assert abs(oracle.au2si(out[0]) - blk["nAT"]) <= 5.1e-7


@pytest.mark.parametrize("case,uhf,key", [("c4h4", False, "c4h4_integration"),
                                          ("open-shell", True, "openshell_integration")])
def test_integration_goldens(golden_dir, case, uhf, key):
    i, o = _load(golden_dir, case, "integration.inp", uhf)
    atoms, _ = o.atoms()
    g = ggrid.new_grid(i, atoms)
    assert g.npts == [36, 36, 1]  # 30 points rounded up to a multiple of gauss_order 9
    bb, _ = ggrid.get_magnet(g, i)
    for blk in GOLD[key]:
        out = o.integrate(g.origin, g.basv, g.axes(), g.radius, bb, what=blk["kind"], spin=blk["spin"])
        _check_block(out, blk)


def test_c4h4_readgrid_jvec(golden_dir):
    i, o = _load(golden_dir, "c4h4", "read-grid.inp", False)
    g = ggrid.new_grid(i, o.atoms()[0], workdir=str(golden_dir / "c4h4"))
    assert g.npts[0] == 4110
    bb, flipped = ggrid.get_magnet(g, i)
    assert not flipped and np.allclose(bb, [0, 0, -1])
    ref = np.load(os.path.join(GOLDEN, "c4h4_readgrid.npz"))["jvec"]
    jt = o.jtensor(g.points())
    jv = np.einsum("pmb,b->pm", jt.reshape(-1, 3, 3).transpose(0, 2, 1), bb)
    # jvec.vtu is written with 3e20.10 (10 significant digits)
    err = np.abs(jv - ref)
    assert np.all(err <= 1e-9 * np.abs(ref) + 1e-14 * np.abs(ref).max())


def _e14_6_ulp(v):
    """Half a unit of the last printed digit of Fortran e14.6 (0.dddddd E+nn)."""
    a = np.abs(v)
    e = np.floor(np.log10(np.where(a > 0, a, 1e-300))) + 1
    return np.where(a > 0, 0.5e-6 * 10.0 ** e, 0.5e-6 * 1e-300)


def _signed_modulus(points, v, mag):
    # jmod2_vtkplot, src/fgimic/jfield.f90:117-160
    val = np.sqrt(np.sum(v ** 2, axis=1))
    coord = points - (points @ mag)[:, None] * mag
    norm = np.cross(mag, coord)
    sgn = np.sum(norm * v, axis=1)
    return np.where(sgn < 0.0, -val, val)


@pytest.mark.parametrize("spin", ["total", "alpha", "beta", "spindens"])
def test_openshell_3d_vti(golden_dir, spin):
    i, o = _load(golden_dir, "open-shell", "3d.inp", True)
    g = ggrid.new_grid(i, o.atoms()[0])
    assert g.npts == [33, 33, 33]
    bb, _ = ggrid.get_magnet(g, i)
    ref = np.load(os.path.join(GOLDEN, "openshell_3d.npz"))
    pts = g.points()[ref["index"]]
    jt = o.jtensor(pts, spin=spin)
    jv = np.einsum("pmb,b->pm", jt.reshape(-1, 3, 3).transpose(0, 2, 1), bb)
    want = ref["jvec_" + spin]
    # e14.6 output: 6 significant digits
    assert np.all(np.abs(jv - want) <= 1.01 * _e14_6_ulp(want) + 1e-3 * _e14_6_ulp(np.abs(want).max()))
    jm = _signed_modulus(pts, jv, bb)
    wm = ref["jmod_" + spin]
    assert np.all(np.abs(jm - wm) <= 1.01 * _e14_6_ulp(wm) + 1e-3 * _e14_6_ulp(np.abs(wm).max()))
