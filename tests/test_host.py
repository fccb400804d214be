"""Host-side checks that need no GPU: the C ABI library loads and exports
every declared symbol, the C++ readers agree with the oracle's, quadrature is
bit-identical to the oracle's restatement of gaussint.f90, the input parser
accepts the reference's inputs, and errors come back as status codes."""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, ROOT
from gimic_gb300 import _lib, api, synth
from gimic_gb300 import grid as ggrid
from gimic_gb300 import inp as ginp


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "gimic_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gimic_\w+|gg_\w+|mkgausspoints)\s*\(", text)))


def test_library_exports_header_symbols():
    L = _lib.load()
    names = _declared_symbols()
    assert len(names) >= 25
    for name in names:
        assert hasattr(L, name), name
        assert name in _lib.SIGNATURES, name


def _ctx(mol, xd, uhf=False, thr=1e-8):
    h = C.c_void_p()
    rc = _lib.load().gg_ctx_create(mol.encode(), xd.encode(), int(uhf), thr, C.byref(h))
    return rc, h


@pytest.mark.parametrize("case,uhf", [("c4h4", False), ("open-shell", True)])
def test_readers_agree_with_oracle(golden_dir, case, uhf):
    mol, xd = str(golden_dir / case / "MOL"), str(golden_dir / case / "XDENS")
    rc, h = _ctx(mol, xd, uhf)
    assert rc == 0
    L = _lib.load()
    o = oracle.Oracle(mol, xd, uhf=uhf, screening=1e-8)
    nbf, nat, nsh, tm = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    L.gg_basis_info(h, C.byref(nbf), C.byref(nat), C.byref(nsh), C.byref(tm))
    assert (nbf.value, nat.value, bool(tm.value)) == (o.nbf, o.natoms, o.turbomole)
    assert nsh.value == len(o.shells()["l"])
    xyz = np.zeros((nat.value, 3))
    L.gg_atoms(h, xyz.ctypes.data_as(C.POINTER(C.c_double)), None)
    assert np.array_equal(xyz, o.atoms()[0])
    L.gg_ctx_destroy(h)


def test_synthetic_inputs_roundtrip(c6h6):
    mp, xp, mol = c6h6
    o = oracle.Oracle(mp, xp)
    assert o.nbf == mol.nbf == 120
    d = o.density(0, 0)
    assert np.array_equal(d, d.T)
    for b in (1, 2, 3):
        p = o.density(0, b)
        assert np.array_equal(p, -p.T)
    assert np.allclose(o.atoms()[0], mol.coords, atol=1e-11)


@pytest.mark.parametrize("quad", ["gauss", "lobatto"])
@pytest.mark.parametrize("order", [2, 3, 5, 7, 9, 10, 12, 13])
def test_quadrature_bit_identical_to_oracle(quad, order):
    for nblock, b in ((1, 1.0), (3, 7.25614), (20, 16.0)):
        p, w = api.gauss_data(0.0, b, order, order * nblock, quad)
        po, wo = oracle.gauss_data(0.0, b, order, order * nblock, quad)
        assert np.array_equal(p, po) and np.array_equal(w, wo)


def test_quadrature_known_answers():
    # exact for polynomials of degree 2n-1 (Gauss) / 2n-3 (Lobatto) on [0, b]
    for quad, deg in (("gauss", 17), ("lobatto", 15)):
        p, w = api.gauss_data(0.0, 2.0, 9, 9, quad)
        assert abs(np.sum(w * p ** deg) - 2.0 ** (deg + 1) / (deg + 1)) < 1e-9 * 2.0 ** (deg + 1)
    # int exp(-x^2) over [-10, 10]^3 = pi^(3/2) (src/pygimic/quadrature.py:27-49)
    p, w = api.gauss_data(0.0, 20.0, 10, 200, "gauss")
    x = p - 10.0
    s1 = np.sum(w * np.exp(-x * x))
    assert abs(s1 ** 3 - math.pi ** 1.5) < 1e-10
    with pytest.raises(ValueError):
        api.gauss_data(0.0, 1.0, 9, 20)  # not a multiple of the order
    assert api.gauss_data(0.0, 5.0, 9, 1)[0].tolist() == [0.0]


def test_plane_records_packed_like_the_structured_path():
    """The gg_grid records of one to four planes (packed field by field)
    hold the same fields as the concatenated path of five or more, and
    point into the caller's axis arrays."""
    ax = [(np.linspace(0, 8, 60), np.full(60, 0.5)), (np.linspace(-8, 8, 61), np.full(61, 0.25)),
          (np.zeros(1), np.ones(1))]
    pl = (np.array([1.0, -2.0, 3.5]), np.arange(9.0).reshape(3, 3), ax, 7.5)
    few, keep = api._grid_records([pl, pl])
    many, flat = api._grid_records([pl] * 5)
    for f in ("origin", "basv", "npts", "radius"):
        assert np.array_equal(few[f][:2], many[f][:2]), f
    assert few["basv"][0].tolist() == np.arange(9.0).reshape(3, 3).T.reshape(9).tolist()
    rec = _lib.GridSpec.from_buffer_copy(few[1].tobytes())
    assert rec.npts[:] == [60, 61, 1] and rec.radius == 7.5
    assert rec.pts[1] is not None
    arrs = keep[1]
    assert C.cast(rec.pts[1], C.c_void_p).value == arrs[2].__array_interface__["data"][0]
    assert C.cast(rec.wgt[0], C.c_void_p).value == arrs[1].__array_interface__["data"][0]


def test_au2si():
    assert abs(api.au2si(1.0) - 28.179409) < 5e-7
    assert api.au2si(-0.708546) == pytest.approx(oracle.au2si(-0.708546), rel=1e-15)


def test_error_codes(tmp_path, c6h6):
    mp, xp, _ = c6h6
    L = _lib.load()
    rc, h = _ctx(str(tmp_path / "nope.mol"), xp)
    assert rc == -2 and not h.value and b"open failed" in L.gg_last_error(None)
    short = tmp_path / "short.xdens"
    short.write_text("\n".join(open(xp).read().splitlines()[:1000]) + "\n")
    rc, h = _ctx(mp, str(short))
    assert rc == -2 and b"too short" in L.gg_last_error(None)
    bad = tmp_path / "bad.mol"
    bad.write_text("NOT AN INTGRL FILE\n")
    rc, _ = _ctx(str(bad), xp)
    assert rc == -2
    rc, h = _ctx(mp, xp)
    assert rc == 0
    assert L.gg_set_spin(h, b"sideways") == -1
    assert L.gg_set_flags(h, 1, 0, 0) == -1  # both dia and para off
    assert L.gg_set_precision(h, 7) == -1
    assert L.gg_set_max_batch(h, 1) == -1
    L.gg_ctx_destroy(h)
    with pytest.raises(_lib.GimicError):
        api.Gimic(str(tmp_path / "nope.mol"), xp)


def test_closed_shell_spin_cases_rejected_before_compute(c6h6):
    # beta/spindens on a closed shell (jtensor.F90:77-98) is a host-side error
    mp, xp, _ = c6h6
    o = oracle.Oracle(mp, xp)
    with pytest.raises(ValueError):
        o.jtensor(np.zeros((1, 3)), spin="beta")


def test_reference_inputs_parse(golden_dir):
    for case, name in (("c4h4", "integration.inp"), ("c4h4", "read-grid.inp"),
                       ("open-shell", "integration.inp"), ("open-shell", "3d.inp")):
        i = ginp.read(str(golden_dir / case / name))
        assert i.get("calc") in ("integral", "cdens")
    i = ginp.read(str(golden_dir / "c4h4" / "integration.inp"))
    assert i.grid_arg == "bond" and i.get("Grid.bond") == [2, 1] and i.get("Grid.gauss_order") == 9
    assert i.get("Advanced.screening_thrs") == 1e-8 and i.get("Advanced.screening") is True
    assert not i.is_set("Grid.radius") and i.is_set("Grid.rotation")


@pytest.mark.parametrize("text,msg", [
    ("calc=foo\nmagnet_axis=z\n", "unknown option calc"),
    ("calc=cdens\n", "Direction of magnetic field must be set"),
    ("calc=cdens\nmagnet=[0,0,1]\nmagnet_axis=z\n", "Both magnet vector and axis"),
    ("calc=cdens\nmagnet_axis=z\nGrid(base){\ntype=even\norigin=[0,0,0]\n}\n", "Required option 'ivec'"),
    ("calc=integral\nmagnet_axis=z\nGrid(bond){\ntype=gauss\ndistance=1.0\nbond=[1,2]\n}\n", "fixpoint or fixcoord"),
    ("calc=cdens\nmagnet_axis=z\nGrid(base){\norigin=[0,0]\n}\n", "length mismatch"),
    ("calc=cdens\nmagnet_axis=z\nGrid(base){\norigin=[0,0,0]\n", "unterminated section"),
    ("calc=cdens\nmagnet_axis=z\nbogus=1\n", "Unknown keyword"),
    ("calc=cdens\nmagnet_axis=z\nAdvanced{\nscreening=maybe\n}\n", "Not a bool"),
])
def test_input_errors(text, msg):
    with pytest.raises(ginp.InputError, match=msg):
        ginp.read(text, is_text=True)


def test_input_syntax_features():
    text = ('calc=integral  # comment\nmagnet_axis=T\ntitle="a b # c"\n'
            'Advanced {\n screening_thrs=1.d-8\n GIAO=off\n}\n'
            'Grid(bond) {\n type=lobatto\n bond=[1,|\n 2]\n fixpoint=3\n distance=0.5\n'
            ' height=[-5.0, 5.0]\n width=[0.0, 8.0]\n grid_points=[60, 60, 0]\n gauss_order=10\n}\n')
    i = ginp.read(text, is_text=True)
    assert i.get("magnet_axis") == "X"  # T and X both mean "perpendicular" (gimic.in:277-283)
    assert i.get("title") == "a b # c"
    assert i.get("Advanced.screening_thrs") == 1e-8 and i.get("Advanced.GIAO") is False
    assert i.get("Grid.bond") == [1, 2]


def test_bond_grid_geometry(c6h6):
    """Bond-plane frame of grid.f90:165-276 for a benzene C-C bond: normal
    along the bond, plane spanned by -ortho and the in-plane direction."""
    mp, xp, mol = c6h6
    text = ('calc=integral\nmagnet_axis=z\nGrid(bond) {\n type=lobatto\n bond=[1,2]\n fixcoord=[0,0,0]\n'
            ' distance=1.313\n height=[-8.0, 8.0]\n width=[0.0, 8.0]\n grid_points=[60, 60, 0]\n'
            ' gauss_order=10\n}\n')
    i = ginp.read(text, is_text=True)
    g = ggrid.new_grid(i, mol.coords)
    assert g.npts == [60, 60, 1]
    bond = mol.coords[1] - mol.coords[0]
    assert np.allclose(g.basv[:, 2], bond / np.linalg.norm(bond))
    assert np.allclose(np.abs(g.basv[:, 0]), [0, 0, 1])
    assert np.allclose(g.basv.T @ g.basv, np.eye(3), atol=1e-14)
    bb, flipped = ggrid.get_magnet(g, i)
    assert np.allclose(np.abs(bb), [0, 0, 1])
    pts = g.points()
    assert pts.shape == (3600, 3)
    assert np.array_equal(pts[61], g.gridpoint(1, 1, 0))
    assert g.warnings == []
    # above 13 Lobatto points per panel the reference warns and goes on
    # (gaussint.f90:68-75); the rule itself is then not reliable
    i14 = ginp.read(text.replace("gauss_order=10", "gauss_order=14").replace("[60, 60, 0]", "[56, 56, 0]"),
                    is_text=True)
    g14 = ggrid.new_grid(i14, mol.coords)
    assert g14.warnings[0] == "lobattomy(): Warning, too many Gauss points:  14"


def test_property_files_and_report(tmp_path):
    """get_property's inputs (coord.au, gridfile.grd, grid_w.grd, nelpts.info)
    are read as the reference reads them, and the printed blocks sum the
    per-block records (jfield.f90:700-928)."""
    import io

    from gimic_gb300 import properties

    (tmp_path / "coord.au").write_text("0.0 0.0 0.0\n1.5D0 0.0 0.0\n")
    pts = np.array([[0.1, 0.2, 0.3], [1.0, -0.5, 0.2], [2.0, 0.1, 0.1], [1.4, 0.3, -0.2], [0.5, 0.5, 0.5]])
    (tmp_path / "gridfile.grd").write_text("".join("%.17g %.17g %.17g\n" % tuple(p) for p in pts))
    (tmp_path / "grid_w.grd").write_text("".join("%r\n" % w for w in (0.1, 0.2, 0.3, 0.4, 0.5)))
    assert properties.read_inputs(str(tmp_path)) is not None
    coord, p, w, blocks = properties.read_inputs(str(tmp_path))
    assert blocks is None and np.allclose(coord[1], [1.5, 0, 0]) and np.allclose(p, pts) and len(w) == 5
    (tmp_path / "nelpts.info").write_text("1 2\n2 3\n")
    assert list(properties.read_inputs(str(tmp_path))[3]) == [2, 3]

    class Fake:
        def properties(self, pts, w, centres, blocks):
            sig = np.arange(2 * 2 * 5, dtype=float).reshape(2, 2, 5)
            chi = np.arange(10, dtype=float).reshape(2, 5) * -0.01
            return sig, chi

    out = io.StringIO()
    sig, chi = properties.run(Fake(), out, str(tmp_path))
    text = out.getvalue()
    # totals of centre 1: sigma_xx = 0 + 5, shielding = (5 + 7 + 9) / 3
    # Fortran (X, A10, 2X, F14.6)
    assert " sigma_xx    " + "%14.6f" % 5.0 in text
    assert "%14.6f" % 7.0 in text
    assert "chi_xx " in text and "isotropic magnetizability chi" in text
    missing = io.StringIO()
    (tmp_path / "grid_w.grd").unlink()
    assert properties.run(Fake(), missing, str(tmp_path)) is None
    assert "property calculation is skipped" in missing.getvalue()


def test_shell_order_permutation(synth_dir):
    """The locality order is a permutation of the file's shells; switching to
    the file order and back restores both, and without screening radii the
    file order is kept."""
    mp, xp, mol = synth.make_workload("c24h24", str(synth_dir), seed=2024)
    g = api.Gimic(mp, xp, screening=1e-8)
    mode, order = g.shell_order()
    assert mode == "locality"
    assert sorted(order) == list(range(g.nshells)) and order != list(range(g.nshells))
    g.set_shell_order("file")
    assert g.shell_order() == ("file", list(range(g.nshells)))
    g.set_shell_order("locality")
    assert g.shell_order() == ("locality", order)
    with pytest.raises(_lib.GimicError):
        g.set_shell_order(2)
    g0 = api.Gimic(mp, xp, screening=0.0)
    assert g0.shell_order()[1] == list(range(g0.nshells))


def test_density_injections_rejected_at_creation(tmp_path, c6h6, golden_dir):
    """A non-finite density value, or an XDENS that holds more values than
    the basis needs (a density of another basis, an open-shell file read as
    closed shell), is an error when the context is created: the reference
    would read past or stop short of the right blocks silently
    (src/libgimic/dens.f90:72-131)."""
    mp, xp, _ = c6h6
    L = _lib.load()
    lines = open(xp).read().splitlines()
    nan = tmp_path / "nan.xdens"
    bad = list(lines)
    assert lines[0].strip() == ""  # the file opens with a blank record
    bad[4321] = "NaN"  # the 4321st value
    nan.write_text("\n".join(bad) + "\n")
    rc, h = _ctx(mp, str(nan))
    assert rc == -2 and not h.value and b"value 4321 is not finite" in L.gg_last_error(None)
    inf = tmp_path / "inf.xdens"
    bad = list(lines)
    bad[17] = "-inf"
    inf.write_text("\n".join(bad) + "\n")
    rc, h = _ctx(mp, str(inf))
    assert rc == -2 and b"not finite" in L.gg_last_error(None)
    # one value too many: the density of a basis one function larger would
    # hold far more, but a single extra value already shows the mismatch
    extra = tmp_path / "extra.xdens"
    extra.write_text("\n".join(lines + ["0.5"]) + "\n")
    rc, h = _ctx(mp, str(extra))
    assert rc == -2 and b"more values" in L.gg_last_error(None)
    # the open-shell golden read as closed shell: the beta blocks are left over
    d = golden_dir / "open-shell"
    rc, h = _ctx(str(d / "MOL"), str(d / "XDENS"), uhf=False)
    assert rc == -2 and b"more values" in L.gg_last_error(None)
    rc, h = _ctx(str(d / "MOL"), str(d / "XDENS"), uhf=True)
    assert rc == 0
    L.gg_ctx_destroy(h)
    # trailing blank lines are not data
    blank = tmp_path / "blank.xdens"
    blank.write_text("\n".join(lines) + "\n\n   \n")
    rc, h = _ctx(mp, str(blank))
    assert rc == 0
    L.gg_ctx_destroy(h)


def test_zero_field_rejected_before_compute(c6h6):
    """A zero magnetic field stops the reference's driver ("Magnetic field is
    zero, not wasting more CPU.", src/fgimic/magnet.f90:56-59); the plane
    integrals and jvector evaluation refuse it before any device work, the
    driver's grid set-up raises it, and the reference C ABI keeps its
    behaviour (no stop there)."""
    mp, xp, mol = c6h6
    g = api.Gimic(mp, xp, screening=1e-8)
    assert np.all(g.get_magnet() == 0.0)
    ax = (np.array([0.0, 1.0]), np.array([0.5, 0.5]))
    with pytest.raises(_lib.GimicError, match="Magnetic field is zero"):
        g.plane_integral(np.zeros(3), np.eye(3), (ax, ax, (np.zeros(1), np.ones(1))))
    jv = np.zeros((1, 3))
    rc = g._L.gg_jvector_batch(g._h, C.c_void_p(np.zeros((1, 3)).ctypes.data), 1, C.c_void_p(jv.ctypes.data), None)
    assert rc == -1 and b"Magnetic field is zero" in g._L.gg_last_error(g._h)
    text = ("calc=integral\nmagnet=[0.0, 0.0, 0.0]\nGrid(bond) {\n type=gauss\n bond=[1,2]\n fixcoord=[0.0,0.0,0.0]\n"
            " distance=1.0\n height=[-2.0, 2.0]\n width=[-2.0, 2.0]\n grid_points=[9, 9, 0]\n gauss_order=9\n}\n")
    i = ginp.read(text, is_text=True)
    grd = ggrid.new_grid(i, mol.coords)
    with pytest.raises(ValueError, match="Magnetic field is zero"):
        ggrid.get_magnet(grd, i)


def test_scalar_vtu_layout(tmp_path):
    """write_scalar_unstructured follows write_vtk_scalar_unstructuredgrid
    (src/fgimic/vtkplot.f90:318-390) record by record."""
    from gimic_gb300 import vtk
    pts = np.array([[0.0, 1.5, -2.25], [1e-3, 0.0, 3.0], [2.0, 2.0, 2.0], [-1.0, 0.5, 0.25], [0.0, 0.0, 0.0]])
    val = np.array([1.25, -3.5e-7, 0.0, 42.0, -1.0])
    cells = np.array([[1, 2, 3, 4], [2, 3, 4, 5]])
    path = tmp_path / "s.vtu"
    vtk.write_scalar_unstructured(str(path), pts, val, cells)
    lines = path.read_text().split("\n")
    assert lines[0] == '<?xml version="1.0"?>'
    assert lines[3] == '    <Piece NumberOfPoints="         5" NumberOfCells="         2">'
    pad = " " * 8  # the records' leading "(a, ...)" field
    assert lines[6] == pad + "    0.0000000000E+00    0.1500000000E+01   -0.2250000000E+01"  # 3e20.10
    assert lines[15] == pad + "    0.1250000000E+01"  # e20.10
    assert lines[16] == pad + "   -0.3500000000E-06"
    assert lines[24] == pad + "         0         1         2         3"  # 4i10, 0-based
    assert lines[28] == pad + "         4         8"  # i10 offsets
    assert lines[31] == pad + "   10   10"  # i5 types
    assert lines[35] == pad + " 0.0 0.0"  # f4.1
    assert lines[-2] == "</VTKFile>"


def test_property_integrands_match_oracle_restatement():
    """The per-point integrands written to the VTU files agree with the
    oracle's restatement of jfield.f90:693-711 and :824-842."""
    import prop_oracle
    from gimic_gb300 import properties
    rng = np.random.default_rng(0)
    jt, pts, coord = rng.normal(size=(50, 9)), rng.normal(size=(50, 3)) * 3, rng.normal(size=(4, 3))
    s1, c1 = properties.per_point(jt, pts, coord)
    s2, c2 = prop_oracle.integrands(jt, pts, coord)
    assert np.abs(s1 - s2).max() <= 1e-14 * np.abs(s2).max()
    assert np.abs(c1 - c2).max() <= 1e-14 * np.abs(c2).max()
