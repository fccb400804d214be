"""GPU parity on the benchmark configurations themselves, against the FP64
C oracle:

  * the timed C24H24 cube workload (seed 2024, Cartesian basis, nbf 720): the
    split path on random points of the 128^3 cube plus points next to every
    nucleus, per tensor component and overall, e_j <= 1e-6;
  * the C6H6 bond plane (60 x 60 Gauss-Lobatto, order 10, +-8 Bohr about
    the ring plane, from the ring centre 8 Bohr outward): current, signed
    modulus and ACID against og_integrate (src/fgimic/integral.f90:50-511),
    within 1e-4 nA/T on the split path and 1e-9 nA/T on the FP64 path;
  * the ACID field of calc=cdens (acid.vti) against the oracle's get_acid
    (src/libgimic/acid.f90:11-43) point by point.
"""
import io
import os
import re

import numpy as np
import pytest

import oracle
from conftest import rel_max_err
from gimic_gb300 import api, driver, synth
from gimic_gb300 import grid as ggrid
from gimic_gb300 import inp as ginp

pytestmark = pytest.mark.gpu

TOL_SPLIT = 1e-6
TOL_NAT = 1e-4


def cube_sample(coords, n_cube, n_near, seed):
    """Points of the benchmark's 128^3 cube (half-width 16 Bohr) and points
    within ~0.1 Bohr of the nuclei, where |j| is largest."""
    rng = np.random.default_rng(seed)
    ax = np.linspace(-16.0, 16.0, 128)
    ijk = rng.integers(0, 128, (n_cube, 3))
    cube = ax[ijk]
    near = coords[rng.integers(0, len(coords), n_near)] + rng.normal(0.0, 0.1, (n_near, 3))
    return np.vstack([cube, near])


def test_c24h24_cube_workload_against_oracle(synth_dir):
    mp, xp, mol = synth.make_workload("c24h24", str(synth_dir), seed=2024)
    assert mol.nbf == 720
    g = api.Gimic(mp, xp, screening=1e-8, precision="split16")
    o = oracle.Oracle(mp, xp, screening=1e-8)
    pts = cube_sample(mol.coords, 4096, 1024, seed=17)
    ref, rho_ref = o.jtensor(pts, with_rho=True)
    jt, rho = g.jtensor_batch(pts, rho=True)
    scale = np.abs(ref).max()
    per_comp = np.abs(jt - ref).max(axis=0) / scale
    assert per_comp.max() <= TOL_SPLIT, per_comp
    assert rel_max_err(jt, ref) <= TOL_SPLIT
    assert rel_max_err(rho, rho_ref) <= TOL_SPLIT


def _c1_plane(synth_dir):
    mp, xp, mol = synth.make_workload("c6h6", str(synth_dir), seed=2024)
    i = ginp.read(synth.ring_bond_plane_input(mol), is_text=True)
    grd = ggrid.new_grid(i, mol.coords)
    bb, _ = ggrid.get_magnet(grd, i)
    return mp, xp, mol, grd, bb


def test_c1_plane_geometry(synth_dir):
    """The plane reaches from the ring centre to 8 Bohr out and +-8 Bohr
    about the ring, 60 x 60 Lobatto points."""
    _, _, _, grd, bb = _c1_plane(synth_dir)
    p = grd.points()
    assert p.shape == (3600, 3) and grd.npts[:2] == [60, 60]
    r = np.linalg.norm(p[:, :2], axis=1)
    assert abs(r.min()) < 1e-12 and abs(r.max() - 8.0) < 1e-12
    assert abs(p[:, 2].min() + 8.0) < 1e-12 and abs(p[:, 2].max() - 8.0) < 1e-12
    assert np.array_equal(bb, [0.0, 0.0, 1.0])


@pytest.mark.parametrize("precision,tol_nat", [("split16", TOL_NAT), ("fp64", 1e-9)])
def test_c1_plane_integrals_against_oracle(synth_dir, precision, tol_nat):
    mp, xp, _, grd, bb = _c1_plane(synth_dir)
    g = api.Gimic(mp, xp, screening=1e-8, precision=precision)
    g.set_magnet(bb)
    o = oracle.Oracle(mp, xp, screening=1e-8)
    res = g.plane_integral(grd.origin, grd.basv, grd.axes(), grd.radius)
    for kind in ("current", "modulus"):
        want = o.integrate(grd.origin, grd.basv, grd.axes(), grd.radius, bb, what=kind)
        for got, ref in zip(res[kind], want):
            assert abs(api.au2si(got) - api.au2si(ref)) <= tol_nat, (kind, got, ref)
    acid = o.integrate(grd.origin, grd.basv, grd.axes(), grd.radius, bb, what="acid")
    assert abs(api.au2si(res["acid"]) - api.au2si(acid[0])) <= tol_nat
    assert abs(res["acid_sum"] - acid[1]) <= 1e-6 * acid[1]
    # the ring current crosses the plane: a sizeable signal, not noise
    assert abs(api.au2si(res["current"][0])) > 1.0


def test_integral_driver_acid_block(tmp_path, synth_dir):
    """calc=integral with Essential.acid=on prints the ACID block
    (integral.f90:502-510) with the oracle's sqrt of the weighted sum."""
    mp, xp, mol, grd, bb = _c1_plane(synth_dir)
    d = tmp_path / "c1"
    d.mkdir()
    os.symlink(mp, d / "MOL")
    os.symlink(xp, d / "XDENS")
    text = ('basis="MOL"\nxdens="XDENS"\n' + synth.ring_bond_plane_input(mol)
            + "Advanced {\n spherical=off\n screening=on\n screening_thrs=1.d-8\n}\nEssential {\n acid=on\n}\n")
    (d / "gimic.inp").write_text(text)
    buf = io.StringIO()
    driver.Driver(str(d / "gimic.inp"), precision="split16", stream=buf).run()
    out = buf.getvalue()
    m = re.search(r"ACID \(au\) sqrt\(delta J\^2\):\s*([-0-9.]+)", out)
    m2 = re.search(r"ACID \(nA/T\)\s*:\s*([-0-9.]+)", out)
    assert m and m2, out
    o = oracle.Oracle(mp, xp, screening=1e-8)
    acid = o.integrate(grd.origin, grd.basv, grd.axes(), grd.radius, bb, what="acid")[0]
    assert abs(float(m.group(1)) - acid) <= 1.5e-6  # printed with 6 decimals
    assert abs(float(m2.group(1)) - api.au2si(acid)) <= 1.5e-6 + TOL_NAT


def _vti_scalars(path):
    text = open(path).read()
    m = re.search(r'<DataArray Name="scalars"[^>]*>(.*?)</DataArray>', text, re.S)
    return np.array(m.group(1).split(), dtype=np.float64)


@pytest.mark.parametrize("precision,tol", [("split16", 1e-5), ("fp64", 1e-10)])
def test_cdens_acid_field_against_oracle(tmp_path, synth_dir, precision, tol):
    mp, xp, mol = synth.make_workload("c6h6", str(synth_dir), seed=2024)
    d = tmp_path / precision
    d.mkdir()
    os.symlink(mp, d / "MOL")
    os.symlink(xp, d / "XDENS")
    (d / "gimic.inp").write_text(
        'calc=cdens\nbasis="MOL"\nxdens="XDENS"\nmagnet_axis=z\n'
        "Grid(base) {\n type=even\n origin=[-6.0, -6.0, -3.0]\n ivec=[1.0, 0.0, 0.0]\n"
        " jvec=[0.0, 1.0, 0.0]\n lengths=[12.0, 12.0, 6.0]\n spacing=[0.75, 0.75, 0.75]\n}\n"
        "Advanced {\n spherical=off\n screening=on\n screening_thrs=1.d-8\n}\nEssential {\n acid=on\n jmod=off\n}\n")
    drv = driver.Driver(str(d / "gimic.inp"), precision=precision, stream=io.StringIO())
    drv.run()
    pts = drv.grid.points()
    got = _vti_scalars(d / "acid.vti")
    assert got.shape == (len(pts),) == (17 * 17 * 9,)
    o = oracle.Oracle(mp, xp, screening=1e-8)
    t = o.jtensor(pts)
    L = oracle.lib()
    want = np.array([L.og_acid(np.ascontiguousarray(ti).ctypes.data_as(oracle._dp)) for ti in t])
    # both sides compared after the file's e14.6 print: the path's error plus
    # one unit of the printed digit
    ax = np.abs(want)
    ulp = np.where(ax > 0, 10.0 ** (np.floor(np.log10(np.where(ax > 0, ax, 1.0))) + 1.0 - 6.0), 0.0)
    assert np.all(np.abs(got - want) <= tol * want.max() + 1.01 * ulp)


def test_plane_graph_replay_matches_eager_passes(synth_dir):
    """gg_plane_integrals captures a pass as a CUDA graph on the second call
    with the same layout and replays it afterwards.  Replays with new plane
    data, a new field, or after a flag change (which forces an eager pass
    and a new capture) are bit-identical to eager passes in fresh contexts."""
    mp, xp, mol = synth.make_workload("c6h6", str(synth_dir), seed=2024)
    planes = []
    for bond in ((1, 2), (2, 3)):
        i = ginp.read(synth.ring_bond_plane_input(mol, bond=bond), is_text=True)
        grd = ggrid.new_grid(i, mol.coords)
        bb, _ = ggrid.get_magnet(grd, i)
        planes.append(((grd.origin, grd.basv, grd.axes(), grd.radius), bb))

    def fresh(plane, bb, flags=(1, 1, 1)):
        h = api.Gimic(mp, xp, screening=1e-8)
        h.set_flags(*flags)
        h.set_magnet(bb)
        return h.plane_integrals([plane])[0]

    g = api.Gimic(mp, xp, screening=1e-8)
    (pa, ba), (pb, bbb) = planes
    g.set_magnet(ba)
    want_a = fresh(pa, ba)
    got = [g.plane_integrals([pa])[0] for _ in range(4)]  # eager, capture, replay, replay
    assert all(r == want_a for r in got)
    g.set_magnet(bbb)
    assert g.plane_integrals([pb])[0] == fresh(pb, bbb)
    tilted = np.array([0.3, -0.2, 0.9])
    g.set_magnet(tilted)
    assert g.plane_integrals([pa])[0] == fresh(pa, tilted)
    g.set_flags(1, 1, 0)
    for _ in range(3):
        assert g.plane_integrals([pb])[0] == fresh(pb, tilted, flags=(1, 1, 0))
    # the kernel count goes on through the replays
    g.profile(False)
    g.plane_integrals([pb])
    assert g.profile_read()["kernels"] > 0


@pytest.mark.parametrize("name", ["c6h6", "c24h24"])
def test_short_and_long_passes_agree(synth_dir, name):
    """A short pass (no more tiles than SMs) spreads each tile's column
    chunks over SMs and adds their partial sums in chunk order as
    double-floats; a long pass runs one fp32 sum per function group over all
    chunks of a tile on one SM.  The fp32 roundings therefore differ between
    the two (measured: 1.2e-7 of max |rho|, about 3e-8 of max |j|, against
    the path's 1e-6 tolerance); both match the oracle."""
    mp, xp, mol = synth.make_workload(name, str(synth_dir), seed=2024)
    g = api.Gimic(mp, xp, screening=1e-8)
    pts = cube_sample(mol.coords, 1800, 248, seed=23)  # 16 tiles: a short pass
    short, rho_s, dv_s = g.jtensor_batch(pts, rho=True, divj=True)
    rng = np.random.default_rng(5)
    filler = rng.uniform(-16.0, 16.0, (160 * 128, 3))  # 160 more tiles: a long pass
    long_, rho_l, dv_l = g.jtensor_batch(np.vstack([pts, filler]), rho=True, divj=True)
    n = len(pts)
    assert rel_max_err(short, long_[:n]) <= 1e-7
    assert rel_max_err(rho_s, rho_l[:n]) <= 3e-7
    assert rel_max_err(dv_s, dv_l[:n]) <= 1e-6
    o = oracle.Oracle(mp, xp, screening=1e-8)
    ref = o.jtensor(pts)
    assert rel_max_err(short, ref) <= TOL_SPLIT and rel_max_err(long_[:n], ref) <= TOL_SPLIT


@pytest.mark.parametrize("precision,tol", [("split16", 1e-6), ("fp64", 1e-11)])
def test_property_integrand_files_against_oracle(tmp_path, synth_dir, precision, tol):
    """calc=cdens with Essential.prop=on on the molecular grid of
    gridfile.grd / grid_w.grd / coord.au / nelpts.info writes, when
    grid.1.ele is present, the per-point files of get_property
    (src/fgimic/jfield.f90:785-806, :905-910): sigma<k>.vtu and its three
    diagonal parts for every nucleus k, and intchi*.vtu.  Their values are
    the oracle's integrands (its tensors through the FP64 restatement)."""
    import prop_oracle

    mp, xp, mol = synth.make_workload("c6h6", str(synth_dir), seed=2024)
    d = tmp_path / precision
    d.mkdir()
    os.symlink(mp, d / "MOL")
    os.symlink(xp, d / "XDENS")
    rng = np.random.default_rng(41)
    xyz = mol.coords
    blocks = rng.integers(30, 60, len(xyz))
    pts = np.vstack([xyz[a] + rng.normal(0.0, 1.0, (blocks[a], 3)) for a in range(len(xyz))])
    w = rng.uniform(0.01, 0.1, len(pts))
    (d / "gridfile.grd").write_text("".join("%.15e %.15e %.15e\n" % tuple(p) for p in pts))
    (d / "grid_w.grd").write_text("".join("%.15e\n" % v for v in w))
    (d / "coord.au").write_text("".join("%.15e %.15e %.15e\n" % tuple(p) for p in xyz))
    (d / "nelpts.info").write_text("".join("%d %d\n" % (a + 1, blocks[a]) for a in range(len(xyz))))
    ncell = 40
    cells = rng.integers(1, len(pts) + 1, (ncell, 4))
    (d / "grid.1.ele").write_text("%d 4 0\n" % ncell + "".join("%d %d %d %d %d\n" % (i + 1, *c)
                                                              for i, c in enumerate(cells)))
    (d / "gimic.inp").write_text('calc=cdens\nbasis="MOL"\nxdens="XDENS"\nmagnet=[0.0, 0.0, 1.0]\n'
                                 "Grid(file) {\n file=gridfile.grd\n}\n"
                                 "Advanced {\n spherical=off\n screening=on\n screening_thrs=1.d-8\n}\n"
                                 "Essential {\n prop=on\n}\n")
    drv = driver.Driver(str(d / "gimic.inp"), precision=precision, stream=io.StringIO())
    drv.run()
    o = oracle.Oracle(mp, xp, screening=1e-8)
    sig, chi = prop_oracle.integrands(o.jtensor(pts), pts, xyz)

    def values(name):
        text = open(d / name).read()
        m = re.search(r'<DataArray Name="scalars"[^>]*>(.*?)</DataArray>', text, re.S)
        return np.array(m.group(1).split(), dtype=np.float64)

    def close(got, want):
        # the path's error relative to the largest integrand, plus one unit
        # of the e20.10 print (0.dddddddddd E+ee)
        aw = np.abs(want)
        ulp = np.where(aw > 0, 10.0 ** (np.floor(np.log10(np.where(aw > 0, aw, 1.0))) + 1.0 - 10.0), 0.0)
        return np.all(np.abs(got - want) <= tol * aw.max() + ulp)

    for k in range(len(xyz)):
        assert close(values("sigma%d.vtu" % (k + 1)), sig[k].sum(axis=1)), k
        for c, ax in enumerate(("xx", "yy", "zz")):
            assert close(values("sigma_%s%d.vtu" % (ax, k + 1)), sig[k][:, c]), (k, ax)
    assert close(values("intchi.vtu"), chi.sum(axis=1))
    for c, ax in enumerate(("xx", "yy", "zz")):
        assert close(values("intchi_%s.vtu" % ax), chi[:, c])
