"""Spherical basis (gimic.inp Advanced.spherical, src/libgimic/cao2sao.f90).

The reference projects its Cartesian basis values per point onto integer-
rescaled real solid harmonics (sbf = po . bf, src/libgimic/bfeval.f90:116-117
and dfdr :330-333), with the densities given over the spherical functions.
The oracle restates that per-point projection; the library folds it into the
densities once (D_cart = po^T D_sph po) and evaluates in the Cartesian basis.

No reference golden covers spherical=on (every reference test sets
spherical=off), so these cases are checked against the oracle only:
  * CPU: the projection rows are the known solid harmonics for l <= 3; the
    library's projection equals the oracle's; the oracle's spherical mode
    equals its Cartesian mode on the projected densities (1e-12);
  * GPU: e_j <= 1e-12 on the FP64 path and 1e-6 on the split path, plane
    integrals within 1e-4 nA/T.
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from conftest import rel_max_err, sample_points
from gimic_gb300 import _lib, api, synth

# rows m = -l..l over the standard component order (x, y, z; xx xy xz yy yz
# zz; xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz)
SOLID = {
    0: [[1]],
    1: [[0, 1, 0], [0, 0, 1], [1, 0, 0]],
    2: [[0, 1, 0, 0, 0, 0], [0, 0, 0, 0, 1, 0], [-1, 0, 0, -1, 0, 2], [0, 0, 1, 0, 0, 0], [1, 0, 0, -1, 0, 0]],
    3: [[0, 3, 0, 0, 0, 0, -1, 0, 0, 0],     # 3x^2y - y^3
        [0, 0, 0, 0, 1, 0, 0, 0, 0, 0],      # xyz
        [0, -1, 0, 0, 0, 0, -1, 0, 4, 0],    # y(4z^2 - x^2 - y^2)
        [0, 0, -3, 0, 0, 0, 0, -3, 0, 2],    # z(2z^2 - 3x^2 - 3y^2)
        [-1, 0, 0, -1, 0, 4, 0, 0, 0, 0],    # x(4z^2 - x^2 - y^2)
        [0, 0, 1, 0, 0, 0, 0, -1, 0, 0],     # (x^2 - y^2) z
        [1, 0, 0, -3, 0, 0, 0, 0, 0, 0]],    # x^3 - 3xy^2
}


@pytest.fixture(scope="module")
def c6h6_sph(synth_dir):
    return synth.make_workload("c6h6", str(synth_dir), seed=31, spherical=True)


def _lib_projection(l):
    L = _lib.load()
    nc = (l + 1) * (l + 2) // 2
    out = np.zeros((2 * l + 1) * nc)
    assert L.gg_spherical_projection(l, out.ctypes.data_as(C.POINTER(C.c_double))) == 0
    return out.reshape(2 * l + 1, nc)


def test_projection_rows_are_solid_harmonics(c6h6_sph):
    mp, xp, mol = c6h6_sph
    o = oracle.Oracle(mp, xp, spherical=True)
    assert (o.nbf, o.ncart) == (mol.nsph, mol.nbf)
    for l, rows in SOLID.items():
        assert np.array_equal(_lib_projection(l), np.asarray(rows, dtype=float)), l
    # the oracle's block-diagonal projection holds the same blocks shell by shell
    T = o.c2s()
    sh = o.shells()
    r = 0
    for a, l, pos in zip(sh["atom"], sh["l"], sh["pos"]):
        c0 = sum(int(n) for n in _atom_sizes(o)[:a]) + int(pos)
        nc = (l + 1) * (l + 2) // 2
        assert np.array_equal(T[r:r + 2 * l + 1, c0:c0 + nc], _lib_projection(int(l)))
        r += 2 * l + 1
    assert r == o.nbf


def _atom_sizes(o):
    sh = o.shells()
    sizes = np.zeros(o.natoms, dtype=int)
    for a, l in zip(sh["atom"], sh["l"]):
        sizes[a] += (l + 1) * (l + 2) // 2
    return sizes


def test_library_projection_beyond_f_matches_oracle(tmp_path):
    """l = 4, 5 (no GPU evaluation above f, but the operator is exported):
    the library keeps the reference's term-by-term assignment, as the oracle."""
    mol = synth.Molecule(["C"], [[0.0, 0.0, 0.0]], {"C": [(4, [1.0], [1.0]), (5, [0.5], [1.0])]})
    mp = str(tmp_path / "g.mol")
    synth.write_mol(mp, mol)
    o = oracle.Oracle(mp, None, spherical=True)
    T = o.c2s()
    assert np.array_equal(T[:9, :15], _lib_projection(4))
    assert np.array_equal(T[9:, 15:], _lib_projection(5))


def test_oracle_spherical_equals_projected_cartesian(c6h6_sph, tmp_path):
    mp, xp, _ = c6h6_sph
    o = oracle.Oracle(mp, xp, spherical=True)
    T = o.c2s()
    xc = str(tmp_path / "cart.xdens")
    synth.write_xdens(xc, [T.T @ o.density(0, b) @ T for b in range(4)])
    oc = oracle.Oracle(mp, xc)
    pts = sample_points(o.atoms()[0], 300, 100, 8.0, seed=2)
    j1, r1 = o.jtensor(pts, with_rho=True)
    j2, r2 = oc.jtensor(pts, with_rho=True)
    assert rel_max_err(j1, j2) <= 1e-12
    assert rel_max_err(r1, r2) <= 1e-12


def test_spherical_rejects_turbomole(golden_dir):
    d = golden_dir / "c4h4"
    with pytest.raises(RuntimeError, match="TURBOMOLE"):
        oracle.Oracle(str(d / "MOL"), str(d / "XDENS"), spherical=True)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c6h6", "c24h24"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("split16", 1e-6)])
def test_spherical_points(synth_dir, name, precision, tol):
    mp, xp, mol = synth.make_workload(name, str(synth_dir), seed=31, spherical=True)
    g = api.Gimic(mp, xp, screening=1e-8, precision=precision, spherical=True)
    o = oracle.Oracle(mp, xp, screening=1e-8, spherical=True)
    n = (900, 300) if name == "c6h6" else (300, 100)
    pts = sample_points(o.atoms()[0], n[0], n[1], 8.0 if name == "c6h6" else 14.0, seed=4)
    ref, rho_ref = o.jtensor(pts, with_rho=True)
    jt, rho = g.jtensor_batch(pts, rho=True)
    assert rel_max_err(jt, ref) <= tol
    assert rel_max_err(rho, rho_ref) <= tol


@pytest.mark.gpu
def test_spherical_plane_integral(c6h6_sph):
    mp, xp, _ = c6h6_sph
    o = oracle.Oracle(mp, xp, screening=1e-8, spherical=True)
    coords = o.atoms()[0]
    # a 40 x 40 Gauss-Lobatto plane through the midpoint of the first C-C
    # bond, perpendicular to it, from the ring centre outwards
    a, b = coords[0], coords[1]
    mid = 0.5 * (a + b)
    v = (b - a) / np.linalg.norm(b - a)
    w = mid / np.linalg.norm(mid)
    zax = np.cross(v, w)
    basv = np.stack([w, zax, v], axis=1)
    origin = mid - np.linalg.norm(mid) * w - 8.0 * zax
    p1, w1 = oracle.gauss_data(0.0, np.linalg.norm(mid) + 8.0, 10, 40, "lobatto")
    p2, w2 = oracle.gauss_data(0.0, 16.0, 10, 40, "lobatto")
    axes = ((p1, w1), (p2, w2), (np.zeros(1), np.ones(1)))
    bb = np.array([0.0, 0.0, -1.0])
    want = o.integrate(origin, basv, axes, 1e10, bb)
    for precision in ("fp64", "split16"):
        g = api.Gimic(mp, xp, screening=1e-8, precision=precision, spherical=True)
        g.set_magnet(bb)
        got = g.plane_integral(origin, basv, axes)["current"]
        for x, y in zip(got, want):
            assert abs(api.au2si(x) - api.au2si(y)) <= 1e-4
