"""GPU parity: libgimic_gb300 (through its C ABI) against the FP64 CPU oracle
and the reference's golden outputs.

Tolerances:
  * plain FP64 GPU path: e_j <= 1e-12 (max |dj| / max |j|);
  * split-FP16 tensor-core path: e_j <= 1e-6, integrated currents within
    1e-4 nA/T of the oracle;
  * div j: against central finite differences of the oracle's tensor.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, rel_max_err, sample_points
from gimic_gb300 import _lib, api
from gimic_gb300 import grid as ggrid
from gimic_gb300 import inp as ginp

pytestmark = pytest.mark.gpu

TOL_SPLIT = 1e-6
TOL_FP64 = 1e-12
TOL_NAT = 1e-4
GOLD = json.load(open(os.path.join(GOLDEN, "golden.json")))


def _pair(mol, xdens, uhf=False, screening=1e-8, precision="split16"):
    g = api.Gimic(mol, xdens, uhf=uhf, screening=screening, precision=precision)
    o = oracle.Oracle(mol, xdens, uhf=uhf, screening=screening)
    return g, o


@pytest.mark.parametrize("precision,tol", [("fp64", TOL_FP64), ("split16", TOL_SPLIT)])
def test_c6h6_points(c6h6, precision, tol):
    mp, xp, _ = c6h6
    g, o = _pair(mp, xp, precision=precision)
    pts = sample_points(o.atoms()[0], 1500, 500, 8.0)
    ref, rho_ref = o.jtensor(pts, with_rho=True)
    jt, rho = g.jtensor_batch(pts, rho=True)
    assert rel_max_err(jt, ref) <= tol
    assert rel_max_err(rho, rho_ref) <= tol


def test_divj_against_finite_differences(c6h6):
    mp, xp, _ = c6h6
    g, o = _pair(mp, xp, precision="fp64")
    pts = sample_points(o.atoms()[0], 30, 10, 4.0, seed=3)
    _, dv = g.jtensor_batch(pts, divj=True)
    # fourth-order central differences (tight primitives vary on 0.01 Bohr)
    h = 2e-4
    fd = np.zeros((len(pts), 3))
    for m in range(3):
        e = np.zeros(3)
        e[m] = h
        t2p, t1p, t1m, t2m = (o.jtensor(pts + k * e) for k in (2, 1, -1, -2))
        for b in range(3):
            i = m + 3 * b
            fd[:, b] += (-t2p[:, i] + 8 * t1p[:, i] - 8 * t1m[:, i] + t2m[:, i]) / (12 * h)
    assert rel_max_err(dv, fd) <= 1e-6
    g.set_precision("split16")
    _, dv16 = g.jtensor_batch(pts, divj=True)
    assert rel_max_err(dv16, dv) <= 1e-5


@pytest.mark.parametrize("giao,dia,para", [(0, 1, 1), (1, 0, 1), (1, 1, 0), (0, 0, 1)])
def test_flags(c6h6, giao, dia, para):
    mp, xp, _ = c6h6
    g, o = _pair(mp, xp, precision="fp64")
    g.set_flags(giao, dia, para)
    lib = oracle.lib()
    lib.og_set_flags(o._h, giao, dia, para)
    pts = sample_points(o.atoms()[0], 300, 100, 8.0, seed=5)
    ref = o.jtensor(pts)
    assert rel_max_err(g.jtensor_batch(pts), ref) <= TOL_FP64
    g.set_precision("split16")
    assert rel_max_err(g.jtensor_batch(pts), ref) <= TOL_SPLIT


def test_c4h4_turbomole_readgrid(golden_dir):
    """TURBOMOLE component order and density reordering; jvec on the
    reference's external grid against jvec.vtu."""
    d = golden_dir / "c4h4"
    i = ginp.read(str(d / "read-grid.inp"))
    g, o = _pair(str(d / "MOL"), str(d / "XDENS"))
    assert g.turbomole and g.nbf == 168
    grd = ggrid.new_grid(i, g.atoms()[0], workdir=str(d))
    bb, _ = ggrid.get_magnet(grd, i)
    g.set_magnet(bb)
    pts = grd.points()
    want = np.load(os.path.join(GOLDEN, "c4h4_readgrid.npz"))["jvec"]
    jv = np.asarray(g.jvector_batch(pts))
    assert rel_max_err(jv, want) <= TOL_SPLIT
    g.set_precision("fp64")
    assert rel_max_err(np.asarray(g.jvector_batch(pts)), want) <= 1e-9


@pytest.mark.parametrize("spin", ["total", "alpha", "beta", "spindens"])
def test_openshell_spin_cases(golden_dir, spin):
    d = golden_dir / "open-shell"
    g, o = _pair(str(d / "MOL"), str(d / "XDENS"), uhf=True)
    pts = sample_points(o.atoms()[0], 800, 200, 8.0, seed=11)
    ref = o.jtensor(pts, spin=spin)
    g.set_spin(spin)
    assert rel_max_err(g.jtensor_batch(pts), ref) <= TOL_SPLIT
    g.set_precision("fp64")
    assert rel_max_err(g.jtensor_batch(pts), ref) <= TOL_FP64


@pytest.mark.parametrize("case,uhf,key", [("c4h4", False, "c4h4_integration"),
                                          ("open-shell", True, "openshell_integration")])
@pytest.mark.parametrize("precision", ["split16", "fp64"])
def test_plane_integral_goldens(golden_dir, case, uhf, key, precision):
    d = golden_dir / case
    i = ginp.read(str(d / "integration.inp"))
    g = api.Gimic(str(d / "MOL"), str(d / "XDENS"), uhf=uhf, screening=i.get("Advanced.screening_thrs"),
                  precision=precision)
    grd = ggrid.new_grid(i, g.atoms()[0])
    bb, _ = ggrid.get_magnet(grd, i)
    g.set_magnet(bb)
    for blk in GOLD[key]:
        g.set_spin(blk["spin"])
        res = g.plane_integral(grd.origin, grd.basv, grd.axes(), grd.radius)[blk["kind"]]
        tol = 6e-7 if precision == "fp64" else 2e-6
        for got, want in zip(res, (blk["au"], blk["pos"], blk["neg"])):
            assert abs(got - want) <= tol, (blk, res)
        assert abs(api.au2si(res[0]) - blk["nAT"]) <= (6e-7 if precision == "fp64" else TOL_NAT)


def test_edge_cases(c6h6):
    mp, xp, _ = c6h6
    g, o = _pair(mp, xp)
    assert g.jtensor_batch(np.zeros((0, 3))).shape == (0, 9)
    coords = o.atoms()[0]
    # a point on a nucleus, a ragged count (not a multiple of the 128-point tile)
    pts = np.vstack([coords[:1], sample_points(coords, 120, 9, 6.0, seed=2)])
    assert len(pts) % 128 != 0
    assert rel_max_err(g.jtensor_batch(pts), o.jtensor(pts)) <= TOL_SPLIT
    # far from every atom: all shells screened, exactly zero
    far = np.array([[1e3, 0.0, 0.0], [0.0, -500.0, 40.0]])
    assert np.all(g.jtensor_batch(far) == 0.0)
    # one point through the single-point API
    assert rel_max_err(np.array(g.jtensor(pts[5])), o.jtensor(pts[5:6])[0]) <= 1e-5


def test_batching_is_invariant(c6h6):
    """Tiles are independent: with the cross-product skip off, any batch
    split gives bit-identical results.  With it on (the default) the blocks
    whose cross products are skipped depend on a tile's points, so a point's
    result may change in its last bits with the split (one fp32 rounding of
    the main product per skipped block)."""
    mp, xp, _ = c6h6
    g = api.Gimic(mp, xp, screening=1e-8)
    pts = sample_points(g.atoms()[0], 3000, 100, 8.0, seed=9)

    def splits():
        g.set_max_batch(0)
        a = g.jtensor_batch(pts)
        g.set_max_batch(256)
        b = g.jtensor_batch(pts)
        c = np.vstack([g.jtensor_batch(pts[s:s + 777]) for s in range(0, len(pts), 777)])
        return a, b, c

    a, b, c = splits()  # skip on
    assert rel_max_err(b, a) <= 1e-7 and rel_max_err(c, a) <= 1e-7
    g.set_cross_skip(False)
    a0, b0, c0 = splits()
    assert np.array_equal(a0, b0) and np.array_equal(a0, c0)
    assert rel_max_err(a, a0) <= 1e-7


def test_tile_screening_is_exact(c6h6):
    """Tile screening only skips exact zeros: results are bit-identical with
    and without it, for compact, scattered and far-away points (with the
    cross-product skip off; on, within one fp32 rounding)."""
    mp, xp, _ = c6h6
    g = api.Gimic(mp, xp, screening=1e-8)
    rng = np.random.default_rng(12)
    ax = np.linspace(-12.0, 12.0, 24)
    cube = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    pts = np.vstack([cube, sample_points(g.atoms()[0], 2000, 300, 9.0, seed=13),
                     rng.uniform(-60.0, 60.0, (500, 3))])
    pts = pts[rng.permutation(len(pts))]
    g.set_cross_skip(False)  # the skip needs the tile lists: compare like with like
    a = g.jtensor_batch(pts, rho=True, divj=True)
    g.set_tile_screening(False)
    b = g.jtensor_batch(pts, rho=True, divj=True)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    g.set_tile_screening(True)
    g.set_cross_skip(True)
    for x, y in zip(g.jtensor_batch(pts, rho=True, divj=True), a):
        assert rel_max_err(x, y) <= 1e-7
    o = oracle.Oracle(mp, xp, screening=1e-8)
    sel = rng.choice(len(pts), 800, replace=False)
    assert rel_max_err(a[0][sel], o.jtensor(pts[sel])) <= TOL_SPLIT


@pytest.mark.parametrize("precision,tol", [("fp64", TOL_FP64), ("split16", TOL_SPLIT)])
def test_shell_order_does_not_change_results(c6h6_uhf, precision, tol):
    """The locality order permutes the functions and density rows/columns:
    every output agrees with the file order (and with the oracle) for all
    spin cases of an open-shell density, and tile screening issues fewer
    GEMM blocks on a cube."""
    mp, xp, _ = c6h6_uhf
    g = api.Gimic(mp, xp, uhf=True, screening=1e-8, precision=precision)
    o = oracle.Oracle(mp, xp, uhf=True, screening=1e-8)
    assert g.shell_order()[0] == "locality"
    pts = sample_points(g.atoms()[0], 1200, 300, 8.0, seed=21)
    for spin in ("alpha", "beta", "total", "spindens"):
        g.set_spin(spin)
        g.set_shell_order("locality")
        a = g.jtensor_batch(pts, rho=True, divj=True)
        g.set_shell_order("file")
        b = g.jtensor_batch(pts, rho=True, divj=True)
        for x, y in zip(a, b):
            assert rel_max_err(x, y) <= tol
        assert rel_max_err(a[0], o.jtensor(pts, spin=spin)) <= tol
    ax = np.linspace(-16.0, 16.0, 48)
    cube = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    g.set_spin("total")
    blocks = {}
    for mode in ("file", "locality"):
        g.set_shell_order(mode)
        g.profile(True)
        g.jtensor_batch(cube)
        blocks[mode] = g.profile_read()["gemm_blocks"][0]
        g.profile(False)
    if precision == "split16":
        assert blocks["locality"] < blocks["file"]


def test_profile_counts_screened_work(c6h6):
    mp, xp, _ = c6h6
    g = api.Gimic(mp, xp, screening=1e-8)
    ax = np.linspace(-16.0, 16.0, 32)
    cube = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    g.profile(True)
    g.jtensor_batch(cube)
    pr = g.profile_read()
    issued, dense = pr["gemm_blocks"]
    g.profile(False)
    assert 0 < issued < dense
    # blocks small for a whole tile issue only the main product
    assert 0 < pr["cross_blocks"] < issued
    g.set_cross_skip(False)
    g.profile(True)
    g.jtensor_batch(cube)
    pr = g.profile_read()
    g.profile(False)
    assert pr["cross_blocks"] == pr["gemm_blocks"][0] == issued


def test_device_and_host_buffers_agree(c6h6):
    torch = pytest.importorskip("torch")
    mp, xp, _ = c6h6
    g = api.Gimic(mp, xp, screening=1e-8)
    pts = sample_points(g.atoms()[0], 1000, 100, 8.0, seed=4)
    host = g.jtensor_batch(pts, rho=True, divj=True)
    dev = g.jtensor_batch(torch.as_tensor(pts, device="cuda"), rho=True, divj=True)
    for h, d in zip(host, dev):
        assert np.array_equal(h, d.cpu().numpy())


def test_host_buffers_in_uneven_batches_agree_with_device_buffers(c6h6):
    """Host buffers of 2^20 + 3,000 points go through the overlapped copy
    pipeline in batches of 2^18, a full pass and 2^18 points, each prepared
    while the previous one is contracted; device buffers take one pass.  With
    the cross-product skip off the results are bit-identical (tiles are
    independent); with it on they agree to the skip's rounding."""
    torch = pytest.importorskip("torch")
    mp, xp, _ = c6h6
    g = api.Gimic(mp, xp, screening=1e-8)
    rng = np.random.default_rng(31)
    pts = np.vstack([rng.uniform(-10.0, 10.0, ((1 << 20) + 2000, 3)),
                     sample_points(g.atoms()[0], 900, 100, 8.0, seed=32)])
    dpts = torch.as_tensor(pts, device="cuda")
    g.set_cross_skip(False)
    host = g.jtensor_batch(pts, rho=True, divj=True)
    dev = g.jtensor_batch(dpts, rho=True, divj=True)
    for h, d in zip(host, dev):
        assert np.array_equal(h, d.cpu().numpy())
    g.set_cross_skip(True)
    host = g.jtensor_batch(pts, rho=True, divj=True)
    dev = g.jtensor_batch(dpts, rho=True, divj=True)
    for h, d in zip(host, dev):
        assert rel_max_err(h, d.cpu().numpy()) <= 1e-7


def test_reference_compat_interface(golden_dir):
    """gimic_init / gimic_calc_jtensor / gimic_calc_jvector / mkgausspoints
    (src/libgimic/gimic_interface.h, gausspoints.h) through ctypes."""
    L = _lib.load()
    d = golden_dir / "c4h4"
    L.gimic_init(str(d / "MOL").encode(), str(d / "XDENS").encode())
    o = oracle.Oracle(str(d / "MOL"), str(d / "XDENS"), screening=1e-6)
    b = (C.c_double * 3)(0.0, 0.0, 1.0)
    L.gimic_set_magnet(b)
    pts = sample_points(o.atoms()[0], 50, 10, 5.0, seed=8)
    ref = o.jtensor(pts)
    for p, t in zip(pts, ref):
        r = (C.c_double * 3)(*p)
        jt = (C.c_double * 9)()
        jv = (C.c_double * 3)()
        L.gimic_calc_jtensor(r, jt)
        L.gimic_calc_jvector(r, jv)
        assert np.abs(np.array(jt[:]) - t).max() <= TOL_SPLIT * np.abs(ref).max()
        assert np.abs(np.array(jv[:]) - t[6:9]).max() <= TOL_SPLIT * np.abs(ref).max()
    L.gimic_finalize()
    a, bb, n, order = C.c_double(0.0), C.c_double(2.0), C.c_int(18), C.c_int(9)
    pts_, wgt_ = (C.c_double * 18)(), (C.c_double * 18)()
    L.mkgausspoints(C.byref(a), C.byref(bb), C.byref(n), C.byref(order), pts_, wgt_)
    p_ref, w_ref = oracle.gauss_data(0.0, 2.0, 9, 18)
    assert np.array_equal(np.array(pts_[:]), p_ref) and np.array_equal(np.array(wgt_[:]), w_ref)


def test_full_cube_properties(synth_dir):
    """The 128^3 C24H24 cube at full size: density non-negative (D = 2 C C^T
    is positive semidefinite), split path against the FP64 path on a random
    subset, and finite everywhere."""
    torch = pytest.importorskip("torch")
    from gimic_gb300 import synth
    mp, xp, _ = synth.make_workload("c24h24", str(synth_dir), seed=2024)
    g = api.Gimic(mp, xp, screening=1e-8)
    ax = torch.linspace(-16.0, 16.0, 128, dtype=torch.float64, device="cuda")
    pts = torch.stack(torch.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3).contiguous()
    jt, rho, dv = g.jtensor_batch(pts, rho=True, divj=True)
    assert bool(torch.isfinite(jt).all()) and bool(torch.isfinite(dv).all())
    assert float(rho.min()) >= -1e-7 * float(rho.max())
    idx = torch.randint(0, pts.shape[0], (2048,), generator=torch.Generator().manual_seed(1)).cuda()
    g64 = api.Gimic(mp, xp, screening=1e-8, precision="fp64")
    ref = g64.jtensor_batch(pts[idx].contiguous())
    assert rel_max_err(jt[idx].cpu().numpy(), ref.cpu().numpy()) <= TOL_SPLIT


@pytest.mark.parametrize("precision", ["split16", "fp64"])
def test_fp32_outputs_are_the_fp64_results_rounded(c6h6, precision):
    """gg_jtensor_batch_f32 stores each fp64 result rounded once to fp32, on
    host and device buffers alike."""
    torch = pytest.importorskip("torch")
    mp, xp, _ = c6h6
    g = api.Gimic(mp, xp, screening=1e-8, precision=precision)
    pts = sample_points(g.atoms()[0], 900, 300, 8.0, seed=11)
    jt, rho, dv = g.jtensor_batch(pts, rho=True, divj=True)
    jt32, rho32, dv32 = g.jtensor_batch(pts, rho=True, divj=True, dtype=np.float32)
    assert jt32.dtype == np.float32
    assert np.array_equal(jt32, jt.astype(np.float32))
    assert np.array_equal(rho32, rho.astype(np.float32))
    assert np.array_equal(dv32, dv.astype(np.float32))
    djt = g.jtensor_batch(torch.as_tensor(pts, device="cuda"), dtype=np.float32)
    assert djt.dtype == torch.float32 and np.array_equal(djt.cpu().numpy(), jt32)


@pytest.mark.parametrize("precision,tol", [("split16", 1e-6), ("fp64", 1e-11)])
def test_properties_against_oracle(c6h6, precision, tol):
    """gg_properties (shielding of every nucleus, magnetizability, per-block
    decomposition) against the FP64 restatement of get_property on the C
    oracle's tensors; errors relative to the sums of |terms|."""
    import prop_oracle

    mp, xp, _ = c6h6
    g, o = _pair(mp, xp, precision=precision)
    xyz = o.atoms()[0]
    rng = np.random.default_rng(21)
    blocks = rng.integers(150, 400, len(xyz))
    pts = np.vstack([xyz[a] + rng.normal(0.0, 1.2, (blocks[a], 3)) for a in range(len(xyz))])
    w = rng.uniform(0.01, 0.2, len(pts))
    sig, chi = g.properties(pts, w, xyz, blocks)
    jt = o.jtensor(pts)
    ref_sig, ref_chi = prop_oracle.properties(jt, pts, w, xyz, blocks)
    assert sig.shape == ref_sig.shape == (len(xyz), len(xyz), 5) and chi.shape == ref_chi.shape
    # error bound: tol * max|j| times the sum of |weight * kernel|
    jmax = np.max(np.abs(jt))
    for k, R in enumerate(xyz):
        d = np.linalg.norm(pts - R, axis=1)
        scale = jmax * np.sum(w * 1.0e6 * d / d ** 3 / 137.0359998 ** 2)
        assert np.max(np.abs(sig[k] - ref_sig[k])) <= tol * scale, k
    scale = jmax * np.sum(w * 0.5 * np.linalg.norm(pts, axis=1))
    assert np.max(np.abs(chi - ref_chi)) <= tol * scale
    # one block when no decomposition is given: the totals
    s1, c1 = g.properties(pts, w, xyz)
    assert s1.shape == (len(xyz), 1, 5)
    assert np.allclose(s1[:, 0, :], sig.sum(axis=1), rtol=1e-9, atol=1e-12)
    assert np.allclose(c1[0], chi.sum(axis=0), rtol=1e-9, atol=1e-15)


def test_queued_plane_passes_match_blocking_calls(c6h6, c6h6_uhf):
    """gg_plane_integrals_enqueue / _collect over several contexts gives the
    blocking call's sums; a second enqueue before collecting, and a collect
    with nothing queued, are rejected."""
    from gimic_gb300 import scan

    jobs = []
    for (mp, xp, mol), uhf in ((c6h6, False), (c6h6_uhf, True)):
        g = api.Gimic(mp, xp, uhf=uhf, screening=1e-8)
        bond = scan.first_cc_bond(mol.symbols, mol.coords)
        planes, bb = scan.profile_planes(mol.coords, bond=bond, start=-2.0, out=8.0, nstrips=7, npts=(30, 30),
                                         order=10, quadrature="lobatto",
                                         fixcoord=tuple(scan.plane_fixcoord(mol.coords, bond)))
        g.set_magnet(bb)
        jobs.append((g, planes))
    want = [g.plane_integrals(planes) for g, planes in jobs]
    for _ in range(2):
        got, ms = api.plane_integrals_multi(jobs, timings=True)
        assert all(t > 0 for t in ms)
        for a, b in zip(got, want):
            for ra, rb in zip(a, b):
                assert np.allclose(ra["current"], rb["current"], rtol=1e-12, atol=1e-15)
                assert np.allclose(ra["modulus"], rb["modulus"], rtol=1e-12, atol=1e-15)
    g, planes = jobs[0]
    specs, flat = api._grid_records(planes)
    L = g._L
    p = specs.ctypes.data_as(C.POINTER(_lib.GridSpec))
    assert L.gg_plane_integrals_enqueue(g._h, p, len(planes), None) == 0
    assert L.gg_plane_integrals_enqueue(g._h, p, len(planes), None) != 0
    out = np.zeros((len(planes), 7))
    assert L.gg_plane_integrals_collect(g._h, out.ctypes.data_as(C.POINTER(C.c_double)), None) == 0
    assert np.allclose(out[:, 0], [r["current"][0] for r in want[0]], rtol=1e-12, atol=1e-15)
    assert L.gg_plane_integrals_collect(g._h, out.ctypes.data_as(C.POINTER(C.c_double)), None) != 0


def test_fp64_path_screens_tiles_like_the_split_path(c6h6):
    """The plain FP64 path runs the split path's tile screening (Z order,
    per-tile active chunks and K blocks; the skipped basis values are exact
    zeros): with and without it the results agree to FP64 rounding (the
    GEMM sums in another order), for compact, scattered and far points, and
    both match the oracle."""
    mp, xp, _ = c6h6
    g = api.Gimic(mp, xp, screening=1e-8, precision="fp64")
    rng = np.random.default_rng(21)
    ax = np.linspace(-12.0, 12.0, 20)
    cube = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    pts = np.vstack([cube, sample_points(g.atoms()[0], 1500, 300, 9.0, seed=22),
                     rng.uniform(-60.0, 60.0, (300, 3))])
    pts = pts[rng.permutation(len(pts))]
    g.profile(True)
    a = g.jtensor_batch(pts, rho=True, divj=True)
    issued, dense = g.profile_read()["gemm_blocks"]
    g.profile(False)
    assert 0 < issued < dense
    g.set_tile_screening(False)
    b = g.jtensor_batch(pts, rho=True, divj=True)
    for x, y in zip(a, b):
        assert rel_max_err(x, y) <= 1e-13
    o = oracle.Oracle(mp, xp, screening=1e-8)
    sel = rng.choice(len(pts), 600, replace=False)
    ref, rho_ref = o.jtensor(pts[sel], with_rho=True)
    assert rel_max_err(a[0][sel], ref) <= TOL_FP64 and rel_max_err(a[1][sel], rho_ref) <= TOL_FP64
