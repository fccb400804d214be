"""CPU checks of the fp32 geometry the kernels use for r - R_A and
|r - R_A|^2, and of the fp32 tile screen, restated with numpy float32
operations (and the directed roundings) in the kernels' order
(gimic_gb300/csrc/gg_device.cuh: grid_split, atom_offset_g, two_sum;
gimic_gb300/csrc/gg_tiles.cuh: warp_tile_sphere, mark_shell).
The kernels' results are checked against the FP64 oracle by the GPU tests;
these tests pin the error bounds the device code states, over many random
points, without a GPU.  A fused multiply-add is restated as the float64
product (exact for float32 inputs) plus the addend, rounded once to float32."""
import numpy as np

f32 = np.float32


def fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    e = f32(f32(a - f32(s - bb)) + f32(b - bb))
    return s, e


def df_split(x):
    h = f32(x)
    return h, f32(x - np.float64(h))


def grid_split(h, l):
    g = f32(f32(np.rint(f32(h * f32(4096.0)))) * f32(1.0 / 4096.0))
    return g, f32(f32(h - g) + l)


def atom_offset_g(rg, ag):
    dh = [f32(rg[c][0] - ag[c][0]) for c in range(3)]
    s, p, lo = [], [], f32(0.0)
    for c in range(3):
        dl = f32(rg[c][1] - ag[c][1])
        s.append(f32(dh[c] + dl))
        p.append(f32(dh[c] * dh[c]))
        lo = f32(lo + fma(dh[c], dh[c], -p[c]))
        lo = fma(dl, fma(f32(2.0), dh[c], dl), lo)
    a1 = two_sum(p[0], p[1])
    a2 = two_sum(a1[0], p[2])
    d2 = two_sum(a2[0], f32(f32(a1[1] + a2[1]) + lo))
    return d2, s


def host_grid_split(v):
    g = f32(np.rint(v * 4096.0) / 4096.0)
    return g, f32(v - np.float64(g))


def test_grid_split_parts():
    rng = np.random.default_rng(11)
    for x in np.concatenate([rng.uniform(-60, 60, 3000), rng.uniform(-1e-3, 1e-3, 300)]):
        g, l = grid_split(*df_split(x))
        assert float(g) * 4096.0 == np.rint(float(g) * 4096.0)  # on the 2^-12 grid
        assert abs(float(l)) <= 2.0 ** -13 + 2.0 ** -24 * abs(x)
        assert abs(float(g) + float(l) - x) <= 2.0 ** -36 * max(1.0, abs(x))


def test_atom_offsets_within_stated_bounds():
    """|r - R_A|^2 within 2^-33 |d| + 2^-45 Bohr^2, from 1e-5 to 20 Bohr from
    the nucleus (the low parts carry about 2^-36 Bohr of rounding); the fp32
    offset s within half an ulp of r - R_A plus 2^-35 Bohr."""
    rng = np.random.default_rng(12)
    for _ in range(4000):
        A = rng.uniform(-20, 20, 3)
        r = A + rng.normal(size=3) * 10.0 ** rng.uniform(-5, 1.3)
        rg = [grid_split(*df_split(v)) for v in r]
        ag = [host_grid_split(v) for v in A]
        (h, l), s = atom_offset_g(rg, ag)
        d = r - A
        exact = float(np.sum(d.astype(np.longdouble) ** 2))
        assert abs(float(h) + float(l) - exact) <= 2.0 ** -33 * np.sqrt(exact) + 2.0 ** -45
        for c in range(3):
            assert abs(float(s[c]) - d[c]) <= 2.0 ** -24 * abs(d[c]) + 2.0 ** -35


# ---- tile screening (gimic_gb300/csrc/gg_tiles.cuh) -------------------------

def _rd(x):
    f = f32(x)
    return np.nextafter(f, f32(-np.inf)) if float(f) > x else f


def _ru(x):
    f = f32(x)
    return np.nextafter(f, f32(np.inf)) if float(f) < x else f


def _outward(x):
    """A coordinate converted to fp32 once (to nearest) and widened by
    2^-23 |v| + 2^-126 with directed roundings, as warp_tile_sphere does."""
    v = f32(x)
    e = _ru(abs(float(v)) * 2.0 ** -23 + 2.0 ** -126)
    return _rd(float(v) - float(e)), _ru(float(v) + float(e))


def _tile_sphere(pts):
    """warp_tile_sphere: the box from outward-widened fp32 coordinates, its
    centre and the radius widened against the centre's rounding."""
    ends = [[_outward(v) for v in pts[:, d]] for d in range(3)]
    lo = [min(a for a, _ in ends[d]) for d in range(3)]
    hi = [max(b for _, b in ends[d]) for d in range(3)]
    cf, rho2, cmax = [], f32(0.0), f32(0.0)
    for d in range(3):
        cf.append(f32(f32(0.5) * f32(lo[d] + hi[d])))
        h = _ru(0.5 * float(_ru(float(hi[d]) - float(lo[d]))))
        rho2 = _ru(float(h) * float(h) + float(rho2))
        cmax = max(cmax, abs(cf[d]))
    s = f32(np.sqrt(rho2))
    return cf, f32(_ru(float(s) * float(f32(1.0 + 1e-6))) + f32(f32(1.6e-5) * f32(1.0 + cmax)))


def _in_range(cf, rhof, atom, radius):
    """mark_shell's test: out of range when |R_A - c|^2 > (radius + rho)^2,
    widened."""
    at = [f32(v) for v in atom]
    dx, dy, dz = (f32(at[d] - cf[d]) for d in range(3))
    d2 = fma(dx, dx, fma(dy, dy, f32(dz * dz)))
    reach = f32(_ru(min(radius, 1e30)) + rhof)
    return not (d2 > fma(f32(reach * reach), f32(1.00001), f32(1e-4)))


def test_tile_screen_is_conservative():
    """A shell the fp32 tile test drops is out of range (|r - R_A| > radius,
    in FP64) for every point of the tile, over tiles up to 8 Bohr wide
    anywhere within 40 Bohr, with shells placed to just reach the tile; half
    the tiles have points on their box's corners, where the bounding sphere
    is tight and only the widening against the fp32 roundings keeps the test
    conservative (without it, about 5% of such needed shells are dropped)."""
    rng = np.random.default_rng(13)
    dropped = kept = 0
    for it in range(300):
        centre = rng.uniform(-40, 40, 3)
        half = rng.uniform(0.05, 1.0, 3) * 10.0 ** rng.uniform(-2, 0.6)
        pts = centre + rng.uniform(-1.0, 1.0, (128, 3)) * half
        if it % 2:  # a box whose corners are tile points: the sphere passes through them
            pts[:8] = centre + np.array([[sx, sy, sz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)]) * half
        cf, rhof = _tile_sphere(pts)
        for _ in range(20):
            radius = 10.0 ** rng.uniform(-1, 1.3)
            direction = rng.normal(size=3)
            if it % 2 and rng.uniform() < 0.5:
                direction = np.sign(direction) * half  # towards a corner
            direction /= np.linalg.norm(direction)
            # nuclei at about the distance where the shell just reaches the tile
            dmin = np.min(np.linalg.norm(pts - centre, axis=1))
            if rng.uniform() < 0.5:
                atom = centre + direction * (radius + rng.uniform(-1.0, 1.0) * 0.05 * radius + dmin)
            else:
                # within a few 1e-7 of just reaching the tile's outermost point
                # in that direction: the fp32 roundings decide
                far = pts[np.argmax(pts @ direction)]
                atom = far + direction * radius * (1.0 + rng.uniform(-3e-7, 3e-7))
            need = bool(np.any(np.sum((pts - atom) ** 2, axis=1) <= radius * radius))
            got = _in_range(cf, rhof, atom, radius)
            if need:
                assert got, "a shell some point needs was dropped"
            dropped += not got
            kept += got
    assert dropped > 100 and kept > 100  # the test exercises both sides


# ---- cross-product skip (gimic_gb300/csrc/gg_kernels.h, kCrossSkipScaled) ----

def test_cross_products_of_small_blocks_within_bound():
    """For scaled basis values below 1 (2^-14 of the row bound 2^14) and
    scaled matrix entries up to 2^14, the cross products hi*lo + lo*hi of the
    fp16 splits stay within 2^-24 of the row bound times the entry."""
    rng = np.random.default_rng(14)
    a = np.concatenate([rng.uniform(-1, 1, 20000), 10.0 ** rng.uniform(-12, 0, 20000)]).astype(np.float32)
    b = (rng.uniform(-1, 1, a.size) * 10.0 ** rng.uniform(-6, np.log10(16383.0), a.size)).astype(np.float32)
    ah = a.astype(np.float16)
    al = (a - ah.astype(np.float32)).astype(np.float16)
    bh = b.astype(np.float16)
    bl = (b - bh.astype(np.float32)).astype(np.float16)
    cross = np.abs(ah.astype(np.float64) * bl.astype(np.float64) + al.astype(np.float64) * bh.astype(np.float64))
    assert np.all(cross <= 2.0 ** -24 * 2.0 ** 14 * np.abs(b.astype(np.float64)) + 2.0 ** -48)
