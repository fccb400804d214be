"""CPU checks of the fp32 geometry the kernels use for r - R_A and
|r - R_A|^2, restated with numpy float32 operations in the kernels' order
(gimic_gb300/csrc/gg_device.cuh: grid_split, atom_offset_g, two_sum).
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
