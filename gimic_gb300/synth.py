"""Seeded synthetic molecules, basis sets and density matrices.

The workloads are planar hydrocarbons with random contracted Cartesian
Gaussian shells, written in the reference's own input formats (an INTGRL
``MOL`` file and an ``XDENS`` file, see src/libgimic/intgrl.f90:20-264 and
src/libgimic/dens.f90:56-135), so that every consumer (the GPU path, the CPU
oracle, the reference itself) reads identical inputs.

Recipe (per workload ``seed``):
  * geometry: planar ring or fused-hexagon flake in the xy-plane, lengths in
    Angstrom converted with A2AU = 1.889725949 (src/libgimic/globals.f90:53);
  * one basis per element: C gets 3 s, 2 p and 1 d shells (+1 f when asked),
    H gets 2 s and 1 p shells; every shell has 1-6 primitives with exponents
    log-uniform in [0.1, 5000] Bohr^-2 and contraction coefficients uniform
    in [0.1, 1] (the reader normalises them, basis.f90:164-191);
  * D = 2 C_occ C_occ^T from the first ``nocc`` columns of a random
    orthonormal matrix (QR of a Gaussian matrix), exactly symmetric;
  * dD/dB_b, b = x, y, z: random antisymmetric matrices scaled to
    1e-2 * ||D||_F.
"""
import math
import os

import numpy as np

A2AU = 1.889725949

# (l, count) shells per element
_SHELLS = {
    "C": [(0, 3), (1, 2), (2, 1)],
    "H": [(0, 2), (1, 1)],
}
_CHARGE = {"C": 6.0, "H": 1.0}


def ncomp(l):
    return (l + 1) * (l + 2) // 2


class Molecule:
    """Atoms (symbols, coordinates in Bohr) plus per-element shell lists."""

    def __init__(self, symbols, coords_bohr, basis):
        self.symbols = list(symbols)
        self.coords = np.asarray(coords_bohr, dtype=np.float64)
        self.basis = basis  # element -> list of (l, exps[npf], coefs[npf])

    @property
    def natoms(self):
        return len(self.symbols)

    @property
    def nbf(self):
        return sum(sum(ncomp(l) for l, _, _ in self.basis[s]) for s in self.symbols)

    @property
    def nsph(self):
        """Functions of the spherical basis (2l + 1 per shell)."""
        return sum(sum(2 * l + 1 for l, _, _ in self.basis[s]) for s in self.symbols)

    def function_atoms(self):
        out = []
        for a, s in enumerate(self.symbols):
            out += [a] * sum(ncomp(l) for l, _, _ in self.basis[s])
        return np.asarray(out)


def random_basis(rng, with_f=False):
    basis = {}
    for el in ("C", "H"):
        shells = list(_SHELLS[el])
        if el == "C" and with_f:
            shells.append((3, 1))
        out = []
        for l, count in shells:
            for _ in range(count):
                npf = int(rng.integers(1, 7))
                exps = np.sort(np.exp(rng.uniform(math.log(0.1), math.log(5000.0), npf)))[::-1]
                coefs = rng.uniform(0.1, 1.0, npf)
                out.append((l, exps.copy(), coefs))
        basis[el] = out
    return basis


# ----------------------------------------------------------------------------
# geometries (Angstrom in, Bohr out)
# ----------------------------------------------------------------------------
def ring(ncarbon, cc=1.39, ch=1.09):
    """Planar regular ring of ``ncarbon`` C atoms with one H per carbon."""
    rad = cc / (2.0 * math.sin(math.pi / ncarbon))
    sym, xyz = [], []
    for i in range(ncarbon):
        t = 2.0 * math.pi * i / ncarbon
        sym.append("C")
        xyz.append((rad * math.cos(t), rad * math.sin(t), 0.0))
    for i in range(ncarbon):
        t = 2.0 * math.pi * i / ncarbon
        sym.append("H")
        xyz.append(((rad + ch) * math.cos(t), (rad + ch) * math.sin(t), 0.0))
    return sym, np.asarray(xyz) * A2AU


def hex_flake(nedge, cc=1.42, ch=1.09):
    """Hexagonal graphene flake with ``nedge`` hexagons per edge: 6 n^2 C
    atoms and 6 n H atoms (n=1 benzene, 2 coronene, ..., 4 C96H24)."""
    m = nedge - 1
    e1 = np.array([1.5 * cc, math.sqrt(3.0) / 2.0 * cc])
    e2 = np.array([0.0, math.sqrt(3.0) * cc])
    carbons = {}
    for u in range(-m, m + 1):
        for v in range(-m, m + 1):
            if max(abs(u), abs(v), abs(u + v)) > m:
                continue
            c = u * e1 + v * e2
            for k in range(6):
                t = math.pi / 3.0 * k
                p = (c[0] + cc * math.cos(t), c[1] + cc * math.sin(t))
                carbons[(round(p[0], 6), round(p[1], 6))] = p
    cpos = np.array([carbons[k] for k in sorted(carbons)])
    sym, xyz, hxyz = [], [], []
    for p in cpos:
        d = np.linalg.norm(cpos - p, axis=1)
        nb = cpos[(d > 0.1) & (d < cc * 1.1)]
        sym.append("C")
        xyz.append((p[0], p[1], 0.0))
        if len(nb) == 2:  # perimeter carbon: one H, pointing outward
            out = 2 * p - nb.sum(axis=0)
            out = out / np.linalg.norm(out)
            hxyz.append((p[0] + ch * out[0], p[1] + ch * out[1], 0.0))
    sym += ["H"] * len(hxyz)
    xyz += hxyz
    return sym, np.asarray(xyz) * A2AU


def benzene():
    return ring(6, cc=1.39, ch=1.09)


def honeycomb_patch(ncarbon, rng, cc=1.42, ch=1.09):
    """Planar sheet of exactly ``ncarbon`` C atoms cut from a honeycomb lattice
    around a random centre (jittered so that shapes vary), dangling carbons
    pruned and refilled, one H on every perimeter carbon (two C neighbours).
    Returns None when no carbon set of that size with at least two C
    neighbours per carbon was found."""
    a = math.sqrt(3.0) * cc
    lat = []
    m = 8
    for i in range(-m, m + 1):
        for j in range(-m, m + 1):
            x = a * (i + 0.5 * j)
            y = a * (math.sqrt(3.0) / 2.0) * j
            lat.append((x, y))
            lat.append((x, y + cc))
    lat = np.asarray(lat)
    centre = rng.uniform(-0.5, 0.5, 2) * cc
    order = np.argsort(np.linalg.norm(lat - centre, axis=1) + rng.uniform(0, 0.3 * cc, len(lat)))
    chosen = list(order[:ncarbon])
    rest = list(order[ncarbon:])

    def nbrs(idx, pool):
        d = np.linalg.norm(lat[pool] - lat[idx], axis=1)
        return int(np.sum((d > 0.1) & (d < 1.1 * cc)))

    for _ in range(4 * ncarbon):  # replace carbons with fewer than two C neighbours
        bad = [k for k in chosen if nbrs(k, chosen) < 2]
        if not bad:
            break
        chosen.remove(bad[0])
        for r in rest:
            if nbrs(r, chosen) >= 2:
                chosen.append(r)
                rest.remove(r)
                break
    if len(chosen) != ncarbon or any(nbrs(k, chosen) < 2 for k in chosen):
        return None  # no such patch near this centre (e.g. 4, 5 or 7 carbons)
    cpos = lat[chosen]
    sym, xyz, hxyz = [], [], []
    for p in cpos:
        d = np.linalg.norm(cpos - p, axis=1)
        nb = cpos[(d > 0.1) & (d < cc * 1.1)]
        sym.append("C")
        xyz.append((p[0], p[1], 0.0))
        if len(nb) == 2:
            out = 2 * p - nb.sum(axis=0)
            out = out / np.linalg.norm(out)
            hxyz.append((p[0] + ch * out[0], p[1] + ch * out[1], 0.0))
    sym += ["H"] * len(hxyz)
    xyz += hxyz
    return sym, np.asarray(xyz) * A2AU


def random_hydrocarbon(rng, cmin=4, cmax=40):
    """A planar ring (C <= 30, at random) or honeycomb sheet with a C count
    drawn uniformly from [cmin, cmax], H on every perimeter carbon."""
    nc = int(rng.integers(cmin, cmax + 1))
    if nc <= 30 and rng.uniform() < 0.5:
        return ring(nc, cc=1.39, ch=1.09)
    sheet = honeycomb_patch(nc, rng)
    if sheet is None:
        return ring(nc, cc=1.39, ch=1.09) if nc <= 30 else random_hydrocarbon(rng, cmin, cmax)
    return sheet


# ----------------------------------------------------------------------------
# densities
# ----------------------------------------------------------------------------
def random_densities(rng, nbf, nocc, pert_scale=1e-2):
    g = rng.standard_normal((nbf, nbf))
    q, _ = np.linalg.qr(g)
    c = q[:, :nocc]
    d = 2.0 * c @ c.T
    d = 0.5 * (d + d.T)
    norm = np.linalg.norm(d)
    pert = []
    for _ in range(3):
        a = rng.standard_normal((nbf, nbf))
        a = a - a.T
        a *= pert_scale * norm / np.linalg.norm(a)
        pert.append(a)
    return d, pert


# ----------------------------------------------------------------------------
# writers in the reference's formats
# ----------------------------------------------------------------------------
def write_mol(path, mol, title="synthetic molecule"):
    """INTGRL file as read by intgrl.f90:20-264 (standard component order)."""
    lines = ["INTGRL        1    0    1    0    0    0    0    0    0",
             "GIMIC-GB300",
             "              " + title,
             "%d    0            0.10E-08              0    0" % mol.natoms,
             "9999.00      3.00"]
    for a, s in enumerate(mol.symbols):
        shells = mol.basis[s]
        lmax = max(l for l, _, _ in shells)
        counts = [sum(1 for l, _, _ in shells if l == ll) for ll in range(lmax + 1)]
        lines.append("%.1f    1 %d  %s" % (_CHARGE[s], lmax + 1, "  ".join(str(c) for c in counts)))
        x, y, z = mol.coords[a]
        lines.append("%-2s%-2d %19.12f %19.12f %19.12f" % (s, a % 99 + 1, x, y, z))
        for ll in range(lmax + 1):
            for l, exps, coefs in shells:
                if l != ll:
                    continue
                lines.append("%6d %3d" % (len(exps), 1))
                for e, c in zip(exps, coefs):
                    lines.append("%24.16E %24.16E" % (e, c))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_xdens(path, blocks):
    """XDENS (dens.f90:56-135): per spin four nbf x nbf blocks (D, dD/dBx,
    dD/dBy, dD/dBz), column-major, one value per line, a blank line before
    each block.  Values are written with 17 significant digits so that the
    file round-trips to the same doubles."""
    with open(path, "w") as f:
        for m in blocks:
            f.write(" \n")
            flat = np.asarray(m, dtype=np.float64).reshape(-1, order="F")
            f.write("\n".join("%.16E" % v for v in flat))
            f.write("\n")


# ----------------------------------------------------------------------------
# named workloads
# ----------------------------------------------------------------------------
WORKLOADS = {
    # name: (geometry builder, with_f, nocc)
    "c6h6": (benzene, False, 21),
    "c24h24": (lambda: ring(24, cc=1.39, ch=1.09), True, 84),
    "c96h24": (lambda: hex_flake(4, cc=1.42, ch=1.09), False, 324),
}


def make_batch_molecule(outdir, index, seed=77):
    """Molecule ``index`` of the batched-scan generator: a random ring or sheet
    (C 4..40) with the seeded basis recipe and nocc = number of C atoms x 3.5
    (rounded).  Returns (mol_path, xdens_path, Molecule)."""
    rng = np.random.default_rng([seed, index])
    sym, xyz = random_hydrocarbon(rng)
    mol = Molecule(sym, xyz, random_basis(rng, with_f=False))
    os.makedirs(outdir, exist_ok=True)
    tag = "batch_s%d_%03d" % (seed, index)
    mol_path, xd_path = os.path.join(outdir, tag + ".mol"), os.path.join(outdir, tag + ".xdens")
    if not (os.path.exists(mol_path) and os.path.exists(xd_path)):
        nocc = max(1, int(round(3.5 * sym.count("C"))))
        d, pert = random_densities(rng, mol.nbf, min(nocc, mol.nbf))
        tmp = ".tmp%d" % os.getpid()
        write_mol(mol_path + tmp, mol, "batch molecule %d seed %d" % (index, seed))
        write_xdens(xd_path + tmp, [d] + pert)
        os.replace(xd_path + tmp, xd_path)
        os.replace(mol_path + tmp, mol_path)
    return mol_path, xd_path, mol


def make_workload(name, outdir, seed=2024, uhf=False, spherical=False):
    """Write MOL and XDENS for a named workload; returns (mol_path, xdens_path,
    Molecule).  Files are reused when already present for the same seed.
    With ``spherical`` the densities are over the spherical functions (2l + 1
    per shell, as a producer run with a spherical basis writes them); the MOL
    file is the same."""
    geo, with_f, nocc = WORKLOADS[name]
    os.makedirs(outdir, exist_ok=True)
    tag = "%s_s%d%s%s" % (name, seed, "_uhf" if uhf else "", "_sph" if spherical else "")
    mol_path = os.path.join(outdir, tag + ".mol")
    xd_path = os.path.join(outdir, tag + ".xdens")
    rng = np.random.default_rng(seed)
    sym, xyz = geo()
    mol = Molecule(sym, xyz, random_basis(rng, with_f))
    if os.path.exists(mol_path) and os.path.exists(xd_path):
        return mol_path, xd_path, mol  # the MOL file is written last
    n = mol.nsph if spherical else mol.nbf
    blocks = []
    for _ in range(2 if uhf else 1):
        d, pert = random_densities(rng, n, nocc if not uhf else max(1, nocc // 2))
        blocks += [d] + pert
    tmp = ".tmp%d" % os.getpid()
    write_mol(mol_path + tmp, mol, "synthetic %s seed %d" % (name, seed))
    write_xdens(xd_path + tmp, blocks)
    os.replace(xd_path + tmp, xd_path)
    os.replace(mol_path + tmp, mol_path)
    return mol_path, xd_path, mol


def ring_bond_plane_input(mol, bond=(1, 2), height=8.0, reach=8.0, npts=60, order=10):
    """gimic.inp text of the bond plane of the C6H6 workload: a Grid(bond)
    Gauss-Lobatto plane (``npts`` x ``npts`` points, composite order
    ``order``) through the midpoint of the C-C bond ``bond`` (1-based atom
    numbers), perpendicular to it, from ``height`` Bohr below to ``height``
    above the ring plane and from the ring centre to ``reach`` Bohr from it
    outward; magnet_axis=z.  The ring centre is the mean of the carbon
    positions; the width keyword is measured from the bond midpoint
    (src/fgimic/grid.f90:165-276), so it starts at minus the centre-midpoint
    distance."""
    c = np.asarray(mol.coords, dtype=np.float64)
    carbons = [i for i, s in enumerate(mol.symbols) if s == "C"]
    centre = c[carbons].mean(axis=0)
    a1, a2 = bond
    mid = 0.5 * (c[a1 - 1] + c[a2 - 1])
    dc = float(np.linalg.norm(mid - centre))
    half = 0.5 * float(np.linalg.norm(c[a2 - 1] - c[a1 - 1]))
    return ("calc=integral\nmagnet_axis=z\nGrid(bond) {\n type=lobatto\n bond=[%d,%d]\n fixcoord=[%r, %r, %r]\n"
            " distance=%r\n height=[%r, %r]\n width=[%r, %r]\n grid_points=[%d, %d, 0]\n gauss_order=%d\n}\n"
            % (a1, a2, float(centre[0]), float(centre[1]), float(centre[2]), half, -float(height), float(height),
               -dc, float(reach) - dc, npts, npts, order))
