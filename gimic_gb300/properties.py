"""Nuclear shielding and magnetizability from the current density on a
molecular grid: the `Essential.prop` step of calc=cdens
(src/fgimic/jfield.f90:584-929, get_property).

The grid is read from the files the reference reads: gridfile.grd (points,
Bohr), grid_w.grd (weights), coord.au (nuclei, Bohr) and nelpts.info (per
nucleus the number of grid points it generated, for the atom
decomposition).  The quadratures run on the GPU (gg_properties); this module
reads the files, prints the reference's result blocks and writes the
per-point VTU files when grid.1.ele is present.
"""
import os

import numpy as np

FAC_AU2SIMAG = 7.89104e-29  # J/T^2 per au of magnetizability
C_AU = 137.0359998


def _read_rows(path, ncol):
    rows = []
    with open(path) as f:
        for line in f:
            v = line.replace("D", "E").replace("d", "e").split()
            if v:
                rows.append([float(x) for x in v[:ncol]])
    return np.asarray(rows, dtype=np.float64).reshape(-1, ncol)


def read_inputs(workdir="."):
    """(coord, points, weights, block_npts) or None when a file is missing
    (the reference then skips the property calculation)."""
    need = [os.path.join(workdir, f) for f in ("coord.au", "gridfile.grd", "grid_w.grd")]
    if not all(os.path.exists(f) for f in need):
        return None
    coord = _read_rows(need[0], 3)
    pts = _read_rows(need[1], 3)
    w = _read_rows(need[2], 1)[:, 0]
    if len(w) != len(pts):
        raise ValueError("gridfile.grd and grid_w.grd have different lengths")
    nel = os.path.join(workdir, "nelpts.info")
    blocks = _read_rows(nel, 2)[:, 1].astype(np.int64) if os.path.exists(nel) else None
    return coord, pts, w, blocks


def per_point(jt, pts, coord):
    """Per-point values of the reference's VTU files: for every centre the
    three shielding integrands (ppm) and their sum, and the three
    magnetizability integrands and their sum (numpy, host side)."""
    t = np.asarray(jt).reshape(-1, 9)

    def cross_diag(d):
        return np.stack([-(d[:, 1] * t[:, 2] - d[:, 2] * t[:, 1]), -(d[:, 2] * t[:, 3] - d[:, 0] * t[:, 5]),
                         -(d[:, 0] * t[:, 7] - d[:, 1] * t[:, 6])], axis=1)

    sig = []
    for R in coord:
        d = pts - R
        r2 = np.sum(d * d, axis=1)
        f = -1.0 / (r2 * np.sqrt(r2)) / (C_AU * C_AU)
        sig.append(1.0e6 * f[:, None] * cross_diag(d))
    return np.asarray(sig), 0.5 * cross_diag(pts)


def report(stream, sigma, chi):
    """The reference's printed blocks (jfield.f90:700-928)."""
    def out(s=""):
        stream.write(s + "\n")

    def contrib(blocks):
        out(" atom contributions, total, positive, negative")
        csum = np.zeros(3)
        for l, b in enumerate(blocks):
            v = np.array([b[0] + b[1] + b[2], b[3], b[4]]) / 3.0
            out("atom %5d%14.6f%14.6f%14.6f" % (l + 1, v[0], v[1], v[2]))
            csum += v
        out("sum       %14.6f%14.6f%14.6f" % (csum[0], csum[1], csum[2]))

    for k, blocks in enumerate(sigma):
        tot = blocks.sum(axis=0)
        out(" atom %d" % (k + 1))
        out(" in ppm")
        for name, v in zip(("sigma_xx ", "sigma_yy ", "sigma_zz "), tot[:3]):
            out(" %-10s  %14.6f" % (name, v))
        iso = tot[:3].sum() / 3.0
        out("%30s  %14.6f" % ("shielding constant    = ", iso))
        out("%30s  %14.6f" % ("positive contribution = ", tot[3] / 3.0))
        out("%30s  %14.6f" % ("negative contribution = ", tot[4] / 3.0))
        out("%30s  %14.6f" % ("sum = ", (tot[3] + tot[4]) / 3.0))
        out("  ")
        contrib(blocks)
        out(" " + "*" * 52)
    out("")
    tot = chi.sum(axis=0)
    out("")
    for name, v in zip(("chi_xx ", "chi_yy ", "chi_zz "), tot[:3]):
        out(" %-7s  %14.8f" % (name, v))
    iso = tot[:3].sum() / 3.0
    out(" in au")
    out(" %30s  %14.6f" % ("isotropic magnetizability chi = ", iso))
    out(" %30s  %14.6f" % ("positive contribution         = ", tot[3] / 3.0))
    out(" %30s  %14.6f" % ("negative contribution         = ", tot[4] / 3.0))
    out(" %30s  %14.6f" % ("sum ", (tot[3] + tot[4]) / 3.0))
    out("")
    out(" in SI units J/T^2 ")
    out(" conversion factor: 7.89104*10^-29 J/T^2 ")
    out("")
    out("%30s  %14.6E" % ("isotropic magnetizability = ", iso * FAC_AU2SIMAG))
    out("%30s  %14.6E" % ("positive contribution     = ", tot[3] / 3.0 * FAC_AU2SIMAG))
    out("%30s  %14.6E" % ("negative contribution     = ", tot[4] / 3.0 * FAC_AU2SIMAG))
    out("%30s  %14.6E" % ("sum ", (tot[3] + tot[4]) / 3.0 * FAC_AU2SIMAG))
    out(" " + "*" * 52)
    out("")
    contrib(chi)


def integrand_file_name(kind, k=None):
    """File names of jfield.f90:785-806 and :905-910: sigma<k>.vtu,
    sigma_xx<k>.vtu, ... per nucleus k (1-based) and intchi*.vtu.  The
    reference formats k with I1 or I2, so from nucleus 100 on all its files
    share one name made of asterisks; here k is written in full instead."""
    return ("%s%d.vtu" % (kind, k)) if k is not None else ("%s.vtu" % kind)


def write_integrand_files(workdir, pts, jt, coord, cells):
    """The per-point VTU files of get_property (written only when
    grid.1.ele is present): for every nucleus the summed shielding
    integrand and its three diagonal parts, then the same for the
    magnetizability.  jt: (N, 9) tensors at pts (N, 3); returns the names."""
    from . import vtk

    sig, chi = per_point(jt, pts, coord)
    names = []
    for k, s3 in enumerate(sig, start=1):
        for kind, vals in (("sigma", s3.sum(axis=1)), ("sigma_xx", s3[:, 0]), ("sigma_yy", s3[:, 1]),
                           ("sigma_zz", s3[:, 2])):
            name = integrand_file_name(kind, k)
            vtk.write_scalar_unstructured(os.path.join(workdir, name), pts, vals, cells)
            names.append(name)
    for kind, vals in (("intchi", chi.sum(axis=1)), ("intchi_xx", chi[:, 0]), ("intchi_yy", chi[:, 1]),
                       ("intchi_zz", chi[:, 2])):
        name = integrand_file_name(kind)
        vtk.write_scalar_unstructured(os.path.join(workdir, name), pts, vals, cells)
        names.append(name)
    return names


def run(gimic, stream, workdir=".", grid_points=None, grid_jt=None):
    """Read the grid files, evaluate, print and, with grid.1.ele present,
    write the per-point integrand files; returns (sigma, chi) or None.
    grid_points / grid_jt: tensors the caller already has (calc=cdens on
    the same file grid), reused for the files when the points agree."""
    inputs = read_inputs(workdir)
    if inputs is None:
        stream.write(" at least one of the files coord.au, gridfile.grd, and grid_w.grd is missing. Therefore any "
                     "property calculation is skipped.\n")
        return None
    coord, pts, w, blocks = inputs
    sigma, chi = gimic.properties(pts, w, coord, blocks)
    report(stream, sigma, chi)
    ele = os.path.join(workdir, "grid.1.ele")
    if os.path.exists(ele):
        from . import vtk

        if grid_jt is not None and grid_points is not None and np.array_equal(np.asarray(grid_points), pts):
            jt = np.asarray(grid_jt)
        else:
            jt = gimic.jtensor_batch(pts)
        write_integrand_files(workdir, pts, jt, coord, vtk.read_tetgen_ele(ele))
    return sigma, chi
