"""Field output files in the formats of src/fgimic/vtkplot.f90 and
src/fgimic/jfield.f90 (jvec*.vti, jmod*.vti, acid.vti, jvec.vtu, jmod*.txt).

Numbers use the reference's edit descriptors (e14.6, 3e14.6, 3e20.10,
6f11.7); list-directed header fields follow gfortran's layout.
"""
import math

import numpy as np


def fortran_e(x, w, d):
    """Fortran Ew.d: 0.ddddddE+xx right-justified in w columns."""
    x = float(x)
    if x == 0.0 or not math.isfinite(x):
        body = "0." + "0" * d + "E+00" if x == 0.0 else str(x)
        return body.rjust(w)
    m, e = "%.*e" % (d - 1, abs(x)), 0
    mant, exp = m.split("e")
    digits = mant.replace(".", "")
    e = int(exp) + 1
    s = "%s0.%sE%s%02d" % ("-" if x < 0 else "", digits, "+" if e >= 0 else "-", abs(e))
    if abs(e) > 99:
        s = "%s0.%s%s%03d" % ("-" if x < 0 else "", digits, "+" if e >= 0 else "-", abs(e))
    return s.rjust(w)


def _ld_int(i):
    return "%12d" % i


def _ld_real(x):
    """gfortran list-directed real(8): 17 significant digits, F form for
    0.1 <= |x| < 1e16, in a 26-column field."""
    ax = abs(x)
    if ax == 0.0:
        t = "0.0000000000000000"
    elif 0.1 <= ax < 1e16:
        ndig = int(math.floor(math.log10(ax))) + 1
        t = "%.*f" % (max(17 - max(ndig, 0), 1), x)
    else:
        t = "%.16E" % x
    return ("  " + t).ljust(26)


def _header(npts, qmin, step):
    ext = "".join(_ld_int(v) for p in npts for v in (0, p - 1))
    org = "".join(_ld_real(v) for v in qmin)
    spc = "".join(_ld_real(v) for v in step)
    return (' <VTKFile type="ImageData" version="0.1" byte_order="LittleEndian">\n'
            '   <ImageData WholeExtent="%s " Origin="%s" Spacing="%s">\n'
            '   <Piece Extent="%s ">\n' % (ext, org, spc, ext))


def _extent(grid):
    npts = grid.npts
    qmin = grid.gridpoint(0, 0, 0)
    qmax = grid.gridpoint(npts[0] - 1, npts[1] - 1, npts[2] - 1)
    step = qmax - qmin
    step = np.where(step > 1e-8, step / np.maximum(np.array(npts) - 1, 1), step)
    return npts, qmin, step


def write_imagedata(path, grid, values):
    """write_vtk_imagedata (vtkplot.f90:14-86): scalars, e14.6, a line break
    after the first value and then every four."""
    npts, qmin, step = _extent(grid)
    v = np.asarray(values, dtype=np.float64).reshape(-1)
    out = ['<?xml version="1.0"?>\n', _header(npts, qmin, step),
           '   <PointData Scalars="scalars">\n',
           '   <DataArray Name="scalars" type="Float64" NumberOfComponents="1" Format="ascii">\n']
    line = []
    for l, x in enumerate(v):
        line.append(fortran_e(x, 14, 6))
        if l % 4 == 0:
            out.append("".join(line) + "\n")
            line = []
    out.append("".join(line) + "\n")
    out.append("    </DataArray>\n    </PointData>\n    </Piece>\n    </ImageData>\n </VTKFile>\n")
    with open(path, "w") as f:
        f.writelines(out)


def write_vector_imagedata(path, grid, vec):
    """write_vtk_vector_imagedata (vtkplot.f90:88-234): 3e14.6 per point and
    the norm of the 8- (or 4-) point average as cell data."""
    npts, qmin, step = _extent(grid)
    v = np.asarray(vec, dtype=np.float64).reshape(npts[2], npts[1], npts[0], 3)
    out = ['<?xml version="1.0"?>\n', _header(npts, qmin, step),
           '   <PointData Scalars="scalars">\n',
           '   <DataArray Name="vectors" type="Float64" NumberOfComponents="3" Format="ascii">\n']
    for row in v.reshape(-1, 3):
        out.append("".join(fortran_e(x, 14, 6) for x in row) + "\n")
    out.append("\n    </DataArray>\n    </PointData>\n    <CellData Scalars=\"foo\">\n")
    n1, n2, n3 = npts
    if n1 > 1 and n2 > 1 and n3 > 1:
        avg = (v[:-1, :-1, :-1] + v[:-1, :-1, 1:] + v[:-1, 1:, :-1] + v[1:, :-1, :-1] + v[:-1, 1:, 1:]
               + v[1:, :-1, 1:] + v[1:, 1:, :-1] + v[1:, 1:, 1:]) / 8.0
    elif n1 > 1 and n2 > 1 and n3 == 1:
        w = v[0]
        avg = (w[:-1, :-1] + w[:-1, 1:] + w[1:, :-1] + w[1:, 1:]) / 4.0
    elif n1 > 1 and n2 == 1 and n3 > 1:
        w = v[:, 0]
        avg = (w[:-1, :-1] + w[:-1, 1:] + w[1:, :-1] + w[1:, 1:]) / 4.0
    elif n1 == 1 and n2 > 1 and n3 > 1:
        w = v[:, :, 0]
        avg = (w[:-1, :-1] + w[:-1, 1:] + w[1:, :-1] + w[1:, 1:]) / 4.0
    else:
        avg = np.zeros((0, 3))
    for x in np.sqrt(np.sum(np.asarray(avg).reshape(-1, 3) ** 2, axis=1)):
        out.append(fortran_e(x, 14, 6) + "\n")
    out.append("    </CellData>\n    </Piece>\n    </ImageData>\n </VTKFile>\n")
    with open(path, "w") as f:
        f.writelines(out)


def write_vector_unstructured(path, points, vec, cells):
    """write_vtk_vector_unstructuredgrid (vtkplot.f90:241-316): tetrahedra
    (VTK type 10) with 0-based connectivity, vectors in 3e20.10."""
    pts = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    v = np.asarray(vec, dtype=np.float64).reshape(-1, 3)
    cells = np.asarray(cells, dtype=np.int64).reshape(-1, 4)
    out = ['<?xml version="1.0"?>\n',
           '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian">\n',
           '  <UnstructuredGrid>\n',
           '    <Piece NumberOfPoints="%10d" NumberOfCells="%10d">\n' % (len(pts), len(cells)),
           '      <Points>\n',
           '        <DataArray type="Float32" NumberOfComponents="3" Format="ascii">\n']
    for p in pts:
        out.append("        " + "".join(fortran_e(x, 20, 10) for x in p) + "\n")
    out.append("        </DataArray>\n      </Points>\n      <PointData Scalars=\"scalars\">\n"
               '        <DataArray Name="vectors" type="Float64" NumberOfComponents="3" Format="ascii">\n')
    for p in v:
        out.append("        " + "".join(fortran_e(x, 20, 10) for x in p) + "\n")
    out.append("        </DataArray>\n      </PointData>\n      <Cells>\n"
               '        <DataArray type="Int32" Name="connectivity" Format="ascii">\n')
    for c in cells:
        out.append("        " + "".join("%10d" % (x - 1) for x in c) + "\n")
    out.append("        </DataArray>\n        <DataArray type=\"Int32\" Name=\"offsets\" Format=\"ascii\">\n")
    out.append("        " + " ".join(str(4 * (i + 1)) for i in range(len(cells))) + "\n")
    out.append("        </DataArray>\n        <DataArray type=\"Int32\" Name=\"types\" Format=\"ascii\">\n")
    out.append("        " + " ".join("10" for _ in range(len(cells))) + "\n")
    out.append("        </DataArray>\n      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n")
    with open(path, "w") as f:
        f.writelines(out)


def write_scalar_unstructured(path, points, values, cells):
    """write_vtk_scalar_unstructuredgrid (vtkplot.f90:318-390): tetrahedra
    (VTK type 10) with 0-based connectivity, points in 3e20.10, one scalar
    per point in e20.10, offsets in i10, types in i5 and an all-zero cell
    array in f4.1, laid out as the reference writes them."""
    pts = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    v = np.asarray(values, dtype=np.float64).reshape(-1)
    cells = np.asarray(cells, dtype=np.int64).reshape(-1, 4)
    nc = len(cells)
    out = ['<?xml version="1.0"?>\n',
           '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian">\n',
           '  <UnstructuredGrid>\n',
           '    <Piece NumberOfPoints="%10d" NumberOfCells="%10d">\n' % (len(pts), nc),
           '      <Points>\n',
           '        <DataArray type="Float32" NumberOfComponents="3" Format="ascii">\n']
    for p in pts:
        out.append("        " + "".join(fortran_e(x, 20, 10) for x in p) + "\n")
    out.append('        </DataArray>\n      </Points>\n      <PointData Scalars="scalars">\n'
               '        <DataArray Name="scalars" type="Float64" NumberOfComponents="1" Format="ascii">\n')
    for x in v:
        out.append("        " + fortran_e(x, 20, 10) + "\n")
    out.append('        </DataArray>\n      </PointData>\n      <Cells>\n'
               '        <DataArray type="Int32" Name="connectivity" Format="ascii">\n')
    for c in cells:
        out.append("        " + "".join("%10d" % (x - 1) for x in c) + "\n")
    out.append('        </DataArray>\n        <DataArray type="Int32" Name="offsets" Format="ascii">\n')
    out.append("        " + "".join("%10d" % (4 * (i + 1)) for i in range(nc)) + "\n")
    out.append('        </DataArray>\n        <DataArray type="Int32" Name="types" Format="ascii">\n')
    out.append("        " + "%5d" % 10 * nc + "\n")
    out.append('        </DataArray>\n      </Cells>\n      <CellData Scalars="foo">\n')
    out.append("        " + " 0.0" * nc + "\n")
    out.append("      </CellData>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n")
    with open(path, "w") as f:
        f.writelines(out)


def read_tetgen_ele(path):
    """grid.1.ele as read in jfield.f90:421-433: count on the first line, then
    'index n1 n2 n3 n4' per cell (1-based)."""
    lines = open(path).read().split("\n")
    ncells = int(lines[0].split()[0])
    cells = np.array([[int(t) for t in lines[1 + i].split()[1:5]] for i in range(ncells)], dtype=np.int64)
    return cells


def write_jmod_txt(path, points_angstrom, vec, npts):
    """jmod*.txt of gauss-type grids (jfield.f90:293-301, write_jmod): 6f11.7
    rows of coordinate (Angstrom) and |j|, a blank line after each row of i."""
    p = np.asarray(points_angstrom).reshape(-1, 3)
    m = np.sqrt(np.sum(np.asarray(vec).reshape(-1, 3) ** 2, axis=1))
    out = []
    for idx in range(len(p)):
        out.append("".join("%11.7f" % x for x in p[idx]) + "%11.7f" % m[idx] + "\n")
        if (idx + 1) % npts[0] == 0:
            out.append("\n")
    with open(path, "w") as f:
        f.writelines(out)
