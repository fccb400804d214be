"""The drop-in driver (python -m gimic_gb300 gimic.inp) on the reference's
own test inputs, compared the way the reference's runtest filters do: the
10 lines after ' *** Integrating current' of stdout, and whole VTK files."""
import io
import json
import os
import re
import shutil

import numpy as np
import pytest

from conftest import GOLDEN
from gimic_gb300 import driver

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(GOLDEN, "golden.json")))


def _workdir(tmp_path, golden_dir, case, inpname):
    d = tmp_path / case
    d.mkdir()
    for f in ("MOL", "XDENS"):
        os.symlink(golden_dir / case / f, d / f)
    shutil.copy(golden_dir / case / inpname, d / "gimic.inp")
    return d


def _blocks(text):
    nums = []
    for line in text.splitlines():
        if re.search(r"Induced (mod )?current \(au\)|contribution", line):
            nums.append(float(line.split(":")[1].split("(")[0]))
    return nums


@pytest.mark.parametrize("case,key", [("c4h4", "c4h4_integration"), ("open-shell", "openshell_integration")])
@pytest.mark.parametrize("precision", ["fp64", "split16"])
def test_integration_stdout(tmp_path, golden_dir, case, key, precision):
    d = _workdir(tmp_path, golden_dir, case, "integration.inp")
    buf = io.StringIO()
    drv = driver.Driver(str(d / "gimic.inp"), precision=precision, stream=buf)
    drv.run()
    text = buf.getvalue()
    assert "*** Integrating current" in text
    got = _blocks(text)
    # The c4h4 input leaves Essential.jmod at its default (off), so only the
    # current block is printed; the reference's filter compares just the 10
    # lines after ' *** Integrating current' (test/c4h4/integration/test).
    kinds = ("modulus", "current") if drv.kw.get("Essential.jmod") else ("current",)
    want = [v for b in GOLD[key] if b["kind"] in kinds for v in (b["au"], b["pos"], b["neg"])]
    assert len(got) == len(want)
    tol = 5.1e-7 if precision == "fp64" else 2e-6
    assert np.abs(np.array(got) - np.array(want)).max() <= tol


def _vtk_vectors(path, name):
    text = open(path).read()
    m = re.search(r'<DataArray Name="%s"[^>]*>(.*?)</DataArray>' % name, text, re.S)
    return np.array(m.group(1).split(), dtype=np.float64)


def _print_ulp(x):
    """One unit in the last place of Fortran e14.6 output (0.dddddd E+ee)."""
    ax = np.abs(x)
    e = np.floor(np.log10(np.where(ax > 0, ax, 1.0))) + 1.0
    return np.where(ax > 0, 10.0 ** (e - 6), 0.0)


def _agree_printed(got, ref, tol=1e-6):
    """Both sides are e14.6 prints: each element may differ by the path's
    error (tol x the largest value) plus one unit of the print, since the two
    roundings can fall on either side of a digit."""
    bound = tol * np.abs(ref).max() + np.maximum(_print_ulp(got), _print_ulp(ref))
    return bool(np.all(np.abs(got - ref) <= bound))


def test_openshell_3d_cdens_files(tmp_path, golden_dir):
    d = _workdir(tmp_path, golden_dir, "open-shell", "3d.inp")
    drv = driver.Driver(str(d / "gimic.inp"), precision="split16", stream=io.StringIO())
    drv.run()
    ref = np.load(os.path.join(GOLDEN, "openshell_3d.npz"))
    idx = ref["index"]
    for tag, spin in (("", "total"), ("alpha", "alpha"), ("beta", "beta"), ("spindens", "spindens")):
        jv = _vtk_vectors(d / ("jvec%s.vti" % tag), "vectors").reshape(-1, 3)
        assert jv.shape == (33 ** 3, 3)
        assert _agree_printed(jv[idx], ref["jvec_" + spin])
        jm = _vtk_vectors(d / ("jmod%s.vti" % tag), "scalars")
        assert _agree_printed(jm[idx], ref["jmod_" + spin])


def test_readgrid_vtu(tmp_path, golden_dir):
    d = _workdir(tmp_path, golden_dir, "c4h4", "read-grid.inp")
    shutil.copy(golden_dir / "c4h4" / "gridfile.grd", d / "gridfile.grd")
    # a two-cell mesh is enough to exercise the writer
    (d / "grid.1.ele").write_text("2 4 0\n1 1 2 3 4\n2 2 3 4 5\n")
    drv = driver.Driver(str(d / "gimic.inp"), precision="fp64", stream=io.StringIO())
    drv.run()
    jv = _vtk_vectors(d / "jvec.vtu", "vectors").reshape(-1, 3)
    want = np.load(os.path.join(GOLDEN, "c4h4_readgrid.npz"))["jvec"]
    assert np.all(np.abs(jv - want) <= 2e-9 * np.abs(want) + 1e-14 * np.abs(want).max())
