"""Extract golden fixtures from the reference's regression tests.

Run in a checkout that has the reference tree (default /root/reference):

    python tests/golden/make_golden.py [REFERENCE_ROOT]

It copies the inputs of the four reference tests whose densities are present
(test/c4h4/{integration,read-grid}, test/open-shell/{integration,3d}: MOL,
XDENS compressed with xz, the grid file, the gimic.inp files) and turns their
committed outputs into numbers:

  golden.json            integration blocks of reference/stdout
                         (integral.f90:167-183, :306-322 print format)
  c4h4_readgrid.npz      jvec.vtu point data (4110 points, 3e20.10)
  openshell_3d.npz       every 17th point of jvec*.vti / jmod*.vti (e14.6)
"""
import json
import lzma
import os
import re
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _num(s):
    return float(s.replace("D", "E"))


def parse_stdout(path):
    """Sequence of (kind, spin, au, pos, neg, nAT) integration blocks."""
    out = []
    spin = "total"
    kind = None
    lines = open(path).read().splitlines()
    for i, line in enumerate(lines):
        m = re.search(r"Integrating (total|alpha|beta|spin) density", line)
        if m:
            spin = {"spin": "spindens"}.get(m.group(1), m.group(1))
        if "Induced mod current (au)" in line:
            kind = "modulus"
        elif "Induced current (au)" in line:
            kind = "current"
        else:
            continue
        au = _num(line.split(":")[1])
        pos = _num(lines[i + 1].split(":")[1].split("(")[0])
        neg = _num(lines[i + 2].split(":")[1].split("(")[0])
        nat = _num(lines[i + 4].split(":")[1])
        out.append({"kind": kind, "spin": spin, "au": au, "pos": pos, "neg": neg, "nAT": nat})
    return out


def vtk_arrays(path):
    text = open(path).read()
    arrays = {}
    for m in re.finditer(r"<DataArray([^>]*)>(.*?)</DataArray>", text, re.S):
        attrs, body = m.group(1), m.group(2)
        name = re.search(r'Name="([^"]+)"', attrs)
        name = name.group(1) if name else "points"
        arrays.setdefault(name, np.array(body.split(), dtype=np.float64))
    return arrays


def xz_copy(src, dst):
    with open(src, "rb") as f, lzma.open(dst, "wb", preset=9) as g:
        shutil.copyfileobj(f, g)


def main(ref):
    t = os.path.join(ref, "test")
    gold = {}
    for case in ("c4h4", "open-shell"):
        d = os.path.join(HERE, case)
        os.makedirs(d, exist_ok=True)
        shutil.copy(os.path.join(t, case, "MOL"), os.path.join(d, "MOL"))
        xz_copy(os.path.join(t, case, "XDENS"), os.path.join(d, "XDENS.xz"))
    shutil.copy(os.path.join(t, "c4h4/integration/gimic.inp"), os.path.join(HERE, "c4h4", "integration.inp"))
    shutil.copy(os.path.join(t, "c4h4/read-grid/gimic.inp"), os.path.join(HERE, "c4h4", "read-grid.inp"))
    xz_copy(os.path.join(t, "c4h4/read-grid/gridfile.grd"), os.path.join(HERE, "c4h4", "gridfile.grd.xz"))
    shutil.copy(os.path.join(t, "open-shell/integration/gimic.inp"), os.path.join(HERE, "open-shell", "integration.inp"))
    shutil.copy(os.path.join(t, "open-shell/3d/gimic.inp"), os.path.join(HERE, "open-shell", "3d.inp"))

    gold["c4h4_integration"] = parse_stdout(os.path.join(t, "c4h4/integration/reference/stdout"))
    gold["openshell_integration"] = parse_stdout(os.path.join(t, "open-shell/integration/reference/stdout"))
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(gold, f, indent=1)

    a = vtk_arrays(os.path.join(t, "c4h4/read-grid/reference/jvec.vtu"))
    np.savez_compressed(os.path.join(HERE, "c4h4_readgrid.npz"), jvec=a["vectors"].reshape(-1, 3),
                        points=a["points"].reshape(-1, 3))

    sub = {}
    idx = None
    for tag in ("", "alpha", "beta", "spindens"):
        v = vtk_arrays(os.path.join(t, "open-shell/3d/reference/jvec%s.vti" % tag))["vectors"].reshape(-1, 3)
        mval = vtk_arrays(os.path.join(t, "open-shell/3d/reference/jmod%s.vti" % tag))["scalars"]
        if idx is None:
            idx = np.arange(0, v.shape[0], 17)
        sub["jvec_" + (tag or "total")] = v[idx]
        sub["jmod_" + (tag or "total")] = mval[idx]
    np.savez_compressed(os.path.join(HERE, "openshell_3d.npz"), index=idx, **sub)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
