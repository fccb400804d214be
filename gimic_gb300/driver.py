"""Drop-in driver for ``gimic gimic.inp`` on the GB300 path.

Replaces the Fortran program's initialize/driver/run_integral/run_cdens
sequence (src/fgimic/gimic.F90:60-261) with the same keyword handling, the
same order of spin cases and the same printed result blocks
(src/fgimic/integral.f90:167-183, :306-322, :502-510), evaluating every
current tensor through libgimic_gb300.
"""
import argparse
import os
import sys

import numpy as np

from . import api, inp, properties, vtk
from . import grid as ggrid

AU2A = 0.52917726


def _out(stream, s=""):
    stream.write(" " + s + "\n" if s else "\n")


def _print_integral(stream, kind, res):
    xs, ps, ns = res
    au2si = api.au2si
    _out(stream)
    _out(stream, "*" * 60)
    if kind == "modulus":
        _out(stream, "Induced mod current (au)   :%13.6f" % xs)
    else:
        _out(stream, "   Induced current (au)    :%13.6f" % xs)
    _out(stream, "      Positive contribution:%13.6f  (%11.6f )" % (ps, au2si(ps)))
    _out(stream, "      Negative contribution:%13.6f  (%11.6f )" % (ns, au2si(ns)))
    _out(stream)
    if kind == "modulus":
        _out(stream, "Induced mod current (nA/T) :%13.6f" % au2si(xs))
    else:
        _out(stream, "   Induced current (nA/T)  :%13.6f" % au2si(xs))
    _out(stream, "      (conversion factor)  :%13.6f" % au2si(1.0))
    _out(stream, "*" * 60)
    _out(stream)


def _spin_note(stream, uhf, spin):
    if uhf:
        name = {"spindens": "spin"}.get(spin, spin)
        _out(stream, "*** Integrating %s density" % name)


class Driver:
    def __init__(self, inp_path, precision="split16", stream=None, workdir=None):
        self.stream = stream or sys.stdout
        self.workdir = workdir or os.path.dirname(os.path.abspath(inp_path))
        self.kw = inp.read(inp_path)
        kw = self.kw
        if not kw.get("Advanced.diamag") and not kw.get("Advanced.paramag"):
            raise inp.InputError("PLEASE SEEK PROFESSIONAL HELP, ASAP!  (diamag and paramag both off)")
        self.uhf = bool(kw.get("openshell"))
        path = lambda k: os.path.join(self.workdir, kw.get(k))
        thr = kw.get("Advanced.screening_thrs") if kw.get("Advanced.screening") else -1.0
        self.g = api.Gimic(path("basis"), path("xdens"), uhf=self.uhf, screening=thr, precision=precision,
                           spherical=bool(kw.get("Advanced.spherical")))
        self.g.set_flags(kw.get("Advanced.GIAO"), kw.get("Advanced.diamag"), kw.get("Advanced.paramag"))
        self.atoms = self.g.atoms()[0]
        self.grid = ggrid.new_grid(kw, self.atoms, workdir=self.workdir)
        self.magnet, self.flipped = ggrid.get_magnet(self.grid, kw)
        self.g.set_magnet(self.magnet)

    def run(self):
        calc = self.kw.get("calc")
        for w in getattr(self.grid, "warnings", []):
            self.stream.write(" WARNING: %s\n" % w)
        if self.kw.get("dryrun"):
            _out(self.stream, "Dry run, not calculating ...")
            return {}
        if calc == "integral":
            return self.run_integral()
        if calc == "cdens":
            return self.run_cdens()
        raise inp.InputError("gimic(): Unknown operation!")

    def _spins(self):
        return ["total", "alpha", "beta", "spindens"] if self.uhf else ["total"]

    def run_integral(self):
        s = self.stream
        grd = self.grid
        _out(s, "Integrating current density")
        _out(s, "*" * 41)
        results = {"modulus": {}, "current": {}, "acid": None}
        cache = {}
        for spin in self._spins():
            self.g.set_spin(spin)
            cache[spin] = self.g.plane_integral(grd.origin, grd.basv, grd.axes(), grd.radius)
        if self.kw.get("Essential.jmod"):
            _out(s, "*** Integrating |J|")
            for spin in self._spins():
                _spin_note(s, self.uhf, spin)
                results["modulus"][spin] = cache[spin]["modulus"]
                _print_integral(s, "modulus", cache[spin]["modulus"])
        else:
            s.write(" Jmod integration skipped.\n")
        _out(s, "*** Integrating current")
        for spin in self._spins():
            _spin_note(s, self.uhf, spin)
            results["current"][spin] = cache[spin]["current"]
            _print_integral(s, "current", cache[spin]["current"])
        if self.kw.get("Essential.acid"):
            # integrate_acid uses the module's spin, 'total' after the loops above
            acid = cache["total"]["acid"]
            results["acid"] = acid
            _out(s, "*** Integrating ACID density")
            _out(s)
            _out(s, "*" * 60)
            _out(s, "  ACID (au) sqrt(delta J^2):%13.6f" % acid)
            _out(s, "  ACID (nA/T)              :%13.6f" % api.au2si(acid))
            _out(s)
            _out(s, "*" * 60)
            _out(s)
        return results

    def run_cdens(self):
        """calc_jvectors + jvector_plots (src/fgimic/jfield.f90:140-433)."""
        grd = self.grid
        pts = grd.points()
        out = {}
        for spin in self._spins():
            tag = "" if spin == "total" else spin
            self.g.set_spin(spin)
            jt = self.g.jtensor_batch(pts)
            t = jt.reshape(-1, 3, 3).transpose(0, 2, 1)
            jv = t @ self.magnet
            out[spin] = {"jt": jt, "jvec": jv}
            self._write_fields(tag, pts, jt, jv)
            if self.kw.get("Essential.prop"):
                # get_property (jfield.f90:404-405): shielding and magnetizability
                # over the molecular grid of gridfile.grd / grid_w.grd
                out[spin]["properties"] = properties.run(self.g, self.stream, self.workdir, grid_points=pts,
                                                         grid_jt=jt)
        return out

    def _write_fields(self, tag, pts, jt, jv):
        grd, kw, wd = self.grid, self.kw, self.workdir
        if grd.gtype == "file":
            ele = os.path.join(wd, "grid.1.ele")
            if os.path.exists(ele):
                vtk.write_vector_unstructured(os.path.join(wd, "jvec.vtu"), pts, jv, vtk.read_tetgen_ele(ele))
            return
        if grd.gauss:
            vtk.write_jmod_txt(os.path.join(wd, "jmod%s.txt" % tag), pts * AU2A, jv, grd.npts)
        if grd.is_3d() and kw.get("Essential.acid"):
            t = jt
            acid = (0.3333333 * ((t[:, 0] - t[:, 4]) ** 2 + (t[:, 4] - t[:, 8]) ** 2 + (t[:, 8] - t[:, 0]) ** 2)
                    + 0.5 * ((t[:, 3] + t[:, 1]) ** 2 + (t[:, 6] + t[:, 2]) ** 2 + (t[:, 7] + t[:, 5]) ** 2))
            vtk.write_imagedata(os.path.join(wd, "acid.vti"), grd, acid)
        if grd.is_3d() and kw.get("Essential.jmod"):
            mag = self.magnet
            val = np.sqrt(np.sum(jv ** 2, axis=1))
            coord = pts - (pts @ mag)[:, None] * mag
            sgn = np.sum(np.cross(mag, coord) * jv, axis=1)
            vtk.write_imagedata(os.path.join(wd, "jmod%s.vti" % tag), grd, np.where(sgn < 0.0, -val, val))
        if grd.gtype == "even":
            vtk.write_vector_imagedata(os.path.join(wd, "jvec%s.vti" % tag), grd, jv)


def main(argv=None):
    ap = argparse.ArgumentParser(description="GIMIC current densities on GB300")
    ap.add_argument("infile", nargs="?", default="gimic.inp")
    ap.add_argument("--precision", default="split16", choices=("split16", "fp64"))
    ap.add_argument("-y", "--dryrun", action="store_true")
    a = ap.parse_args(argv)
    try:
        d = Driver(a.infile, precision=a.precision)
        if a.dryrun:
            d.kw._val["dryrun"] = [True]
        d.run()
    except (inp.InputError, ValueError) as e:
        sys.stderr.write("%s\n" % e)
        return 1
    return 0
