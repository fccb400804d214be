"""ctypes front-end of the FP64 CPU oracle (``og_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` as the checker.  The shipped package
``gimic_gb300`` never imports this module.

The C library restates the reference's FP64 algorithm (caos.f90, bfeval.f90,
basis.f90, intgrl.f90, dens.f90, reorder.f90, jtensor.F90, gaussint.f90,
integral.f90, acid.f90); see the per-function citations in og_oracle.c.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build(force=False):
    """Compile the oracle with its Makefile (gcc, a second or two)."""
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "og_oracle.c"))):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.og_load.restype = C.c_void_p
        L.og_load.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_double, C.c_char_p, C.c_int]
        L.og_load_sph.restype = C.c_void_p
        L.og_load_sph.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_double, C.c_int, C.c_char_p, C.c_int]
        L.og_c2s.argtypes = [C.c_void_p, _dp]
        L.og_c2s.restype = C.c_int
        L.og_free.argtypes = [C.c_void_p]
        for f in ("og_ncgto", "og_nfun", "og_ngto", "og_natoms", "og_is_turbomole", "og_nctr_total"):
            getattr(L, f).argtypes = [C.c_void_p]
            getattr(L, f).restype = C.c_int
        L.og_atom_info.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        L.og_set_flags.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.og_get_dens.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp]
        L.og_get_dens.restype = C.c_int
        L.og_shell_table.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip, _dp, _dp, _dp, C.c_int]
        L.og_basis_eval.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.og_jtensor_batch.argtypes = [C.c_void_p, C.c_char_p, C.c_long, _dp, _dp, _dp, C.c_int]
        L.og_jtensor_batch.restype = C.c_int
        L.og_gauss_data.argtypes = [C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, _dp, _dp]
        L.og_gauss_data.restype = C.c_int
        L.og_acid.argtypes = [_dp]
        L.og_acid.restype = C.c_double
        L.og_au2si.argtypes = [C.c_double]
        L.og_au2si.restype = C.c_double
        L.og_integrate_flat.argtypes = [C.c_void_p, C.c_char_p, _dp, _dp, _ip, _dp, _dp, _dp, _dp, _dp, _dp,
                                        C.c_double, _dp, C.c_int, _dp, C.c_int]
        L.og_integrate_flat.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def au2si(au):
    return lib().og_au2si(float(au))


def gauss_data(a, b, order, npts, quadrature="gauss"):
    """setup_gauss_data (gaussint.f90:267-319): composite nodes on [0, b-a]."""
    pts = np.zeros(npts)
    wgt = np.zeros(npts)
    rc = lib().og_gauss_data(float(a), float(b), int(order), int(npts), 1 if quadrature == "lobatto" else 0,
                             _p(pts), _p(wgt))
    if rc != 0:
        raise RuntimeError("oracle quadrature failed (rc=%d)" % rc)
    return pts, wgt


class Oracle:
    """One molecule + density, evaluated on the CPU in FP64."""

    def __init__(self, mol, xdens=None, uhf=False, screening=1e-8, giao=True, dia=True, para=True,
                 spherical=False):
        L = lib()
        err = C.create_string_buffer(512)
        h = L.og_load_sph(mol.encode(), xdens.encode() if xdens else None, int(bool(uhf)),
                          float(screening) if screening else -1.0, int(bool(spherical)), err, 512)
        if not h:
            raise RuntimeError(err.value.decode())
        self._h = C.c_void_p(h)
        self.uhf = bool(uhf)
        L.og_set_flags(self._h, int(giao), int(dia), int(para))
        self.nbf = L.og_nfun(self._h)        # functions of the densities (spherical or Cartesian)
        self.ncart = L.og_ncgto(self._h)     # Cartesian functions
        self.spherical = bool(spherical)
        self.natoms = L.og_natoms(self._h)
        self.turbomole = bool(L.og_is_turbomole(self._h))

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.og_free(self._h)
            self._h = None

    def atoms(self):
        coords = np.zeros((self.natoms, 3))
        charges = np.zeros(self.natoms)
        for a in range(self.natoms):
            c = np.zeros(3)
            q = C.c_double()
            lib().og_atom_info(self._h, a, _p(c), C.byref(q))
            coords[a] = c
            charges[a] = q.value
        return coords, charges

    def density(self, spin=0, b=0):
        out = np.zeros(self.nbf * self.nbf)
        if lib().og_get_dens(self._h, spin, b, _p(out)) != 0:
            raise ValueError("no such density block")
        return out.reshape(self.nbf, self.nbf, order="F")

    def c2s(self):
        """The Cartesian -> spherical projection (nfun x ncart) of a spherical context."""
        out = np.zeros(self.nbf * self.ncart)
        if lib().og_c2s(self._h, _p(out)) != 0:
            raise ValueError("not a spherical context")
        return out.reshape(self.nbf, self.ncart)

    def shells(self, maxprim=16):
        L = lib()
        ns = L.og_nctr_total(self._h)
        atom, l, npf, pos = (np.zeros(ns, dtype=np.int32) for _ in range(4))
        thrs = np.zeros(ns)
        xp = np.zeros((ns, maxprim))
        ncc = np.zeros((ns, maxprim))
        ip = lambda a: a.ctypes.data_as(_ip)
        L.og_shell_table(self._h, ip(atom), ip(l), ip(npf), ip(pos), _p(thrs), _p(xp), _p(ncc), maxprim)
        return dict(atom=atom, l=l, npf=npf, pos=pos, thrs=thrs, xp=xp, ncc=ncc)

    def basis(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        bf = np.zeros(self.ncart)
        dr = np.zeros(3 * self.ncart)
        lib().og_basis_eval(self._h, _p(r), _p(bf), _p(dr))
        return bf, dr.reshape(3, self.ncart)

    def jtensor(self, points, spin="total", nthreads=0, with_rho=False):
        """ctensor at points (N,3) -> (N,9) column-major tensors (+ rho)."""
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
        n = pts.shape[0]
        jt = np.zeros((n, 9))
        rho = np.zeros(n)
        rc = lib().og_jtensor_batch(self._h, spin.encode(), n, _p(pts), _p(jt), _p(rho), int(nthreads))
        if rc != 0:
            raise ValueError("oracle jtensor failed (rc=%d, spin=%s)" % (rc, spin))
        return (jt, rho) if with_rho else jt

    def integrate(self, origin, basv, axes, radius, bb, what="current", spin="total", nthreads=0):
        """Plane/volume integral over a product grid.

        axes: three (pts, wgt) pairs; basv: 3x3 with basv[:, d] the d-th axis.
        Returns (total, positive, negative) in au (acid: (sqrt(sum), sum, 0)).
        """
        origin = np.ascontiguousarray(origin, dtype=np.float64)
        bv = np.ascontiguousarray(np.asarray(basv, dtype=np.float64).T.reshape(9))
        npts = np.array([len(a[0]) for a in axes], dtype=np.int32)
        ax = [(np.ascontiguousarray(p, dtype=np.float64), np.ascontiguousarray(w, dtype=np.float64))
              for p, w in axes]
        bb = np.ascontiguousarray(bb, dtype=np.float64)
        out = np.zeros(3)
        code = {"current": 0, "modulus": 1, "acid": 2}[what]
        rc = lib().og_integrate_flat(self._h, spin.encode(), _p(origin), _p(bv), npts.ctypes.data_as(_ip),
                                     _p(ax[0][0]), _p(ax[0][1]), _p(ax[1][0]), _p(ax[1][1]), _p(ax[2][0]),
                                     _p(ax[2][1]), float(radius), _p(bb), code, _p(out), int(nthreads))
        if rc != 0:
            raise ValueError("oracle integrate failed (rc=%d)" % rc)
        return out
