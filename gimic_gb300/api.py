"""Python host interface of the GB300 GIMIC path.

``Gimic`` mirrors the reference's Cython class (src/libgimic/gimic.pyx:6-57,
a ``GimicConnector``, src/pygimic/connector.pxd:6-9): ``jvector(r)``,
``jtensor(r)`` and ``set_property(name, value)`` for one point, plus batched
evaluation on numpy arrays or CUDA torch tensors and plane integrals.  All
evaluation runs in libgimic_gb300.so on the GPU.
"""
import ctypes as C
import math
import struct

import numpy as np

from . import _lib
from ._lib import GG_PREC_FP64, GG_PREC_SPLIT16, check

# gg_grid as a numpy record (same offsets as _lib.GridSpec; checked below)
_GRID_DTYPE = np.dtype({"names": ["origin", "basv", "npts", "pts", "wgt", "radius"],
                        "formats": [(np.float64, 3), (np.float64, 9), (np.int32, 3), (np.uint64, 3), (np.uint64, 3),
                                    np.float64],
                        "offsets": [_lib.GridSpec.origin.offset, _lib.GridSpec.basv.offset, _lib.GridSpec.npts.offset,
                                    _lib.GridSpec.pts.offset, _lib.GridSpec.wgt.offset, _lib.GridSpec.radius.offset],
                        "itemsize": C.sizeof(_lib.GridSpec)})
# the same record as one struct format (native byte order), padding included
_GRID_PACK = struct.Struct("=3d9d3i%dx3Q3Q%dxd%dx" % (
    _lib.GridSpec.pts.offset - (_lib.GridSpec.npts.offset + 12),
    _lib.GridSpec.radius.offset - (_lib.GridSpec.wgt.offset + 24),
    C.sizeof(_lib.GridSpec) - (_lib.GridSpec.radius.offset + 8)))
assert _GRID_PACK.size == C.sizeof(_lib.GridSpec) and _lib.GridSpec.basv.offset == 24 and _lib.GridSpec.npts.offset == 96

try:  # torch is optional: used only to accept device tensors
    import torch
except Exception:  # pragma: no cover
    torch = None

SPINS = ("total", "alpha", "beta", "spindens")
PRECISIONS = {"fp64": GG_PREC_FP64, "split16": GG_PREC_SPLIT16}


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _is_cuda(t):
    return torch is not None and isinstance(t, torch.Tensor) and t.is_cuda


def au2si(au):
    """Current in atomic units -> nA/T (src/libgimic/globals.f90 au2si)."""
    return _lib.load().gg_au2si(float(au))


def gauss_data(a, b, order, npts, quadrature="gauss"):
    """Composite Gauss(-Lobatto) nodes and weights on [0, b - a]
    (src/libgimic/gaussint.f90:267-319)."""
    pts = np.zeros(int(npts))
    wgt = np.zeros(int(npts))
    rc = _lib.load().gg_gauss_data(float(a), float(b), int(order), int(npts),
                                   1 if quadrature == "lobatto" else 0, _dptr(pts), _dptr(wgt))
    if rc != 0:
        raise ValueError("quadrature: npts=%d is not a multiple of order=%d (or Newton failed)" % (npts, order))
    return pts, wgt


class Gimic:
    """One molecule with its (perturbed) densities on the current CUDA device.

    Defaults follow gimic_init (src/libgimic/gimic_interface.f90:26-70):
    closed shell, screening 1e-6, GIAO/diamagnetic/paramagnetic terms on,
    magnetic field zero until set.
    """

    def __init__(self, mol, xdens, uhf=False, screening=1e-6, precision="split16", spherical=False):
        """``spherical``: the XDENS densities are over spherical functions
        (the gimic.inp keyword Advanced.spherical); the basis values are
        their projections from the Cartesian functions."""
        L = _lib.load()
        h = C.c_void_p()
        rc = L.gg_ctx_create_ex(str(mol).encode(), str(xdens).encode(), int(bool(uhf)),
                                float(screening) if screening else -1.0, int(bool(spherical)), C.byref(h))
        check(rc, None)
        self._h = h
        self._L = L
        self.uhf = bool(uhf)
        self.spherical = bool(spherical)
        nbf, nat, nsh, tm = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        L.gg_basis_info(h, C.byref(nbf), C.byref(nat), C.byref(nsh), C.byref(tm))
        self.nbf, self.natoms, self.nshells, self.turbomole = nbf.value, nat.value, nsh.value, bool(tm.value)
        self.set_precision(precision)

    def close(self):
        if getattr(self, "_h", None):
            self._L.gg_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- settings -------------------------------------------------------
    def set_precision(self, mode):
        check(self._L.gg_set_precision(self._h, PRECISIONS[mode] if isinstance(mode, str) else int(mode)), self._h)

    def set_flags(self, giao=True, diamag=True, paramag=True):
        check(self._L.gg_set_flags(self._h, int(giao), int(diamag), int(paramag)), self._h)

    def set_tile_screening(self, on=True):
        check(self._L.gg_set_tile_screening(self._h, int(bool(on))), self._h)

    def set_cross_skip(self, on=True):
        """Issue only the main product of the split for K blocks that are
        small for a whole tile (on by default; gg_set_cross_skip).  Off:
        results are bit-identical across batch splits."""
        check(self._L.gg_set_cross_skip(self._h, int(bool(on))), self._h)

    def set_shell_order(self, mode="locality"):
        """'locality' (default): shells grouped by screening radius along a
        tour of the atoms, which lets tile screening skip more work; 'file':
        the MOL file's order.  Results agree up to rounding."""
        code = {"file": 0, "locality": 1}[mode] if isinstance(mode, str) else int(mode)
        check(self._L.gg_set_shell_order(self._h, code), self._h)

    def shell_order(self):
        """(mode, order): order[k] is the file index of the shell at position k."""
        nshells = self.nshells
        mode = C.c_int()
        order = (C.c_int * max(1, nshells))()
        check(self._L.gg_get_shell_order(self._h, C.byref(mode), order), self._h)
        return ("file", "locality")[mode.value], list(order[:nshells])

    def set_max_batch(self, n):
        """Points per device pass (at least 128); 0 restores the default."""
        check(self._L.gg_set_max_batch(self._h, int(n)), self._h)

    def set_uhf(self, onoff):
        if not isinstance(onoff, int):
            raise TypeError
        if bool(onoff) != self.uhf:
            raise ValueError("open-shell mode is fixed when the context is created (pass uhf=True)")

    def set_magnet(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64).reshape(3)
        check(self._L.gg_set_magnet(self._h, _dptr(b)), self._h)

    def get_magnet(self):
        b = np.zeros(3)
        check(self._L.gg_get_magnet(self._h, _dptr(b)), self._h)
        return b

    def set_spin(self, spin):
        if not isinstance(spin, str):
            raise TypeError
        check(self._L.gg_set_spin(self._h, spin.encode()), self._h)

    def set_screening(self, thrs):
        if not isinstance(thrs, float):
            raise TypeError
        check(self._L.gg_set_screening(self._h, thrs), self._h)

    def set_property(self, prop, val):
        """GimicConnector.set_property: dispatches to set_<prop>(val)."""
        getattr(self, "set_" + prop)(val)

    def atoms(self):
        xyz = np.zeros((self.natoms, 3))
        q = np.zeros(self.natoms)
        check(self._L.gg_atoms(self._h, _dptr(xyz), _dptr(q)), self._h)
        return xyz, q

    def profile(self, enable=True):
        """Start (and zero) or stop per-kernel event timing inside the library."""
        check(self._L.gg_profile(self._h, int(enable)), self._h)

    def profile_read(self):
        """{group: (milliseconds, launches)} since profile(True), plus the
        total number of kernels this context launched."""
        ms = np.zeros(5)
        n = (C.c_int64 * 5)()
        tot = C.c_int64()
        check(self._L.gg_profile_read(self._h, _dptr(ms), n, C.byref(tot)), self._h)
        names = ("basis", "tc", "fp64", "plane", "order")
        out = {k: (float(ms[i]), int(n[i])) for i, k in enumerate(names)}
        out["kernels"] = int(tot.value)
        issued, dense = C.c_int64(), C.c_int64()
        check(self._L.gg_profile_blocks(self._h, C.byref(issued), C.byref(dense)), self._h)
        out["gemm_blocks"] = (int(issued.value), int(dense.value))
        cross = C.c_int64()
        check(self._L.gg_profile_cross(self._h, C.byref(cross)), self._h)
        out["cross_blocks"] = int(cross.value)  # of the issued blocks, those with the cross products
        return out

    # ---- evaluation -----------------------------------------------------
    def jtensor_batch(self, points, rho=False, divj=False, stream=None, dtype=np.float64):
        """Current tensors t(m,b) = dj_m/dB_b at points (N,3), returned as
        (N,9) column-major (index m + 3b); optionally the density (N,) and
        the tensor divergence (N,3).  numpy in -> numpy out; CUDA torch
        tensors in -> CUDA torch tensors out (no host round trip).  dtype
        float32 stores the outputs in fp32 (gg_jtensor_batch_f32)."""
        f32 = np.dtype(dtype) == np.float32
        fn = self._L.gg_jtensor_batch_f32 if f32 else self._L.gg_jtensor_batch
        if _is_cuda(points):
            p = points.to(torch.float64).contiguous().reshape(-1, 3)
            n = p.shape[0]
            tdt = torch.float32 if f32 else torch.float64
            jt = torch.empty((n, 9), dtype=tdt, device=p.device)
            rh = torch.empty(n, dtype=tdt, device=p.device) if rho else None
            dv = torch.empty((n, 3), dtype=tdt, device=p.device) if divj else None
            st = stream if stream is not None else torch.cuda.current_stream(p.device).cuda_stream
            rc = fn(self._h, C.c_void_p(p.data_ptr()), n, C.c_void_p(jt.data_ptr()),
                    C.c_void_p(rh.data_ptr()) if rh is not None else None,
                    C.c_void_p(dv.data_ptr()) if dv is not None else None, C.c_void_p(st))
        else:
            p = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
            n = p.shape[0]
            ndt = np.float32 if f32 else np.float64
            jt = np.zeros((n, 9), dtype=ndt)
            rh = np.zeros(n, dtype=ndt) if rho else None
            dv = np.zeros((n, 3), dtype=ndt) if divj else None
            rc = fn(self._h, C.c_void_p(p.ctypes.data), n, C.c_void_p(jt.ctypes.data),
                    C.c_void_p(rh.ctypes.data) if rh is not None else None,
                    C.c_void_p(dv.ctypes.data) if dv is not None else None, C.c_void_p(stream) if stream else None)
        check(rc, self._h)
        out = [jt]
        if rho:
            out.append(rh)
        if divj:
            out.append(dv)
        return out[0] if len(out) == 1 else tuple(out)

    def jvector_batch(self, points, magnet=None):
        """j = t . B at points (N,3) for the context's (or the given) field."""
        jt = self.jtensor_batch(points)
        b = self.get_magnet() if magnet is None else np.asarray(magnet, dtype=np.float64)
        if _is_cuda(jt):
            t = jt.reshape(-1, 3, 3).transpose(1, 2)  # t[p, m, b]
            return t @ torch.as_tensor(b, dtype=torch.float64, device=jt.device)
        return jt.reshape(-1, 3, 3).transpose(0, 2, 1) @ b

    def jtensor(self, r):
        """One point, as Gimic.jtensor in gimic.pyx:14-21 (a list of 9)."""
        return list(self.jtensor_batch(np.asarray(r, dtype=np.float64).reshape(1, 3))[0])

    def jvector(self, r):
        """One point, as Gimic.jvector in gimic.pyx:23-32 (a list of 3)."""
        return list(self.jvector_batch(np.asarray(r, dtype=np.float64).reshape(1, 3))[0])

    def properties(self, points, weights, centres, block_npts=None):
        """Shielding of every centre (ppm) and magnetizability (au) over a
        molecular grid (gg_properties).  Returns (sigma, chi) with sigma of
        shape (ncentres, nblocks, 5) and chi of shape (nblocks, 5): the
        three diagonal sums, then the positive and negative parts."""
        p = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
        w = np.ascontiguousarray(np.asarray(weights, dtype=np.float64).reshape(-1))
        c = np.ascontiguousarray(np.asarray(centres, dtype=np.float64).reshape(-1, 3))
        nb = 1
        bp = None
        if block_npts is not None and len(block_npts):
            bp = np.ascontiguousarray(np.asarray(block_npts, dtype=np.int64))
            nb = len(bp)
        sig = np.zeros((len(c), nb, 5))
        chi = np.zeros((nb, 5))
        rc = self._L.gg_properties(self._h, _dptr(p), _dptr(w), len(p), _dptr(c), len(c),
                                   bp.ctypes.data_as(C.POINTER(C.c_int64)) if bp is not None else None,
                                   nb if bp is not None else 0, _dptr(sig), _dptr(chi), None)
        check(rc, self._h)
        return sig, chi

    def plane_integral(self, origin, basv, axes, radius=1e10, stream=None):
        """Quadrature over the product grid origin + x1 basv[:,0] + x2 basv[:,1]
        + x3 basv[:,2] with axes = ((x1, w1), (x2, w2), (x3, w3)).  Returns a
        dict of atomic-unit sums: current (total, positive, negative),
        modulus (total, positive, negative) and acid (sqrt of the sum), as
        printed by src/fgimic/integral.f90."""
        return self.plane_integrals([(origin, basv, axes, radius)], stream=stream)[0]

    def plane_integrals(self, planes, stream=None):
        """Many planes (origin, basv, axes, radius) in one device pass, e.g. a
        bond-current profile scan; returns one dict per plane."""
        specs, flat = _records(planes)
        n = len(planes)
        out = np.zeros((n, 7))
        check(self._L.gg_plane_integrals(self._h, specs.ctypes.data_as(C.POINTER(_lib.GridSpec)), n, _dptr(out),
                                         C.c_void_p(stream) if stream else None), self._h)
        return _plane_results(out)


class PlaneSet:
    """Planes whose gg_grid records are built once, for planes integrated
    again and again (the strips of a profile scan at every step): building
    the records of a few thousand planes costs tens of milliseconds of host
    time, which a single launch over many molecules cannot hide.  Accepted
    wherever a list of planes is."""

    def __init__(self, planes):
        self.planes = list(planes)
        self.specs, self._keep = _grid_records(self.planes)

    def __len__(self):
        return len(self.planes)


def _records(planes):
    """(records, what keeps their axis buffers alive) of a list of planes or
    a PlaneSet."""
    if isinstance(planes, PlaneSet):
        return planes.specs, planes
    return _grid_records(planes)


def _plane_results(out):
    return [{"current": tuple(o[0:3]), "modulus": tuple(o[3:6]), "acid": math.sqrt(max(o[6], 0.0)),
             "acid_sum": o[6]} for o in out.tolist()]


def _grid_records(planes):
    """gg_grid records of (origin, basv, axes, radius) planes, and the buffer
    of axis points and weights they point into (keep it referenced until the
    library call returns)."""
    n = len(planes)
    if n <= 4:
        # a few planes: the records point straight into the callers' axis
        # arrays and are packed field by field into one buffer (a third of
        # the time of filling a structured array for one plane)
        buf = bytearray(_GRID_DTYPE.itemsize * n)
        keep = []
        for q, (origin, basv, axes, radius) in enumerate(planes):
            arrs = [np.ascontiguousarray(v, dtype=np.float64).reshape(-1) for ax in axes for v in ax]
            keep.append(arrs)
            addr = [a.__array_interface__["data"][0] for a in arrs]
            b = np.asarray(basv, dtype=np.float64)
            _GRID_PACK.pack_into(buf, q * _GRID_DTYPE.itemsize, *np.asarray(origin, dtype=np.float64).reshape(3).tolist(),
                                 *b.T.reshape(9).tolist(), arrs[0].shape[0], arrs[2].shape[0], arrs[4].shape[0],
                                 addr[0], addr[2], addr[4], addr[1], addr[3], addr[5], float(radius))
        return np.frombuffer(buf, dtype=_GRID_DTYPE), keep
    # the gg_grid records are filled as one numpy structured array (a
    # per-field ctypes loop cost about 25 us per plane); the axis
    # arrays are concatenated, and the records point into that buffer
    lens = np.array([[len(ax[0]) for ax in pl[2]] for pl in planes], dtype=np.int64).reshape(n, 3)
    flat = np.concatenate([np.asarray(v, dtype=np.float64).reshape(-1)
                           for pl in planes for ax in pl[2] for v in ax])
    specs = np.zeros(n, dtype=_GRID_DTYPE)
    specs["origin"] = np.asarray([pl[0] for pl in planes], dtype=np.float64).reshape(n, 3)
    # basv[3 d + c] = basv[c, d]
    specs["basv"] = np.asarray([pl[1] for pl in planes], dtype=np.float64).reshape(n, 3, 3).transpose(0, 2, 1).reshape(n, 9)
    specs["npts"] = lens
    specs["radius"] = np.asarray([pl[3] for pl in planes], dtype=np.float64)
    # layout of flat: per plane, per axis d, the points then the weights
    sizes = np.repeat(lens.reshape(-1), 2)
    starts = np.concatenate([[0], np.cumsum(sizes)[:-1]]).reshape(n, 3, 2)
    base = flat.ctypes.data
    specs["pts"] = base + 8 * starts[:, :, 0]
    specs["wgt"] = base + 8 * starts[:, :, 1]
    return specs, flat


def plane_integrals_multi(jobs, stream=None, timings=False):
    """Plane batches of many molecules, queued one after the other on one
    stream and collected at the end (gg_plane_integrals_enqueue / _collect):
    the host work of molecule i+1 overlaps the device work of molecule i.
    jobs = [(Gimic, planes), ...] with distinct contexts.  Returns one list of
    result dicts per molecule, and with ``timings`` also each molecule's
    stream milliseconds."""
    st = C.c_void_p(stream) if stream else None
    queued = []
    try:
        keep = []
        for g, planes in jobs:
            specs, flat = _records(planes)
            keep.append(flat)
            check(g._L.gg_plane_integrals_enqueue(g._h, specs.ctypes.data_as(C.POINTER(_lib.GridSpec)), len(planes),
                                                  st), g._h)
            queued.append((g, len(planes)))
    finally:
        # every queued pass is collected, also when a later one failed
        res, ms, err = [], [], None
        for g, n in queued:
            out = np.zeros((n, 7))
            t = C.c_double()
            try:
                check(g._L.gg_plane_integrals_collect(g._h, _dptr(out), C.byref(t)), g._h)
            except Exception as e:  # keep collecting; report the first failure
                err = err or e
            res.append(_plane_results(out))
            ms.append(t.value)
    if err is not None:
        raise err
    return (res, ms) if timings else res


def plane_integrals_batch(jobs, stream=None, order="cost", timings=False):
    """Plane batches of many molecules in one contraction launch
    (gg_plane_integrals_batch): jobs = [(Gimic, planes), ...] with distinct
    contexts on one device.  ``order`` "cost" runs the most expensive
    molecules' tiles first, "given" in the order of ``jobs``.  Returns one
    list of result dicts per molecule, and with ``timings`` also each
    molecule's completion time (ms) within the launch."""
    n = len(jobs)
    if n == 0:
        return ([], []) if timings else []
    L = jobs[0][0]._L
    recs = [_records(planes) for _, planes in jobs]  # keep the axis buffers referenced
    counts = (C.c_int * n)(*[len(planes) for _, planes in jobs])
    hs = (C.c_void_p * n)(*[g._h.value for g, _ in jobs])
    gp = (C.POINTER(_lib.GridSpec) * n)(*[specs.ctypes.data_as(C.POINTER(_lib.GridSpec)) for specs, _ in recs])
    out = np.zeros((sum(counts), 7))
    ms = np.zeros(n)
    rc = L.gg_plane_integrals_batch(hs, gp, counts, n, {"given": 0, "cost": 1}[order], _dptr(out), _dptr(ms),
                                    C.c_void_p(stream) if stream else None)
    check(rc, jobs[0][0]._h)
    res, off = [], 0
    for k in counts:
        res.append(_plane_results(out[off:off + k]))
        off += k
    return (res, ms.tolist()) if timings else res
