"""Learned proposal for adaptive plane integration (no reference counterpart).

The reference integrates the current through a plane on a fixed product grid
of Gauss(-Lobatto) points (src/fgimic/integral.f90:50-511 over the grid of
src/fgimic/grid.f90:165-276 and src/libgimic/gaussint.f90:267-319).  Here a
small network predicts ln|j| over the plane from five cheap features; the
prediction drives a quadtree of Gauss-Lobatto panels (refined where the
predicted current mass is large), and j is evaluated on the GPU only at the
nodes of the final panels.  The uniform-grid integral stays both the judge
of the result and the fallback when a plane lies outside what the network
was trained on.

Everything numerical runs in libgimic_gb300.so: the features
(gg_mlp_features), the network's training step (gg_mlp_grad + gg_mlp_adam,
hand-written forward/backward and Adam kernels, fp32 weights), its bf16
inference (gg_mlp_infer), the current density (gg_jtensor_batch) and the
panel quadratures (gg_plane_integrals).  PyTorch only holds device buffers.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _lib, api, scan
from . import grid as ggrid
from . import inp as ginp

N_IN = 5
J_FLOOR = 1e-9  # au; targets are ln(|j| + J_FLOOR)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check(rc, what):
    if rc != 0:
        raise _lib.GimicError(rc, what)


# ---------------------------------------------------------------------------
# integration planes
# ---------------------------------------------------------------------------
class Region:
    """A rectangular integration plane: points origin + x e1 + y e2 with
    x in [0, lx], y in [0, ly]; ``centre`` is the point the in-plane feature
    coordinates are measured from (the bond crossing of a bond plane)."""

    def __init__(self, origin, e1, e2, normal, lx, ly, centre, radius=1e10):
        self.origin = np.asarray(origin, dtype=np.float64)
        self.e1 = np.asarray(e1, dtype=np.float64)
        self.e2 = np.asarray(e2, dtype=np.float64)
        self.normal = np.asarray(normal, dtype=np.float64)
        self.lx, self.ly = float(lx), float(ly)
        self.centre = np.asarray(centre, dtype=np.float64)
        self.radius = float(radius)

    @classmethod
    def bond_plane(cls, coords, bond, start=None, out=8.0, up=8.0, down=8.0, fixcoord=None, magnet_axis="z"):
        """The plane through the midpoint of ``bond`` (1-based atoms)
        perpendicular to it, as grid type 'bond' builds it
        (src/fgimic/grid.f90:165-276): height [-down, up] about the molecular
        plane, width from ``start`` (default: the molecule's centroid side,
        at most 8 Bohr) to ``out`` past the bond.  Returns (Region, magnet)."""
        coords = np.asarray(coords, dtype=np.float64)
        fix = scan.plane_fixcoord(coords, bond) if fixcoord is None else np.asarray(fixcoord, dtype=np.float64)
        a1, a2 = bond
        mid = 0.5 * (coords[a1 - 1] + coords[a2 - 1])
        if start is None:
            start = -min(float(np.linalg.norm(mid - coords.mean(axis=0))), 8.0)
        dist = 0.5 * float(np.linalg.norm(coords[a2 - 1] - coords[a1 - 1]))
        text = ("calc=integral\nmagnet_axis=%s\nGrid(bond) {\n type=lobatto\n bond=[%d,%d]\n"
                " fixcoord=[%r, %r, %r]\n distance=%r\n height=[%r, %r]\n width=[%r, %r]\n"
                " grid_points=[10, 10, 0]\n gauss_order=10\n}\n"
                % (magnet_axis, a1, a2, float(fix[0]), float(fix[1]), float(fix[2]), dist, -float(down), float(up),
                   float(start), float(out)))
        i = ginp.read(text, is_text=True)
        g = ggrid.new_grid(i, coords)
        b, _ = ggrid.get_magnet(g, i)
        reg = cls(g.origin, g.basv[:, 0], g.basv[:, 1], g.basv[:, 2], g.l[0], g.l[1], g.bond_center, g.radius)
        reg.basv = g.basv.copy()
        return reg, np.asarray(b, dtype=np.float64)

    def basis(self):
        return getattr(self, "basv", np.stack([self.e1, self.e2, self.normal], axis=1))

    def points(self, xy):
        xy = np.asarray(xy, dtype=np.float64).reshape(-1, 2)
        return self.origin + xy[:, :1] * self.e1 + xy[:, 1:] * self.e2

    def uv(self, xy):
        """In-plane coordinates relative to ``centre`` (Bohr)."""
        p = self.points(xy) - self.centre
        return np.stack([p @ self.e1, p @ self.e2], axis=1)

    def panel(self, x0, x1, y0, y1, qx, qy):
        """One Gauss-Lobatto panel as a plane for Gimic.plane_integrals."""
        ax = [api.gauss_data(0.0, x1 - x0, qx, qx, "lobatto"), api.gauss_data(0.0, y1 - y0, qy, qy, "lobatto"),
              (np.zeros(1), np.ones(1))]
        return (self.origin + x0 * self.e1 + y0 * self.e2, self.basis(), ax, self.radius)

    def uniform(self, npts, order=10):
        """The whole plane as one uniform grid of npts x npts points."""
        ax = [api.gauss_data(0.0, self.lx, order, npts, "lobatto"),
              api.gauss_data(0.0, self.ly, order, npts, "lobatto"), (np.zeros(1), np.ones(1))]
        return (self.origin, self.basis(), ax, self.radius)


def integrate_uniform(gimic, region, npts, order=10):
    """Current (nA/T) through the plane on an npts x npts Gauss-Lobatto grid
    (panels of ``order`` points), as the reference's integral does it."""
    r = gimic.plane_integrals([region.uniform(npts, order)])[0]
    return api.au2si(r["current"][0])


# ---------------------------------------------------------------------------
# features and the network
# ---------------------------------------------------------------------------
def features(gimic, pts, uv):
    """The five network inputs (N, 5) fp32 on the device for points pts (N, 3)
    with in-plane coordinates uv (N, 2); both device or host arrays."""
    dev = torch.device("cuda", torch.cuda.current_device())
    p = torch.as_tensor(pts, dtype=torch.float64, device=dev).reshape(-1, 3).contiguous()
    q = torch.as_tensor(uv, dtype=torch.float64, device=dev).reshape(-1, 2).contiguous()
    f = torch.empty((p.shape[0], N_IN), dtype=torch.float32, device=dev)
    _check(gimic._L.gg_mlp_features(gimic._h, _ptr(p), _ptr(q), p.shape[0], _ptr(f), _stream()), "gg_mlp_features")
    return f


class ProposalNet:
    """5 -> 64 -> 64 -> 1 SiLU network predicting ln(|j| + 1e-9) (|j| in au).

    Weights are fp32 on the device; targets are standardised with the
    training set's mean and deviation.  ``box`` is the per-feature range seen
    in training, used to decide when a plane falls back to the uniform grid.
    """

    def __init__(self, seed=0, device=None):
        L = _lib.load()
        self._L = L
        self.n_params = int(L.gg_mlp_nparams())
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
        rng = np.random.default_rng(seed)
        h = 64
        parts = []
        for fan_in, fan_out in ((N_IN, h), (h, h), (h, 1)):
            bound = math.sqrt(6.0 / fan_in) / 1.6  # He-uniform, tempered for SiLU
            parts.append(rng.uniform(-bound, bound, fan_in * fan_out))
            parts.append(np.zeros(fan_out))
        p = np.concatenate(parts).astype(np.float32)
        assert p.size == self.n_params
        self.params = torch.as_tensor(p, device=self.device)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grad = torch.zeros_like(self.params)
        self.step = 0
        self.t_mean, self.t_std = 0.0, 1.0
        self.box = None

    # -- raw kernels --------------------------------------------------------
    def loss_grad(self, x, t, loss=True):
        """Mean squared error of standardised predictions and its gradient
        (a device tensor, overwritten on every call)."""
        x = x.contiguous()
        t = t.contiguous()
        lo = torch.zeros(1, dtype=torch.float32, device=self.device) if loss else None
        _check(self._L.gg_mlp_grad(_ptr(self.params), _ptr(x), _ptr(t), x.shape[0], _ptr(self.grad), _ptr(lo),
                                   _stream()), "gg_mlp_grad")
        return lo, self.grad

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step += 1
        _check(self._L.gg_mlp_adam(_ptr(self.params), _ptr(self.grad), _ptr(self.m), _ptr(self.v), float(lr),
                                   float(beta1), float(beta2), float(eps), self.step, _stream()), "gg_mlp_adam")

    def infer(self, x):
        """Standardised bf16 predictions for features x (N, 5)."""
        x = x.contiguous()
        y = torch.empty(x.shape[0], dtype=torch.float32, device=self.device)
        _check(self._L.gg_mlp_infer(_ptr(self.params), _ptr(x), x.shape[0], _ptr(y), _stream()), "gg_mlp_infer")
        return y

    # -- training and prediction ---------------------------------------------
    def fit(self, x, target, epochs=20, batch=4096, lr=3e-3, lr_min=1e-4, seed=0):
        """Train on features x (N, 5) and targets ln(|j| + 1e-9) (N,), both
        device tensors.  Returns the mean training loss of each epoch."""
        target = target.to(torch.float32)
        self.t_mean = float(target.mean())
        self.t_std = float(target.std()) or 1.0
        t = ((target - self.t_mean) / self.t_std).contiguous()
        self.box = (x.min(dim=0).values.cpu().numpy(), x.max(dim=0).values.cpu().numpy())
        n = x.shape[0]
        gen = torch.Generator(device=self.device)
        gen.manual_seed(seed)
        steps = epochs * ((n + batch - 1) // batch)
        k = 0
        hist = []
        nb = (n + batch - 1) // batch
        losses = torch.zeros(nb, dtype=torch.float32, device=self.device)  # one slot per step of an epoch
        x = x.contiguous()
        for _ in range(epochs):
            perm = torch.randperm(n, device=self.device, generator=gen)
            # the epoch's samples in shuffled order, gathered once: every
            # minibatch is then a contiguous slice (the same samples as
            # indexing each batch), and each step writes its loss to its own
            # slot, so a step launches only the library's kernels
            xs, ts = x[perm], t[perm]
            for b, s in enumerate(range(0, n, batch)):
                _check(self._L.gg_mlp_grad(_ptr(self.params), _ptr(xs[s:s + batch]), _ptr(ts[s:s + batch]),
                                           min(batch, n - s), _ptr(self.grad), _ptr(losses[b:b + 1]), _stream()),
                       "gg_mlp_grad")
                frac = k / max(steps - 1, 1)
                self.adam(lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * frac)))
                k += 1
            hist.append(float(losses.sum()) / nb)
        return hist

    def predict(self, x):
        """ln(|j| + 1e-9) predicted for features x (device tensor)."""
        return self.infer(x) * self.t_std + self.t_mean

    def in_box(self, x, margin=0.1):
        """Fraction of feature rows inside the training range widened by
        ``margin`` of its width on each side."""
        if self.box is None:
            return 0.0
        lo, hi = (torch.as_tensor(b, device=self.device) for b in self.box)
        w = (hi - lo) * margin
        ok = ((x >= lo - w) & (x <= hi + w)).all(dim=1)
        return float(ok.float().mean())

    def state(self):
        return {"params": self.params.cpu().numpy(), "t_mean": self.t_mean, "t_std": self.t_std,
                "box_lo": self.box[0] if self.box else None, "box_hi": self.box[1] if self.box else None}

    def save(self, path):
        s = self.state()
        np.savez(path, params=s["params"], t_mean=s["t_mean"], t_std=s["t_std"],
                 box_lo=s["box_lo"] if s["box_lo"] is not None else np.zeros(0),
                 box_hi=s["box_hi"] if s["box_hi"] is not None else np.zeros(0))

    @classmethod
    def load(cls, path):
        z = np.load(path)
        net = cls()
        net.params = torch.as_tensor(z["params"].astype(np.float32), device=net.device)
        net.t_mean, net.t_std = float(z["t_mean"]), float(z["t_std"])
        if z["box_lo"].size:
            net.box = (z["box_lo"], z["box_hi"])
        return net


# ---------------------------------------------------------------------------
# training data produced by the method itself
# ---------------------------------------------------------------------------
def sample_plane(gimic, region, n, rng, core_frac=0.5, floor=J_FLOOR):
    """n points on the plane with their features and targets ln(|j| + floor)
    (|j| in au, from the GPU path).  A fraction ``core_frac`` is drawn within 3 Bohr
    of the molecular plane, where the current lives; the rest uniformly."""
    nc = int(n * core_frac)
    xy = np.empty((n, 2))
    xy[:, 0] = rng.uniform(0.0, region.lx, n)
    xy[:, 1] = rng.uniform(0.0, region.ly, n)
    u0 = float((region.centre - region.origin) @ region.e1)
    xy[:nc, 0] = np.clip(u0 + rng.uniform(-3.0, 3.0, nc), 0.0, region.lx)
    dev = torch.device("cuda", torch.cuda.current_device())
    pts = torch.as_tensor(region.points(xy), device=dev)
    f = features(gimic, pts, torch.as_tensor(region.uv(xy), device=dev))
    j = gimic.jvector_batch(pts)
    t = torch.log(torch.linalg.norm(j, dim=1) + floor).to(torch.float32)
    return f, t


# ---------------------------------------------------------------------------
# adaptive integration
# ---------------------------------------------------------------------------
# Calibrated on 64 bond planes of 32 training molecules (bench.py --config
# proposal builds the same set): the cheapest rule of a grid search over
# kappa, initial panels, tau, depth and orders with every training plane
# within 0.01 nA/T of its 200 x 200 uniform judge (largest error 0.0075).
DEFAULT_RULE = {"kappa_u": 2.0, "kappa_v": 2.0, "tau": 1.0, "q_hi": 7, "q_hi_v": None, "q_lo": 4, "frac": 0.02,
                "max_depth": 1, "n0u": 3, "n0v": 3, "lattice": 96}


class AxisMap:
    """Smooth monotone map x(t) = c + s sinh(t) of t in [t0, t1] onto [0, L]:
    Gauss-Lobatto nodes equally spaced in t crowd around x = c, on the
    length scale s; s = None is the identity (t = x)."""

    def __init__(self, L, c=None, s=None):
        self.L, self.c, self.s = float(L), c, s
        if s is None:
            self.t0, self.t1 = 0.0, self.L
        else:
            self.t0, self.t1 = float(np.arcsinh((0.0 - c) / s)), float(np.arcsinh((self.L - c) / s))

    def x(self, t):
        t = np.asarray(t, dtype=np.float64)
        if self.s is None:
            return t
        return np.clip(self.c + self.s * np.sinh(t), 0.0, self.L)

    def nodes(self, ta, tb, q):
        """Gauss-Lobatto nodes of order q on [ta, tb] mapped to x, with the
        weights times dx/dt."""
        t, w = api.gauss_data(0.0, tb - ta, q, q, "lobatto")
        t = t + ta
        if self.s is None:
            return t, w
        return self.x(t), w * self.s * np.cosh(t)


def _weighted_quantiles(centres, w, qs):
    cw = np.cumsum(w)
    if cw[-1] <= 0.0:
        return [float(np.quantile(centres, q)) for q in qs]
    return [float(np.interp(q * cw[-1], cw, centres)) for q in qs]


def estimate_maps(mass, region, rule=None):
    """The two axis maps from the predicted mass lattice: centred on the
    mass-weighted median of each marginal, with s = kappa times the
    interquartile range of that marginal (at least 0.25 Bohr)."""
    r = dict(DEFAULT_RULE, **(rule or {}))
    G = mass.shape[0]
    maps = []
    for axis, L, kappa in ((0, region.lx, r["kappa_u"]), (1, region.ly, r["kappa_v"])):
        marg = np.abs(mass).sum(axis=1 - axis)
        centres = (np.arange(G) + 0.5) / G * L
        q25, q50, q75 = _weighted_quantiles(centres, marg, (0.25, 0.5, 0.75))
        maps.append(AxisMap(L, q50, max(kappa * (q75 - q25), 0.25)) if kappa is not None else AxisMap(L))
    return maps


class _MassTable:
    """Predicted mass of any rectangle [x0, x1] x [y0, y1] from the lattice,
    by interpolating its 2-D cumulative sums."""

    def __init__(self, mass, region):
        G = mass.shape[0]
        self.S = np.zeros((G + 1, G + 1))
        self.S[1:, 1:] = mass.cumsum(0).cumsum(1)
        self.gx = np.linspace(0.0, region.lx, G + 1)
        self.gy = np.linspace(0.0, region.ly, G + 1)

    def _cum(self, x, y):
        fx = np.interp(x, self.gx, np.arange(len(self.gx)))
        fy = np.interp(y, self.gy, np.arange(len(self.gy)))
        i, j = min(int(fx), len(self.gx) - 2), min(int(fy), len(self.gy) - 2)
        ax, ay = fx - i, fy - j
        S = self.S
        return ((1 - ax) * (1 - ay) * S[i, j] + ax * (1 - ay) * S[i + 1, j] + (1 - ax) * ay * S[i, j + 1]
                + ax * ay * S[i + 1, j + 1])

    def __call__(self, x0, x1, y0, y1):
        return self._cum(x1, y1) - self._cum(x0, y1) - self._cum(x1, y0) + self._cum(x0, y0)


def propose_panels(mass, region, rule=None):
    """The proposal: axis maps from the predicted mass, then a quadtree in the
    mapped coordinates.  The mapped domain starts as n0u x n0v panels; a
    panel is split in four while its predicted current mass exceeds ``tau``
    (nA/T) and it is shallower than ``max_depth``; a leaf gets ``q_hi``
    Gauss-Lobatto points along u and ``q_hi_v`` (default q_hi) along v when
    its mass exceeds frac * tau, else ``q_lo`` along both.  Returns
    (map_u, map_v, [(ta, tb, wa, wb, q_u, q_v)])."""
    r = dict(DEFAULT_RULE, **(rule or {}))
    mu, mv = estimate_maps(mass, region, r)
    table = _MassTable(mass, region)
    tu = np.linspace(mu.t0, mu.t1, int(r["n0u"]) + 1)
    tv = np.linspace(mv.t0, mv.t1, int(r["n0v"]) + 1)
    stack = [(tu[i], tu[i + 1], tv[j], tv[j + 1], 0) for i in range(len(tu) - 1) for j in range(len(tv) - 1)]
    panels = []
    while stack:
        ta, tb, wa, wb, d = stack.pop()
        m = table(float(mu.x(ta)), float(mu.x(tb)), float(mv.x(wa)), float(mv.x(wb)))
        if m > r["tau"] and d < r["max_depth"]:
            tm, wm = 0.5 * (ta + tb), 0.5 * (wa + wb)
            stack += [(ta, tm, wa, wm, d + 1), (tm, tb, wa, wm, d + 1), (ta, tm, wm, wb, d + 1),
                      (tm, tb, wm, wb, d + 1)]
        elif m > r["frac"] * r["tau"]:
            panels.append((ta, tb, wa, wb, r["q_hi"], r["q_hi_v"] or r["q_hi"]))
        else:
            panels.append((ta, tb, wa, wb, r["q_lo"], r["q_lo"]))
    return mu, mv, panels


def panel_planes(region, mu, mv, panels):
    """Each mapped panel as a plane for Gimic.plane_integrals."""
    out = []
    for ta, tb, wa, wb, qu, qv in panels:
        ax = [mu.nodes(ta, tb, qu), mv.nodes(wa, wb, qv), (np.zeros(1), np.ones(1))]
        out.append((region.origin, region.basis(), ax, region.radius))
    return out


def integrate_panels(gimic, region, mu, mv, panels):
    """Current (nA/T) summed over the mapped Gauss-Lobatto panels, all in
    one device pass."""
    res = gimic.plane_integrals(panel_planes(region, mu, mv, panels))
    return sum(api.au2si(r["current"][0]) for r in res)


def predict_mass(net, gimic, region, lattice=96):
    """Predicted current mass per cell of a lattice x lattice partition of
    the plane (|j| predicted at the cell centre times the cell area, nA/T),
    and the fraction of those cells whose features lie in the training
    range."""
    G = int(lattice)
    cx = (np.arange(G) + 0.5) / G * region.lx
    cy = (np.arange(G) + 0.5) / G * region.ly
    X, Y = np.meshgrid(cx, cy, indexing="ij")
    xy = np.stack([X.reshape(-1), Y.reshape(-1)], axis=1)
    dev = torch.device("cuda", torch.cuda.current_device())
    f = features(gimic, torch.as_tensor(region.points(xy), device=dev), torch.as_tensor(region.uv(xy), device=dev))
    inside = net.in_box(f)
    lnj = net.predict(f).double().cpu().numpy().reshape(G, G)
    return np.exp(lnj) * api.au2si(1.0) * (region.lx / G) * (region.ly / G), inside


def integrate_adaptive(gimic, net, region, rule=None, min_inside=0.99, fallback_npts=200):
    """Current (nA/T) through the plane on the proposed panels.  When fewer
    than ``min_inside`` of the lattice features lie in the training range
    (or no network is given), the uniform grid of fallback_npts^2 points is
    used instead.  Returns a dict: current, points, panels, method."""
    inside = None
    if net is not None:
        r = dict(DEFAULT_RULE, **(rule or {}))
        mass, inside = predict_mass(net, gimic, region, r["lattice"])
        if inside >= min_inside:
            mu, mv, panels = propose_panels(mass, region, r)
            cur = integrate_panels(gimic, region, mu, mv, panels)
            return {"current": cur, "points": int(sum(p[4] * p[5] for p in panels)), "panels": panels,
                    "maps": (mu, mv), "method": "adaptive", "inside": inside}
    cur = integrate_uniform(gimic, region, fallback_npts)
    return {"current": cur, "points": fallback_npts * fallback_npts, "panels": None, "method": "uniform-fallback",
            "inside": inside}


def uniform_points_to_reach(gimic, region, judge, tol=0.01, order=10, kmax=20):
    """Smallest uniform grid (order-``order`` panels, k per axis) from which
    every finer grid up to kmax panels stays within ``tol`` nA/T of ``judge``.
    Returns (points, {k: error})."""
    errs = {}
    planes = [region.uniform(order * k, order) for k in range(1, kmax + 1)]
    res = gimic.plane_integrals(planes)
    for k, r in zip(range(1, kmax + 1), res):
        errs[k] = api.au2si(r["current"][0]) - judge
    first = None
    for k in range(kmax, 0, -1):
        if abs(errs[k]) <= tol:
            first = k
        else:
            break
    return (None if first is None else (order * first) ** 2), errs
