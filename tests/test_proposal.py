"""Integration proposal network: the CPU oracle pinned by finite differences,
the CUDA kernels (features, gradient, Adam, bf16 inference) against it, and
the quadtree integrator against the uniform Gauss-Lobatto judge."""
import numpy as np
import pytest

import mlp_oracle as MO


def _rand_params(rng, scale=0.4):
    return rng.standard_normal(MO.N_PARAMS) * scale


# ---------------------------------------------------------------------------
# CPU: the oracle itself
# ---------------------------------------------------------------------------
def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = _rand_params(rng)
    x = rng.standard_normal((37, 5))
    t = rng.standard_normal(37)
    _, g = MO.loss_and_grad(p, x, t)
    idx = rng.choice(MO.N_PARAMS, 60, replace=False)
    idx = np.concatenate([idx, [0, 319, 320, 383, 384, 4479, 4480, 4543, 4544, 4607, 4608]])
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (MO.loss_and_grad(p + e, x, t)[0] - MO.loss_and_grad(p - e, x, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_oracle_layout_and_bf16():
    assert MO.N_PARAMS == 4609
    # bf16 keeps 7 fraction bits: the spacing above 1.0 is 2^-7
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 3 * 2 ** -9, -3.14159, 0.0], dtype=np.float32)
    r = MO.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0  # halfway: to the even neighbour 1.0
    assert r[2] == np.float32(1.0 + 2 ** -6)  # halfway: to the even neighbour 1 + 2^-6
    assert r[3] == np.float32(1.0 + 2 ** -7)  # nearest
    assert r[4] == np.float32(-3.140625) and r[5] == 0.0


def test_oracle_adam_first_step_is_signed_lr():
    g = np.array([0.5, -2.0, 1e-3])
    p, m, v = MO.adam(np.zeros(3), g, np.zeros(3), np.zeros(3), 0.01, 0.9, 0.999, 1e-12, 1)
    assert np.allclose(p, -0.01 * np.sign(g), rtol=1e-6)


def _mapped_rule_sum(P, reg, mu, mv, panels, f):
    tot = 0.0
    for ta, tb, wa, wb, qu, qv in panels:
        x, wx = mu.nodes(ta, tb, qu)
        y, wy = mv.nodes(wa, wb, qv)
        tot += np.sum(np.outer(wx, wy) * f(x[:, None], y[None, :]))
    return tot


def test_mapped_quadtree_integrates_a_peaked_function():
    """The proposal machinery on an analytic integrand (no GPU): axis maps
    and panels built from the function's own mass lattice integrate it far
    more accurately than a uniform grid with the same number of points."""
    pytest.importorskip("torch")
    from gimic_gb300 import proposal as P
    from gimic_gb300 import api

    reg = P.Region(np.zeros(3), [1, 0, 0], [0, 1, 0], [0, 0, 1], 16.0, 13.0, [8.0, 6.0, 0.0])
    c, d = 8.3, 5.1

    def f(x, y):
        return np.exp(-((x - c) / 0.6) ** 2) * (1.0 + 0.5 * np.cos(2.0 * (y - d))) * np.exp(-((y - d) / 1.2) ** 2)

    # both factors are negligible (< 1e-8) at the plane's edges
    exact = 0.6 * np.sqrt(np.pi) * (1.2 * np.sqrt(np.pi) * (1.0 + 0.5 * np.exp(-(2.0 * 1.2) ** 2 / 4.0)))
    G = 96
    cx = (np.arange(G) + 0.5) / G * reg.lx
    cy = (np.arange(G) + 0.5) / G * reg.ly
    mass = f(cx[:, None], cy[None, :]) * (reg.lx / G) * (reg.ly / G)
    mu, mv, panels = P.propose_panels(mass, reg, dict(kappa_u=1.0, kappa_v=1.0, n0u=3, n0v=3, max_depth=0, tau=1.0,
                                                      q_hi=6, q_lo=4, frac=0.0))
    # the maps cover the plane and put their centres on the peak
    assert abs(mu.x(mu.t0)) < 1e-12 and abs(mu.x(mu.t1) - reg.lx) < 1e-9
    assert abs(mv.x(mv.t0)) < 1e-12 and abs(mv.x(mv.t1) - reg.ly) < 1e-9
    assert abs(mu.c - c) < 0.2 and abs(mv.c - d) < 0.2
    n = sum(p[4] * p[5] for p in panels)
    assert n == 324
    got = _mapped_rule_sum(P, reg, mu, mv, panels, f)
    assert abs(got - exact) < 1e-4 * exact, (got, exact)
    # the uniform composite Lobatto grid needs 1600 points to get near it
    for k, worse in ((2, True), (3, True), (4, True)):
        xu, wu = api.gauss_data(0.0, reg.lx, 10, 10 * k, "lobatto")
        yu, wv = api.gauss_data(0.0, reg.ly, 10, 10 * k, "lobatto")
        uni = np.sum(np.outer(wu, wv) * f(xu[:, None], yu[None, :]))
        assert (abs(uni - exact) > abs(got - exact)) == worse, k


def test_quadtree_refines_where_the_mass_is():
    pytest.importorskip("torch")
    from gimic_gb300 import proposal as P

    reg = P.Region(np.zeros(3), [1, 0, 0], [0, 1, 0], [0, 0, 1], 16.0, 10.0, [8.0, 5.0, 0.0])
    m = np.full((64, 64), 1e-6)
    m[30:34, 20:28] = 1.0
    rule = dict(kappa_u=None, kappa_v=None, n0u=1, n0v=1, max_depth=4, tau=2.0, q_hi=10, q_lo=4, frac=0.02)
    mu, mv, pan = P.propose_panels(m, reg, rule)
    assert mu.s is None and mv.s is None  # identity maps: panels in plane coordinates
    area = sum((tb - ta) * (wb - wa) for ta, tb, wa, wb, _, _ in pan)
    assert abs(area - 160.0) < 1e-9
    assert {p[4] for p in pan} == {4, 10} and all(p[4] == p[5] for p in pan)
    hot = [p for p in pan if p[0] < 8.5 and p[1] > 7.5 and p[2] < 4.375 and p[3] > 3.125]
    assert hot and all(p[4] == 10 and abs(p[1] - p[0] - 1.0) < 1e-12 for p in hot)
    mu, mv, pan = P.propose_panels(np.full((64, 64), 1e-9), reg, rule)
    assert len(pan) == 1 and pan[0][4:] == (4, 4)
    # different orders along the two axes
    _, _, pan = P.propose_panels(m, reg, dict(rule, q_hi_v=6))
    assert {(p[4], p[5]) for p in pan} == {(4, 4), (10, 6)}


# ---------------------------------------------------------------------------
# GPU: kernels against the oracle
# ---------------------------------------------------------------------------
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from gimic_gb300 import _lib
    return torch, _lib.load()


def _ptr(t):
    import ctypes as C
    return C.c_void_p(t.data_ptr())


@pytest.mark.gpu
def test_mlp_gradient_matches_oracle():
    torch, L = _cuda()
    rng = np.random.default_rng(1)
    for n in (1, 31, 128, 1000, 4099):
        p = _rand_params(rng, 0.25).astype(np.float32)
        x = rng.standard_normal((n, 5)).astype(np.float32)
        # targets away from the outputs, so that y - t is well conditioned
        y0 = MO.forward(p.astype(np.float64), x.astype(np.float64))[0]
        t = (y0 + np.where(rng.uniform(size=n) < 0.5, -1.0, 1.0) * rng.uniform(0.5, 2.0, n)).astype(np.float32)
        loss_ref, g_ref = MO.loss_and_grad(p.astype(np.float64), x.astype(np.float64), t.astype(np.float64))
        dp, dx, dt = (torch.as_tensor(a, device="cuda") for a in (p, x, t))
        grad = torch.full((MO.N_PARAMS,), 7.0, device="cuda")  # overwritten, not accumulated
        loss = torch.zeros(1, device="cuda")
        assert L.gg_mlp_grad(_ptr(dp), _ptr(dx), _ptr(dt), n, _ptr(grad), _ptr(loss), None) == 0
        torch.cuda.synchronize()
        g = grad.cpu().numpy().astype(np.float64)
        # fp32 kernel vs fp64 oracle: relative to the gradient's scale
        assert np.max(np.abs(g - g_ref)) <= 2e-5 * np.max(np.abs(g_ref)), n
        assert abs(float(loss) - loss_ref) <= 1e-5 * max(1.0, loss_ref)


@pytest.mark.gpu
def test_mlp_adam_matches_oracle():
    torch, L = _cuda()
    rng = np.random.default_rng(2)
    p = _rand_params(rng)
    m = rng.standard_normal(MO.N_PARAMS) * 1e-2
    v = np.abs(rng.standard_normal(MO.N_PARAMS)) * 1e-4
    g = rng.standard_normal(MO.N_PARAMS) * 1e-2
    dp, dg, dm, dv = (torch.as_tensor(a.astype(np.float32), device="cuda") for a in (p, g, m, v))
    p32, g32, m32, v32 = (a.astype(np.float32).astype(np.float64) for a in (p, g, m, v))
    for step in (1, 2, 3):
        assert L.gg_mlp_adam(_ptr(dp), _ptr(dg), _ptr(dm), _ptr(dv), 1e-3, 0.9, 0.999, 1e-8, step, None) == 0
        p32, m32, v32 = MO.adam(p32, g32, m32, v32, 1e-3, 0.9, 0.999, 1e-8, step)
    torch.cuda.synchronize()
    # fp32 kernel vs fp64 oracle, tolerances relative to each array's scale
    for got, ref in ((dp, p32), (dm, m32), (dv, v32)):
        got = got.cpu().numpy().astype(np.float64)
        assert np.max(np.abs(got - ref)) <= 1e-6 * np.max(np.abs(ref))


@pytest.mark.gpu
def test_mlp_bf16_inference_matches_oracle():
    torch, L = _cuda()
    rng = np.random.default_rng(3)
    p = _rand_params(rng).astype(np.float32)
    x = rng.standard_normal((5000, 5)).astype(np.float32)
    dp, dx = torch.as_tensor(p, device="cuda"), torch.as_tensor(x, device="cuda")
    y = torch.empty(5000, device="cuda")
    assert L.gg_mlp_infer(_ptr(dp), _ptr(dx), 5000, _ptr(y), None) == 0
    torch.cuda.synchronize()
    ref = MO.infer_bf16(p, x)
    full = MO.forward(p.astype(np.float64), x.astype(np.float64))[0]
    err = np.abs(y.cpu().numpy() - ref)
    # fp32 accumulation may flip the bf16 rounding of an activation now and then
    assert np.median(err) < 1e-5 * np.max(np.abs(ref))
    assert np.max(err) < 2e-2 * np.max(np.abs(ref))
    # bf16 inference stays close to the fp32 network
    assert np.max(np.abs(ref - full)) < 0.05 * np.max(np.abs(full))


@pytest.mark.gpu
def test_mlp_rejects_host_pointers_and_bad_sizes():
    torch, L = _cuda()
    p = torch.zeros(MO.N_PARAMS, device="cuda")
    x = np.zeros((4, 5), dtype=np.float32)
    y = torch.empty(4, device="cuda")
    import ctypes as C
    assert L.gg_mlp_infer(_ptr(p), C.c_void_p(x.ctypes.data), 4, _ptr(y), None) != 0
    assert L.gg_mlp_infer(_ptr(p), _ptr(p), -1, _ptr(y), None) != 0
    assert L.gg_mlp_adam(_ptr(p), _ptr(p), _ptr(p), _ptr(p), 1e-3, 0.9, 0.999, 1e-8, 0, None) != 0
    assert L.gg_mlp_infer(_ptr(p), _ptr(p), 0, _ptr(y), None) == 0


@pytest.mark.gpu
def test_features_match_oracle(c6h6):
    torch, L = _cuda()
    from gimic_gb300 import api
    from oracle import Oracle
    from gimic_gb300 import proposal as P

    mol, xdens, _ = c6h6
    o = Oracle(mol, xdens)
    xyz, _ = o.atoms()
    sh = o.shells()
    amin = np.array([sh["xp"][s, :sh["npf"][s]].min() for s in range(len(sh["atom"]))])
    rng = np.random.default_rng(4)
    pts = rng.uniform(-6, 6, (3000, 3))
    pts[:3] = xyz[:3]  # on nuclei: distance floor
    uv = rng.uniform(-8, 8, (3000, 2))
    g = api.Gimic(mol, xdens)
    f = P.features(g, pts, uv).cpu().numpy()
    ref = MO.features(xyz, sh["atom"], amin, pts, uv)
    assert np.allclose(f, ref, rtol=2e-6, atol=2e-6)


@pytest.mark.gpu
def test_training_reduces_loss_and_matches_oracle_step():
    torch, L = _cuda()
    from gimic_gb300 import proposal as P

    rng = np.random.default_rng(5)
    x = rng.standard_normal((20000, 5)).astype(np.float32)
    t = (np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2] - 0.5 * x[:, 3] ** 2 + 0.3 * x[:, 4]).astype(np.float32)
    net = P.ProposalNet(seed=3)
    p0 = net.params.cpu().numpy().astype(np.float64)
    dx, dt = torch.as_tensor(x, device="cuda"), torch.as_tensor(t, device="cuda")
    # one step by hand against the oracle
    tt = (t - t.mean()) / t.std(ddof=1)
    _, g = net.loss_grad(dx[:4096], torch.as_tensor(tt[:4096].astype(np.float32), device="cuda"))
    _, g_ref = MO.loss_and_grad(p0, x[:4096].astype(np.float64), tt[:4096].astype(np.float64))
    assert np.max(np.abs(g.cpu().numpy() - g_ref)) <= 2e-5 * np.max(np.abs(g_ref))
    hist = net.fit(dx, dt, epochs=20, batch=2048, lr=3e-3)
    assert hist[-1] < 0.2 * hist[0], hist
    pred = net.predict(dx).cpu().numpy()
    assert np.sqrt(np.mean((pred - t) ** 2)) < 0.4 * t.std()


# ---------------------------------------------------------------------------
# GPU: the trained proposal against the uniform grid and the untrained one
# ---------------------------------------------------------------------------
def _bond_planes(P, api, synth, outdir, seed, n, per):
    out = []
    for i in range(n):
        mp, xp, mol = synth.make_batch_molecule(outdir, i, seed=seed)
        g = api.Gimic(mp, xp, screening=1e-8)
        c = mol.coords
        ci = [k for k, s in enumerate(mol.symbols) if s == "C"]
        bonds = [(a + 1, b + 1) for a in ci for b in ci if b > a and np.linalg.norm(c[a] - c[b]) < 3.0]
        rng = np.random.default_rng([seed, i, 7])
        pick = [bonds[0]] + [bonds[k] for k in rng.choice(len(bonds), min(per - 1, len(bonds)), replace=False)]
        for bd in pick[:per]:
            reg, bb = P.Region.bond_plane(c, bd)
            out.append((g, reg, bb))
    return out


@pytest.mark.gpu
def test_learned_proposal_gains_over_uniform_and_untrained(tmp_path_factory):
    """Trained on 10^6 samples from 64 bond planes of 32 generated molecules
    (the calibration set of the default rule), the proposal integrates 16
    held-out planes (other seed) within 0.01 nA/T of the 200 x 200 judge
    with fewer evaluated points than the smallest converged uniform grid,
    and with at least 4x fewer than the standard 60 x 60 Gauss-Lobatto grid
    (order 10), which is itself within 0.01 nA/T on every plane; the same
    network untrained misses the tolerance."""
    torch, L = _cuda()
    from gimic_gb300 import api, synth
    from gimic_gb300 import proposal as P

    d = str(tmp_path_factory.mktemp("proposal"))
    train = _bond_planes(P, api, synth, d, 1077, 32, 2)
    held = _bond_planes(P, api, synth, d, 2077, 16, 1)
    rng = np.random.default_rng(5)
    F, T = [], []
    for g, reg, bb in train:
        g.set_magnet(bb)
        f, t = P.sample_plane(g, reg, 1000000 // len(train), rng)
        F.append(f)
        T.append(t)
    net = P.ProposalNet(seed=1)
    hist = net.fit(torch.cat(F), torch.cat(T), epochs=20, batch=4096, lr=3e-3)
    assert hist[-1] < 0.8 * hist[0]
    net0 = P.ProposalNet(seed=1)
    net0.t_mean, net0.t_std, net0.box = net.t_mean, net.t_std, net.box
    uni, ada, err, err0, err60 = 0, 0, [], [], []
    for g, reg, bb in held:
        g.set_magnet(bb)
        judge = P.integrate_uniform(g, reg, 200)
        upts, _ = P.uniform_points_to_reach(g, reg, judge)
        err60.append(abs(P.integrate_uniform(g, reg, 60) - judge))
        res = P.integrate_adaptive(g, net, reg)
        assert res["method"] == "adaptive"
        res0 = P.integrate_adaptive(g, net0, reg, min_inside=0.0)
        uni += upts
        ada += res["points"]
        err.append(abs(res["current"] - judge))
        err0.append(abs(res0["current"] - judge))
    assert max(err) <= 0.01, err
    assert ada < uni, (ada, uni)
    assert max(err60) <= 0.01, err60
    assert 3600 * len(held) / ada >= 4.0, (ada, 3600 * len(held))
    assert sum(e > 0.01 for e in err0) >= 8, err0
