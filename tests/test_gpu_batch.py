"""Plane passes of many molecules in one contraction launch
(gg_plane_integrals_batch), against the per-molecule blocking passes and the
FP64 oracle: long and short passes, open and closed shells, molecules of
different nbf, both job orders, and the eager, captured and replayed forms
of the batch."""
import numpy as np
import pytest

import oracle
from gimic_gb300 import _lib, api, scan, synth

pytestmark = pytest.mark.gpu


def _jobs(synth_dir, c6h6, c6h6_uhf):
    specs = [(c6h6, False, 7, 60), (c6h6_uhf, True, 5, 40),
             (synth.make_workload("c24h24", str(synth_dir), seed=2024), False, 3, 50)]
    jobs = []
    for (mp, xp, mol), uhf, nstrips, p in specs:
        g = api.Gimic(mp, xp, uhf=uhf, screening=1e-8)
        bond = scan.first_cc_bond(mol.symbols, mol.coords)
        planes, bb = scan.profile_planes(mol.coords, bond=bond, start=-2.0, out=8.0, nstrips=nstrips, npts=(p, p),
                                         order=10, quadrature="lobatto",
                                         fixcoord=tuple(scan.plane_fixcoord(mol.coords, bond)))
        g.set_magnet(bb)
        jobs.append((g, planes, mp, xp, uhf, bb))
    return jobs


def test_batch_matches_per_molecule_passes_and_oracle(synth_dir, c6h6, c6h6_uhf):
    jobs = _jobs(synth_dir, c6h6, c6h6_uhf)
    pairs = [(g, planes) for g, planes, *_ in jobs]
    want = [g.plane_integrals(planes) for g, planes in pairs]
    for order in ("given", "cost"):
        for _ in range(3):  # eager, captured, replayed
            got, ms = api.plane_integrals_batch(pairs, order=order, timings=True)
            assert len(ms) == len(pairs) and all(t > 0.0 for t in ms)
            for a, b in zip(got, want):
                assert len(a) == len(b)
                for ra, rb in zip(a, b):
                    for kind in ("current", "modulus"):
                        x, y = np.array(ra[kind]), np.array(rb[kind])
                        # short passes split each tile's chunks over SMs:
                        # fp32 chunk sums round differently (about 3e-8)
                        assert np.all(np.abs(x - y) <= 1e-7 * np.abs(y).max() + 1e-12), (kind, x, y)
    # the first and the last strip of every molecule against the oracle
    got = api.plane_integrals_batch(pairs)
    for (g, planes, mp, xp, uhf, bb), res in zip(jobs, got):
        o = oracle.Oracle(mp, xp, uhf=uhf, screening=1e-8)
        for k in (0, len(planes) - 1):
            origin, basv, axes, radius = planes[k]
            ref = o.integrate(origin, basv, axes, radius, bb, what="current")
            assert abs(api.au2si(res[k]["current"][0]) - api.au2si(ref[0])) <= 1e-4


def test_batch_rejects_bad_batches(synth_dir, c6h6, c6h6_uhf):
    jobs = _jobs(synth_dir, c6h6, c6h6_uhf)
    g0, p0 = jobs[0][0], jobs[0][1]
    with pytest.raises(_lib.GimicError, match="appears twice"):
        api.plane_integrals_batch([(g0, p0), (g0, p0)])
    g1, p1 = jobs[1][0], jobs[1][1]
    g1.set_flags(1, 1, 0)
    with pytest.raises(_lib.GimicError, match="same GIAO"):
        api.plane_integrals_batch([(g0, p0), (g1, p1)])
    g1.set_flags(1, 1, 1)
    g1.set_precision("fp64")
    with pytest.raises(_lib.GimicError, match="split-FP16"):
        api.plane_integrals_batch([(g0, p0), (g1, p1)])
    g1.set_precision("split16")
    # still usable afterwards, and a one-molecule batch is a plain pass
    assert api.plane_integrals_batch([(g1, p1)])[0] == api.plane_integrals_batch([(g1, p1)])[0]


def test_autotuner_picks_a_candidate_that_gives_the_same_sums(synth_dir, c6h6, c6h6_uhf):
    """gimic_gb300.autotune times every launch layout on the batch (queued
    passes, one blocking call per molecule, one batched launch) and keeps
    the fastest per nbf class; every layout gives the same plane sums."""
    torch = pytest.importorskip("torch")
    from gimic_gb300 import autotune
    pairs = [(g, planes) for g, planes, *_ in _jobs(synth_dir, c6h6, c6h6_uhf)]
    best, times = autotune.tune_scan(pairs, reps=1, sync=torch.cuda.synchronize)
    assert best in autotune.CANDIDATES and set(times) == set(autotune.CANDIDATES)
    assert all(t > 0 for t in times.values())
    assert autotune.choice_for(pairs) == best
    assert ("sequential", None) in autotune.CANDIDATES and autotune.label(("sequential", None)) == "sequential"
    # 0 restores the default pass size; other sizes below 128 are rejected
    pairs[0][0].set_max_batch(0)
    with pytest.raises(_lib.GimicError):
        pairs[0][0].set_max_batch(100)
    ref = autotune.run(pairs, ("batch", "cost"))
    for cand in autotune.CANDIDATES:
        got = autotune.run(pairs, cand)
        for a, b in zip(got, ref):
            for ra, rb in zip(a, b):
                x, y = np.array(ra["current"]), np.array(rb["current"])
                assert np.all(np.abs(x - y) <= 1e-7 * np.abs(y).max() + 1e-12), cand


def test_plane_sets_give_the_same_sums(synth_dir, c6h6, c6h6_uhf):
    """Records built once (api.PlaneSet) and plain plane lists give the same
    sums through the single, queued and batched entry points."""
    pairs = [(g, planes) for g, planes, *_ in _jobs(synth_dir, c6h6, c6h6_uhf)]
    sets = [(g, api.PlaneSet(planes)) for g, planes in pairs]
    assert [g.plane_integrals(p) for g, p in pairs] == [g.plane_integrals(p) for g, p in sets]
    assert api.plane_integrals_multi(pairs) == api.plane_integrals_multi(sets)
    assert api.plane_integrals_batch(pairs) == api.plane_integrals_batch(sets)
