"""Failure paths on the GPU, in the forms that fault, trap or hang nothing:

  * a bounded device wait that nothing satisfies gives up after its limit,
    the host reports GG_ETIMEDOUT, and the next evaluation on the same
    context succeeds and matches the oracle;
  * an error already recorded in the device error word (as a failed wait of
    another thread would leave it) makes the contraction kernel's roles leave
    their pipelines early; the call reports it and the context stays usable;
  * two threads that create contexts and make their first evaluation at the
    same moment (in a fresh process, so that the kernels' one-time set-up
    per device runs under that race) both match the oracle.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import oracle
from conftest import ROOT, rel_max_err, sample_points
from gimic_gb300 import _lib, api

pytestmark = pytest.mark.gpu

TOL_SPLIT = 1e-6


def test_wait_timeout_reports_and_context_recovers(c6h6):
    mp, xp, _ = c6h6
    g = api.Gimic(mp, xp, screening=1e-8)
    o = oracle.Oracle(mp, xp, screening=1e-8)
    L = _lib.load()
    import ctypes as C
    for limit in (1.0, 20.0):
        waited = C.c_double()
        rc = L.gg_selftest_wait_timeout(g._h, limit, C.byref(waited), None)
        assert rc == -5, L.gg_last_error(g._h)  # GG_ETIMEDOUT
        assert b"code 100" in L.gg_last_error(g._h)
        # gave up after its limit, not long after (one poll round is ~us)
        assert limit <= waited.value <= limit + 50.0, waited.value
    pts = sample_points(o.atoms()[0], 700, 100, 7.0, seed=31)
    assert rel_max_err(g.jtensor_batch(pts), o.jtensor(pts)) <= TOL_SPLIT
    assert L.gg_selftest_wait_timeout(g._h, 0.0, None, None) == -1
    assert L.gg_selftest_wait_timeout(g._h, 5000.0, None, None) == -1


@pytest.mark.parametrize("precision", ["split16", "fp64"])
def test_recorded_error_ends_the_call_and_clears(c6h6, precision):
    mp, xp, _ = c6h6
    g = api.Gimic(mp, xp, screening=1e-8, precision=precision)
    o = oracle.Oracle(mp, xp, screening=1e-8)
    L = _lib.load()
    pts = sample_points(o.atoms()[0], 3000, 200, 8.0, seed=32)
    ref = o.jtensor(pts)
    g.jtensor_batch(pts[:10])  # prepared
    assert L.gg_selftest_fail_next(g._h, 0) == -1
    assert L.gg_selftest_fail_next(g._h, 42) == 0
    with pytest.raises(_lib.GimicError, match="code 42"):
        g.jtensor_batch(pts)
    # the word is clear again: the same call now succeeds
    assert rel_max_err(g.jtensor_batch(pts), ref) <= TOL_SPLIT
    # the same through a multi-batch call (pipelined batches)
    g.set_max_batch(512)
    assert L.gg_selftest_fail_next(g._h, 43) == 0
    with pytest.raises(_lib.GimicError, match="code 43"):
        g.jtensor_batch(pts)
    assert rel_max_err(g.jtensor_batch(pts), ref) <= TOL_SPLIT


_TWO_THREADS = textwrap.dedent("""
    import sys, threading
    import numpy as np
    sys.path.insert(0, {root!r}); sys.path.insert(0, {oracle_dir!r})
    import oracle
    from gimic_gb300 import api
    mp, xp = {mp!r}, {xp!r}
    o = oracle.Oracle(mp, xp, screening=1e-8)
    rng = np.random.default_rng(5)
    sets = [np.vstack([rng.uniform(-8, 8, (1500, 3)), o.atoms()[0] + rng.normal(0, 0.1, (12, 3))]) for _ in range(2)]
    refs = [o.jtensor(p) for p in sets]
    start = threading.Barrier(2)
    res = [None, None]
    def work(k):
        start.wait()
        g = api.Gimic(mp, xp, screening=1e-8)       # context creation at the same moment
        res[k] = g.jtensor_batch(sets[k])  # both race on the same kernels' one-time set-up
    th = [threading.Thread(target=work, args=(k,)) for k in range(2)]
    for t in th: t.start()
    for t in th: t.join()
    for k in range(2):
        err = np.abs(res[k] - refs[k]).max() / np.abs(refs[k]).max()
        assert err <= 1e-6, (k, err)
    print("two threads ok")
""")


def test_two_threads_first_calls_at_once(c6h6):
    mp, xp, _ = c6h6
    code = _TWO_THREADS.format(root=ROOT, oracle_dir=os.path.join(ROOT, "oracle"), mp=mp, xp=xp)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "two threads ok" in r.stdout, r.stdout + r.stderr
