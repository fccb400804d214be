"""Measured choice of the launch configuration for batched plane scans.

The contraction's tile (128 points x 224 columns x 64-deep K blocks) is fixed
by the tensor memory and shared memory of one SM, so what is left to choose
at run time is how a batch of molecules is laid out over launches:

  * "batch/cost":  one persistent contraction launch over all molecules,
    the most expensive molecules' tiles first (gg_plane_integrals_batch);
  * "batch/given": the same launch with the molecules in the caller's order;
  * "queued/<n>":  one pass per molecule, all queued on one stream before any
    is collected, with at most n points per device pass
    (gg_plane_integrals_enqueue / _collect, gg_set_max_batch);
  * "sequential":  one blocking call per molecule (gg_plane_integrals), which
    replays each context's captured CUDA graph once its layout repeats.

``tune_scan`` times every candidate on the batch itself (after one warm-up
call, which also builds the device tables and, for the batch forms, captures
the CUDA graph) and returns the fastest.  Choices are remembered per nbf
class of the batch (how many molecules have nbf < 200, < 500 and above), so
later batches of the same make-up reuse the measurement.
"""
import time

from . import api

# the queued forms first: their set_max_batch calls would otherwise make the
# batch forms recapture their graph once more after tuning
CANDIDATES = (("queued", 1 << 21), ("queued", 1 << 20), ("sequential", None), ("batch", "given"), ("batch", "cost"))
_CHOICE = {}


def nbf_class(jobs):
    """The batch's make-up: counts of molecules with nbf < 200, < 500, >= 500."""
    nb = [g.nbf for g, _ in jobs]
    return (sum(n < 200 for n in nb), sum(200 <= n < 500 for n in nb), sum(n >= 500 for n in nb))


def run(jobs, choice, timings=False):
    """One scan step with the given candidate; returns what
    api.plane_integrals_batch / plane_integrals_multi return."""
    mode, arg = choice
    if mode == "batch":
        return api.plane_integrals_batch(jobs, order=arg, timings=timings)
    if mode == "sequential":
        if timings:
            raise ValueError("the sequential layout has no per-molecule stream timings")
        for g, _ in jobs:
            g.set_max_batch(0)  # the library's default pass size
        return [g.plane_integrals(planes) for g, planes in jobs]
    for g, _ in jobs:
        g.set_max_batch(arg)
    return api.plane_integrals_multi(jobs, timings=timings)


def label(choice):
    """'queued/2097152', 'sequential', 'batch/cost', ..."""
    return choice[0] if choice[1] is None else "%s/%s" % choice


def tune_scan(jobs, reps=2, sync=None, candidates=CANDIDATES):
    """Times each candidate on ``jobs`` and returns (best, {candidate: s}).
    ``sync`` (optional) waits for the device between measurements."""
    key = nbf_class(jobs)
    times = {}
    for cand in candidates:
        run(jobs, cand)  # warm-up: tables, scratch, graph capture
        if sync:
            sync()
        t0 = time.perf_counter()
        for _ in range(reps):
            run(jobs, cand)
        if sync:
            sync()
        times[cand] = (time.perf_counter() - t0) / reps
    best = min(times, key=times.get)
    _CHOICE[key] = best
    return best, times


def choice_for(jobs):
    """The remembered choice for a batch of this make-up, or None."""
    return _CHOICE.get(nbf_class(jobs))
