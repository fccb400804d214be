"""gg_jtensor_batch_noalloc: the evaluation entry point for callers that
cannot let the library allocate device memory (applications that budget all
device memory themselves, or loops that must not stall on cudaMalloc /
cudaFree).  Its results must match gg_jtensor_batch, call after call, while
the scratch lives in a fixed static device array.

The file name makes pytest collect it last; it also passes on its own in a
fresh process (it builds its own inputs)."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_max_err, sample_points
from gimic_gb300 import _lib, api

pytestmark = pytest.mark.gpu

TOL = 1e-6  # the split-path tolerance of the parity tests


def _call(g, pts, n, jt, rho, dv):
    return g._L.gg_jtensor_batch_noalloc(g._h, C.c_void_p(pts.data_ptr()), n, C.c_void_p(jt.data_ptr()),
                                         C.c_void_p(rho.data_ptr()), C.c_void_p(dv.data_ptr()), None)


def test_noalloc_matches_allocating_entry_point(c6h6):
    torch = pytest.importorskip("torch")
    mp, xp, _ = c6h6
    g = api.Gimic(mp, xp, screening=1e-8, precision="split16")
    L = _lib.load()
    coords = g.atoms()[0]
    first = torch.as_tensor(sample_points(coords, 2500, 300, 8.0, seed=21), device="cuda")
    second = torch.as_tensor(sample_points(coords, 700, 100, 6.0, seed=22), device="cuda")

    # before preparation the entry point refuses (preparing would allocate)
    out = [torch.empty((len(first), k), dtype=torch.float64, device="cuda") for k in (9, 1, 3)]
    assert _call(g, first, len(first), *out) == -1
    assert b"not prepared" in L.gg_last_error(g._h)

    refs = [g.jtensor_batch(p, rho=True, divj=True) for p in (first, second)]  # prepares the context
    for call, (pts, ref) in enumerate(zip((first, second), refs)):
        n = len(pts)
        jt = torch.full((n, 9), float("nan"), dtype=torch.float64, device="cuda")
        rho = torch.full((n, 1), float("nan"), dtype=torch.float64, device="cuda")
        dv = torch.full((n, 3), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        assert _call(g, pts, n, jt, rho, dv) == 0, L.gg_last_error(g._h)
        torch.cuda.synchronize()
        if call == 1:
            # (the first call may load the module that holds the static array)
            assert torch.cuda.mem_get_info()[0] == free_before
        assert rel_max_err(jt.cpu().numpy(), ref[0].cpu().numpy()) <= TOL
        assert rel_max_err(rho.cpu().numpy()[:, 0], ref[1].cpu().numpy()) <= TOL
        assert rel_max_err(dv.cpu().numpy(), ref[2].cpu().numpy()) <= 1e-5


def test_noalloc_rejects_oversized_and_host_buffers(c6h6):
    torch = pytest.importorskip("torch")
    mp, xp, _ = c6h6
    g = api.Gimic(mp, xp, screening=1e-8, precision="split16")
    L = _lib.load()
    small = torch.zeros((4, 3), dtype=torch.float64, device="cuda")
    g.jtensor_batch(small)
    # nbf 120 -> kpad 128: (32 MiB - 768) / (4 * 128 + 4) = 65,026 points at most
    n = 65027
    big = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    jt = torch.empty((n, 9), dtype=torch.float64, device="cuda")
    rc = g._L.gg_jtensor_batch_noalloc(g._h, C.c_void_p(big.data_ptr()), n, C.c_void_p(jt.data_ptr()), None, None,
                                       None)
    assert rc == -1 and b"exceed its limit of 65026 points" in L.gg_last_error(g._h)
    host = np.zeros((4, 3))
    hjt = np.zeros((4, 9))
    rc = g._L.gg_jtensor_batch_noalloc(g._h, C.c_void_p(host.ctypes.data), 4, C.c_void_p(hjt.ctypes.data), None,
                                       None, None)
    assert rc == -1 and b"device pointers only" in L.gg_last_error(g._h)
