"""FP64 restatement of the property quadratures of the reference's
get_property (src/fgimic/jfield.f90:584-929): nuclear shielding of every
centre and the magnetizability, from current tensors at weighted grid
points, with the positive/negative split and the per-block (per-atom)
decomposition.  Test infrastructure only: tests/test_gpu_parity.py checks
gg_properties against it, with the tensors from the C oracle."""
import numpy as np

C_AU = 137.0359998  # jfield.f90:690


def _jvec(t, a):
    """jvec = matmul(reshape(jtens(:,i), (3,3)), bb) with bb = -e_a."""
    return -t[:, 3 * a:3 * a + 3]


def integrands(jt, pts, centres):
    """Per-point integrands of get_property (jfield.f90:693-711 intsigma,
    :824-842 intchi): (ncentres, N, 3) shielding terms in ppm and (N, 3)
    magnetizability terms."""
    t = np.asarray(jt, dtype=np.float64).reshape(-1, 9)
    pts = np.asarray(pts, dtype=np.float64).reshape(-1, 3)
    j = [_jvec(t, a) for a in range(3)]

    def terms(d, scale):
        return np.stack([scale * (d[:, 1] * j[0][:, 2] - d[:, 2] * j[0][:, 1]),
                         scale * (d[:, 2] * j[1][:, 0] - d[:, 0] * j[1][:, 2]),
                         scale * (d[:, 0] * j[2][:, 1] - d[:, 1] * j[2][:, 0])], axis=1)

    sig = []
    for R in np.asarray(centres, dtype=np.float64).reshape(-1, 3):
        d = pts - R
        f = -1.0 / ((d * d).sum(axis=1) ** 1.5) / C_AU ** 2.0
        sig.append(terms(d, 1.0) * (1.0e6 * f)[:, None])
    return np.asarray(sig), terms(pts, 0.5)


def properties(jt, pts, w, centres, block_npts=None):
    """(sigma (ncentres, nblocks, 5), chi (nblocks, 5)) as gg_properties."""
    t = np.asarray(jt, dtype=np.float64).reshape(-1, 9)
    pts = np.asarray(pts, dtype=np.float64).reshape(-1, 3)
    w = np.asarray(w, dtype=np.float64).reshape(-1)
    n = len(pts)
    sizes = [n] if block_npts is None else [int(v) for v in block_npts]
    off = np.concatenate([[0], np.cumsum(sizes)])
    j = [_jvec(t, a) for a in range(3)]

    def terms(d, scale):
        # intsigma / intchi of jfield.f90:693-711 and :824-842
        return np.stack([scale * (d[:, 1] * j[0][:, 2] - d[:, 2] * j[0][:, 1]),
                         scale * (d[:, 2] * j[1][:, 0] - d[:, 0] * j[1][:, 2]),
                         scale * (d[:, 0] * j[2][:, 1] - d[:, 1] * j[2][:, 0])], axis=1)

    def sums(v):
        out = np.zeros((len(sizes), 5))
        p = v.sum(axis=1)
        for l in range(len(sizes)):
            s = slice(off[l], off[l + 1])
            out[l, :3] = (w[s, None] * v[s]).sum(axis=0)
            pw = p[s] * w[s]
            out[l, 3] = pw[p[s] >= 0.0].sum()
            out[l, 4] = pw[p[s] < 0.0].sum()
        return out

    sig = []
    for R in np.asarray(centres, dtype=np.float64).reshape(-1, 3):
        d = pts - R
        f = -1.0 / ((d * d).sum(axis=1) ** 1.5) / C_AU ** 2.0
        sig.append(sums(terms(d, 1.0) * (1.0e6 * f)[:, None]))
    chi = sums(terms(pts, 0.5))
    return np.asarray(sig), chi
