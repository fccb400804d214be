import lzma
import os
import shutil
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden_dir(tmp_path_factory):
    """Decompressed copies of the reference test inputs (MOL, XDENS, grid)."""
    d = tmp_path_factory.mktemp("golden")
    for case in ("c4h4", "open-shell"):
        os.makedirs(d / case)
        shutil.copy(os.path.join(GOLDEN, case, "MOL"), d / case / "MOL")
        with lzma.open(os.path.join(GOLDEN, case, "XDENS.xz"), "rb") as f, open(d / case / "XDENS", "wb") as g:
            shutil.copyfileobj(f, g)
        for name in os.listdir(os.path.join(GOLDEN, case)):
            if name.endswith(".inp"):
                shutil.copy(os.path.join(GOLDEN, case, name), d / case / name)
    with lzma.open(os.path.join(GOLDEN, "c4h4", "gridfile.grd.xz"), "rb") as f, \
            open(d / "c4h4" / "gridfile.grd", "wb") as g:
        shutil.copyfileobj(f, g)
    return d


@pytest.fixture(scope="session")
def synth_dir(tmp_path_factory):
    return tmp_path_factory.mktemp("synth")


@pytest.fixture(scope="session")
def c6h6(synth_dir):
    from gimic_gb300 import synth
    return synth.make_workload("c6h6", str(synth_dir), seed=2024)


@pytest.fixture(scope="session")
def c6h6_uhf(synth_dir):
    from gimic_gb300 import synth
    return synth.make_workload("c6h6", str(synth_dir), seed=77, uhf=True)


def sample_points(coords, n_random, n_near, half, seed=0):
    """Random points in a cube plus points within ~0.15 Bohr of nuclei (where
    |j| peaks, so the max-normalised error is dominated there)."""
    rng = np.random.default_rng(seed)
    pts = rng.uniform(-half, half, (n_random, 3))
    near = coords[rng.integers(0, len(coords), n_near)] + rng.normal(0.0, 0.15, (n_near, 3))
    return np.vstack([pts, near])


def rel_max_err(a, b):
    """e_j: max |a - b| over all points and components / max |b|."""
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())
