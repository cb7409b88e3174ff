import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (the GB300 host); calls the CUDA library")


def has_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def load_golden(name: str):
    """Inputs and expected results of a golden case.

    Returns dict(meshes=[Mesh...], pairs=array or None, frames=[[xyz per mesh], ...],
    hits=[sorted uint32[n,4] per frame], candidates=[int per frame]).
    """
    from cases import CASES, REGENERATED
    from oibvh_gb300.meshes import Mesh, mesh_digest

    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    n = int(z["n_meshes"])
    if name in REGENERATED:
        meshes = CASES[name]()["meshes"]
    else:
        meshes = [Mesh(z[f"xyz_{i}"], z[f"tri_{i}"]) for i in range(n)]
    for i, m in enumerate(meshes):
        want = z[f"digest_{i}"].item().decode()
        assert mesh_digest(m.xyz, m.tri) == want, f"{name}: input mesh {i} differs from the fixture"
    nf = int(z["n_frames"])
    frames = [[z[f"frame{f}_xyz_{i}"] for i in range(n)] for f in range(1, nf)]
    return dict(
        meshes=meshes,
        pairs=z["pairs"] if "pairs" in z else None,
        frames=frames,
        hits=[z[f"hits_{f}"] for f in range(nf)],
        candidates=[int(z[f"candidates_{f}"]) for f in range(nf)],
    )


@pytest.fixture(scope="session")
def gpu():
    """Skip unless a GPU is visible; make sure the CUDA library is built and loaded."""
    if not has_gpu():
        pytest.skip("no CUDA device")
    from oibvh_gb300 import _native

    return _native.lib()
