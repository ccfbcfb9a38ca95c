import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def cases(tmp_path_factory):
    """Small seeded cases in the reference's input formats, written once per session."""
    from sysu_cfd_parallel_gb300 import meshgen

    root = tmp_path_factory.mktemp("cases")
    made = {}

    def get(name):
        if name in made:
            return made[name]
        d = str(root / name)
        if name == "cavity4":
            p = meshgen.write_case(d, "cavity", n=4, steps=50)
        elif name == "cavity8":
            p = meshgen.write_case(d, "cavity", n=8, steps=50)
        elif name == "cavity8j":
            p = meshgen.write_case(d, "cavity", n=8, jitter=0.1, seed=3, steps=50, mu=0.02)
        elif name == "cavity12":
            p = meshgen.write_case(d, "cavity", n=12, steps=50)
        elif name == "cavity36":  # > 152 * 256 cells: the persistent kernels use every SM
            p = meshgen.write_case(d, "cavity", n=36, steps=50)
        elif name == "channel_tiny":
            p = meshgen.write_case(d, "channel", nx=10, ny=2, nz=2, steps=20)
        elif name == "channel_small":
            p = meshgen.write_case(d, "channel", nx=20, ny=4, nz=4, steps=20)
        else:
            raise KeyError(name)
        made[name] = p
        return p

    return get
