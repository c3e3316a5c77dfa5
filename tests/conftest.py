import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def native():
    from zim_gb300 import _build, _lib
    _build.build_all()
    return _lib.load()


@pytest.fixture(scope="session")
def ctx(native):
    from zim_gb300 import api
    return api.Context(0)


_scene_cache = {}


def scene_data(name, **kw):
    """(spec, left frames, right frames, left ground-truth xyz) -- cached per session."""
    key = (name, tuple(sorted(kw.items())))
    if key not in _scene_cache:
        from zim_gb300 import synth
        spec = getattr(synth, name)(**kw)
        L, gt = spec.render(0, with_xyz=True)
        R = spec.render(1)
        _scene_cache[key] = (spec, L, R, gt)
    return _scene_cache[key]


SMALL_SCENES = [
    ("config0", {}),
    ("config1", {"width": 612, "height": 512}),
    ("ref_heterodyne", {"width": 612, "height": 512}),
]
