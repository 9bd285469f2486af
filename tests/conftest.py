import os
import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "tatsy-pppm_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libpppm_gb300.so")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(GOLDEN / f"{name}.npz")
    return load


@pytest.fixture(scope="session")
def ctx():
    import pppm_gb300 as P
    c = P.Context(0)
    yield c
    c.close()


def scene_from(tris, mat_id=None, mats=None, env=None):
    import scenes as S
    tris = np.asarray(tris, np.float32).reshape(-1, 9)
    if mat_id is None:
        mat_id = np.zeros(tris.shape[0], np.int32)
    if mats is None:
        mats = np.array([S.material(S.LAMBERTIAN, (0.5, 0.5, 0.5))], S.MATERIAL_DTYPE)
    cam = S.look_camera((0, 0, -10), (0, 0, 0), 0.8, 8, 8)
    return S.Scene("fixture", tris, np.asarray(mat_id, np.int32), mats, env, cam)
