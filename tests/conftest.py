import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI of libmcrt_cuda.so)")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def mcrt():
    import mcrt_gb300
    mcrt_gb300.lib()
    return mcrt_gb300


@pytest.fixture(scope="session")
def ctx(mcrt):
    c = mcrt.Context(0)
    yield c
    c.close()


GOLDEN = os.path.join(ROOT, "tests", "golden")


def golden(name):
    return os.path.join(GOLDEN, name)


def load_fixture_scene(name):
    """A regression scene loaded by the product's YAML loader and frozen as arrays."""
    import mcrt_gb300 as m
    z = np.load(golden(f"scene_{name}.npz"), allow_pickle=False)
    d = {k: z[k] for k in z.files}
    out = dict(spheres=d["spheres"].view(m.SPHERE).reshape(-1), vertices=d["vertices"].view(m.VERTEX).reshape(-1),
               triangles=d["triangles"].view(m.TRIANGLE).reshape(-1),
               materials=d["materials"].view(m.MATERIAL_DATA).reshape(()), camera=d["camera"].view(m.CAMERA).reshape(()),
               width=int(d["render"][0]), height=int(d["render"][1]), spp=int(d["render"][2]),
               threshold_mse=float(d["thresholds"][0]), threshold_psnr=float(d["thresholds"][1]))
    return out
