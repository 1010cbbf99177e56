import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "reference: needs the reference checkout (oracle/_ref)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle.Oracle()


@pytest.fixture(scope="session")
def ref():
    import oracle
    if not oracle.reference_available():
        try:
            oracle.build(reference=None)
        except Exception:
            pass
    if not oracle.reference_available():
        pytest.skip("reference checkout not available here")
    return oracle.Reference()


def load_fixture(name):
    import numpy as np
    z = np.load(GOLDEN / f"{name}.npz")
    return {k: z[k] for k in z.files}


@pytest.fixture(scope="session", params=["spheres64", "terrain64"])
def golden(request):
    return request.param, load_fixture(request.param)


@pytest.fixture(scope="session")
def digests():
    import json
    return json.loads((GOLDEN / "digests.json").read_text())


def subdags_of(fx):
    return [((int(r[0]), int(r[1]), int(r[2])), int(r[3]), int(r[4])) for r in fx["subdags"]]
