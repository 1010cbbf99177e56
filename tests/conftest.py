import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def _ensure_library():
    """Builds libcbq.so before the test modules import the package, when a
    session starts without it (the package itself refuses to import without
    the library: there is no CPU fallback)."""
    if (ROOT / "cubiquity_gb300" / "libcbq.so").exists():
        return
    import importlib.util
    spec = importlib.util.spec_from_file_location("_cbq_build", ROOT / "cubiquity_gb300" / "_build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()


_ensure_library()


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


def relocate(nodes, root, edge_log2, origin):
    """Moves a scene built at the origin (box [0, 2^edge_log2)^3) so that its
    box starts at `origin` (multiples of 2^edge_log2): re-links the chain of
    single-child nodes between the scene's top node and the root."""
    import numpy as np
    n = nodes.reshape(-1, 8)
    node = int(n[root][7])                      # height 31: unsigned bit 31 set on every axis
    for _ in range(31 - edge_log2):
        node = int(n[node][0])                  # heights 30 .. edge_log2: bits clear
    extra = []
    count = n.shape[0]
    u = [(int(o) + (1 << 31)) & 0xFFFFFFFF for o in origin]
    for hh in range(edge_log2 + 1, 33):
        b = hh - 1
        cid = ((u[0] >> b) & 1) | (((u[1] >> b) & 1) << 1) | (((u[2] >> b) & 1) << 2)
        row = [0] * 8
        row[cid] = node
        extra.append(row)
        node = count + len(extra) - 1
    out = np.concatenate([nodes.reshape(-1), np.array(extra, dtype=np.uint32).reshape(-1)])
    return out, node


def subdags_of(fx):
    return [((int(r[0]), int(r[1]), int(r[2])), int(r[3]), int(r[4])) for r in fx["subdags"]]
