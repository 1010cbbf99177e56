"""The wavefront pathtracer (cbq_pathtrace): every traversal it issues (camera,
bounce and shadow rays, with the LOD footprint) is checked bit for bit against
the oracle on the same rays, and frames are reproducible."""
import numpy as np
import pytest

import cubiquity_gb300 as cbq
import oracle
from cubiquity_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def city():
    torch.cuda.set_device(0)
    spec = W.SceneSpec(cbq.SCENE_CITY, 9, 31337)
    nodes, root = spec.build()
    return nodes, root, cbq.Dag(nodes, root)


def test_every_wave_matches_the_oracle(city, orc):
    nodes, root, dag = city
    eye, target = W.city_camera(9)
    rec = cbq.WaveRecorder()
    image, stats = cbq.pathtrace(dag, 64, 40, 2, 4, eye, target, W.city_materials(), max_footprint=0.0035,
                                 seed=5, on_wave=rec)
    kinds = {k for k, *_ in rec.waves}
    assert kinds == {0, 1}
    assert max(dp for _, dp, *_ in rec.waves) >= 2  # bounces happened
    assert sum(w[3].shape[0] for w in rec.waves if w[0] == 0) == stats["extension_rays"]
    assert sum(w[3].shape[0] for w in rec.waves if w[0] == 1) == stats["shadow_rays"]
    sd = orc.find_subdags(nodes, root)
    checked = 0
    for kind, depth, sample, o, d, hits, (cs, mf) in rec.waves:
        want = orc.intersect(nodes, sd, o, d, cs, mf)
        for k, v in hits.items():
            w = want[k]
            assert oracle.same_bits_nan_equal(v.astype(w.dtype) if k == "material" else v, w), \
                f"wave kind={kind} depth={depth} sample={sample}: {k}"
        checked += o.shape[0]
    assert checked == stats["extension_rays"] + stats["shadow_rays"]
    img = image.cpu().numpy()
    assert np.isfinite(img).all() and img.max() > 0


def test_frames_are_reproducible(city):
    nodes, root, dag = city
    eye, target = W.city_camera(9)
    a, _ = cbq.pathtrace(dag, 48, 32, 3, 3, eye, target, W.city_materials(), seed=9)
    b, _ = cbq.pathtrace(dag, 48, 32, 3, 3, eye, target, W.city_materials(), seed=9)
    c, _ = cbq.pathtrace(dag, 48, 32, 3, 3, eye, target, W.city_materials(), seed=10)
    # Float atomics accumulate in a different order from run to run: equal to rounding.
    assert torch.allclose(a, b, rtol=1e-5, atol=1e-6)
    assert not torch.allclose(a, c, rtol=1e-3, atol=1e-3)


def test_emissive_materials_light_the_image(city):
    nodes, root, dag = city
    eye, target = W.city_camera(9)
    mats = W.city_materials()
    dark = mats.copy()
    dark[:, 1] = 0.0
    a, _ = cbq.pathtrace(dag, 32, 24, 2, 2, eye, target, mats, seed=3)
    b, _ = cbq.pathtrace(dag, 32, 24, 2, 2, eye, target, dark, seed=3)
    assert (a >= b - 1e-4).all() and a.sum() >= b.sum()
