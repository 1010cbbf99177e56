"""The FP32 traversal's distance error against an FP64 exact-box ray cast.

The reference checks its ESVO ray cast against a brute-force tracer with a
0.001 tolerance (test_rendering.cpp:75-80).  Here the FP32 path (the oracle,
bit-identical to the GPU kernels on these rays: tests/golden/digests.json and
test_gpu_parity) is compared with orc_trace_fp64_batch, which intersects the
exact voxel boxes in double precision, over the full spheres-256 camera
(1,048,576 rays).  The relative distance error |d32 - d64| / max(d64, 1) stays
below 1e-7 for 99.9% of the hits; the rays above 1e-5 are grazing rays, where
FP32 decides an edge or corner the other way and so meets a neighbouring voxel
of the same material.  They are counted and listed, not hidden.
"""
import numpy as np

from cubiquity_gb300 import workloads as W

# Rays of the spheres-256 camera above 1e-5 (grazing an edge or corner).
GRAZING = [575227, 650898]


def _rel_error(fp32, fp64):
    both = (fp32["hit"] == 1) & (fp64["hit"] == 1)
    idx = np.nonzero(both)[0]
    d64 = fp64["distance"][both]
    rel = np.abs(fp32["distance"][both].astype(np.float64) - d64) / np.maximum(np.abs(d64), 1.0)
    return idx, rel


def test_spheres256_distance_error_against_fp64(orc):
    nodes, root = W.SPHERES_256.build()
    o, d = W.SPHERES_256_CAMERA.rays()
    sd = orc.find_subdags(nodes, root)
    fp32 = orc.intersect(nodes, sd, o, d)
    fp64 = orc.trace_fp64(nodes, sd, o, d)
    # Same rays hit, with the same material.
    assert np.array_equal(fp32["hit"], fp64["hit"])
    hits = fp32["hit"] == 1
    assert np.array_equal(fp32["material"][hits], fp64["material"][hits])
    idx, rel = _rel_error(fp32, fp64)
    assert idx.size == 395_256
    assert np.quantile(rel, 0.999) < 2e-7
    over = idx[rel > 1e-5].tolist()
    assert over == GRAZING, over
    # The grazing rays still hit a voxel of the same material, a fraction of a voxel away.
    for i in GRAZING:
        assert abs(float(fp32["distance"][i]) - fp64["distance"][i]) < 2.0
