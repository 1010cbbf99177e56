"""The C++ drop-in shim (include/cubiquity_gb300.hpp) compiled as a user would."""
import subprocess

import numpy as np
import pytest

import cubiquity_gb300 as cbq
from conftest import ROOT, load_fixture

SRC = ROOT / "tests" / "shim_check.cpp"


def compile_shim(tmp_path):
    exe = tmp_path / "shim_check"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(SRC), "-o", str(exe),
           f"-L{cbq.LIB_PATH.parent}", "-lcbq", f"-Wl,-rpath,{cbq.LIB_PATH.parent}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_shim_compiles_and_links(tmp_path):
    assert compile_shim(tmp_path).exists()


@pytest.mark.gpu
def test_shim_results_match_reference_records(tmp_path):
    fx = load_fixture("spheres64")
    exe = compile_shim(tmp_path)
    cbq.save_dag(tmp_path / "v.dag", fx["nodes"], int(fx["root"]))
    rays = np.concatenate([fx["origin_tmax"][:, :3], fx["direction"][:, :3]], axis=1).astype(np.float32)
    rays = rays[:600]
    rays.tofile(tmp_path / "rays.bin")
    subprocess.run([str(exe), str(tmp_path / "v.dag"), str(tmp_path / "rays.bin"), str(tmp_path / "out.bin")],
                   check=True, capture_output=True, text=True, timeout=120)
    rec = np.dtype({"names": ["hit", "distance", "material", "position", "normal"],
                    "formats": [np.uint8, np.float64, np.uint32, (np.float32, 3), (np.float32, 3)],
                    "offsets": [0, 8, 16, 20, 32], "itemsize": 48})
    got = np.fromfile(tmp_path / "out.bin", dtype=rec)
    n = rays.shape[0]
    assert got.shape[0] == n
    assert np.array_equal(got["hit"], fx["surface_hit"][:n])
    assert np.array_equal(got["material"], fx["surface_material"][:n])
    assert np.array_equal(got["distance"], fx["surface_distance"][:n].astype(np.float64))
    assert np.array_equal(got["position"].view(np.uint32), fx["surface_position"][:n].view(np.uint32))
    assert np.array_equal(got["normal"].view(np.uint32), fx["surface_normal"][:n].view(np.uint32))
