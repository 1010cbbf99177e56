"""Material metadata (.toml) I/O, and the multi-rank (replicas) timing path on
CPU with gloo, world size 2."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT
from cubiquity_gb300 import metadata as md

SAMPLE = """# Dimensions
dimensions = [256, 256, 64]

[[materials]] # Material index 0
name = "EmptySpace"

[[materials]] # Material index 1
name = "Rock"
base_color = [0.5000, 0.4500, 0.4000]

[[materials]] # Material index 2
base_color = [0.1000, 0.8000, 0.1000]
"""


def test_metadata_reads_reference_layout(tmp_path):
    p = tmp_path / "v.toml"
    p.write_text(SAMPLE)
    m = md.load(p)
    assert m.dimensions == (256, 256, 64)
    assert [x.name for x in m.materials] == ["EmptySpace", "Rock", None]
    assert m.materials[0].base_color is None and m.materials[0].color() == md.DEFAULT_COLOR
    assert m.materials[1].base_color == (0.5, 0.45, 0.4)


def test_metadata_round_trip_and_material_table(tmp_path):
    m = md.Metadata((64, 64, 64), [md.Material("a", (0.1, 0.2, 0.3)), md.Material(None, None),
                                   md.Material('q"uote', (1.0, 0.0, 0.5))])
    p = tmp_path / "r.toml"
    md.save(p, m)
    text = p.read_text()
    assert "[[materials]] # Material index 2" in text and "base_color = [0.1000, 0.2000, 0.3000]" in text
    m2 = md.load(p)
    assert m2.dimensions == m.dimensions
    assert [(x.name, x.base_color) for x in m2.materials] == [(x.name, x.base_color) for x in m.materials]
    t = md.material_table(m2, {2: (3.0, 2.0, 1.0)})
    assert t.shape == (256, 2, 3)
    assert np.allclose(t[0, 0], (0.1, 0.2, 0.3)) and np.allclose(t[1, 0], 0.8) and np.allclose(t[2, 1], (3, 2, 1))


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    q.put((rank, bench.max_over_ranks(world, 10.0 * (rank + 1))))
    dist.destroy_process_group()


def test_max_over_ranks_with_gloo():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    assert all(p.exitcode == 0 for p in ps)
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 20.0), (1, 20.0)]


def test_reference_arm_under_torchrun_two_ranks():
    """bench.py --impl reference with 2 ranks: rank 0 alone prints one JSON line;
    the other rank exits 0 without work."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    env = dict(os.environ, PYTHONPATH=str(ROOT))
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
                        "--impl", "reference", "--workload", "spheres-256", "--gpus", "2", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    import json
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["value"] > 0 and j["n_gpus"] == 2
    for key in ("metric", "unit", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling", "vs_baseline",
                "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in j, key
    assert j["config"]["workload"] == "spheres-256" and j["unit"] == "Mrays/s" and j["higher_is_better"] is True
    cb = j["cpu_baseline"]
    assert cb["value"] == j["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    assert j["e2e"] == {"value": j["value"], "unit": j["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


@pytest.mark.parametrize("script", ["bench.py", "__graft_entry__.py"])
def test_entry_scripts_compile_without_warnings(script):
    """The bench and the entry module compile with warnings as errors (a
    SyntaxWarning such as a string literal followed by a parenthesised
    expression is a call that fails only when the line runs)."""
    import warnings
    src = (ROOT / script).read_text()
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        compile(src, script, "exec")
