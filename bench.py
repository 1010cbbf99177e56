"""Benchmark: sparse-voxel-DAG ray traversal throughput on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload terrain-4096|spheres-256] [--kernel plain|persistent]

Workload (default terrain-4096): the seeded 4096^3 terrain DAG; one step traces
4,194,304 primary rays (2048x2048 pinhole) and 4,194,304 cosine-weighted bounce
rays from the primary hits, i.e. two traversal launches over 8,388,608 rays.
Inputs are resident in HBM before timing; the ray and hit arrays (654 MB per
step) exceed the 129 MB L2, so each step streams them; the 115 MB DAG is the
traversal's working set and stays in L2.

`value` is device throughput (CUDA events on the launching stream); `e2e` is the
same workload through the host-buffer C ABI (cbq_intersect_host) with pinned
host rays in and hits out, copies inside the timed region.

Multi-GPU (torchrun, N > 1): replicas only.  Rays are independent and the DAG is
read-only, so every rank traces its own full replica; there is no data-path
collective, only the timing barrier and a max-over-ranks of the elapsed time.

--impl reference times the reference's CPU ray cast on the host cores on the
same workload: the reference's own library (oracle/_ref, where it could be
compiled from the reference checkout) or else the oracle's C restatement of it.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

HIT_BYTES = 1 + 4 + 4 + 12 + 12 + 12 + 1  # hit, distance, material, position, normal, voxel, status
REF_HIT_BYTES = 1 + 4 + 4 + 12 + 12  # the reference's result fields only
RAY_BYTES = 32
SECTOR = 32


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--workload", choices=["terrain-4096", "spheres-256", "batch-64", "serve-8", "city-8192"],
                   default="terrain-4096")
    p.add_argument("--kernel", choices=["auto", "flat", "nested"], default="auto")
    p.add_argument("--form", choices=["tuned", "persistent", "plain"], default="tuned",
                   help="tuned: the autotuner's choice per batch (form, block, refill, stack); persistent: grid "
                        "pulling rays from a work counter; plain: one thread per ray")
    p.add_argument("--block", type=int, default=0)
    p.add_argument("--chunk", type=int, default=0, help="persistent: refill threshold (flat) / grab size (nested)")
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--layout", choices=["reference", "compact"], default="reference",
                   help="device node store: the reference's array, or the compact store (occupied children only)")
    p.add_argument("--serve-inflight", type=int, default=8, help="serve-8: launches in flight")
    p.add_argument("--serve-batch-rays", type=int, default=4 << 20, help="serve-8: rays per launch at most")
    p.add_argument("--serve-buffers", choices=["staged", "in-place"], default="staged",
                   help="serve-8: stage requests through device memory with copies, or traverse the page-locked "
                        "request buffers in place")
    args = p.parse_args()
    args.persistent = args.form == "persistent"
    return args


# ------------------------------------------------------------------ workload

def make_workload(name: str):
    """Returns (nodes, root, [(label, origin_tmax, direction), ...])."""
    import cubiquity_gb300 as cbq
    from cubiquity_gb300 import workloads as W

    if name == "spheres-256":
        nodes, root = W.SPHERES_256.build()
        o, d = W.SPHERES_256_CAMERA.rays()
        return nodes, root, [("primary", o, d)], None
    nodes, root = W.TERRAIN_4096.build()
    o, d = W.TERRAIN_4096_CAMERA.rays()
    return nodes, root, [("primary", o, d)], "bounce"


def bounce_batch(dag, o, d):
    """Bounce rays from the primary hits (traced once on the GPU during set-up)."""
    import torch
    import cubiquity_gb300 as cbq
    from cubiquity_gb300 import workloads as W

    out = cbq.intersect_volume(dag, torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda())
    torch.cuda.synchronize()
    bo, bd = W.bounce_from_hits(out, o.shape[0])
    return bo, bd


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ helpers

def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            j = json.loads(p.read_text())
            return float(j["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def profiled_traffic(workload: str):
    """DRAM bytes per launch from the committed ncu summary, if one exists."""
    f = ROOT / "profiles" / f"traverse_{workload}.md"
    if not f.exists():
        return None
    m = re.search(r"dram_bytes_per_ray:\s*([0-9.]+)", f.read_text())
    return float(m.group(1)) if m else None


def profiled_issue_active(workload: str):
    """smsp__issue_active (% of issue slots) of the traversal from the committed ncu summary."""
    f = ROOT / "profiles" / f"traverse_{workload}.md"
    if not f.exists():
        return None
    m = re.search(r"\| smsp__issue_active \| ([0-9.]+)%", f.read_text())
    return float(m.group(1)) if m else None


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "gb300" else "gloo"
        if args.impl == "gb300":
            import torch
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value: float) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ CPU arms

def cpu_trace(nodes, root, batches, threads=0):
    """Times the reference CPU ray cast over the batches; returns (seconds, kind)."""
    import oracle

    if oracle.reference_available():
        ref = oracle.Reference()
        vol = ref.volume_from_nodes(nodes, root)
        sd = vol.find_subdags()
        t0 = time.perf_counter()
        for _, o, d in batches:
            vol.intersect(sd, o, d, True, -1.0, threads)
        return time.perf_counter() - t0, "reference"
    orc = oracle.Oracle()
    sd = orc.find_subdags(nodes, root)
    t0 = time.perf_counter()
    for _, o, d in batches:
        orc.intersect(nodes, sd, o, d, True, -1.0, threads=threads)
    return time.perf_counter() - t0, "port"


def host_cpu() -> str:
    """The host CPU's model (for the CPU baseline record)."""
    import platform
    try:
        info = Path("/proc/cpuinfo").read_text()
    except OSError:
        return platform.machine()
    m = re.search(r"^model name\s*:\s*(.+)$", info, re.M)
    if m:
        return m.group(1).strip()
    part = re.search(r"^CPU part\s*:\s*(\S+)$", info, re.M)
    names = {"0xd4f": "Arm Neoverse V2 (NVIDIA Grace)"}
    return names.get(part.group(1), f"{platform.machine()} CPU part {part.group(1)}") if part else platform.machine()


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args, world, rank):
    if rank != 0:
        return
    nodes, root, batches, bounce = make_workload(args.workload)
    if bounce:
        import oracle
        orc = oracle.Oracle()
        prim = orc.intersect(nodes, orc.find_subdags(nodes, root), batches[0][1], batches[0][2])
        from cubiquity_gb300 import workloads as W
        bo, bd = W.bounce_from_hits(prim, batches[0][1].shape[0])
        batches.append(("bounce", bo, bd))
    rays = sum(b[1].shape[0] for b in batches)
    for _ in range(args.warmup):
        cpu_trace(nodes, root, batches)
    total = 0.0
    kind = "port"
    for _ in range(args.steps):
        dt, kind = cpu_trace(nodes, root, batches)
        total += dt
    value = rays * args.steps / total / 1e6
    cores = host_cores()
    line = {
        "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene, generated rays)",
        "impl": "reference",
        "config": {"workload": args.workload, "rays_per_step": rays},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": cores, "cpu": host_cpu(), "kind": kind,
                         "sample": f"full workload ({rays} rays) per step, intersectVolume with "
                                   f"computeSurfaceProperties=true on {cores} host threads"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


LAYOUTS = {"reference": 0, "compact": 1}  # CBQ_DAG_LAYOUT_*


# ------------------------------------------------------------------ GPU arm

def run_gpu(args, world, rank, local):
    import torch
    import cubiquity_gb300 as cbq

    torch.cuda.set_device(local)
    nodes, root, batches, bounce = make_workload(args.workload)
    dag = cbq.Dag(nodes, root, LAYOUTS[args.layout])
    kernel_id = {"auto": cbq.KERNEL_AUTO, "flat": cbq.KERNEL_FLAT, "nested": cbq.KERNEL_NESTED}[args.kernel]
    dag.set_launch_config(kernel_id, args.block, args.chunk if not args.persistent else 0, 0)
    cfg = dag.launch_config()
    kernel_name = ("cbq_k_flat" if cfg["kernel"] == cbq.KERNEL_FLAT else
                   ("cbq_k_intersect_persistent" if args.persistent else "cbq_k_intersect_plain"))
    if bounce:
        bo, bd = bounce_batch(dag, batches[0][1], batches[0][2])
        batches.append(("bounce", bo, bd))
    stream = torch.cuda.current_stream()
    dev_batches = []
    for label, o, d in batches:
        to = torch.from_numpy(o).cuda()
        td = torch.from_numpy(d).cuda()
        out = cbq.alloc_hits(o.shape[0])
        f = cbq.count_fetches(dag, to, td).double().mean().item()
        dev_batches.append((label, to, td, out, f))
    counter = torch.zeros(1, dtype=torch.int64, device="cuda")
    rays_per_step = sum(b[1].shape[0] for b in dev_batches)
    tuned = {}
    if args.form == "tuned":
        from cubiquity_gb300 import autotune
        scratch = cbq.scratch_for(max(b[1].shape[0] for b in dev_batches))
        for label, to, td, out, _ in dev_batches:
            tuned[label] = autotune.tune(dag, to, td, scratch, out, stream=stream)
        torch.cuda.synchronize()

    def launch(label, to, td, out):
        if tuned:
            c = tuned[label]
            dag.set_launch_config(c["kernel"], c["block"], c["chunk"], c["refill_min"], c["stack"], c["form"],
                                  c.get("steps", 1), c.get("registers", 0))
            cbq.intersect_auto(dag, to, td, scratch, out=out, stream=stream)
        elif args.persistent:
            cbq.intersect_volume_persistent(dag, to, td, counter, chunk=args.chunk, out=out, stream=stream)
        else:
            cbq.intersect_volume(dag, to, td, out=out, stream=stream)

    def step(events=None):
        for i, (label, to, td, out, _) in enumerate(dev_batches):
            if events is not None:
                events[i][0].record(stream)
            launch(label, to, td, out)
            if events is not None:
                events[i][1].record(stream)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    per_launch = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in dev_batches] for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for k in range(args.steps):
        step(per_launch[k])
    t1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    elapsed_ms = max_over_ranks(world, t0.elapsed_time(t1))
    value = rays_per_step * args.steps * world / (elapsed_ms * 1e-3) / 1e6

    launch_ms = {b[0]: float(np.mean([per_launch[k][i][0].elapsed_time(per_launch[k][i][1])
                                      for k in range(args.steps)])) for i, b in enumerate(dev_batches)}

    # Roofline of the traversal kernel: algorithmic bytes per launch / launch time.
    peak, peak_kind = measured_peaks()
    alg_bytes = {b[0]: b[1].shape[0] * (RAY_BYTES + b[4] * SECTOR + HIT_BYTES) for b in dev_batches}
    tot_bytes = sum(alg_bytes.values())
    tot_ms = sum(launch_ms.values())
    achieved = tot_bytes / (tot_ms * 1e-3) / 1e9
    l2_stream, l2_rand = cbq.measure_l2(64 << 20, 20)
    sectors = sum(b[1].shape[0] * b[4] for b in dev_batches)
    sector_rate = sectors / (tot_ms * 1e-3) / 1e9
    traffic_per_ray = profiled_traffic(args.workload)
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
        "peak_source": f"{peak_kind} hbm_gbs", "kernel": kernel_name,
        "traffic": None if traffic_per_ray is None else traffic_per_ray * rays_per_step / len(dev_batches),
        "limiter": {"kind": "instruction issue (dependent node fetches are served from L2)",
                    "issue_active_pct": profiled_issue_active(args.workload), "source": "ncu --set full"},
        "bytes_per_ray": {b[0]: RAY_BYTES + b[4] * SECTOR + HIT_BYTES for b in dev_batches},
        "fetches_per_ray": {b[0]: b[4] for b in dev_batches},
        "l2": {"achieved_gbs": achieved, "stream_peak_gbs": l2_stream, "frac_stream": achieved / l2_stream,
               "sector_rate_gsps": sector_rate, "random_sector_peak_gsps": l2_rand,
               "frac_sector": sector_rate / l2_rand, "peak_source": "cbq_measure_l2 (this run)"},
    }

    # End to end through the host-buffer C ABI, pinned host memory, copies inside.
    host = []
    for label, o, d in batches:
        po = torch.from_numpy(o).pin_memory()
        pd = torch.from_numpy(d).pin_memory()
        n = o.shape[0]
        # The reference's RayVolumeIntersection fields (raytracing.h:48-55): what a drop-in
        # caller receives.  voxel and status are extra outputs it does not have.
        outs = {"hit": torch.empty(n, dtype=torch.uint8).pin_memory(),
                "distance": torch.empty(n, dtype=torch.float32).pin_memory(),
                "material": torch.empty(n, dtype=torch.int32).pin_memory(),
                "position": torch.empty((n, 3), dtype=torch.float32).pin_memory(),
                "normal": torch.empty((n, 3), dtype=torch.float32).pin_memory()}
        host.append((label, po.numpy(), pd.numpy(), {k: v.numpy() for k, v in outs.items()}))

    def e2e_step():
        for label, po, pd, outs in host:
            if tuned:  # the launch shape tuned for this batch, as a caller who tuned would set it
                c = tuned[label]
                dag.set_launch_config(c["kernel"], c["block"], c["chunk"], c["refill_min"], c["stack"], c["form"],
                                      c.get("steps", 1), c.get("registers", 0))
            cbq.intersect_volume_host(dag, po, pd, out=outs)

    e2e_step()
    barrier(world)
    t = time.perf_counter()
    for _ in range(args.e2e_steps):
        e2e_step()
    e2e_s = max_over_ranks(world, time.perf_counter() - t)
    e2e_value = rays_per_step * args.e2e_steps * world / e2e_s / 1e6

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        dt, kind = cpu_trace(nodes, root, batches)
        cores = host_cores()
        cpu = {"value": rays_per_step / dt / 1e6, "unit": "Mrays/s", "cores": cores, "cpu": host_cpu(), "kind": kind,
               "sample": f"one pass over the full workload ({rays_per_step} rays), {cores} host threads"}

    launches = args.steps * len(dev_batches)
    line = {
        "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene built by libcbq, generated rays)",
        "config": {"workload": args.workload, "rays_per_step": rays_per_step, "kernel": kernel_name,
                   "form": args.form, "launch_config": tuned if tuned else cfg,
                   "batches": {b[0]: int(b[1].shape[0]) for b in dev_batches},
                   "dag_nodes": int(dag.node_count), "dag_bytes": int(dag.bytes),
                   "layout": args.layout, "device_node_bytes": int(dag.device_bytes),
                   "l2": "inputs larger than L2 (rays + hits %.0f MB per step); DAG read through L2"
                         % (rays_per_step * (RAY_BYTES + HIT_BYTES) / 1e6),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "breakdown_mrays": {lbl: b[1].shape[0] / (ms * 1e-3) / 1e6 for (lbl, ms), b in
                            zip(launch_ms.items(), dev_batches)},
        "launch_ms": launch_ms,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": rays_per_step * RAY_BYTES,
                "d2h_bytes_per_step": rays_per_step * REF_HIT_BYTES,
                "api": "cbq_intersect_host (pinned host buffers, copies pipelined with the traversal inside)",
                "fields": "hit, distance, material, position, normal (the reference's RayVolumeIntersection)"},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    dag.destroy()


def batch_jobs():
    """The 64-volume batching workload as [(nodes, root, origin_tmax, direction)]."""
    from cubiquity_gb300 import workloads as W

    jobs = []
    for v in W.batch_volumes():
        nodes, root = v.scene.build()
        o, d = v.make_rays()
        jobs.append((nodes, root, o, d))
    return jobs


def run_reference_batch(args, world, rank):
    if rank != 0:
        return
    import oracle

    jobs = batch_jobs()
    rays = sum(j[2].shape[0] for j in jobs)
    use_ref = oracle.reference_available()
    if use_ref:
        ref = oracle.Reference()
        vols = [ref.volume_from_nodes(n, r) for n, r, _, _ in jobs]
        sds = [v.find_subdags() for v in vols]
    else:
        orc = oracle.Oracle()
        sds = [orc.find_subdags(n, r) for n, r, _, _ in jobs]

    def step():
        t0 = time.perf_counter()
        for k, (n, r, o, d) in enumerate(jobs):
            if use_ref:
                vols[k].intersect(sds[k], o, d, True, -1.0)
            else:
                orc.intersect(n, sds[k], o, d, True, -1.0)
        return time.perf_counter() - t0

    for _ in range(args.warmup):
        step()
    total = sum(step() for _ in range(args.steps))
    value = rays * args.steps / total / 1e6
    cores = host_cores()
    kind = "reference" if use_ref else "port"
    print(json.dumps({
        "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (64 seeded volumes, generated rays)",
        "impl": "reference", "config": {"workload": "batch-64", "rays_per_step": rays, "volumes": len(jobs)},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": cores, "cpu": host_cpu(), "kind": kind,
                         "sample": f"all 64 volumes ({rays} rays) per step on {cores} host threads"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}), flush=True)


def run_gpu_batch(args, world, rank, local):
    """batch-64: many volumes of uneven size in one persistent, graph-captured,
    autotuned launch, against the plain kernel launched once per volume."""
    import torch
    import cubiquity_gb300 as cbq

    torch.cuda.set_device(local)
    host_jobs = batch_jobs()
    dags = [cbq.Dag(n, r, LAYOUTS[args.layout]) for n, r, _, _ in host_jobs]
    dev = [(torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()) for _, _, o, d in host_jobs]
    rays_per_step = sum(o.shape[0] for o, _ in dev)
    stream = torch.cuda.current_stream()
    plain_out = [cbq.alloc_hits(o.shape[0]) for o, _ in dev]
    batch = cbq.Batch([(g, o, d) for g, (o, d) in zip(dags, dev)])
    tuned = batch.autotune(3, stream=stream)

    def plain_step():
        for g, (o, d), out in zip(dags, dev, plain_out):
            cbq.intersect_volume(g, o, d, out=out, stream=stream)

    def batched_step():
        batch.launch(stream=stream)

    def timed(fn, steps):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        return max_over_ranks(world, e0.elapsed_time(e1))

    plain_ms = timed(plain_step, args.steps)
    clocks = ClockSampler(local)
    clocks.start()
    batched_ms = timed(batched_step, args.steps)
    clk = clocks.stop()
    # Same answers from both forms.
    for out_b, out_p in zip(batch.outputs, plain_out):
        for k in ("hit", "material", "voxel", "distance", "status"):
            if not torch.equal(out_b[k], out_p[k]):
                raise SystemExit(f"batched and plain results differ in {k}")
    value = rays_per_step * args.steps * world / (batched_ms * 1e-3) / 1e6
    plain_value = rays_per_step * args.steps * world / (plain_ms * 1e-3) / 1e6

    # Roofline of the batched launch.
    fetches = sum(cbq.count_fetches(g, o, d).double().sum().item() for g, (o, d) in zip(dags, dev))
    peak, peak_kind = measured_peaks()
    step_s = batched_ms / args.steps * 1e-3
    alg_bytes = rays_per_step * (RAY_BYTES + HIT_BYTES) + fetches * SECTOR
    achieved = alg_bytes / step_s / 1e9
    l2_stream, l2_rand = cbq.measure_l2(64 << 20, 20)

    # End to end from host buffers: each step submits the 64 volumes' pinned rays to the request
    # server as one request each and waits for all hits (the reference's result fields) in host
    # memory; the server overlaps each group's copies with other groups' traversals.
    ref_fields = ("hit", "distance", "material", "position", "normal")
    pinned_in = [(torch.from_numpy(o).pin_memory().numpy(), torch.from_numpy(d).pin_memory().numpy())
                 for _, _, o, d in host_jobs]
    pinned_out = [{k: torch.from_numpy(v).pin_memory().numpy() for k, v in cbq.alloc_host_hits(o.shape[0]).items()
                   if k in ref_fields} for o, _ in pinned_in]
    server = cbq.Server(device_memory_budget=4 << 30, max_inflight_launches=8, max_batch_requests=64,
                        max_batch_rays=1 << 20)

    def e2e_step():
        tickets = [server.submit(g, po, pd, queries_batch, out=out)[0]
                   for g, (po, pd), out in zip(dags, pinned_in, pinned_out)]
        for t_ in tickets:
            server.wait(t_)

    queries_batch = cbq.Query()
    e2e_step()
    server.reset_stats()
    t = time.perf_counter()
    for _ in range(args.e2e_steps):
        e2e_step()
    e2e_value = rays_per_step * args.e2e_steps * world / max_over_ranks(world, time.perf_counter() - t) / 1e6
    e2e_launches = server.stats()["launches"]
    server.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        orc = oracle.Oracle()
        t0 = time.perf_counter()
        for n, r, o, d in host_jobs:
            orc.intersect(n, orc.find_subdags(n, r), o, d)
        dt = time.perf_counter() - t0
        cpu = {"value": rays_per_step / dt / 1e6, "unit": "Mrays/s", "cores": host_cores(), "cpu": host_cpu(), "kind": "port",
               "sample": f"one pass over all 64 volumes ({rays_per_step} rays), {host_cores()} host threads"}
    batch_traffic = profiled_traffic("batch-64")  # DRAM bytes per ray, one launch (ncu)
    line = {
        "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": batched_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (64 seeded sphere/terrain volumes, edges 2^7..2^11, generated rays)",
        "config": {"workload": "batch-64", "volumes": len(dags), "rays_per_step": rays_per_step,
                   "dag_bytes": int(sum(g.bytes for g in dags)), "layout": args.layout,
                   "device_node_bytes": int(sum(g.device_bytes for g in dags)), "batch_config": tuned,
                   "form": "one persistent launch replayed from a CUDA graph",
                   "l2": "inputs larger than L2 (rays + hits %.0f MB per step)" % (rays_per_step * 78 / 1e6)},
        "plain": {"value": plain_value, "unit": "Mrays/s", "ms_per_step": plain_ms / args.steps,
                  "form": "cbq_intersect once per volume (64 launches per step)"},
        "batched_over_plain": value / plain_value,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": f"{peak_kind} hbm_gbs", "kernel": "cbq_k_flat_batch",
                     "traffic": None if batch_traffic is None else batch_traffic * rays_per_step,
                     "limiter": {"kind": "instruction issue", "issue_active_pct": profiled_issue_active("batch-64"),
                                 "source": "ncu --set full"},
                     "fetches_per_ray": fetches / rays_per_step,
                     "l2": {"stream_peak_gbs": l2_stream, "frac_stream": achieved / l2_stream,
                            "sector_rate_gsps": fetches / step_s / 1e9, "random_sector_peak_gsps": l2_rand}},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": rays_per_step * RAY_BYTES,
                "d2h_bytes_per_step": rays_per_step * REF_HIT_BYTES,
                "api": "cbq_server_submit/wait, one request per volume (pinned host buffers)",
                "fields": "hit, distance, material, position, normal (the reference's RayVolumeIntersection)",
                "launches_per_step": e2e_launches / args.e2e_steps},
        "gpu_launches": args.steps,
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_gpu_serve(args, world, rank, local):
    """serve-8: 8 resident terrain DAGs (edges 1024-4096); requests of 1k-256k
    rays (log-uniform), 70% tmax-bounded collision rays and 30% view rays.
    Finds the peak request rate closed-loop, then drives an open-loop Poisson
    stream at half of it and reports p50/p99 latency (submit -> hits in host
    memory, timed by the server) and Mrays/s."""
    import random
    import threading
    import torch
    import cubiquity_gb300 as cbq
    from cubiquity_gb300 import workloads as W

    # The generator spins on the clock while the waiter thread blocks in the
    # library: a short switch interval keeps the spinning thread from holding
    # the GIL for whole 5 ms slices, which would make arrivals bursty.
    sys.setswitchinterval(5e-5)
    torch.cuda.set_device(local)
    scenes = W.serve_volumes()
    dags, pools = [], []
    for i, s in enumerate(scenes):
        nodes, root = s.build()
        dags.append(cbq.Dag(nodes, root))
        (co, cd), (vo, vd) = W.serve_ray_pools(s, 1 << 19, 724, 7000 + i)
        pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
        pools.append(((pin(co), pin(cd)), (pin(vo), pin(vd))))
    sizes = (1 << 19, 724 * 724)
    reqs = W.serve_requests(20000, sizes, seed=1234)
    ring = 64
    max_n = 262144
    outs = [{"hit": torch.empty(max_n, dtype=torch.uint8).pin_memory().numpy(),
             "distance": torch.empty(max_n, dtype=torch.float32).pin_memory().numpy(),
             "material": torch.empty(max_n, dtype=torch.int32).pin_memory().numpy(),
             "voxel": torch.empty((max_n, 3), dtype=torch.int32).pin_memory().numpy(),
             "status": torch.empty(max_n, dtype=torch.uint8).pin_memory().numpy()} for _ in range(ring)]
    in_place = args.serve_buffers == "in-place"
    server = cbq.Server(device_memory_budget=2 << 30, max_inflight_launches=args.serve_inflight,
                        max_batch_requests=128, max_batch_rays=args.serve_batch_rays, in_place=in_place)
    queries = {True: cbq.Query(True, cbq.MAX_FOOTPRINT_DISABLED, True), False: cbq.Query()}

    def submit(k, r):
        (co, cd), (vo, vd) = pools[r.volume]
        o, d = (co, cd) if r.collision else (vo, vd)
        out = {f: v[: r.count] for f, v in outs[k % ring].items()}
        t, _ = server.submit(dags[r.volume], o[r.start:r.start + r.count], d[r.start:r.start + r.count],
                             queries[r.collision], out=out)
        return t

    # Peak: closed loop with up to `ring` requests outstanding for a fixed count.
    def closed_loop(first, count):
        pending = []
        t0 = time.perf_counter()
        for k in range(first, first + count):
            if len(pending) >= ring:
                server.wait(pending.pop(0))
            pending.append(submit(k, reqs[k % len(reqs)]))
        for t in pending:
            server.wait(t)
        return time.perf_counter() - t0

    n_peak = 3000
    # The same closed loop through a server of the other buffer mode.
    live = server
    server = cbq.Server(device_memory_budget=2 << 30, max_inflight_launches=args.serve_inflight,
                        max_batch_requests=128, max_batch_rays=args.serve_batch_rays, in_place=not in_place)
    closed_loop(0, 300)
    server.reset_stats()
    dt_other = closed_loop(300, n_peak)
    other = server.stats()
    server.close()
    server = live

    closed_loop(0, 300)  # warm-up
    server.reset_stats()
    dt = closed_loop(300, n_peak)
    peak = server.stats()
    peak_rps = n_peak / dt
    peak_mrays = peak["rays_completed"] / dt / 1e6

    def open_loop(rate, duration, first):
        """Poisson arrivals at `rate` requests/s for `duration` seconds."""
        rng = random.Random(rate * 1000.0 + first)
        times, t = [], 0.0
        while t < duration:
            t += rng.expovariate(rate)
            times.append(t)
        tickets = [None] * len(times)
        done = threading.Semaphore(ring)
        issued = threading.Event()

        def waiter():
            for i in range(len(times)):
                while tickets[i] is None:
                    time.sleep(0)
                server.wait(tickets[i])
                done.release()

        server.reset_stats()
        th = threading.Thread(target=waiter)
        th.start()
        backpressure = 0
        t0 = time.perf_counter()
        for i, at in enumerate(times):
            while time.perf_counter() - t0 < at:
                pass
            if not done.acquire(blocking=False):
                backpressure += 1
                done.acquire()
            tickets[i] = submit(first + i, reqs[(first + i) % len(reqs)])
        th.join()
        wall = time.perf_counter() - t0
        st = server.stats()
        return {"rate_rps": rate, "requests": len(times), "p50_ms": st["latency_p50_us"] / 1e3,
                "p99_ms": st["latency_p99_us"] / 1e3, "max_ms": st["latency_max_us"] / 1e3,
                "mrays_per_s": st["rays_completed"] / wall / 1e6, "requests_per_launch": st["mean_requests_per_launch"],
                "generator_backpressure": backpressure, "direct_requests": st["direct_requests"],
                "launches": st["launches"]}

    clocks = ClockSampler(local)
    clocks.start()
    # Three 4 s runs at half load; the line reports the run with the median p99
    # (host jitter from other work on the machine moves single-run tails).
    import gc
    gc.collect()
    gc.disable()  # no collector pauses in the Python load generator while it runs
    halves = [open_loop(0.5 * peak_rps, 4.0, 5000 + 40000 * k) for k in range(3)]
    clk = clocks.stop()
    half = dict(sorted(halves, key=lambda r: r["p99_ms"])[1])
    half["p99_ms_runs"] = [r["p99_ms"] for r in halves]
    sweep = [open_loop(f * peak_rps, 2.0, 9000 + int(f * 1000)) for f in (0.25, 0.75)]
    gc.enable()
    server.close()
    line = {
        "metric": "p99 latency at 50% of peak load", "value": half["p99_ms"], "unit": "ms", "n_gpus": world,
        "steps": half["requests"], "warmup": 300, "ms_per_step": half["p50_ms"], "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (8 seeded terrain DAGs, 1k-256k-ray requests: 70% collision tmax<=64, 30% view)",
        "config": {"workload": "serve-8", "edges": [1 << s.edge_log2 for s in scenes],
                   "server": {"memory_budget_gb": 2, "inflight_launches": args.serve_inflight,
                              "max_batch_requests": 128, "max_batch_rays": args.serve_batch_rays,
                              "buffers": "page-locked host, served in place" if in_place else
                              "page-locked host, staged through device memory"},
                   "arrivals": "open-loop Poisson"},
        "peak": {"requests_per_s": peak_rps, "mrays_per_s": peak_mrays, "p50_ms": peak["latency_p50_us"] / 1e3,
                 "p99_ms": peak["latency_p99_us"] / 1e3, "direct_requests": peak["direct_requests"]},
        "peak_other_buffers": {"buffers": "staged" if in_place else "in-place", "requests_per_s": n_peak / dt_other,
                               "mrays_per_s": other["rays_completed"] / dt_other / 1e6,
                               "p50_ms": other["latency_p50_us"] / 1e3, "p99_ms": other["latency_p99_us"] / 1e3},
        "half_load": half, "sweep": sweep,
        "e2e": {"value": half["mrays_per_s"], "unit": "Mrays/s", "note": "host rays in, host hits out, per request"},
        "gpu_launches": half["launches"], "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_gpu_city(args, world, rank, local):
    """city-8192: the wavefront pathtracer on the seeded 8192^3 city,
    1920x1080, 16 samples per pixel, 4 bounces, LOD footprint 0.0035.  One
    step = one frame.  A 1-sample frame is also traced with every traversal
    wave checked against the oracle on the host."""
    import torch
    import cubiquity_gb300 as cbq
    import oracle
    from cubiquity_gb300 import workloads as W

    torch.cuda.set_device(local)
    nodes, root = W.CITY_8192.build()
    dag = cbq.Dag(nodes, root)
    eye, target = W.city_camera(13)
    mats = W.city_materials()
    w, h, spp, bounces = 1920, 1080, 16, 4

    # Verification frame (1 spp, every wave checked).
    checked = mismatched = 0
    if not args.no_cpu_baseline:
        orc = oracle.Oracle()
        sd = orc.find_subdags(nodes, root)
        rec = cbq.WaveRecorder()
        cbq.pathtrace(dag, w, h, 1, bounces, eye, target, mats, seed=1, on_wave=rec)
        t0 = time.perf_counter()
        for kind, depth, sample, o, d, hits, (cs, mf) in rec.waves:
            want = orc.intersect(nodes, sd, o, d, cs, mf)
            bad = np.zeros(o.shape[0], bool)
            for k, v in hits.items():
                x = v.astype(want[k].dtype) if k == "material" else v
                bad |= (x != want[k]).reshape(o.shape[0], -1).any(axis=1) & ~np.isnan(
                    x.astype(np.float64)).reshape(o.shape[0], -1).any(axis=1)
            checked += o.shape[0]
            mismatched += int(bad.sum())
        cpu_s = time.perf_counter() - t0
        rec = None
    else:
        cpu_s = None

    for _ in range(max(1, args.warmup)):
        cbq.pathtrace(dag, w, h, spp, bounces, eye, target, mats, seed=2)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    rays = 0
    launches = 0
    ms = []
    t0 = time.perf_counter()
    for k in range(args.steps):
        img, st = cbq.pathtrace(dag, w, h, spp, bounces, eye, target, mats, seed=100 + k)
        rays += st["extension_rays"] + st["shadow_rays"]
        launches += st["kernel_launches"]
        ms.append(st["milliseconds"])
    wall = max_over_ranks(world, time.perf_counter() - t0)
    clk = clocks.stop()
    value = rays * world / wall / 1e6
    line = {
        "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(1, args.warmup), "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded 8192^3 city: boxes on a 64-voxel grid, 32 materials, 2 emissive)",
        "config": {"workload": "city-8192 pathtracer", "image": [w, h], "spp": spp, "bounces": bounces,
                   "max_footprint": 0.0035, "dag_nodes": int(dag.node_count), "rays_per_frame": rays // args.steps,
                   "frame_ms_median": float(np.median(ms))},
        "verification": {"frame": "1 spp, 1920x1080, 4 bounces", "traversals_checked": checked,
                         "mismatches": mismatched, "oracle_seconds": cpu_s},
        "e2e": {"value": value, "unit": "Mrays/s", "note": "camera rays generated on the device; image stays there"},
        "gpu_launches": launches, "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        if args.workload == "batch-64":
            run_reference_batch(args, world, rank)
        else:
            run_reference(args, world, rank)
    elif args.workload == "batch-64":
        run_gpu_batch(args, world, rank, local)
    elif args.workload == "serve-8":
        run_gpu_serve(args, world, rank, local)
    elif args.workload == "city-8192":
        run_gpu_city(args, world, rank, local)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
