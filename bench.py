"""Benchmark: sparse-voxel-DAG ray traversal throughput on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload terrain-4096|spheres-256|batch-64|serve-8|city-8192]
                    [--form tuned|persistent|plain] [--no-extras]

Workload (default terrain-4096): the seeded 4096^3 terrain DAG; one step traces
4,194,304 primary rays (2048x2048 pinhole) and 4,194,304 cosine-weighted bounce
rays from the primary hits, i.e. two traversal launches over 8,388,608 rays.
Inputs are resident in HBM before timing; the ray and hit arrays (654 MB per
step) exceed the 129 MB L2, so each step streams them; the 115 MB DAG is the
traversal's working set and stays in L2.

The camera batch passes its image width (the query's image_width), so the
kernel takes its rays in 4x8 pixel tiles (same results; --no-image-order passes
none); the bounce batch is not an image and goes in order.

`value` is device throughput (CUDA events on the launching stream); `e2e` is the
same workload through the host-buffer C ABI (cbq_intersect_host) with pinned
host rays in and hits out, copies inside the timed region.  `roofline` is that
of the dominant launch against the L2 (the DAG is L2-resident; the same run
measures the L2's read bandwidth and random-sector rate).  `fp64_error` compares
the GPU's distances with the oracle's FP64 exact-box ray cast (CPU leg).

On one GPU the default line also carries the benchmark's two other figures:
`serve` (serve-8: peak request rate and p50/p99 latency at half of it, median
of three runs, with the load generator's lateness; measured first, by a child
process, alone on the GPU) and `batch` (batch-64: the batched persistent
launch against the plain drop-in launched once per volume; measured after the
terrain).  `--no-extras` skips them.

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
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--e2e-threads", type=int, default=0,
                   help="host threads issuing the e2e calls (0: one per batch); threads x calls per thread = "
                        "batches x e2e steps")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-impl", choices=["auto", "port"], default="auto",
                   help="CPU ray cast timed by --impl reference: the reference's own library where it was built "
                        "from the checkout (else the oracle's C restatement), or the restatement always")
    p.add_argument("--no-extras", action="store_true",
                   help="terrain-4096: skip the batch-64 and serve-8 measurements added to the line")
    p.add_argument("--no-image-order", dest="image_order", action="store_false",
                   help="do not pass the camera batch's image width (rays then taken in the order given)")
    p.add_argument("--layout", choices=["reference", "compact"], default="reference",
                   help="device node store: the reference's array, or the compact store (occupied children only)")
    p.add_argument("--node-order", choices=["builder", "bfs"], default="builder",
                   help="batch-64: node stores as built, or renumbered breadth first (same results)")
    p.add_argument("--l2-window", type=float, default=0.0,
                   help="batch-64: persisting L2 window over the largest DAG on the batch graph's kernel nodes "
                        "(fraction of the persisting-L2 limit; 0 = none)")
    p.add_argument("--serve-inflight", type=int, default=8, help="serve-8: launches in flight")
    p.add_argument("--serve-batch-rays", type=int, default=4 << 20, help="serve-8: rays per launch at most")
    p.add_argument("--serve-summary", action="store_true",
                   help="serve-8: print only the summary that the default line carries under `serve`")
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


def image_widths(name: str) -> dict:
    """Batches whose rays are a camera's pixels in row-major order, with the
    image width (passed as the query's image_width: the kernel may take them
    in image tiles; the bounce rays are not an image)."""
    from cubiquity_gb300 import workloads as W
    cam = W.SPHERES_256_CAMERA if name == "spheres-256" else W.TERRAIN_4096_CAMERA
    return {"primary": cam.width}


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


PROFILE_NOTE = "ncu capture committed in profiles/ (not this run)"


def profiled_figure(workload: str, name: str, label: str | None = None):
    """A figure of the committed ncu summary of this workload's traversal
    (`name[label]: value` lines, e.g. `dram_bytes_per_ray[bounce]: 109.2`), or
    None.  These come from an earlier ncu capture, never from the run that
    prints them, and the bench line says so wherever it carries one."""
    f = ROOT / "profiles" / f"traverse_{workload}.md"
    if not f.exists():
        return None
    text = f.read_text()
    for key in ([re.escape(name) + r"\[" + re.escape(label) + r"\]"] if label else []) + [re.escape(name)]:
        m = re.search(r"^" + key + r":\s*([0-9.]+)", text, re.M)
        if m:  # the batch's own figure, else the workload's (one-batch workloads)
            return float(m.group(1))
    return None


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

def cpu_trace(nodes, root, batches, threads=0, impl="auto"):
    """Times the reference CPU ray cast over the batches; returns (seconds, kind).
    impl "auto": the reference's own library where it was built (oracle/_ref),
    else the oracle's C restatement; "port": the restatement always."""
    import oracle

    if impl != "port" and oracle.reference_available():
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
        cpu_trace(nodes, root, batches, impl=args.cpu_impl)
    total = 0.0
    kind = "port"
    for _ in range(args.steps):
        dt, kind = cpu_trace(nodes, root, batches, impl=args.cpu_impl)
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

    # The benchmark's other two measurements ride on the default line (single-GPU
    # runs): the serving latency (serve-8) first, by a child process, before
    # this process creates its CUDA context; the batched form (batch-64) after
    # the terrain.
    extras = world == 1 and args.workload == "terrain-4096" and not args.no_extras
    serve = serve_in_own_process(args, local) if extras else None
    torch.cuda.set_device(local)
    nodes, root, batches, bounce = make_workload(args.workload)
    widths = image_widths(args.workload) if args.image_order else {}
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
            tuned[label] = autotune.tune(dag, to, td, scratch, out, stream=stream, image_width=widths.get(label, 0))
        torch.cuda.synchronize()

    def launch(label, to, td, out):
        if tuned:
            c = tuned[label]
            dag.set_launch_config(c["kernel"], c["block"], c["chunk"], c["refill_min"], c["stack"], c["form"],
                                  c.get("steps", 1), c.get("registers", 0))
            cbq.intersect_auto(dag, to, td, scratch, out=out, stream=stream, image_width=widths.get(label, 0))
        elif args.persistent:
            cbq.intersect_volume_persistent(dag, to, td, counter, chunk=args.chunk, out=out, stream=stream,
                                            image_width=widths.get(label, 0))
        else:
            cbq.intersect_volume(dag, to, td, out=out, stream=stream, image_width=widths.get(label, 0))

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

    # Roofline of the dominant traversal launch.  Its node fetches are dependent
    # 4-byte loads, one 32-byte L2 sector each, from a DAG that stays in L2: the
    # bound is the L2, whose read bandwidth and random-sector rate this run
    # measures itself (cbq_measure_l2).  Algorithmic bytes per ray = 32 (ray in)
    # + F x 32 (one sector per node fetch) + 46 (hit record out).
    hbm_peak, hbm_kind = measured_peaks()
    l2_stream, l2_rand = cbq.measure_l2(64 << 20, 20)
    per_batch = {}
    for label, to, _, _, f in dev_batches:
        n = to.shape[0]
        ms = launch_ms[label]
        bpr = RAY_BYTES + f * SECTOR + HIT_BYTES
        achieved = n * bpr / (ms * 1e-3) / 1e9
        sectors = n * f / (ms * 1e-3) / 1e9
        dram = profiled_figure(args.workload, "dram_bytes_per_ray", label)
        c = tuned.get(label, cfg)
        per_batch[label] = {
            "rays": n, "launch_ms": ms, "fetches_per_ray": f, "bytes_per_ray": bpr,
            "kernel": ("cbq_k_flat_r56" if c.get("registers") == 56 and c.get("form") != 0 and c.get("stack") == 1
                       else kernel_name),
            "achieved_gbs": achieved, "frac_l2_stream": achieved / l2_stream,
            "sector_rate_gsps": sectors, "frac_l2_sector": sectors / l2_rand,
            "dram_bytes_per_launch": None if dram is None else dram * n,
            "frac_hbm": None if dram is None else dram * n / (ms * 1e-3) / 1e9 / hbm_peak}
    dominant = max(launch_ms, key=launch_ms.get)
    dom = per_batch[dominant]
    issue = profiled_figure(args.workload, "issue_active_pct", dominant)
    roofline = {
        "bound": "l2", "achieved": dom["achieved_gbs"], "peak": l2_stream, "unit": "GB/s",
        "frac": dom["frac_l2_stream"], "traffic": dom["dram_bytes_per_launch"],
        "kernel": dom["kernel"], "launch": f"{dominant} batch ({dom['rays']} rays, {dom['launch_ms']:.3f} ms per launch)",
        "peak_source": "cbq_measure_l2 in this run: streaming reads of a 64 MB L2-resident buffer",
        "traffic_source": f"dram__bytes_read.sum + dram__bytes_write.sum per launch, {PROFILE_NOTE}",
        "sector": {"achieved_gsps": dom["sector_rate_gsps"], "peak_gsps": l2_rand, "frac": dom["frac_l2_sector"],
                   "peak_source": "cbq_measure_l2 in this run: independent random 32-byte sector reads"},
        "hbm": {"frac": dom["frac_hbm"], "peak_gbs": hbm_peak, "peak_source": f"{hbm_kind} hbm_gbs",
                "note": "DRAM traffic of the launch (the ray and hit streams plus node-store misses) over its time; "
                        "traffic from the ncu capture, time from this run"},
        "limiter": {"kind": "instruction issue (the node fetches hit in L2)", "issue_active_pct": issue,
                    "source": PROFILE_NOTE},
        "per_batch": per_batch,
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
    # Calls in flight at once: one host thread per batch by default; each thread
    # has its own output buffers.
    e2e_threads = args.e2e_threads or len(host)
    thread_outs = [[h[3] for h in host]]
    for _ in range(1, e2e_threads):
        thread_outs.append([{k: torch.empty(v.shape, dtype=torch.from_numpy(v).dtype).pin_memory().numpy()
                             for k, v in h[3].items()} for h in host])

    # One DAG handle per batch, so each keeps the launch shape tuned for it (a
    # handle's launch configuration is shared by its callers).
    e2e_dags = {}
    for label, _, _, _ in host:
        g = cbq.Dag(nodes, root, LAYOUTS[args.layout])
        if tuned:  # the launch shape tuned for this batch, as a caller who tuned would set it
            c = tuned[label]
            g.set_launch_config(c["kernel"], c["block"], c["chunk"], c["refill_min"], c["stack"], c["form"],
                                c.get("steps", 1), c.get("registers", 0))
        e2e_dags[label] = g

    def e2e_call(item, outs=None):
        label, po, pd, own = item
        cbq.intersect_volume_host(e2e_dags[label], po, pd, out=own if outs is None else outs,
                                  image_width=widths.get(label, 0))

    # The batches are independent streams of work, so a caller issues them from
    # several host threads (one per batch by default, --e2e-threads), and the
    # calls of different threads overlap their copies and traversals (the host
    # entry point is thread-safe).  The threads alternate the batches (thread
    # t's k-th call is batch (t + k) mod the number of batches), so no thread is
    # left running alone at the end; over all threads each batch is called
    # e2e_steps times (threads x calls per thread = batches x e2e_steps).  The
    # clock runs from the start until every thread has made its calls, i.e.
    # every step's rays were copied in and its hits copied out.  The
    # single-thread figure (the batches' calls one after the other) is kept
    # beside it.
    if (args.e2e_steps * len(host)) % e2e_threads:
        raise SystemExit("--e2e-threads must divide the e2e calls (batches x --e2e-steps)")
    calls_per_thread = args.e2e_steps * len(host) // e2e_threads

    def e2e_timed(threaded: bool) -> float:
        errors = []

        def worker(t):
            try:
                for k in range(calls_per_thread):
                    b = (t + k) % len(host)
                    e2e_call(host[b], thread_outs[t][b])
            except Exception as e:  # noqa: BLE001  (re-raised below: a failed call voids the figure)
                errors.append(e)
        for h in host:  # warm-up: staging sets allocated
            e2e_call(h)
        barrier(world)
        t = time.perf_counter()
        if threaded:
            th = [threading.Thread(target=worker, args=(t,)) for t in range(e2e_threads)]
            for x in th:
                x.start()
            for x in th:
                x.join()
            if errors:
                raise errors[0]
        else:
            for _ in range(args.e2e_steps):
                for h in host:
                    e2e_call(h)
        rays = (sum(host[(t + k) % len(host)][1].shape[0] for t in range(e2e_threads) for k in range(calls_per_thread))
                if threaded else rays_per_step * args.e2e_steps)
        return rays * world / max_over_ranks(world, time.perf_counter() - t) / 1e6

    e2e_value = e2e_timed(e2e_threads > 1)
    e2e_one_thread = e2e_timed(False)
    for g in e2e_dags.values():
        g.destroy()

    cpu = None
    fp64 = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        dt, kind = cpu_trace(nodes, root, batches)
        cores = host_cores()
        cpu = {"value": rays_per_step / dt / 1e6, "unit": "Mrays/s", "cores": cores, "cpu": host_cpu(), "kind": kind,
               "sample": f"one pass over the full workload ({rays_per_step} rays), {cores} host threads"}
        fp64 = fp64_error(nodes, root, batches, [b[3] for b in dev_batches])

    launches = args.steps * len(dev_batches)
    line = {
        "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene built by libcbq, generated rays)",
        "config": {"workload": args.workload, "rays_per_step": rays_per_step, "kernel": kernel_name,
                   "form": args.form, "launch_config": tuned if tuned else cfg,
                   "batches": {b[0]: int(b[1].shape[0]) for b in dev_batches},
                   "image_width": widths,
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
                "api": "cbq_intersect_host (pinned host buffers, copies pipelined with the traversal inside), " +
                       ("one call per batch and step, from %d host threads that alternate the batches" % e2e_threads
                        if e2e_threads > 1 else "one call per step"),
                "fields": "hit, distance, material, position, normal (the reference's RayVolumeIntersection)",
                "steps": args.e2e_steps, "one_thread_value": e2e_one_thread},
        "gpu_launches": launches,
        "clocks": clk,
        "fp64_error": fp64,
    }
    dag.destroy()
    if extras:
        line["serve"] = serve
        line["batch"] = measure_batch(args, world, local, e2e_steps=3)[0]
    if rank == 0:
        print(json.dumps(line), flush=True)


def serve_in_own_process(args, local) -> dict:
    """The serve-8 summary, measured by a child process before this one
    touches the GPU.  After large device frees (by any process: this one's
    terrain and batch legs free GBs) GPU completions are delayed by
    milliseconds for tens of seconds (measured: half-load p99 4.4-7.2 ms
    against 0.42-0.43 ms), so the latency is measured as a server runs: alone
    on a GPU where nothing is being freed, in a process of its own."""
    cmd = [sys.executable, str(ROOT / "bench.py"), "--workload", "serve-8", "--serve-summary",
           "--serve-inflight", str(args.serve_inflight), "--serve-batch-rays", str(args.serve_batch_rays),
           "--serve-buffers", args.serve_buffers]
    env = dict(os.environ)
    if "CUDA_VISIBLE_DEVICES" not in env:
        env["CUDA_VISIBLE_DEVICES"] = str(local)
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=env)
    if proc.returncode != 0 or not proc.stdout.strip():
        # The terrain figures stand on their own: report the failure in the line.
        print(f"serve-8 measurement failed:\n{proc.stderr[-2000:]}", file=sys.stderr)
        return {"workload": "serve-8", "error": f"child exited with status {proc.returncode}",
                "stderr_tail": proc.stderr[-400:]}
    summary = json.loads(proc.stdout.strip().splitlines()[-1])
    summary["process"] = "its own (a child of this run)"
    return summary


def fp64_error(nodes, root, batches, gpu_outs) -> dict:
    """The GPU's FP32 hit records against the oracle's FP64 exact-box ray cast
    (the reference's own check compares intersectVolume with traceRayRef,
    test_rendering.cpp:75-80).  Per batch: hit and material disagreements and
    the relative distance error |d32 - d64| / max(d64, 1 voxel) over rays both
    hit, with the rays above 1e-5 (grazing rays: an edge or corner decided the
    other way in FP32) counted and listed.  Part of the CPU leg."""
    import oracle

    orc = oracle.Oracle()
    sd = orc.find_subdags(nodes, root)
    out = {}
    for (label, o, d), g in zip(batches, gpu_outs):
        exact = orc.trace_fp64(nodes, sd, o, d)
        hit = g["hit"].cpu().numpy().astype(bool)
        dist = g["distance"].cpu().numpy().astype(np.float64)
        mat = g["material"].cpu().numpy().astype(np.uint32)
        ehit = exact["hit"].astype(bool)
        both = hit & ehit
        rel = np.abs(dist[both] - exact["distance"][both]) / np.maximum(np.abs(exact["distance"][both]), 1.0)
        idx = np.nonzero(both)[0]
        over = idx[rel > 1e-5]
        hit_mm = np.nonzero(hit != ehit)[0]
        mat_mm = np.nonzero(both & (mat != exact["material"]))[0]
        out[label] = {"rays": int(o.shape[0]), "hits": int(hit.sum()), "hit_mismatches": int(hit_mm.size),
                      "hit_mismatch_rays": hit_mm[:20].tolist(), "material_mismatches": int(mat_mm.size),
                      "material_mismatch_rays": mat_mm[:20].tolist(),
                      "rel_p50": float(np.quantile(rel, 0.5)) if rel.size else None,
                      "rel_p999": float(np.quantile(rel, 0.999)) if rel.size else None,
                      "rel_max": float(rel.max()) if rel.size else None,
                      "over_1e-5": int(over.size), "over_1e-5_rays": over[:20].tolist()}
    return {"batches": out, "oracle": "orc_trace_fp64_batch: exact voxel boxes, double precision",
            "tolerance": "1e-5 relative (distance; grazing rays above it are counted and listed)"}


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


def measure_batch(args, world, local, e2e_steps: int | None = None):
    """batch-64: many volumes of uneven size in one persistent, graph-captured,
    autotuned launch, against the plain drop-in launched once per volume.
    Returns (summary, details): the summary is what the default line carries
    under `batch`; the details make the full `--workload batch-64` line."""
    import torch
    import cubiquity_gb300 as cbq

    torch.cuda.set_device(local)
    host_jobs = batch_jobs()
    if args.node_order == "bfs":  # the same graphs renumbered breadth first: same results
        host_jobs = [cbq.reorder_bfs(n, r) + (o, d) for n, r, o, d in host_jobs]
    dags = [cbq.Dag(n, r, LAYOUTS[args.layout]) for n, r, _, _ in host_jobs]
    dev = [(torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()) for _, _, o, d in host_jobs]
    rays_per_step = sum(o.shape[0] for o, _ in dev)
    stream = torch.cuda.current_stream()
    plain_out = [cbq.alloc_hits(o.shape[0]) for o, _ in dev]
    batch = cbq.Batch([(g, o, d) for g, (o, d) in zip(dags, dev)])
    tuned = batch.autotune(3, stream=stream)
    if args.l2_window > 0:  # persisting window over the largest store, on the graph's kernel nodes
        batch.set_l2_persistence(max(dags, key=lambda g: g.device_bytes), args.l2_window)
    steps = max(3, args.steps)

    def plain_step():
        for g, (o, d), out in zip(dags, dev, plain_out):
            cbq.intersect_volume(g, o, d, out=out, stream=stream)

    def batched_step():
        batch.launch(stream=stream)

    def timed(fn):
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

    plain_ms = timed(plain_step)
    clocks = ClockSampler(local)
    clocks.start()
    batched_ms = timed(batched_step)
    clk = clocks.stop()
    # Same answers from both forms.
    for out_b, out_p in zip(batch.outputs, plain_out):
        for k in ("hit", "material", "voxel", "distance", "status"):
            if not torch.equal(out_b[k], out_p[k]):
                raise SystemExit(f"batched and plain results differ in {k}")
    value = rays_per_step * steps * world / (batched_ms * 1e-3) / 1e6
    plain_value = rays_per_step * steps * world / (plain_ms * 1e-3) / 1e6

    # Roofline of the batched launch (algorithmic bytes as for the single-volume launch).
    fetches = sum(cbq.count_fetches(g, o, d).double().sum().item() for g, (o, d) in zip(dags, dev))
    hbm_peak, hbm_kind = measured_peaks()
    step_s = batched_ms / steps * 1e-3
    alg_bytes = rays_per_step * (RAY_BYTES + HIT_BYTES) + fetches * SECTOR
    achieved = alg_bytes / step_s / 1e9
    l2_stream, l2_rand = cbq.measure_l2(64 << 20, 20)
    dram = profiled_figure("batch-64", "dram_bytes_per_ray")

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
    # One step = the 64 volumes' requests (the reference's query, every hit
    # field the reference returns); the steps are submitted back to back by the
    # library's native trace driver (all arrivals at 0, 64 requests
    # outstanding), so request k of step s + 1 reuses request k's buffers of
    # step s once that one has completed.
    one = np.zeros(len(dags), cbq.REQUEST_DTYPE)
    for k, (g, (po, pd), out) in enumerate(zip(dags, pinned_in, pinned_out)):
        one[k]["dag"] = g.handle.value
        one[k]["origin_tmax"] = po.ctypes.data
        one[k]["direction"] = pd.ctypes.data
        one[k]["ray_count"] = po.shape[0]
        one[k]["compute_surface"] = 1
        one[k]["max_footprint"] = cbq.MAX_FOOTPRINT_DISABLED
        for f, v in out.items():
            one[k][f] = v.ctypes.data

    def e2e_run(steps):
        trace = np.tile(one, steps)
        r = server.replay(trace, np.zeros(trace.shape[0]), len(dags))
        if r["failed"]:
            raise SystemExit("batch-64 end to end: requests failed")
        return r["wall_seconds"]

    n_e2e = e2e_steps if e2e_steps is not None else args.e2e_steps
    e2e_run(1)
    server.reset_stats()
    e2e_value = rays_per_step * n_e2e * world / max_over_ranks(world, e2e_run(n_e2e)) / 1e6
    e2e_launches = server.stats()["launches"]
    server.close()
    batch.destroy()
    for g in dags:
        g.destroy()

    summary = {
        "workload": "batch-64", "volumes": len(dags), "rays_per_step": rays_per_step, "steps": steps,
        "batched_mrays": value, "plain_mrays": plain_value, "batched_over_plain": value / plain_value,
        "batched_ms_per_step": batched_ms / steps, "plain_ms_per_step": plain_ms / steps,
        "batched_form": "one persistent cbq_k_flat_batch launch per step, replayed from a CUDA graph, autotuned",
        "plain_form": "the drop-in cbq_intersect once per volume (64 launches per step)",
        "batch_config": tuned, "fetches_per_ray": fetches / rays_per_step,
        "l2_frac_stream": achieved / l2_stream,
        "e2e_mrays": e2e_value, "clocks": clk,
    }
    details = {
        "rays_per_step": rays_per_step, "steps": steps, "value": value, "ms_per_step": batched_ms / steps, "clk": clk,
        "dag_bytes": int(sum(g.bytes for g in dags)), "device_node_bytes": int(sum(g.device_bytes for g in dags)),
        "tuned": tuned, "plain_value": plain_value, "plain_ms": plain_ms / steps,
        "roofline": {"bound": "l2", "achieved": achieved, "peak": l2_stream, "unit": "GB/s",
                     "frac": achieved / l2_stream, "kernel": "cbq_k_flat_batch",
                     "peak_source": "cbq_measure_l2 in this run: streaming reads of a 64 MB L2-resident buffer",
                     "traffic": None if dram is None else dram * rays_per_step,
                     "traffic_source": f"dram__bytes_read.sum + dram__bytes_write.sum per launch, {PROFILE_NOTE}",
                     "fetches_per_ray": fetches / rays_per_step,
                     "sector": {"achieved_gsps": fetches / step_s / 1e9, "peak_gsps": l2_rand,
                                "frac": fetches / step_s / 1e9 / l2_rand},
                     "hbm": {"frac": None if dram is None else dram * rays_per_step / step_s / 1e9 / hbm_peak,
                             "peak_gbs": hbm_peak, "peak_source": f"{hbm_kind} hbm_gbs"},
                     "limiter": {"kind": "instruction issue",
                                 "issue_active_pct": profiled_figure("batch-64", "issue_active_pct"),
                                 "source": PROFILE_NOTE}},
        "e2e": e2e_value, "e2e_launches_per_step": e2e_launches / max(1, n_e2e), "e2e_steps": n_e2e,
    }
    return summary, details


def run_gpu_batch(args, world, rank, local):
    """The full bench line of batch-64 (`--workload batch-64`)."""
    s, d = measure_batch(args, world, local)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        orc = oracle.Oracle()
        t0 = time.perf_counter()
        for n, r, o, dd in batch_jobs():
            orc.intersect(n, orc.find_subdags(n, r), o, dd)
        dt = time.perf_counter() - t0
        cpu = {"value": d["rays_per_step"] / dt / 1e6, "unit": "Mrays/s", "cores": host_cores(), "cpu": host_cpu(),
               "kind": "port", "sample": f"one pass over all 64 volumes ({d['rays_per_step']} rays), "
                                         f"{host_cores()} host threads"}
    line = {
        "metric": "Mrays/s", "value": d["value"], "unit": "Mrays/s", "n_gpus": world, "steps": d["steps"],
        "warmup": max(3, args.warmup), "ms_per_step": d["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (64 seeded sphere/terrain volumes, edges 2^7..2^11, generated rays)",
        "config": {"workload": "batch-64", "volumes": s["volumes"], "rays_per_step": d["rays_per_step"],
                   "dag_bytes": d["dag_bytes"], "layout": args.layout, "device_node_bytes": d["device_node_bytes"],
                   "batch_config": d["tuned"], "form": "one persistent launch replayed from a CUDA graph",
                   "node_order": args.node_order, "l2_window": args.l2_window,
                   "l2": "inputs larger than L2 (rays + hits %.0f MB per step)" % (d["rays_per_step"] * 78 / 1e6)},
        "plain": {"value": d["plain_value"], "unit": "Mrays/s", "ms_per_step": d["plain_ms"],
                  "form": "cbq_intersect once per volume (64 launches per step)"},
        "batched_over_plain": d["value"] / d["plain_value"],
        "roofline": d["roofline"],
        "cpu_baseline": cpu,
        "e2e": {"value": d["e2e"], "unit": "Mrays/s", "h2d_bytes_per_step": d["rays_per_step"] * RAY_BYTES,
                "d2h_bytes_per_step": d["rays_per_step"] * REF_HIT_BYTES,
                "api": "request server, one request per volume and step (pinned host buffers), submitted by "
                       "the native trace driver (cbq_server_replay) with 64 requests outstanding",
                "fields": "hit, distance, material, position, normal (the reference's RayVolumeIntersection)",
                "launches_per_step": d["e2e_launches_per_step"]},
        "gpu_launches": d["steps"],
        "clocks": d["clk"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_serve(args, world, local, half_runs: int = 3, half_seconds: float = 4.0, sweep: bool = True):
    """serve-8: 8 resident terrain DAGs (edges 1024-4096); requests of 1k-256k
    rays (log-uniform), 70% tmax-bounded collision rays and 30% view rays.
    The load comes from the library's native trace driver (cbq_server_replay),
    so the client's own timing is not the Python interpreter's: the peak
    request rate is found closed loop (every arrival at time 0, 64 requests
    outstanding), then an open-loop Poisson stream at half of it gives p50/p99
    latency (submit -> hits in host memory, timed by the server) and Mrays/s,
    with the trace driver's lateness (actual submit time minus scheduled arrival)
    beside them.  Returns (summary, details)."""
    import torch
    import cubiquity_gb300 as cbq
    from cubiquity_gb300 import workloads as W

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
    r_vol = np.array([r.volume for r in reqs])
    r_coll = np.array([r.collision for r in reqs])
    r_start = np.array([r.start for r in reqs], np.uint64)
    r_count = np.array([r.count for r in reqs], np.uint64)
    ptr = lambda a: a.ctypes.data  # noqa: E731
    dag_h = np.array([g.handle.value for g in dags], np.uint64)
    o_ptr = {True: np.array([ptr(p[0][0]) for p in pools], np.uint64),
             False: np.array([ptr(p[1][0]) for p in pools], np.uint64)}
    d_ptr = {True: np.array([ptr(p[0][1]) for p in pools], np.uint64),
             False: np.array([ptr(p[1][1]) for p in pools], np.uint64)}
    ring = 64
    max_n = 262144
    outs = [{"hit": torch.empty(max_n, dtype=torch.uint8).pin_memory().numpy(),
             "distance": torch.empty(max_n, dtype=torch.float32).pin_memory().numpy(),
             "material": torch.empty(max_n, dtype=torch.int32).pin_memory().numpy(),
             "voxel": torch.empty((max_n, 3), dtype=torch.int32).pin_memory().numpy(),
             "status": torch.empty(max_n, dtype=torch.uint8).pin_memory().numpy()} for _ in range(ring)]
    out_ptr = {k: np.array([ptr(o[k]) for o in outs], np.uint64) for k in outs[0]}
    in_place = args.serve_buffers == "in-place"

    def trace(first: int, count: int) -> np.ndarray:
        """Requests first .. first + count - 1 of the stream; request k writes ring buffer k % ring."""
        k = np.arange(count)
        i = (first + k) % len(reqs)
        vol, coll = r_vol[i], r_coll[i]
        t = np.zeros(count, cbq.REQUEST_DTYPE)
        t["dag"] = dag_h[vol]
        t["origin_tmax"] = np.where(coll, o_ptr[True][vol], o_ptr[False][vol]) + r_start[i] * np.uint64(16)
        t["direction"] = np.where(coll, d_ptr[True][vol], d_ptr[False][vol]) + r_start[i] * np.uint64(16)
        t["ray_count"] = r_count[i]
        t["compute_surface"] = 1
        t["max_footprint"] = cbq.MAX_FOOTPRINT_DISABLED
        t["flags"] = np.where(coll, cbq.QUERY_TMAX, 0)
        for f, p in out_ptr.items():
            t[f] = p[(first + k) % ring]
        return t

    def make_server(place):
        return cbq.Server(device_memory_budget=2 << 30, max_inflight_launches=args.serve_inflight,
                          max_batch_requests=128, max_batch_rays=args.serve_batch_rays, in_place=place)

    def closed_loop(server, first, count):
        server.reset_stats()
        r = server.replay(trace(first, count), np.zeros(count), ring)
        st = server.stats()
        return {"requests_per_s": count / r["wall_seconds"], "mrays_per_s": st["rays_completed"] / r["wall_seconds"] / 1e6,
                "p50_ms": st["latency_p50_us"] / 1e3, "p99_ms": st["latency_p99_us"] / 1e3,
                "direct_requests": st["direct_requests"], "failed": r["failed"]}

    n_peak = 6000
    other = None
    if sweep:  # the same closed loop through a server of the other buffer mode
        server = make_server(not in_place)
        closed_loop(server, 0, 600)
        other = dict(closed_loop(server, 600, n_peak), buffers="staged" if in_place else "in-place")
        server.close()
    server = make_server(in_place)
    closed_loop(server, 0, 600)  # warm-up
    peak = closed_loop(server, 600, n_peak)
    peak_rps = peak["requests_per_s"]

    def open_loop(rate, duration, first):
        """Poisson arrivals at `rate` requests/s for `duration` seconds."""
        rng = np.random.default_rng(int(rate * 1000.0) + first)
        gaps = rng.exponential(1.0 / rate, size=int(rate * duration * 1.2) + 16)
        times = np.cumsum(gaps)
        times = times[times < duration]
        server.reset_stats()
        r = server.replay(trace(first, times.size), times, ring)
        st = server.stats()
        late = r["lateness_us"]
        return {"rate_rps": rate, "requests": int(times.size), "p50_ms": st["latency_p50_us"] / 1e3,
                "p99_ms": st["latency_p99_us"] / 1e3, "max_ms": st["latency_max_us"] / 1e3,
                "mrays_per_s": st["rays_completed"] / r["wall_seconds"] / 1e6,
                "requests_per_launch": st["mean_requests_per_launch"], "launches": st["launches"],
                "direct_requests": st["direct_requests"], "failed": r["failed"],
                "generator_backpressure": r["backpressure"],
                "generator_lateness_ms": {"p50": float(np.quantile(late, 0.5)) / 1e3,
                                          "p99": float(np.quantile(late, 0.99)) / 1e3,
                                          "max": float(late.max()) / 1e3},
                "submit_call_ms": {"p99": r["submit_p99_us"] / 1e3, "max": r["submit_max_us"] / 1e3}}

    clocks = ClockSampler(local)
    clocks.start()
    # `half_runs` runs at half load; the result is the run with the median p99
    # (host jitter from other work on the machine moves single-run tails).
    halves = [open_loop(0.5 * peak_rps, half_seconds, 5000 + 40000 * k) for k in range(half_runs)]
    clk = clocks.stop()
    half = dict(sorted(halves, key=lambda r: r["p99_ms"])[len(halves) // 2])
    half["p99_ms_runs"] = [r["p99_ms"] for r in halves]
    sweep_runs = [open_loop(f * peak_rps, 2.0, 9000 + int(f * 1000)) for f in (0.25, 0.75)] if sweep else []
    server.close()
    for g in dags:
        g.destroy()
    buffers = "page-locked host, served in place" if in_place else "page-locked host, staged through device memory"
    summary = {
        "workload": "serve-8", "edges": [1 << s.edge_log2 for s in scenes],
        "peak_requests_per_s": peak_rps, "peak_mrays_per_s": peak["mrays_per_s"],
        "half_load": {"rate_rps": half["rate_rps"], "p50_ms": half["p50_ms"], "p99_ms": half["p99_ms"],
                      "p99_ms_runs": half["p99_ms_runs"], "seconds_per_run": half_seconds,
                      "mrays_per_s": half["mrays_per_s"], "requests_per_launch": half["requests_per_launch"],
                      "generator_lateness_ms": half["generator_lateness_ms"],
                      "submit_call_ms": half["submit_call_ms"]},
        "latency": "submit -> hits in host memory, timed by the server; p99 = median over the runs",
        "arrivals": "open-loop Poisson, replayed by the library's native driver (cbq_server_replay)",
        "buffers": buffers, "clocks": clk,
    }
    # The generator's threads spin through the last 200 us before each arrival,
    # so their lateness measures how late the host ran this process's threads;
    # the server's threads wait the same way, so a late host delays completions
    # alike and the p99 then describes the host, not the server.
    late_p99 = half["generator_lateness_ms"]["p99"]
    summary["host_threads_stalled"] = bool(late_p99 > 0.2)
    if late_p99 > 0.2:
        summary["host_note"] = ("the load generator's own threads were late by p99 %.2f ms: the host did not run this "
                                "process's threads on time (measured on these hosts for minutes after another "
                                "process freed device memory)" % late_p99)
    details = {"scenes": scenes, "in_place": in_place, "peak": peak, "peak_rps": peak_rps, "other": other,
               "half": half, "sweep": sweep_runs, "clk": clk, "buffers": buffers}
    return summary, details


def run_gpu_serve(args, world, rank, local):
    """The full bench line of serve-8 (`--workload serve-8`); with
    --serve-summary, only the summary the default line carries."""
    if args.serve_summary:
        s, _ = measure_serve(args, world, local, sweep=False)
        if rank == 0:
            print(json.dumps(s), flush=True)
        return
    s, d = measure_serve(args, world, local)
    half, peak = d["half"], d["peak"]
    line = {
        "metric": "p99 latency at 50% of peak load", "value": half["p99_ms"], "unit": "ms", "n_gpus": world,
        "steps": half["requests"], "warmup": 300, "ms_per_step": half["p50_ms"], "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (8 seeded terrain DAGs, 1k-256k-ray requests: 70% collision tmax<=64, 30% view)",
        "config": {"workload": "serve-8", "edges": s["edges"],
                   "server": {"memory_budget_gb": 2, "inflight_launches": args.serve_inflight,
                              "max_batch_requests": 128, "max_batch_rays": args.serve_batch_rays,
                              "buffers": d["buffers"]},
                   "arrivals": "open-loop Poisson (native trace driver, cbq_server_replay)"},
        "peak": peak,
        "peak_other_buffers": d["other"],
        "half_load": half, "sweep": d["sweep"],
        "e2e": {"value": half["mrays_per_s"], "unit": "Mrays/s", "note": "host rays in, host hits out, per request"},
        "gpu_launches": half["launches"], "clocks": d["clk"],
        "host_threads_stalled": s["host_threads_stalled"],
    }
    if "host_note" in s:
        line["host_note"] = s["host_note"]
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
