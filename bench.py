"""Benchmark: the distance-driven projector + backprojector pair at
512^3 voxels (0.5 mm), 720 views over 2 pi, 1024x768 detector (0.75 mm),
SAD 1000 mm, SDD 1500 mm; 30 seeded random ellipsoids.

One step = Reconstruction.forward() then Reconstruction.backward() of the
reference (DD forward projection A x, then the FDK-weighted DD backprojection
of the result), each over all 720 views.  Metric: voxel-views of the pair per
second, in Gvoxel*views/s (nx*ny*nz*nviews per step / step time).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's own CUDA-C kernels compiled for the
host CPU (oracle/_ref, or the oracle port when that library is absent) on a
bounded sample: one view forward + one view backward over the full volume.
Prints one JSON line (rank 0).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORKLOAD = "dd_pair_512cube_720views_det1024x768"


def scan_params(n=512, nviews=720, nu=1024, nv=768):
    return {'SourceInit': [0.0, 1000.0, 0.0], 'DetectorInit': [0.0, -500.0, 0.0], 'StartAngle': 0.0,
            'EndAngle': 2 * np.pi, 'NumberOfDetectorPixels': [nu, nv], 'DetectorPixelSize': [0.75, 0.75],
            'NumberOfViews': nviews, 'ImagePixelSpacing': [0.5, 0.5, 0.5], 'NumberOfImage': [n, n, n],
            'PhantomCenter': [0.0, 0.0, 0.0], 'RotationOrigin': [0.0, 0.0, 0.0], 'ReconCenter': [0.0, 0.0, 0.0],
            'Method': 'Distance', 'FilterType': 'hann', 'cutoff': 1.0, 'GPU': 1, 'DetectorShape': 'Flat',
            'Pitch': 0.0}


METRIC = "DD proj+backproj throughput"
UNIT = "Gvoxel*views/s"


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(kernel):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary
    (a line 'traffic_bytes_per_launch: <N>' in profiles/<kernel>*.md), or None."""
    d = os.path.join(REPO, "profiles")
    if not os.path.isdir(d):
        return None
    for f in sorted(os.listdir(d)):
        if f.startswith(kernel) and f.endswith((".md", ".txt")):
            for line in open(os.path.join(d, f)):
                if line.strip().startswith("traffic_bytes_per_launch:"):
                    try:
                        return float(line.split(":", 1)[1].split()[0])
                    except ValueError:
                        return None
    return None


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", "ctgb_clocks_%d_%d.csv" % (os.getpid(), index))

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---------------------------------------------------------------------------
def cpu_phantom(params):
    from ctreconstruction_gb300 import phantoms
    n = params['NumberOfImage'][0]
    return phantoms.random_ellipsoids((n, n, n), n=30, seed=1, device="cpu").numpy()


def cpu_sample(params, vol, nthreads=None):
    """The reference's CPU path (oracle/_ref) — or the oracle port — on one view
    forward + one view backward over the full volume.  Returns a dict."""
    from oracle import ref_runner
    nthreads = nthreads or os.cpu_count()
    n = params['NumberOfImage'][0]
    view = 37
    if ref_runner.available():
        r = ref_runner.RefScan(dict(params, DetectorOffset=[0.0, 0.0]))
        t0 = time.perf_counter()
        pv = r.forward_view(vol, view, nthreads)
        t1 = time.perf_counter()
        r.backward_view(pv, view, r.angles[1] - r.angles[0], nthreads=nthreads)
        t2 = time.perf_counter()
        kind = "reference"
        what = "reference CUDA-C kernels (distance_project_on_*3, flat_distance_backproj_arb2) as host C++, OpenMP"
    else:
        from oracle.oracle import OracleGeometry
        g = OracleGeometry(params)
        t0 = time.perf_counter()
        pv = g.forward(vol, view, 1, nthreads)
        t1 = time.perf_counter()
        g.backward_fdk(pv.astype(np.float32), view, 1, nthreads)
        t2 = time.perf_counter()
        kind = "port"
        what = "FP64 C oracle port, OpenMP"
    nvox = n ** 3
    return {"seconds": t2 - t0, "fwd_s": t1 - t0, "bwd_s": t2 - t1, "voxel_views": nvox, "kind": kind,
            "cores": nthreads, "what": what}


def run_reference(args):
    ws, rank, local = dist_setup()
    if rank != 0:
        return 0
    params = scan_params()
    vol = cpu_phantom(params)
    for _ in range(args.warmup):
        cpu_sample(params, vol)
    times = []
    last = None
    for _ in range(args.steps):
        last = cpu_sample(params, vol)
        times.append(last["seconds"])
    t = sum(times) / len(times)
    value = last["voxel_views"] / t / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": "1 view forward + 1 view backward, full 512^3 volume"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": last["cores"], "kind": last["kind"],
                             "sample": "one view of DD forward + FDK-weighted DD backprojection over 512^3: "
                                       + last["what"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    import torch.distributed as dist
    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=dev)

    from ctreconstruction_gb300 import Projector, Reconstruction, phantoms

    params = scan_params(*([args.small] if args.small else []))
    if args.small:
        params = scan_params(args.small, nviews=max(8, args.small // 4), nu=2 * args.small, nv=args.small + 16)
    n = params['NumberOfImage'][0]
    nviews = params['NumberOfViews']
    P = Projector(params, device=dev)
    vol = phantoms.random_ellipsoids((n, n, n), n=30, seed=1, device=dev)
    proj = torch.empty(P.proj_shape(), dtype=torch.float32, device=dev)
    bp = torch.empty(P.volume_shape, dtype=torch.float32, device=dev)
    xzy = torch.empty((n, n, n), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    ev = {k: [] for k in ("transpose", "forward", "backproject_fdk")}

    def step(record=False):
        if record:
            e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            e[0].record(stream)
        P.transpose(vol, out=xzy)
        if record:
            e[1].record(stream)
        P.forward(vol, out=proj, transposed=xzy)
        if record:
            e[2].record(stream)
        P.backproject_fdk(proj, out=bp)
        if record:
            e[3].record(stream)
            ev["transpose"].append((e[0], e[1]))
            ev["forward"].append((e[1], e[2]))
            ev["backproject_fdk"].append((e[2], e[3]))

    def barrier():
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        start.record(stream)
        for _ in range(args.steps):
            step(record=True)
        end.record(stream)
        barrier()
    ms = start.elapsed_time(end) / args.steps
    t = torch.tensor([ms], device=dev)
    if ws > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    vv = float(n) ** 3 * nviews
    value = ws * vv / (ms / 1e3) / 1e9

    kern = {k: sum(a.elapsed_time(b) for a, b in v) / len(v) for k, v in ev.items()}
    dom = max(("forward", "backproject_fdk"), key=lambda k: kern[k])
    peak, peak_kind = measured_peaks()
    alg_bytes = 4.0 * vv                 # 4 B per voxel-view per direction
    achieved = alg_bytes / (kern[dom] / 1e3) / 1e9
    kname = {"forward": "dd_forward_kernel", "backproject_fdk": "bp_fdk_kernel"}[dom]
    roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": profiled_traffic(kname),
                "algorithmic_bytes_per_launch": alg_bytes, "ms_per_launch": kern[dom]}

    # matched pair (autograd path): forward + exact adjoint
    matched = None
    if not args.no_matched:
        bpm = torch.empty_like(bp)
        P.backproject_matched(proj, out=bpm)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        P.backproject_matched(proj, out=bpm)
        b.record(stream)
        torch.cuda.synchronize()
        mm = a.elapsed_time(b)
        matched = {"backproject_matched_ms": mm,
                   "pair_value": vv / ((kern["forward"] + kern["transpose"] + mm) / 1e3) / 1e9}

    # end to end through the public API with host arrays (copies inside the timed region)
    host_vol = vol.cpu().numpy()
    R = Reconstruction(params, device=dev)
    e2e_steps = max(1, min(args.steps, 3))
    R.image = host_vol
    R.forward()
    R.backward()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        R.image = host_vol
        R.forward()
        R.backward()
    barrier()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": ws * vv / e2e_s / 1e9, "unit": UNIT, "ms_per_step": e2e_s * 1e3,
           "h2d_bytes_per_step": int(4 * (n ** 3 + nviews * P.params.nu * P.params.nv)),
           "d2h_bytes_per_step": int(4 * (n ** 3 + nviews * P.params.nu * P.params.nv))}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        s = cpu_sample(params, host_vol)
        cpu = {"value": s["voxel_views"] / s["seconds"] / 1e9, "unit": UNIT, "cores": s["cores"], "kind": s["kind"],
               "sample": "one view of DD forward + FDK-weighted DD backprojection over the full volume: "
                         + s["what"], "seconds": s["seconds"]}

    clocks = clk.summary()
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (30 seeded random ellipsoids)",
                "config": {"workload": WORKLOAD if not args.small else "small_%d" % n, "volume": [n, n, n],
                           "views": nviews, "detector": [P.params.nu, P.params.nv], "voxel_mm": 0.5,
                           "pixel_mm": 0.75, "sad_mm": 1000, "sdd_mm": 1500,
                           "step": "forward() + backward() (DD forward, FDK-weighted DD backprojection)",
                           "l2": "inputs larger than L2 (volume 512 MiB, projections 2.16 GiB)",
                           "parallelism": "replicas" if ws > 1 else "single GPU"},
                "kernels_ms": kern, "gpu_launches": 3 * args.steps, "effective_hbm_gbs": 2 * 4 * vv / (ms / 1e3) / 1e9,
                "roofline": roofline, "e2e": e2e, "cpu_baseline": cpu, "clocks": clocks, "matched_pair": matched}
        print(json.dumps(line))
    if ws > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", type=int, default=0, help="cube side for a quick small run (not the workload)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-matched", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
