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


def profiled_traffic(kernel, workload):
    """Per-launch DRAM bytes of `kernel` on `workload` from the committed ncu
    summary profiles/<kernel>_<workload>.md (a line 'traffic_bytes_per_launch:
    <N>'), or None when that workload's launches were not captured."""
    d = os.path.join(REPO, "profiles")
    for ext in (".md", ".txt"):
        path = os.path.join(d, "%s_%s%s" % (kernel, workload, ext))
        if not os.path.exists(path):
            continue
        with open(path) as fh:
            for line in fh:
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

    def __init__(self, index, tag="timed"):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", "ctgb_clocks_%s_%d_%d.csv" % (tag, os.getpid(), index))

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
        with open(self.path) as fh:
            lines = fh.readlines()
        for line in lines:
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
    names = ("transpose", "forward", "backproject_fdk")
    ev = {k: [] for k in names}
    # backward() = one bp_fdk_walk_kernel launch over all views (the full
    # orbit's four-fold symmetry; no integrated copy of the projections).
    launches_per_step = 1 + P.forward_launches() + 1

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
            for k, name in enumerate(names):
                ev[name].append((e[k], e[k + 1]))

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
    # Dominant kernel: bp_fdk_walk_kernel (one launch over all views) or the
    # forward (dd_forward_tma_kernel, one launch per run of same-axis views).
    nfwd = P.forward_launches()
    per_launch = {"forward": kern["forward"] / nfwd, "backproject_fdk": kern["backproject_fdk"]}
    dom = max(("forward", "backproject_fdk"), key=lambda k: kern[k])
    peak, peak_kind = measured_peaks()
    units = {"forward": vv / nfwd, "backproject_fdk": vv}[dom]      # voxel-views per launch
    alg_bytes = 4.0 * units              # 4 B per voxel-view per direction
    achieved = alg_bytes / (per_launch[dom] / 1e3) / 1e9
    kname = {"forward": "dd_forward_tma_kernel", "backproject_fdk": "bp_fdk_walk_kernel"}[dom]
    roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": profiled_traffic(kname, "dd_pair" if not args.small else "small"),
                "algorithmic_bytes_per_launch": alg_bytes, "ms_per_launch": per_launch[dom],
                "per_kernel_frac": {k: 4.0 * vv / (kern[k] / 1e3) / 1e9 / peak for k in ("forward", "backproject_fdk")},
                # the whole step (transpose, forward, backprojection): 4 B per voxel-view each way
                "pair_frac": 2 * 4.0 * vv / (ms / 1e3) / 1e9 / peak}

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

    # end to end through the public API with host data (copies inside the
    # timed region): the volume in pinned host memory goes in, the projections
    # come back to pinned host memory after forward(), go in again for
    # backward(), and the volume comes back.
    host_vol = vol.cpu().numpy()
    pinned_vol = torch.from_numpy(host_vol).pin_memory()
    R = Reconstruction(params, device=dev)
    e2e_steps = max(1, min(args.steps, 10))
    R.image = pinned_vol
    R.forward()
    R.backward()
    barrier()
    fwd_ms, bwd_ms = [], []
    with ClockSampler(local, "e2e") as clk_e2e:
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ta = time.perf_counter()
            R.image = pinned_vol
            R.forward()
            tb = time.perf_counter()
            R.backward()
            tc = time.perf_counter()
            fwd_ms.append((tb - ta) * 1e3)
            bwd_ms.append((tc - tb) * 1e3)
        barrier()
        e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": ws * vv / e2e_s / 1e9, "unit": UNIT, "ms_per_step": e2e_s * 1e3, "steps": e2e_steps,
           "h2d_bytes_per_step": int(4 * (n ** 3 + nviews * P.params.nu * P.params.nv)),
           "d2h_bytes_per_step": int(4 * (n ** 3 + nviews * P.params.nu * P.params.nv)),
           "forward_ms": [round(v, 2) for v in fwd_ms], "backward_ms": [round(v, 2) for v in bwd_ms],
           "clocks": clk_e2e.summary()}

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
                           "l2": "inputs larger than L2 (volume %.0f MiB, projections %.2f GiB)" % (
                               4.0 * n ** 3 / 2 ** 20, 4.0 * proj.numel() / 2 ** 30),
                           "parallelism": "replicas" if ws > 1 else "single GPU"},
                "kernels_ms": kern, "gpu_launches": launches_per_step * args.steps, "effective_hbm_gbs": 2 * 4 * vv / (ms / 1e3) / 1e9,
                "roofline": roofline, "e2e": e2e, "cpu_baseline": cpu, "clocks": clocks, "matched_pair": matched}
        print(json.dumps(line))
    if ws > 1:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# Other BASELINE configurations (one JSON line each; not the headline workload).
def _timed(fn, steps, warmup):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def _timed_stages(stages, steps, warmup):
    """Run the (name, fn) stages in order `steps` times after `warmup` untimed
    rounds; CUDA events on the current stream around every stage.  Returns
    (ms per round, {name: ms per round})."""
    import torch
    for _ in range(warmup):
        for _, fn in stages:
            fn()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    marks = []
    first = torch.cuda.Event(enable_timing=True)
    first.record(stream)
    for _ in range(steps):
        row = []
        for _, fn in stages:
            fn()
            e = torch.cuda.Event(enable_timing=True)
            e.record(stream)
            row.append(e)
        marks.append(row)
    torch.cuda.synchronize()
    per = {name: 0.0 for name, _ in stages}
    prev = first
    for row in marks:
        for (name, _), e in zip(stages, row):
            per[name] += prev.elapsed_time(e)
            prev = e
    total = first.elapsed_time(marks[-1][-1]) / steps
    return total, {k: v / steps for k, v in per.items()}


def _lib_call(name, *args):
    """A C-ABI call whose tensor arguments become device pointers and whose
    float/int arguments pass through; the element count of the first tensor
    and the current stream are appended (the element-wise iterative updates'
    signature)."""
    import ctypes
    import torch
    from ctreconstruction_gb300 import _lib
    conv = [ctypes.c_void_p(a.data_ptr()) if isinstance(a, torch.Tensor) else a for a in args]
    first = next(a for a in args if isinstance(a, torch.Tensor))
    _lib.call(name, *conv, first.numel(), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def hbm_roofline(kernel, ms_per_launch, alg_bytes, what, workload):
    """roofline object for an HBM-bound kernel: algorithmic bytes per launch
    (`what` says how they are counted) over its CUDA-event time per launch,
    against the measured copy bandwidth; DRAM traffic from the workload's own
    ncu summary where one is committed."""
    peak, kind = measured_peaks()
    achieved = alg_bytes / (ms_per_launch / 1e3) / 1e9
    return {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": kind, "traffic": profiled_traffic(kernel, workload),
            "algorithmic_bytes_per_launch": alg_bytes, "ms_per_launch": ms_per_launch, "bytes_model": what}


def ref_voxel_view_rate(params, views, vol=None, nthreads=None):
    """CPU: the reference's CUDA-C kernels compiled for the host
    (distance_project_on_*3 forward, flat_distance_backproj_arb2 backward)
    on `views` of one scan, all host threads.  Returns (seconds per
    voxel-view for forward + backward, forward s, backward s, kind, what)."""
    from oracle import ref_runner
    nthreads = nthreads or os.cpu_count()
    n = params['NumberOfImage']
    nvox = int(n[0]) * int(n[1]) * int(n[2])
    if vol is None:
        vol = np.random.default_rng(0).random((n[2], n[1], n[0]), dtype=np.float32)
    if not ref_runner.available():
        from oracle.oracle import OracleGeometry
        g = OracleGeometry(params)
        t0 = time.perf_counter()
        pv = [g.forward(vol, v, 1, nthreads).astype(np.float32) for v in views]
        t1 = time.perf_counter()
        for v, q in zip(views, pv):
            g.backward_fdk(q, v, 1, nthreads)
        t2 = time.perf_counter()
        return (t2 - t0) / (2.0 * nvox * len(views)), t1 - t0, t2 - t1, "port", "FP64 C oracle port, OpenMP"
    r = ref_runner.RefScan(dict(params, DetectorOffset=[0.0, 0.0]))
    t0 = time.perf_counter()
    pv = [r.forward_view(vol, v, nthreads) for v in views]
    t1 = time.perf_counter()
    out = None
    for v, q in zip(views, pv):
        out = r.backward_view(q, v, r.angles[1] - r.angles[0], out=out, nthreads=nthreads)
    t2 = time.perf_counter()
    return ((t2 - t0) / (2.0 * nvox * len(views)), t1 - t0, t2 - t1, "reference",
            "reference CUDA-C kernels (distance_project_on_*3, flat_distance_backproj_arb2) as host C++, OpenMP")


def run_fdk128(args):
    """FDK 128^3 (1 mm), 360 views, 256x192 detector (1.5 mm), SAD 1000, SDD
    1500; modified Shepp-Logan, DD-forward projections with Poisson noise at
    I0 = 1e5; Filtering() + backward() with a Hann ramp."""
    import torch
    from ctreconstruction_gb300 import Projector, phantoms
    p = {'SourceInit': [0.0, 1000.0, 0.0], 'DetectorInit': [0.0, -500.0, 0.0], 'StartAngle': 0.0,
         'EndAngle': 2 * np.pi, 'NumberOfDetectorPixels': [256, 192], 'DetectorPixelSize': [1.5, 1.5],
         'NumberOfViews': 360, 'ImagePixelSpacing': [1.0, 1.0, 1.0], 'NumberOfImage': [128, 128, 128],
         'FilterType': 'hann', 'cutoff': 1.0}
    P = Projector(p)
    ph = phantoms.shepp_logan_3d((128, 128, 128), device=P.device) * 0.02
    clean = P.forward(ph)
    gen = torch.Generator(device=P.device).manual_seed(0)
    counts = torch.poisson(1e5 * torch.exp(-clean), generator=gen)
    proj = -torch.log(torch.clamp(counts, min=1.0) / 1e5)
    q = torch.empty_like(proj)
    out = torch.empty(P.volume_shape, device=P.device)
    # Filtering() then backward() (one bp_fdk_walk_kernel launch: the full
    # orbit's four-fold symmetry), issued as separate stages so each is timed.
    stages = [("copy", lambda: q.copy_(proj)), ("filter", lambda: P.filter(q)),
              ("backproject", lambda: P.backproject_fdk(q, out=out))]
    ms, per = _timed_stages(stages, args.steps, args.warmup)
    ms -= per["copy"]                      # restoring the input is not part of the step
    vv = 128 ** 3 * 360
    inner = ph.abs() > 0
    rmse = float(torch.sqrt(torch.mean((out - ph)[inner] ** 2)))
    dom = max(("filter", "backproject"), key=lambda k: per[k])
    if dom == "backproject":
        roof = hbm_roofline("bp_fdk_walk_kernel", per["backproject"], 4.0 * vv, "4 B per voxel-view", "fdk128")
    else:
        roof = hbm_roofline("fdk_filter_kernel", per["filter"], 8.0 * 360 * 256 * 192, "8 B per detector pixel",
                            "fdk128")
    roof["per_stage_ms"] = per
    cpu = None
    if not args.no_cpu:
        # The reference's CPU path for this configuration: Filtering() in NumPy
        # (the FP64 restatement, oracle.fdk_filter) and the reference's
        # backprojection kernel for every view, all host threads.
        from oracle import ref_runner
        from oracle.oracle import OracleGeometry
        host = proj.cpu().numpy()
        nthreads = os.cpu_count()
        t0 = time.perf_counter()
        filt = OracleGeometry(p).filtering(host).astype(np.float32)
        t1 = time.perf_counter()
        if ref_runner.available():
            r = ref_runner.RefScan(dict(p, DetectorOffset=[0.0, 0.0], ReconCenter=[0, 0, 0]))
            acc = None
            for v in range(360):
                acc = r.backward_view(filt[v], v, r.angles[1] - r.angles[0], out=acc, nthreads=nthreads)
            kind, what = "reference", "flat_distance_backproj_arb2 as host C++ (OpenMP) + NumPy Filtering"
        else:
            OracleGeometry(p).backward_fdk(filt, 0, 360, nthreads)
            kind, what = "port", "FP64 C oracle port (OpenMP) + NumPy Filtering"
        t2 = time.perf_counter()
        cpu = {"value": vv / (t2 - t0) / 1e9, "unit": UNIT, "cores": nthreads, "kind": kind,
               "sample": "the whole workload (360 views, 128^3): " + what, "filter_s": t1 - t0,
               "backproject_s": t2 - t1}
    return {"metric": "FDK reconstruction throughput", "value": vv / (ms / 1e3) / 1e9, "unit": UNIT,
            "ms_per_step": ms, "higher_is_better": True, "dtype": "f32", "data": "synthetic (Shepp-Logan, Poisson)",
            "config": {"workload": "fdk_128cube_360views_det256x192", "step": "Filtering() + backward()",
                       "l2": "volume 8 MiB and projections 70 MiB fit L2: after the first step the inputs are "
                             "L2-resident (upper bound on HBM-bound throughput)"},
            "gpu_launches": (1 + 2) * args.steps, "rmse_vs_phantom_inside": rmse, "roofline": roof,
            "cpu_baseline": cpu}


def run_fan_batch(args):
    """256 fan-beam slices (86 x 256^2, 85 x 384^2, 85 x 512^2 on a 0.8 mm
    grid), 720 views over 2 pi, 984 channels, SAD 570, SDD 1040 (line
    detector pitch 1.0 mm; arc detector the same pitch as an arc length), 20
    random ellipses per slice with exact line-integral sinograms.  One batch
    = filtering (Hann, cutoff 1.0; the balanced equiangular kernel for the
    arc detector) + one persistent backprojection launch with the autotuned
    tile; both detector shapes are timed.  Quality: scale-fitted relative
    error against the phantom on three slices."""
    import torch
    from ctreconstruction_gb300 import phantoms
    from ctreconstruction_gb300.fanbeam import FanBatch, slice_from_grid
    nviews, nch, sad, sdd, pitch = 720, 984, 570.0, 1040.0, 1.0
    sizes = [256] * 86 + [384] * 85 + [512] * 85
    dev = torch.device("cuda", torch.cuda.current_device())
    out = {}
    rmse = {}
    for arc in (False, True):
        geom = type("G", (), dict(source_to_axis=sad, source_to_detector=sdd, pixel_width=pitch, det_width=nch,
                                  nviews=nviews, angle_coverage=2 * np.pi))()
        slices = [slice_from_grid(n, n, 0.8, geom, arc=arc) for n in sizes]
        sinos, truth = [], []
        for i, (n, s) in enumerate(zip(sizes, slices)):
            half = (n - 1) / 2.0 * 0.8
            ell = [(v, cx * half, cy * half, a * half, b * half, ph)
                   for v, cx, cy, a, b, ph in phantoms.random_ellipses(20, seed=1000 + i)]
            gam = s.g0 + s.dg * np.arange(nch)
            sinos.append(phantoms.ellipse_fan_sinogram(ell, sad, nviews, gam, s.dtheta, arc=arc, device=dev))
            if i in (0, 86, 171):
                grid = torch.linspace(-half, half, n, device=dev)
                truth.append((i, phantoms.ellipse_image(ell, grid, grid)))
        batch = FanBatch(slices, filter_type='hann', cutoff=1.0, arc_kernel='balanced' if arc else 'reference')
        flat = batch.pack(sinos)
        work = torch.empty_like(flat)
        images = torch.empty(batch.image_floats, device=flat.device)
        work.copy_(flat)
        batch.filter(work)
        batch.backproject(work, images)            # autotunes the tile once (untimed)

        stages = [("copy", lambda: work.copy_(flat)), ("filter", lambda: batch.filter(work)),
                  ("backproject", lambda: batch.backproject(work, images))]
        ms, per = _timed_stages(stages, args.steps, args.warmup)
        ms -= per["copy"]
        imgs = batch.unpack(images)
        errs = []
        for i, t in truth:
            k = float((imgs[i] * t).sum() / (t * t).sum())
            errs.append(round(float(torch.linalg.norm(imgs[i] - k * t) / torch.linalg.norm(k * t)), 4))
        rmse["arc" if arc else "line"] = errs
        pv = sum(n * n for n in sizes) * nviews
        out["arc" if arc else "line"] = {"ms_per_batch": ms, "Gpixel_views_per_s": pv / (ms / 1e3) / 1e9,
                                         "per_stage_ms": per, "tile": list(batch.tile),
                                         "fitted_rel_err_slices_0_86_171": rmse["arc" if arc else "line"]}
        if not arc:
            line_sino, line_slice = sinos[0].cpu().numpy(), slices[0]
    total_ms = out["line"]["ms_per_batch"] + out["arc"]["ms_per_batch"]
    pv = sum(n * n for n in sizes) * nviews
    # Dominant kernel: the persistent backprojection (one launch per batch).
    bp_ms = max(out["line"]["per_stage_ms"]["backproject"], out["arc"]["per_stage_ms"]["backproject"])
    roof = hbm_roofline("fan_bp_kernel", bp_ms, 4.0 * pv, "4 B per pixel-view", "fan_batch")
    cpu = None
    if not args.no_cpu:
        # FanBeam.py's own reconstruction restated in FP64 NumPy
        # (oracle/standalone: Filter + per-view interpolated backprojection) on
        # one 256^2 slice over all 720 views (NumPy's own threads).
        from oracle import standalone as osa
        n = 256
        x = (np.arange(n) - (n - 1) / 2.0) * 0.8
        ang = np.arange(nviews) * (2 * np.pi / nviews)
        t0 = time.perf_counter()
        Q, gam = osa.fan_filter(line_sino, sad, sdd, pitch, False, 'hann', 1.0)
        osa.fan_backproject(Q, gam, x, x, sad, sdd, ang, False)
        t1 = time.perf_counter()
        cpu = {"value": n * n * nviews / (t1 - t0) / 1e9, "unit": "Gpixel*views/s", "cores": 1, "kind": "port",
               "sample": "one 256^2 slice, 720 views, line detector: FanBeam.py's filter and backprojection "
                         "restated in FP64 NumPy (oracle/standalone.py)", "seconds": t1 - t0}
    return {"metric": "batched fan-beam FBP throughput", "value": 2 * pv / (total_ms / 1e3) / 1e9,
            "unit": "Gpixel*views/s", "ms_per_step": total_ms, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (20 random ellipses per slice, exact line integrals)",
            "config": {"workload": "fan_batch_256slices_720views_984ch", "detectors": ["line", "arc"],
                       "l2": "sinograms 725 MB and images 172 MB per detector exceed L2"},
            "gpu_launches": 4 * args.steps, "roofline": roof, "cpu_baseline": cpu, "detail": out}


def run_iter(args):
    """Batched OS-SART (10 subsets, lambda 0.8) and MLEM over 16 cone-beam
    scans, volumes 128^3..384^3 (multiples of 16), 90 views, detector 2N x 2N
    at 1.5x the voxel pitch, random ellipsoids with Poisson noise at I0 =
    5e4.  Each method's 16 scans advance together (ctreconstruction_gb300.batch):
    per OS-SART subset, one persistent forward launch per dominant axis and
    one persistent backprojection over all 16 scans, with the update lines
    fused into their stores; one CUDA graph holds one iteration, so an
    iteration is one graph launch.  Reports ms per batch iteration and the
    implied time of the configured runs (20 OS-SART iterations, 50 MLEM
    iterations), and for comparison the same scans as concurrent per-scan
    branches of one graph with separate element-wise kernels."""
    import torch
    from ctreconstruction_gb300 import Projector, iterative, phantoms
    sides = [int(round(v / 16.0)) * 16 for v in np.linspace(128, 384, 16)]
    dev = torch.device("cuda", torch.cuda.current_device())
    scans = []
    for i, n in enumerate(sides):
        vox = 256.0 / n
        p = {'SourceInit': [0.0, 1000.0, 0.0], 'DetectorInit': [0.0, -500.0, 0.0], 'StartAngle': 0.0,
             'EndAngle': 2 * np.pi, 'NumberOfDetectorPixels': [2 * n, 2 * n],
             'DetectorPixelSize': [1.5 * vox, 1.5 * vox], 'NumberOfViews': 90,
             'ImagePixelSpacing': [vox, vox, vox], 'NumberOfImage': [n, n, n]}
        P = Projector(p, device=dev)
        ph = phantoms.random_ellipsoids((n, n, n), n=30, seed=10 + i, device=dev) * 0.01
        clean = P.forward(ph)
        gen = torch.Generator(device=dev).manual_seed(i)
        counts = torch.poisson(5e4 * torch.exp(-clean), generator=gen)
        scans.append((p, -torch.log(torch.clamp(counts, min=1.0) / 5e4), ph))
    vv = sum(float(n) ** 3 * 90 for n in sides)

    def time_batch(batch, iters):
        batch.capture()
        batch.run(max(1, args.warmup))
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        batch.run(iters)
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / iters

    from ctreconstruction_gb300 import batch
    os_batch = batch.batched_os_sart([(Projector(p, device=dev), q) for p, q, _ in scans], nsubsets=10, lam=0.8)
    t_os = time_batch(os_batch, max(1, args.steps))
    os_launches = os_batch.launches_per_step()
    os_rmse = [float(torch.sqrt(torch.mean((s.x - ph) ** 2))) for s, (_, _, ph) in zip(os_batch.solvers, scans)]
    os_ctas = (os_batch.fwd_ctas, os_batch.bp_ctas)
    del os_batch
    em_batch = batch.batched_mlem([(Projector(p, device=dev), q.clamp(min=0)) for p, q, _ in scans])
    t_em = time_batch(em_batch, max(1, args.steps))
    em_launches = em_batch.launches_per_step()
    del em_batch
    # For comparison: the same solvers as concurrent per-scan branches of one
    # CUDA graph, with separate element-wise kernels.
    br = iterative.SolverBatch([iterative.OSSART(Projector(p, device=dev), q, nsubsets=10, lam=0.8)
                                for p, q, _ in scans])
    t_os_branches = time_batch(br, max(1, args.steps))
    del br
    # Dominant kernel: one OS-SART sub-iteration of the largest scan (384^3,
    # 9 views) issued eagerly, each launch group timed alone (inside the graph
    # the launches of 16 scans overlap and cannot be timed one by one).
    p_big, q_big, _ = scans[-1]
    solver = iterative.OSSART(Projector(p_big, device=dev), q_big, nsubsets=10, lam=0.8)
    Ps, ps0, a1, b1 = solver.subsets[0]
    S, x = solver.S, solver.x
    stages = [("forward", lambda: Ps.forward(x, out=S.proj)),
              ("residual", lambda: _lib_call("ctgb_pocs_residual", ps0, S.proj, a1, solver.eps, S.res)),
              ("backproject_matched", lambda: iterative._backproject(Ps, S.res, S.bp, True)),
              ("update", lambda: _lib_call("ctgb_pocs_update", x, S.bp, b1, solver.lam, solver.eps, x))]
    _, per = _timed_stages(stages, 3, 2)
    nb = sides[-1]
    vv_sub = float(nb) ** 3 * 9
    dom = max(("forward", "backproject_matched"), key=lambda k: per[k])
    roof = hbm_roofline({"forward": "dd_forward_tma_kernel",
                         "backproject_matched": "bp_matched_integ_kernel"}[dom], per[dom], 4.0 * vv_sub,
                        "4 B per voxel-view (one 9-view subset of the 384^3 scan; the backprojection's time "
                        "includes its integration pass)", "iter")
    roof["per_stage_ms_384cube_subset"] = per
    del solver
    cpu = None
    if not args.no_cpu:
        spv, tf, tb, kind, what = ref_voxel_view_rate(p_big, [0])
        cpu = {"value": 1.0 / spv / 1e9, "unit": UNIT + " (forward + backprojection)", "cores": os.cpu_count(),
               "kind": kind, "sample": "one view forward + one view backward of the 384^3 scan: " + what,
               "forward_s": tf, "backward_s": tb}
    # voxel-views per batch iteration: one forward + one backprojection per view
    return {"metric": "batched OS-SART iteration throughput", "value": 2 * vv / (t_os / 1e3) / 1e9,
            "unit": UNIT + " (forward + backprojection)", "ms_per_step": t_os, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic (random ellipsoids, Poisson I0=5e4)",
            "config": {"workload": "os_sart_mlem_16scans_128to384_90views", "sides": sides,
                       "graph": "one CUDA graph launch per batch iteration",
                       "launches": "per OS-SART subset: one batched transpose, one persistent forward launch per "
                                   "dominant axis (POCS residual fused), one integration, one persistent matched "
                                   "backprojection (POCS update fused), all 16 scans in each",
                       "persistent_ctas_per_sm_fwd_bp": os_ctas},
            "os_sart_launches_per_iteration": os_launches, "mlem_launches_per_iteration": em_launches,
            "os_sart_ms_per_iteration_per_scan_graph_branches": t_os_branches,
            "os_sart_ms_per_iteration": t_os, "mlem_ms_per_iteration": t_em,
            "mlem_value": 2 * vv / (t_em / 1e3) / 1e9,
            "os_sart_20_iterations_s": 20 * t_os / 1e3, "mlem_50_iterations_s": 50 * t_em / 1e3,
            "gpu_launches": None, "roofline": roof, "cpu_baseline": cpu,
            "os_sart_rmse_after_%d_iterations" % (2 + max(1, args.warmup) + max(1, args.steps)): os_rmse[:4]}


def run_asd256(args):
    """ASD-POCS at 256^3, 60 views, 512x384 detector (plain TV step, alpha
    0.002, 20 TV steps, na = 5): time per outer iteration and RMSE."""
    import torch
    from ctreconstruction_gb300 import Projector, iterative, phantoms
    p = {'SourceInit': [0.0, 1000.0, 0.0], 'DetectorInit': [0.0, -500.0, 0.0], 'StartAngle': 0.0,
         'EndAngle': 2 * np.pi, 'NumberOfDetectorPixels': [512, 384], 'DetectorPixelSize': [0.75, 0.75],
         'NumberOfViews': 60, 'ImagePixelSpacing': [0.5, 0.5, 0.5], 'NumberOfImage': [256, 256, 256],
         'FilterType': 'hann', 'cutoff': 1.0}
    P = Projector(p)
    ph = phantoms.random_ellipsoids((256, 256, 256), n=30, seed=5, device=P.device) * 0.02
    proj = P.forward(ph)
    norms = iterative.normalisers(P)
    iterative.asd_pocs(P, proj, niter=1, alpha=0.002, norms=norms)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    x, rmse, log = iterative.asd_pocs(P, proj, niter=3, alpha=0.002, norms=norms, phantom=ph)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / 3
    roof, cpu = _asd_roofline_cpu(P, x, args)
    return {"metric": "ASD-POCS outer-iteration time", "value": ms, "unit": "ms", "higher_is_better": False,
            "dtype": "f32", "data": "synthetic (random ellipsoids)",
            "config": {"workload": "asd_pocs_256cube_60views_det512x384", "na": 5, "ng": 20, "alpha": 0.002},
            "rmse_per_iteration": rmse, "gpu_launches": None, "roofline": roof, "cpu_baseline": cpu}


def _asd_roofline_cpu(P, x, args, niter_label="outer iteration"):
    """Roofline of the dominant kernel of one ASD-POCS outer iteration at
    256^3 / 60 views (its five data sub-steps' forward and FDK-weighted
    backprojection, and the 20-step TV descent, each timed alone), and the
    reference's CPU cost of one outer iteration extrapolated from one view
    forward + one view backward and one NumPy TV gradient."""
    import torch
    from ctreconstruction_gb300 import iterative
    proj = torch.empty(P.proj_shape(), device=P.device)
    vol = torch.empty(P.volume_shape, device=P.device)
    xt = x.clone()
    stages = [("forward", lambda: P.forward(x, out=proj)), ("backproject", lambda: P.backproject_fdk(proj, out=vol)),
              ("tv20", lambda: iterative.tv_descent(xt, 1e-6, 20))]
    _, per = _timed_stages(stages, 3, 2)
    n = P.volume_shape[0]
    vv = float(n) ** 3 * P.params.NumberOfViews
    nfwd = P.forward_launches()
    cand = {"forward": (per["forward"] / nfwd, 4.0 * vv / nfwd, "dd_forward_tma_kernel", "4 B per voxel-view"),
            "backproject": (per["backproject"], 4.0 * vv, "bp_fdk_walk_kernel", "4 B per voxel-view"),
            "tv20": (per["tv20"] / 20, 12.0 * n ** 3, "tv_norm_kernel + tv_step_kernel",
                     "12 B per voxel per TV step (read for the norm; read + write for the step)")}
    # dominant: the largest share of one outer iteration (5 forward + 5 backprojections + 1 TV descent)
    share = {"forward": 5 * per["forward"], "backproject": 5 * per["backproject"], "tv20": per["tv20"]}
    dom = max(share, key=share.get)
    ms_l, by, kname, what = cand[dom]
    roof = hbm_roofline(kname, ms_l, by, what, "asd256")
    roof["per_stage_ms"] = per
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as ora
        spv, tf, tb, kind, what = ref_voxel_view_rate(P.params.as_dict(), [0])
        xh = x.cpu().numpy()
        t0 = time.perf_counter()
        ora.tv_grad(xh)
        t_tv = time.perf_counter() - t0
        ms_cpu = (5 * 2 * vv * spv + 20 * t_tv) * 1e3
        cpu = {"value": ms_cpu, "unit": "ms per " + niter_label, "cores": os.cpu_count(), "kind": kind,
               "sample": "extrapolated from one view forward + one view backward at 256^3 (" + what + ") and "
                         "one NumPy TV gradient (ASD_POCS.py tv_grad restated): 5 x (60-view forward + "
                         "60-view backward) + 20 TV steps", "tv_grad_s": t_tv, "forward_s": tf, "backward_s": tb}
    return roof, cpu


def run_asd256_learned(args):
    """Learned proximal step at 256^3, 60 views, 512x384 detector: (1) 2,000
    (pre-TV, post-TV) crop pairs (32x32x64) from plain ASD-POCS on 8 training
    phantoms from a zero start (25 pairs x 10 crops each; with --ahead K the
    volume before the TV step of iteration k is paired with the volume after
    the TV step of iteration k + K); (2) training of the 3-D U-Net
    (Adam, batch 8); (3) plain and learned ASD-POCS on a held-out phantom,
    20 iterations each, the learned step judged against the plain TV step on
    every iteration (data residual within 1 %).  Both runs start from a zero
    volume (from the FBP start the plain run's RMSE stays flat within 1 %
    over 20 iterations, so time-to-RMSE would be trivially 0).  Reports RMSE
    vs the phantom, wall time to reach the plain run's final RMSE x 1.01,
    and the U-Net's forward time and TFLOP/s at 256^3."""
    import torch
    from ctreconstruction_gb300 import Projector, iterative, learned, phantoms
    dev = torch.device("cuda", torch.cuda.current_device())
    p = {'SourceInit': [0.0, 1000.0, 0.0], 'DetectorInit': [0.0, -500.0, 0.0], 'StartAngle': 0.0,
         'EndAngle': 2 * np.pi, 'NumberOfDetectorPixels': [512, 384], 'DetectorPixelSize': [0.75, 0.75],
         'NumberOfViews': 60, 'ImagePixelSpacing': [0.5, 0.5, 0.5], 'NumberOfImage': [256, 256, 256],
         'FilterType': 'hann', 'cutoff': 1.0}
    P = Projector(p, device=dev)
    norms = iterative.normalisers(P)
    asd = dict(alpha=0.002, ng=20, na=5)
    t0 = time.perf_counter()
    train_ph = [phantoms.random_ellipsoids((256, 256, 256), n=30, seed=100 + i, device=dev) * 0.02 for i in range(8)]
    zero = torch.zeros((256, 256, 256), device=dev)
    # 25 + K iterations per phantom from a zero start, 10 crops per pair
    # (pre-TV at k, post-TV at k + K): 8 x 25 x 10 = 2,000 pairs.
    pairs = learned.tv_pairs(P, train_ph, niter=25 + args.ahead, crops=10, size=(32, 32, 64), seed=0,
                             ahead=args.ahead, x0=zero, **asd)
    del train_ph
    torch.cuda.synchronize()
    t_pairs = time.perf_counter() - t0
    net = learned.UNet3D(device=dev, seed=0)
    t0 = time.perf_counter()
    losses = learned.train(net, pairs, steps=args.train_steps, batch=8, size=(32, 32, 64), lr=1e-3, seed=0)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    n_pairs = len(pairs)
    del pairs
    ph = phantoms.random_ellipsoids((256, 256, 256), n=30, seed=5, device=dev) * 0.02
    proj0 = P.forward(ph)
    niter = 20
    iterative.asd_pocs(P, proj0, niter=1, norms=norms, x0=zero, **asd)          # warm
    t_plain = []
    _, rmse_plain, _ = iterative.asd_pocs(P, proj0, niter=niter, norms=norms, phantom=ph, times=t_plain, x0=zero,
                                          **asd)
    # Warm the learned step at the full volume size (the network was trained
    # on crops: its first 256^3 call builds tensor maps and sets kernel
    # attributes), as the plain step was warmed above.
    warm = learned.LearnedProx(net, P, proj0, tol=0.01, judge_every=1)
    warm(zero.clone(), lambda: iterative.tv_descent(zero.clone(), 1e-6, asd["ng"]))
    torch.cuda.synchronize()
    prox = learned.LearnedProx(net, P, proj0, tol=0.01, judge_every=1)
    t_learn = []
    _, rmse_learn, _ = iterative.asd_pocs(P, proj0, niter=niter, norms=norms, phantom=ph, prox=prox,
                                          times=t_learn, x0=zero, **asd)
    target = 1.01 * rmse_plain[-1]
    reach = next((i for i, r in enumerate(rmse_learn) if r <= target), None)
    # FDK (Filtering() + backward()) of the same data, for scale: the RMSE
    # the iterative runs are measured against.
    fq = proj0.clone()
    P.filter(fq)
    rmse_fbp = float(torch.sqrt(torch.mean((P.backproject_fdk(fq) - ph) ** 2)))
    # U-Net forward alone at 256^3 and the 20-step TV descent it replaces
    x = ph.clone()
    net.forward(x, net.scale)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(3):
        net.forward(x, net.scale)
    b.record()
    torch.cuda.synchronize()
    unet_ms = a.elapsed_time(b) / 3
    a.record()
    iterative.tv_descent(x, 1e-4, 20)
    b.record()
    torch.cuda.synchronize()
    tv_ms = a.elapsed_time(b)
    flops = learned.FLOPS_PER_VOXEL * 256 ** 3
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            bpeak, bkind = float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        bpeak, bkind = 1900.0, "fallback"
    tf = flops / (unet_ms / 1e3) / 1e12
    roof = {"bound": "tensor", "kernel": "conv3d_tc_dx_kernel (U-Net forward, all layers)", "achieved": tf,
            "peak": bpeak, "unit": "TFLOP/s", "frac": tf / bpeak, "peak_source": bkind, "flops_per_pass": flops,
            "ms_per_pass": unet_ms}
    _, cpu = _asd_roofline_cpu(P, ph, args, "plain outer iteration")
    return {"metric": "learned ASD-POCS wall time to the plain RMSE (x1.01), relative to plain",
            "value": (t_learn[reach] / t_plain[-1]) if reach is not None else None, "unit": "ratio",
            "higher_is_better": False, "dtype": "bf16 U-Net / f32 projectors",
            "data": "synthetic (random ellipsoids, 8 training phantoms + 1 held out)",
            "config": {"workload": "asd_pocs_learned_256cube_60views_det512x384", "alpha": 0.002, "ng": 20,
                       "na": 5, "iterations": niter, "pairs": n_pairs, "train_steps": args.train_steps,
                       "pair_ahead": args.ahead},
            "rmse_plain": rmse_plain, "rmse_learned": rmse_learn, "rmse_fbp": rmse_fbp, "plain_s": t_plain[-1],
            "learned_s_cumulative": t_learn,
            "learned_s_per_iteration": t_learn[-1] / niter, "plain_s_per_iteration": t_plain[-1] / niter,
            "learned_reaches_target_at_iteration": reach, "accepted": prox.accepted, "rejected": prox.rejected,
            "train_loss_first_last": [float(np.mean(losses[:10])), float(np.mean(losses[-10:]))],
            "pairs_s": t_pairs, "train_s": t_train, "unet_forward_ms_256cube": unet_ms,
            "unet_tflops": flops / (unet_ms / 1e3) / 1e12, "tv20_ms_256cube": tv_ms, "roofline": roof,
            "cpu_baseline": cpu}


def run_rows(args):
    """The hot path's other rows at 256^3 (0.5 mm), 360 views, 512x384
    detector (0.75 mm), SAD 1000 mm, SDD 1500 mm, 30 seeded random
    ellipsoids; each timed with CUDA events, inputs and outputs on the
    device, in Gvoxel*views/s: the DD pair (forward + FDK-weighted
    backprojection) on a flat detector, on a curved (equiangular
    cylindrical) detector and on a helical orbit (pitch 0.5); the Siddon
    ray-driven pair (forward + transpose); the voxel-driven ConeBeamGPU
    backprojection (360 views onto 256^3).  `value` is the curved DD pair."""
    import ctypes
    import torch
    from ctreconstruction_gb300 import Projector, _lib, phantoms
    from ctreconstruction_gb300.projector import _ptr, _stream
    from ctreconstruction_gb300.standalone import _cparams
    dev = torch.device("cuda", torch.cuda.current_device())
    n, nviews, nu, nv = (args.small or 256), 360, 512, 384
    base = scan_params(n, nviews, nu, nv)
    ph = phantoms.random_ellipsoids((n, n, n), n=30, seed=1, device=dev) * 0.02
    vv = n ** 3 * nviews
    detail = {}

    def rate(ms):
        return {"ms": ms, "Gvoxel_views_per_s": vv / (ms / 1e3) / 1e9}

    for name, extra in (("dd_pair_curved", {'DetectorShape': 'Curved'}), ("dd_pair_helical", {'Pitch': 0.5}),
                        ("dd_pair_flat", {})):
        P = Projector(dict(base, **extra), device=dev)
        proj = torch.empty(P.proj_shape(), device=dev)
        vol = torch.empty_like(ph)

        stages = [("forward", lambda P=P, proj=proj: P.forward(ph, out=proj)),
                  ("backproject", lambda P=P, proj=proj, vol=vol: P.backproject_fdk(proj, out=vol))]
        ms, per = _timed_stages(stages, args.steps, args.warmup)
        detail[name] = dict(rate(ms), per_stage_ms=per)
    P = Projector(dict(base, Method='Ray'), device=dev)
    proj = torch.empty(P.proj_shape(), device=dev)
    vol = torch.empty_like(ph)

    def ray_pair():
        P.ray_forward(ph, out=proj)
        P.ray_backproject(proj, out=vol)

    detail["siddon_pair"] = rate(_timed(ray_pair, args.steps, args.warmup))
    c = _cparams({'SourceToAxis': 1000.0, 'SourceToDetector': 1500.0, 'DetectorPixelWidth': 0.75,
                  'DetectorPixelHeight': 0.75, 'DetectorWidth': nu, 'DetectorHeight': nv, 'NumberOfViews': nviews,
                  'AngleCoverage': 2 * np.pi, 'ReconX': n, 'ReconY': n, 'ReconZ': n})
    nb = ctypes.c_size_t(0)
    _lib.call("ctgb_conebeam_table_bytes", ctypes.byref(c), ctypes.byref(nb))
    host = np.zeros(nb.value // 4, dtype=np.float32)
    _lib.call("ctgb_conebeam_table_build", ctypes.byref(c), host.ctypes.data_as(ctypes.c_void_p), nb.value)
    table = torch.from_numpy(host).to(dev)
    q = torch.rand((nviews, nv, nu), device=dev, generator=torch.Generator(device=dev).manual_seed(2))
    recon = torch.empty((n, n, n), device=dev)

    def cone_bp():
        _lib.call("ctgb_conebeam_backproject", ctypes.byref(c), _ptr(table), _ptr(q), _ptr(recon), 0, nviews, 0,
                  _stream())

    detail["conebeam_fdk_backprojection"] = rate(_timed(cone_bp, args.steps, args.warmup))
    per = detail["dd_pair_curved"]["per_stage_ms"]
    dom = max(per, key=per.get)
    nfwd = Projector(dict(base, DetectorShape='Curved'), device=dev).forward_launches()
    roof = hbm_roofline({"forward": "dd_forward_tma_kernel", "backproject": "bp_fdk_walk_kernel"}[dom],
                        per[dom] / (nfwd if dom == "forward" else 1), 4.0 * vv / (nfwd if dom == "forward" else 1),
                        "4 B per voxel-view, curved detector", "rows")
    cpu = None
    if not args.no_cpu:
        # Curved detectors run only in the reference's numba flavour (its
        # pycuda curved backprojector is called with 8 of 17 arguments), so
        # the CPU baseline is the FP64 C oracle port of that flavour.
        from oracle.oracle import OracleGeometry
        g = OracleGeometry(dict(base, DetectorShape='Curved'))
        vol_h = ph.cpu().numpy()
        nthreads = os.cpu_count()
        t0 = time.perf_counter()
        pv = g.forward(vol_h, 7, 1, nthreads).astype(np.float32)
        t1 = time.perf_counter()
        g.backward_fdk(pv, 7, 1, nthreads)
        t2 = time.perf_counter()
        cpu = {"value": 2.0 * n ** 3 / (t2 - t0) / 1e9, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": "one view forward + one view FDK-weighted backprojection at %d^3, curved detector: FP64 C "
                         "oracle port (OpenMP)" % n, "forward_s": t1 - t0, "backward_s": t2 - t1}
    return {"metric": "hot-path rows throughput (curved DD pair; detail: helical, flat, Siddon, voxel-driven FDK)",
            "value": detail["dd_pair_curved"]["Gvoxel_views_per_s"], "unit": UNIT,
            "ms_per_step": detail["dd_pair_curved"]["ms"], "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (30 seeded random ellipsoids; uniform random projections for the voxel-driven BP)",
            "config": {"workload": "rows_%dcube_%dviews_det%dx%d" % (n, nviews, nu, nv),
                       "l2": "volume 64 MiB (fits L2), projections 283 MB"},
            "gpu_launches": None, "roofline": roof, "cpu_baseline": cpu, "detail": detail}


def run_unet(args):
    """Forward pass of the learned proximal step's 3-D U-Net on one 256^3
    volume (--small N: N^3), bf16 tcgen05 convolutions; reports ms per pass
    and TFLOP/s against the measured bf16 peak."""
    import torch
    from ctreconstruction_gb300 import learned, phantoms
    dev = torch.device("cuda", torch.cuda.current_device())
    n = args.small or 256
    net = learned.UNet3D(device=dev, seed=0)
    x = phantoms.random_ellipsoids((n, n, n), n=30, seed=5, device=dev) * 0.02
    ms = _timed(lambda: net.forward(x, 0.01), args.steps, args.warmup)
    flops = learned.FLOPS_PER_VOXEL * n ** 3
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peak, kind = float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        peak, kind = 1900.0, "fallback"
    tf = flops / (ms / 1e3) / 1e12
    cpu = None
    if not args.no_cpu:
        # The FP64 NumPy restatement of the network (oracle/unet.py, bf16
        # rounding emulated) on a 16 x 32 x 32 crop.
        from oracle import unet as ounet
        params = {k: v.detach().cpu().numpy() for k, v in net.params.items()}
        xc = x[:16, :32, :32].cpu().numpy()[None]
        t0 = time.perf_counter()
        ounet.forward(params, xc, np.array([0.01]))
        t1 = time.perf_counter()
        cpu = {"value": learned.FLOPS_PER_VOXEL * xc.size / (t1 - t0) / 1e12, "unit": "TFLOP/s", "cores": 1,
               "kind": "port", "sample": "U-Net forward on a 16x32x32 crop: FP64 NumPy restatement "
                                         "(oracle/unet.py)", "seconds": t1 - t0}
    return {"metric": "3-D U-Net forward throughput", "value": tf, "unit": "TFLOP/s", "ms_per_step": ms,
            "higher_is_better": True, "dtype": "bf16 (fp32 accumulate)", "data": "synthetic (random ellipsoids)",
            "config": {"workload": "unet3d_forward_%dcube" % n, "levels": 3, "channels": [16, 32, 64]},
            "roofline": {"bound": "tensor", "achieved": tf, "peak": peak, "unit": "TFLOP/s", "frac": tf / peak,
                         "peak_source": kind, "flops_per_pass": flops}, "cpu_baseline": cpu}


WORKLOADS = {"rows": run_rows, "unet": run_unet, "fdk128": run_fdk128, "fan_batch": run_fan_batch, "iter": run_iter, "asd256": run_asd256,
             "asd256_learned": run_asd256_learned}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", type=int, default=0, help="cube side for a quick small run (not the workload)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-matched", action="store_true")
    ap.add_argument("--train-steps", type=int, default=1500, help="U-Net training steps (asd256_learned)")
    ap.add_argument("--ahead", type=int, default=0,
                    help="training pairs (pre-TV at k, post-TV at k + AHEAD) (asd256_learned)")
    ap.add_argument("--workload", default="dd512", choices=["dd512"] + sorted(WORKLOADS),
                    help="dd512 (default) is the headline DD pair; the others time the remaining configurations")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "dd512":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        line = WORKLOADS[args.workload](args)
        line.update({"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "scaling": "weak",
                     "vs_baseline": None})
        print(json.dumps(line))
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
