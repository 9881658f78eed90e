"""Throughput benchmark: grid-point RK-stage updates/s on one GB300.

Workload (default): config 1 -- two 201^3 curvilinear blocks with seeded
topography and a self-similar rough fault, aging-law rate-and-state friction,
run in the FP32-compensated mode (the production path) with the FP64 mode
timed side by side.  One "step" is one time step = 5 RK stages over both
blocks (src/time_step.f90:68-150).  updates = sum(nq*nr*ns) * 5 * steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With --impl reference the reference's CPU algorithm (the FP64 restatement in
oracle/, all host threads) is timed on the same workload; each step is one
full time step of config 1.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "waveqlab3d-gh_gb300"))

METRIC = "grid-pt RK-stage updates/s + HBM %peak; served solves/s, p50/p99 @FP32 vs FP64"
UNIT = "grid-point RK-stage updates/s"
# time steps each workload is configured for (the end-to-end run's length)
RUN_STEPS = {"config1": 2000, "config2": 3000, "config3_member": 1500, "config4_request": 100,
             "upwind": 2000, "upwind_anelastic": 2000}
# Algorithmic bytes per grid-point RK stage of the fused volume kernel:
# F read 9 + F write 9 + DF read 9 + DF write 9 words of the field type, in
# FP32C plus the Kahan compensation read 9 + write 9 as bfloat16 (9 FP32
# words), + coefficients (J*metric 9, 1/J, lambda, mu, 1/(rho J); Cartesian
# lambda, mu, 1/rho).
BYTES_PER_UPDATE = {("curv", "fp32c"): (45 + 13) * 4, ("curv", "fp64"): (36 + 13) * 8,
                    ("cart", "fp32c"): (45 + 3) * 4, ("cart", "fp64"): (36 + 3) * 8}
L2_BYTES = 129 * 1024 * 1024


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, pw, mx, reasons = [], [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except (ValueError, IndexError):
                continue
            try:
                pw.append(float(f[3]))
            except (ValueError, IndexError):
                pass
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_min_mhz": min(sm) if sm else None,
                "sm_max_mhz": mx, "power_w": statistics.median(pw) if pw else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def workload(args):
    import wql_configs
    if args.workload == "config2":
        # --n scales the blocks to (2n - 1) x n x n (201: the configured 401 x 201 x 201)
        text, media = wql_configs.config2(nq=2 * args.n - 1, nrs=args.n, steps=10 ** 6, seed=args.seed)
    elif args.workload == "config3_member":
        medium = wql_configs.von_karman((2 * 160 - 1, 160, 160), (0.1, 0.1, 0.1), 2.0, 0.2, 0.05, 3131)
        text, media, _ = wql_configs.config3_scenario(args.member, steps=10 ** 6, medium=medium)
    elif args.workload == "config4_request":
        medium = wql_configs.config4_medium(256, h=0.05)
        text, media, _ = wql_configs.config4_request(args.member, steps=10 ** 6, medium=medium)
    elif args.workload in ("upwind", "upwind_anelastic"):
        text, media = wql_configs.upwind_pml12(steps=10 ** 6, anelastic=args.workload == "upwind_anelastic")
    else:
        text, media = wql_configs.config1(n=args.n, steps=10 ** 6, seed=args.seed)
    return text, media, wql_configs.updates_per_step(text)


def time_gpu(wql, ctx, text, media, prec, steps, warmup, world):
    import torch
    s = wql.Scenario(ctx, text=text, precision=prec, media=media)
    st = torch.cuda.ExternalStream(s.stream())
    s.step(warmup)
    s.sync(check_nan=True)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    e0.record(st)
    s.step(steps)
    e1.record(st)
    s.sync()
    torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1)
    # per-kernel times from a separate pass with the library's event markers
    # (their records would otherwise sit between the timed launches)
    prof_steps = max(2, min(steps, 5))
    s.profile(True)
    s.step(prof_steps)
    s.sync()
    kt = s.kernel_times()
    kt["prof_steps"] = prof_steps
    s.profile(False)
    s.sync(check_nan=True)
    info = s.info()
    launches = steps * s.launches_per_step()
    s.close()
    return ms, kt, info, launches


def time_e2e(wql, ctx, text, media, prec, steps):
    """Whole job through the public API with host buffers: scenario creation
    (grid/surface upload), `steps` calls of wql_step(1) with the fault frame
    of every step taken to host memory (the reference writes its fault
    output every step; a longer stride only when the frames would fill more
    than a quarter of the free host memory), and the final velocity fields
    read back.  Returns seconds, H2D and D2H bytes, and the frame stride."""
    import re
    text_f = text.replace("w_fault = F", "w_fault = T")
    # the frames stay in host memory: at most a quarter of what is free
    m = re.search(r"btp\(1\)%nqrs\s*=\s*\d+,\s*(\d+),\s*(\d+)", text)
    frame_bytes = 39 * 4 * int(m.group(1)) * int(m.group(2))
    stride = max(1, -(-steps * frame_bytes // max(1, host_available_bytes() // 4)))
    if stride > 1:
        text_f = re.sub(r"w_stride = \d+", f"w_stride = {stride}", text_f)
    t0 = time.perf_counter()
    s = wql.Scenario(ctx, text=text_f, precision=prec, media=media)
    s.sync()
    t_create = time.perf_counter()
    for _ in range(steps):
        s.step(1)
    s.sync()
    t_steps = time.perf_counter()
    frames = s.frames("Svel")
    v = [s.field(b, c) for b in range(2) for c in range(3)]
    s.sync()
    t1 = time.perf_counter()
    parts = {"create_s": t_create - t0, "steps_s": t_steps - t_create, "read_s": t1 - t_steps}
    info = s.info()
    np_pts = sum(info.nq[b] * info.nr[b] * info.ns[b] for b in range(2))
    h2d = 3 * np_pts * 8 + sum(a.nbytes for k, a in _media_arrays(media))
    d2h = s.frame_count() * frame_bytes + sum(x.nbytes for x in v)
    s.close()
    del frames
    return t1 - t0, h2d, d2h, stride, parts


def host_available_bytes():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 8 << 30


def _media_arrays(media):
    if not media:
        return []
    out = []
    for k, v in media.items():
        if isinstance(v, (list, tuple)):
            out += [(k, a) for a in v if a is not None]
        elif v is not None:
            out.append((k, v))
    return out


def cpu_sample(text, media, steps, warmup=0):
    """The oracle (FP64 CPU restatement of the reference) on the same workload,
    all host threads: `warmup` untimed steps, then `steps` timed ones; returns
    (seconds for the timed steps, threads)."""
    import ctypes
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_oracle
    build_oracle.build()
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "libwqlref.so"))
    L.wqlref_create_ex.restype = ctypes.c_void_p
    L.wqlref_create_ex.argtypes = [ctypes.c_char_p] + [ctypes.c_void_p] * 9
    L.wqlref_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.wqlref_destroy.argtypes = [ctypes.c_void_p]
    L.wqlref_last_error.restype = ctypes.c_char_p
    m = media or {}

    def ptr(a):
        return None if a is None else a.ctypes.data

    topo = m.get("topo_offset") or (None, None)
    lam = m.get("lam") or (None, None)
    mu = m.get("mu") or (None, None)
    rho = m.get("rho") or (None, None)
    h = L.wqlref_create_ex(text.encode(), ptr(m.get("fault_offset")), ptr(topo[0]), ptr(topo[1]),
                           ptr(lam[0]), ptr(mu[0]), ptr(rho[0]), ptr(lam[1]), ptr(mu[1]), ptr(rho[1]))
    if not h:
        raise RuntimeError(L.wqlref_last_error().decode())
    if warmup:
        L.wqlref_step(h, warmup)
    t0 = time.perf_counter()
    L.wqlref_step(h, steps)
    t1 = time.perf_counter()
    L.wqlref_destroy(h)
    return t1 - t0, os.cpu_count()


def perturbed_prestress(text, rel=2.0 ** -24):
    """The workload with its background shear traction s0(5) (the &fault_list
    extension of the parametric presets) scaled by (1 + rel), or None."""
    import re
    m = re.search(r"(s0 = [^,]+, [^,]+, [^,]+, [^,]+, )([-0-9.eEdD+]+)", text)
    if not m:
        return None
    v = float(m.group(2).replace("d", "e").replace("D", "e")) * (1.0 + rel)
    return text[:m.start(2)] + repr(v) + text[m.end(2):]


def accuracy(wql, ctx, text, media, steps, stride=20, checkpoints=8, sensitivity=False):
    """FP32C against FP64 on the same workload after `steps` steps: relative
    L2 of the velocity fields and of the slip, relative error of the peak
    slip rate (over fault frames every `stride` steps) and the largest
    rupture-time difference in time steps over points that ruptured in both,
    with the number of points at each difference; for workloads with
    stations, the relative L2 of the seismograms.  The two runs advance side
    by side, and the velocity error is also recorded at `checkpoints` times
    with the FP64 velocity norm there (a field that has left the domain
    through the PML has a small norm, which inflates the relative error).
    sensitivity: a third run, FP64 with the background shear traction
    scaled by 1 + 2^-24 (one FP32 rounding), recorded against FP64 at the
    same times: how far the workload itself carries a perturbation of FP32
    size."""
    import numpy as np
    text_f = text.replace("w_fault = F", "w_fault = T").replace("w_stride = 1", f"w_stride = {stride}")
    rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))  # noqa: E731
    runs = {name: wql.Scenario(ctx, text=text_f, precision=prec, media=media)
            for name, prec in (("fp64", wql.FP64), ("fp32c", wql.FP32C))}
    text_p = perturbed_prestress(text_f) if sensitivity else None
    if text_p:
        runs["fp64_perturbed"] = wql.Scenario(ctx, text=text_p, precision=wql.FP64, media=media)
    vel = lambda s: [np.concatenate([s.field(b, c).ravel() for c in range(3)]) for b in range(2)]  # noqa: E731
    history = []
    done = 0
    every = max(1, -(-steps // checkpoints))
    while done < steps:
        n = min(every, steps - done)
        for s in runs.values():
            for k in range(0, n, 100):
                s.step(min(100, n - k))
        for s in runs.values():
            s.sync(check_nan=True)
        done += n
        vd, vf = vel(runs["fp64"]), vel(runs["fp32c"])
        h = {"step": done, "velocity_rel_l2": max(rel(vf[b], vd[b]) for b in range(2)),
             "fp64_velocity_l2": float(np.sqrt(sum(np.linalg.norm(v) ** 2 for v in vd)))}
        if "fp64_perturbed" in runs:
            vp = vel(runs["fp64_perturbed"])
            h["fp64_perturbed_velocity_rel_l2"] = max(rel(vp[b], vd[b]) for b in range(2))
            h["fp64_perturbed_slip_rel_l2"] = rel(runs["fp64_perturbed"].iface(0, 3), runs["fp64"].iface(0, 3))
        history.append(h)
    out = {"steps": steps}
    res = {}
    if "fp64_perturbed" in runs:
        tp = runs["fp64_perturbed"].iface(0, 5)
        runs.pop("fp64_perturbed").close()
    else:
        tp = None
    for name, s in runs.items():
        seis = [s.stations(b)[1] for b in range(2)] if "output_seismograms = T" in text_f else None
        res[name] = dict(seis=seis, v=vel(s), slip=s.iface(0, 3), trup=s.iface(0, 5),
                         peak=float(np.sqrt((s.frames("Svel")[:, 1:3].astype(np.float64) ** 2).sum(axis=1)).max()),
                         dt=s.info().dt)
        s.close()
    d, f = res["fp64"], res["fp32c"]
    rup_d, rup_f = d["trup"] < 1e8, f["trup"] < 1e8
    both = rup_d & rup_f
    out["velocity_rel_l2"] = max(rel(f["v"][b], d["v"][b]) for b in range(2))
    out["velocity_history"] = history
    out["ruptured_points_fp64"] = int(rup_d.sum())
    out["ruptured_points_fp32c"] = int(rup_f.sum())
    if rup_d.any():  # slip and slip rate only where the fault slipped
        out["slip_rel_l2"] = rel(f["slip"], d["slip"])
        out["peak_slip_rate_rel"] = abs(f["peak"] - d["peak"]) / max(abs(d["peak"]), 1e-300)
        out["peak_slip_rate_fp64"] = d["peak"]
    out["rupture_time_err_dt"] = float(np.abs(f["trup"][both] - d["trup"][both]).max() / d["dt"]) if both.any() else None
    if both.any():
        k = np.rint(np.abs(f["trup"][both] - d["trup"][both]) / d["dt"]).astype(int)
        out["rupture_time_err_points"] = {str(v): int((k == v).sum()) for v in np.unique(k)}
    if tp is not None:
        bp = rup_d & (tp < 1e8)
        if bp.any():
            k = np.rint(np.abs(tp[bp] - d["trup"][bp]) / d["dt"]).astype(int)
            out["fp64_perturbed_rupture_time_err_points"] = {str(v): int((k == v).sum()) for v in np.unique(k)}
    if d["seis"] is not None:
        out["seismogram_rel_l2"] = max(rel(f["seis"][b][..., 1:], d["seis"][b][..., 1:])
                                       for b in range(2) if d["seis"][b].size)
    return out


def batch_mode(wql, device, args):
    """Config 3: an ensemble of uneven scenarios advanced as one batch (one
    packed stencil launch per stage, tile chunks from the autotuner), against
    the same scenarios stepped one after another (each to the end before the
    next), against all of them queued at once on their own streams, and FP64
    stepped alone."""
    import numpy as np
    import torch
    import wql_configs
    ctx = wql.Context(device)
    n_hi = 160
    medium = wql_configs.von_karman((2 * n_hi - 1, n_hi, n_hi), (0.1, 0.1, 0.1), 2.0, 0.2, 0.05, 3131)
    members, points = [], 0
    t0 = time.perf_counter()
    for i in range(args.members):
        text, media, npts = wql_configs.config3_scenario(i, medium=medium)
        s = wql.Scenario(ctx, text=text, precision=wql.FP32C, media=media)
        s.autotune(reps=2)
        members.append((s, text, media, npts))
        points += npts
    setup_s = time.perf_counter() - t0
    batch = wql.Batch(ctx)
    for s, *_ in members:
        batch.add(s)
    batch.step(args.warmup)
    torch.cuda.synchronize()
    st = torch.cuda.ExternalStream(batch.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(device) as clk:
        # a profiler started with --profile-from-start off sees the timed
        # steps only (no-ops otherwise)
        torch.cuda.profiler.start()
        e0.record(st)
        batch.step(args.steps)
        e1.record(st)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    ms = e0.elapsed_time(e1)
    batched = points * 5 * args.steps / (ms * 1e-3)
    for s, *_ in members:
        s.sync(check_nan=True)
    batch.close()
    # the same members stepped one after another, each to the end of its
    # steps before the next starts (a caller without batching)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s, *_ in members:
        s.step(args.steps)
        s.sync()
    seq = points * 5 * args.steps / (time.perf_counter() - t0)
    # and all of them queued at once, each on its own stream (the streams
    # overlap on the device)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s, *_ in members:
        s.step(args.steps)
    for s, *_ in members:
        s.sync()
    streams = points * 5 * args.steps / (time.perf_counter() - t0)
    for s, *_ in members:
        s.close()
    # FP64 on a few members, one after another
    fp64_pts, fp64_s = 0, 0.0
    for s_, text, media, npts in members[:4]:
        d = wql.Scenario(ctx, text=text, precision=wql.FP64, media=media)
        d.step(1)
        d.sync()
        t0 = time.perf_counter()
        d.step(3)
        d.sync()
        fp64_s += time.perf_counter() - t0
        fp64_pts += npts * 5 * 3
        d.close()
    fp64 = fp64_pts / fp64_s
    return {"mode": "batch", "metric": METRIC, "value": batched, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "dtype": "f32 fields, Kahan-compensated RK update (bf16 compensation term), f64 fault solve",
            "data": "synthetic (seeded)",
            "config": {"workload": f"config3: {args.members} slip-weakening scenarios, blocks of 64^3..160^3 "
                                   f"points, planar/rough faults, homogeneous/von Karman media, 10-point PML, "
                                   f"{points} grid points", "setup_s": setup_s},
            "sequential_fp32c": seq, "batched_over_sequential": batched / seq,
            "own_streams_fp32c": streams, "batched_over_own_streams": batched / streams,
            "fp64_alone": fp64, "batched_fp32c_over_fp64": batched / fp64, "clocks": clk.summary()}


def serve_mode(wql, device, args):
    """Config 4: a Poisson stream of point-source requests (n^3 grids, n in
    96..256, von Karman media, 32 stations) served with admission by device
    memory and continuous batching; latency from each request's scheduled
    arrival to its completion."""
    import numpy as np
    import torch
    import wql_configs
    ctx = wql.Context(device)
    medium = wql_configs.config4_medium(256, h=0.05)
    free, total = torch.cuda.mem_get_info(device)
    budget = int(0.6 * free)
    rng = np.random.default_rng(4242)
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, size=args.requests))
    srv = wql.Server(ctx, hbm_budget_bytes=budget, round_steps=10)
    t_base = time.perf_counter()  # the server clock starts with the server (within ms)
    ids, sizes = [], []
    with Clocks(device) as clk:
        for i, ta in enumerate(arrivals):
            text, media, n = wql_configs.config4_request(i, steps=args.serve_steps, medium=medium)
            wait = ta - (time.perf_counter() - t_base)
            if wait > 0:
                time.sleep(wait)
            ids.append(srv.submit(text, args.serve_steps, media=media))
            sizes.append(n)
            del media
        status = [srv.wait(rid, 3600.0) for rid in ids]
    lat, done = [], []
    for rid, ta in zip(ids, arrivals):
        _, (t_arr, t_adm, t_done) = srv.result(rid, 0)
        lat.append(t_done - ta)
        done.append(t_done)
    srv.close()
    lat = np.array(lat)
    span = max(done) - arrivals[0]
    upd = sum(2 * (n // 2 + 1) * n * n for n in sizes) * 5 * args.serve_steps
    return {"mode": "serve", "metric": METRIC, "value": len(ids) / span, "unit": "solves/s", "n_gpus": 1,
            "higher_is_better": True, "dtype": "f32 fields, Kahan-compensated RK update (bf16 compensation term), f64 sources",
            "data": "synthetic (seeded)",
            "config": {"workload": f"config4: {args.requests} point-source requests, n^3 grids n in 96..256, "
                                   f"von Karman media, 32 stations, {args.serve_steps} steps each",
                       "arrival_rate_per_s": args.rate, "hbm_budget_bytes": budget},
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
            "updates_per_s": upd / span, "completed": int(sum(1 for x in status if x == 1)),
            "clocks": clk.summary()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=201)
    ap.add_argument("--seed", type=int, default=2239)
    ap.add_argument("--cpu-steps", type=int, default=1)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="steps of the end-to-end run (0: the workload's configured run length)")
    ap.add_argument("--mode", default="step", choices=["step", "batch", "serve"],
                    help="step: config 1 (default); batch: config 3 ensemble in one batch; serve: config 4 stream")
    ap.add_argument("--member", type=int, default=0,
                    help="config3_member / config4_request: which seeded member or request")
    ap.add_argument("--workload", default="config1",
                    choices=["config1", "config2", "upwind", "upwind_anelastic", "config3_member", "config4_request"],
                    help="step mode: config1 (2 x n^3 curvilinear, rate and state), config2 (2 x 401x201x201, "
                         "PML, von Karman, plasticity), upwind (2 x 76x101x151 Cartesian, upwind SBP-6, PML, "
                         "point source) or upwind_anelastic (the same with the anelastic response)")
    ap.add_argument("--members", type=int, default=64, help="batch mode: ensemble size")
    ap.add_argument("--requests", type=int, default=32, help="serve mode: number of requests")
    ap.add_argument("--rate", type=float, default=4.0, help="serve mode: Poisson arrival rate (requests/s)")
    ap.add_argument("--serve-steps", type=int, default=100, help="serve mode: time steps per request")
    ap.add_argument("--sensitivity", action="store_true",
                    help="with --accuracy-steps: also FP64 with the shear prestress scaled by 1 + 2^-24")
    ap.add_argument("--accuracy-steps", type=int, default=0,
                    help="instead of timing, run FP32C and FP64 this many steps and report their differences")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    text, media, ups = workload(args)
    wl = (f"config1: 2 x {args.n}^3 curvilinear blocks, seeded topography + self-similar rough fault, "
          f"aging-law rate-and-state, {ups // 5} grid points")
    if args.workload == "config2":
        wl = (f"config2: 2 x {2 * args.n - 1}x{args.n}x{args.n} curvilinear blocks, 20-point PML on 5 sides, "
              f"von Karman medium, "
              f"scec viscoplasticity, TPV26 stress, slip weakening, {ups // 5} grid points")
    if args.workload == "config3_member":
        wl = f"config3 member {args.member} (seeded, 10-point PML, slip weakening), {ups // 5} grid points"
    if args.workload == "config4_request":
        wl = f"config4 request {args.member} (seeded point source, 32 stations), {ups // 5} grid points"
    if args.workload in ("upwind", "upwind_anelastic"):
        wl = (f"{args.workload}: 2 x 76x101x151 Cartesian blocks, upwind SBP-6 operators, 12-point PML on 5 sides, "
              f"locked interface, one moment-tensor source, "
              f"{'anelastic response (4 mechanisms, c = 2, weight_exp = 0.6), ' if 'anelastic' in args.workload else ''}"
              f"{ups // 5} grid points")

    if args.impl == "reference":
        if rank != 0:
            return
        secs, cores = cpu_sample(text, media, args.steps, args.warmup)
        v = ups * args.steps / secs
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
                "config": {"workload": wl, "precision": "fp64"},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                 "sample": f"{args.steps} full time steps of the workload after {args.warmup} "
                                           "untimed ones, oracle/wql_ref.cpp (FP64 restatement), OpenMP on all "
                                           "host threads"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    torch.cuda.set_device(local)
    import wql_build
    wql_build.build()
    import wql
    if args.mode == "batch":
        if rank == 0 or world > 1:
            line = batch_mode(wql, local, args)
            if rank == 0:
                print(json.dumps(line))
        return
    if args.mode == "serve":
        line = serve_mode(wql, local, args)
        if rank == 0:
            print(json.dumps(line))
        return
    if args.accuracy_steps > 0:
        ctx = wql.Context(local)
        res = accuracy(wql, ctx, text, media, args.accuracy_steps, sensitivity=args.sensitivity)
        if rank == 0:
            print(json.dumps({"workload": wl, "fp32c_vs_fp64": res}))
        return
    ctx = wql.Context(local)
    res = {}
    with Clocks(local) as clk:
        for name, prec, steps in (("fp32c", wql.FP32C, args.steps), ("fp64", wql.FP64, max(3, args.steps // 4))):
            ms, kt, info, launches = time_gpu(wql, ctx, text, media, prec, steps, args.warmup, world)
            ms = allmax(world, ms)
            res[name] = dict(ms=ms, steps=steps, kt=kt, launches=launches, info=info)
    clocks = clk.summary()
    total_ups = allsum(world, ups)
    out = {}
    for name, r in res.items():
        per_step = r["ms"] / r["steps"]
        out[name] = {"value": total_ups / (per_step * 1e-3), "ms_per_step": per_step}
    main_r = res["fp32c"]
    peak, peak_kind = peaks()
    vol_ms, vol_n = main_r["kt"]["stencil"]
    # one launch per RK stage covers both blocks (the upwind operators: one
    # per-point launch per block)
    kernel_name = "stencil_kernel_tma2<float,curv,kahan>"
    mesh = "curv"
    if args.workload in ("upwind", "upwind_anelastic"):
        kernel_name, mesh = "stencil_kernel_tma2<float,cart,kahan,upwind>", "cart"
    pts_per_launch = ups * main_r["kt"]["prof_steps"] / vol_n if vol_n else 0
    algo = BYTES_PER_UPDATE[(mesh, "fp32c")] * pts_per_launch
    achieved = algo / (vol_ms / vol_n * 1e-3) / 1e9 if vol_n else None
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic_stencil_tma2_fp32c_curv.json" if mesh == "curv"
                         else "traffic_stencil_tma2_upwind_fp32c_cart.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            t = json.load(f)
        if t.get("kernel") == kernel_name:
            traffic = t.get("bytes_per_point", 0) * pts_per_launch or None
    e2e = None
    if not args.no_e2e:
        e_steps = args.e2e_steps or RUN_STEPS[args.workload]
        with Clocks(local) as eclk:
            secs, h2d, d2h, stride, parts = time_e2e(wql, ctx, text, media, wql.FP32C, e_steps)
        e2e = {"value": total_ups * e_steps / allmax(world, secs), "unit": UNIT, "steps": e_steps,
               "seconds": secs, "parts": parts, "fault_frame_every": stride, "clocks": eclk.summary(),
               "h2d_bytes_per_step": int(h2d / e_steps), "d2h_bytes_per_step": int(d2h / e_steps),
               "includes": "scenario creation (host grid generation, upload), the fault frames to the host "
                           "(every step unless host memory is short), final velocity fields to the host"}
        # the FP64 mode through the same public API path (like for like with
        # the FP64 CPU baseline)
        f_steps = res["fp64"]["steps"]
        secs64, h2d64, d2h64, _, _ = time_e2e(wql, ctx, text, media, wql.FP64, f_steps)
        e2e["fp64"] = {"value": total_ups * f_steps / allmax(world, secs64), "unit": UNIT, "steps": f_steps,
                       "h2d_bytes_per_step": int(h2d64 / f_steps), "d2h_bytes_per_step": int(d2h64 / f_steps)}
    cpu = None
    if rank == 0 and not args.no_cpu:
        secs, cores = cpu_sample(text, media, args.cpu_steps)
        cpu = {"value": ups * args.cpu_steps / secs, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{args.cpu_steps} full time step(s) of the same workload, oracle/wql_ref.cpp "
                         "(FP64 restatement), OpenMP on all host threads"}
    if rank != 0:
        return
    ws_bytes = main_r["info"].device_bytes
    line = {
        "metric": METRIC, "value": out["fp32c"]["value"], "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": out["fp32c"]["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 fields, Kahan-compensated RK update (bf16 compensation term), f64 fault solve",
        "data": {"config1": "synthetic (seeded topography, fault roughness)",
                 "config2": "synthetic (seeded von Karman medium)",
                 "upwind": "synthetic (uniform medium, one point source)",
                 "upwind_anelastic": "synthetic (uniform medium, one point source)"}[args.workload],
        "config": {"workload": wl, "precision": "fp32c", "steps_timed": args.steps,
                   "l2": f"inputs larger than L2: {ws_bytes / 2**20:.0f} MiB resident per GPU vs 129 MiB L2",
                   "parallelism": f"{world} independent replica(s), no collective"},
        "fp64": {"value": out["fp64"]["value"], "ms_per_step": out["fp64"]["ms_per_step"],
                 "steps_timed": res["fp64"]["steps"]},
        "fp32c_over_fp64": out["fp32c"]["value"] / out["fp64"]["value"],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "peak_kind": peak_kind, "kernel": kernel_name,
                     "bytes_per_update": BYTES_PER_UPDATE[(mesh, "fp32c")],
                     "avg_launch_ms": vol_ms / vol_n if vol_n else None,
                     "interface_avg_launch_ms": (main_r["kt"]["interface"][0] / main_r["kt"]["interface"][1])
                     if main_r["kt"]["interface"][1] else None,
                     "corrections_avg_launch_ms": (main_r["kt"]["corrections"][0] / main_r["kt"]["corrections"][1])
                     if main_r["kt"]["corrections"][1] else None},
        "clocks": clocks,
        "gpu_launches": main_r["launches"] + res["fp64"]["launches"],
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
