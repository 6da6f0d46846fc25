"""Benchmark of the LBVH build + closest-hit trace hot path on one GB300.

Workload (one step = one frame): the 1,048,576-triangle fBm terrain (1024 x
512 quads over [-1,1]^2, 30-bit Morton codes), a 1920x1080 pinhole view from
(0, 0.6, 1.6), all primary rays traced closest-hit (child-is order), one
cosine-weighted diffuse bounce ray generated per hit and traced.  The LBVH is
built once before the timed steps (as the reference builds it in
create_rt_set and times only traces, rta/main.cpp:402-405); its build is timed
separately in the same run and reported under "build".

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

value  = rays traced per second over the frame's kernels (device-resident rays;
         the frame is the fused trace launch + the bounce gather)
e2e    = the same frame through the C ABI with host rays, one
         rta_host_frames_run per step: pinned host -> device copy of the primary
         rays, the frame, device -> host copy of all hits and the bounce count;
         the copies run on their own streams beside the neighbouring steps
roofline = the fused frame kernel, timed by events rta_frame_run records
N > 1  = independent replicas, one per GPU (weak scaling); the time is the max
         over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s closest-hit (LBVH terrain, 1920x1080 primary + 1 diffuse bounce)"
UNIT = "Mrays/s"
WORKLOAD = "terrain-1M-tris 1024x512 quads, 1920x1080 primary + 1 diffuse bounce, 30-bit Morton, CIS closest hit"
SEED = 0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=300)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--cpu-sample-rays", type=int, default=262144)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-learned", action="store_true",
                   help="skip the learned-child-order training and evaluation")
    p.add_argument("--no-batch", action="store_true",
                   help="skip the 512-mesh batched build + trace")
    p.add_argument("--no-incoherent", action="store_true",
                   help="skip the 4M-triangle 63-bit build + 8M incoherent rays")
    p.add_argument("--section", choices=["incoherent", "learned", "batched"], default=None,
                   help="run only this workload and print its JSON object (not the bench line)")
    p.add_argument("--learned-samples", type=int, default=1 << 24,
                   help="training decisions recorded over both scene families")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The slowest rank's time: every replica runs the same frame, the job ends
    when the last one does."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def l2_copy_gbs(dev):
    """Copy rate (bytes read + written) between two 32 MiB buffers that stay
    in the L2, as 100 device-to-device copies captured in one CUDA graph (no
    launch gaps): the denominator for kernels whose bytes come from L2
    rather than HBM.  Measured live; not a vendor figure.  (Larger buffers
    spill: 2 x 48 MiB copies ran at 7.6 against 10.7 TB/s for 2 x 32 MiB.)"""
    import torch
    x = torch.ones(8 << 20, dtype=torch.float32, device=dev)
    y = torch.empty_like(x)
    for _ in range(10):
        y.copy_(x)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        with torch.cuda.graph(g):
            for _ in range(100):
                y.copy_(x)
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    e0.record()
    for _ in range(reps):
        g.replay()
    e1.record()
    e1.synchronize()
    return reps * 100 * 2 * x.numel() * 4 / (e0.elapsed_time(e1) * 1e-3) / 1e9


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None
        self.window = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.rows.append((time.time(), parts))

    def mark(self, start: bool):
        """Brackets the timed region; only samples inside it are summarised."""
        if start:
            self.window = [time.time(), None]
        else:
            self.window[1] = time.time()

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = [r for t, r in self.rows
                if self.window is None or (self.window[0] <= t <= (self.window[1] or t))]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# --------------------------------------------------------------------------- #
# CPU baseline: the reference CPU plugin's algorithm (bbvh spatial-median      #
# build + child-is tracer, OpenMP), timed on this machine's host cores.       #
# --------------------------------------------------------------------------- #

def cpu_baseline(tris, orig, dirs, maxt, sample, threads=0):
    from oracle import oracle as O
    t0 = time.perf_counter()
    nodes, leaf_tris = O.bbvh_build(tris)
    build_s = time.perf_counter() - t0
    n = maxt.shape[0]
    idx = np.linspace(0, n - 1, min(sample, n)).astype(np.int64)
    o = orig.reshape(-1, 3)[idx]
    d = dirs.reshape(-1, 3)[idx]
    m = maxt[idx]
    t0 = time.perf_counter()
    O.bbvh_trace_cis(nodes, leaf_tris, o, d, m, threads=threads)
    trace_s = time.perf_counter() - t0
    cores = threads or os.cpu_count()
    return {"rays": int(idx.shape[0]), "trace_s": trace_s, "build_s": build_s,
            "mrays_s": idx.shape[0] / trace_s / 1e6, "cores": cores}


def run_reference(args):
    """--impl reference: the reference CPU plugin's build + child-is trace
    (bbvh/bbvh.h) on the host cores, on a bounded sample of the frame."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    from rta_gb300 import scenes as S
    tris = S.terrain(1024, 512, seed=SEED)
    cam = S.terrain_camera()
    o, d, m = O.shirley_rays(cam.tan_half, cam.aspect, cam.w, cam.h, cam.dir, cam.pos, cam.up)
    # bounce rays of the frame come from the oracle's restatement of the bounce
    lb = O.lbvh_build(tris, 30)
    srt = O.permute(tris, lb.ids)
    hits, _, _ = O.trace(lb.nodes, srt, o, d, m, O.CIS, 64)
    bo, bd, bm, _ = O.diffuse_bounce(srt, o, d, hits, seed=SEED, eps=1e-4)
    allo = np.concatenate([o.reshape(-1, 3), bo.reshape(-1, 3)])
    alld = np.concatenate([d.reshape(-1, 3), bd.reshape(-1, 3)])
    allm = np.concatenate([m, bm])
    t0 = time.perf_counter()
    nodes, leaf_tris = O.bbvh_build(tris)
    build_s = time.perf_counter() - t0
    sample = min(args.cpu_sample_rays, allm.shape[0])
    idx = np.linspace(0, allm.shape[0] - 1, sample).astype(np.int64)
    so, sd, sm = allo[idx], alld[idx], allm[idx]
    for _ in range(args.warmup):
        O.bbvh_trace_cis(nodes, leaf_tris, so, sd, sm)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.bbvh_trace_cis(nodes, leaf_tris, so, sd, sm)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = sample * args.steps / total / 1e6
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": WORKLOAD, "cpu_sample_rays": sample,
                                        "cpu_build_s": build_s},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{sample} rays evenly strided over the frame's primary+bounce rays; "
                                   f"spatial-median bbvh (bbvh/bbvh.h) built once ({build_s:.2f} s)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- #
# learned child order: train on seeds 0-3, evaluate on seed 4                 #
# --------------------------------------------------------------------------- #

def _frame_rays(lib, bvh, cam, seed, dev):
    """Primary rays of `cam` plus one diffuse bounce per hit, on the device."""
    import torch
    from rta_gb300 import lib as L
    from rta_gb300 import plugin as P
    g = P.cam_ray_generator_shirley(cam.w, cam.h)
    g.setup(cam.pos, cam.dir, cam.up, cam.fovy)
    g.generate_rays()
    n = cam.w * cam.h
    hits = torch.empty(4 * n, dtype=torch.float32, device=dev)
    fh = C.c_void_p()
    L.check(lib.rta_frame_create(C.byref(fh), n), "rta_frame_create")
    f = L.FrameView()
    L.check(lib.rta_frame_get(fh, C.byref(f)), "rta_frame_get")
    L.check(lib.rta_frame_run(fh, C.byref(bvh.view), P._ptr(g.gpu_origin), P._ptr(g.gpu_direction),
                              P._ptr(g.gpu_maxt), n, P._ptr(hits), L.TRACE_CIS, seed, np.float32(1e-4),
                              P._stream()), "rta_frame_run")
    torch.cuda.synchronize()
    nb = int(P.device_view(f.count, 1, "<u4").cpu().numpy().view(np.uint32)[0])
    o = torch.cat([g.gpu_origin, P.device_view(f.orig, 3 * nb).clone()])
    d = torch.cat([g.gpu_direction, P.device_view(f.dir, 3 * nb).clone()])
    m = torch.cat([g.gpu_maxt, P.device_view(f.maxt, nb).clone()])
    L.check(lib.rta_frame_destroy(fh), "rta_frame_destroy")
    return o, d, m


def _incoherent(n, seed, dev):
    import torch
    from rta_gb300 import scenes as S
    o, d, m = S.incoherent_rays(n, seed=seed)
    return (torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev), torch.from_numpy(m).to(dev))


def learned_eval(args, dev):
    """Configuration 4: the child-order network, trained per scene family on
    decisions recorded by the plain traversal on seeds 0-3 (half of
    --learned-samples per family), evaluated on the seed-4 scene of each
    family with about 8M rays (primary + bounce frame for terrains, 8,388,608
    incoherent rays for cluster soups)."""
    import torch
    from rta_gb300 import learned as LR
    from rta_gb300 import lib as L
    from rta_gb300 import plugin as P
    from rta_gb300 import scenes as S
    lib = L.load()
    out = {}
    per_family = args.learned_samples // 2
    for fam in ("terrain", "clusters"):
        bits = 30 if fam == "terrain" else 63
        make = (lambda sd: S.terrain(1024, 512, seed=sd)) if fam == "terrain" else (lambda sd: S.clusters(seed=sd))
        model = LR.OrderModel(max_samples=per_family, seed=11)
        ctor = P.lbvh_constructor(morton_bits=bits, keep_triangles=False)
        t0 = time.perf_counter()
        for sd in range(4):
            bvh = ctor.build(P.cuda_ftl(make(sd)))
            if fam == "terrain":
                o, d, m = _frame_rays(lib, bvh, S.terrain_camera(), sd, dev)
            else:
                o, d, m = _incoherent(1 << 22, sd, dev)
            # each seed fills a quarter of the sample store: rays in a seeded
            # random order, recorded in chunks until the quarter is full
            perm = torch.from_numpy(np.random.default_rng(sd).permutation(m.numel())).to(dev)
            target = per_family * (sd + 1) // 4
            for c0 in range(0, m.numel(), 1 << 18):
                if model.sample_count() >= target:
                    break
                idx = perm[c0:c0 + (1 << 18)]
                ro = o.view(-1, 3)[idx].contiguous()
                rd = d.view(-1, 3)[idx].contiguous()
                model.sample(bvh, ro, rd, m[idx].contiguous())
        samples = model.sample_count()
        torch.cuda.synchronize()
        sample_s = time.perf_counter() - t0   # scene generation, builds and recording traces
        loss0 = model.gradient(0, min(samples, 1 << 20))[1]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss = model.train(epochs=4, batch=1 << 16, lr=2e-3)
        torch.cuda.synchronize()
        train_s = time.perf_counter() - t0    # 4 epochs of the forward/backward and Adam kernels
        # the confidence margin is chosen on the last training scene's rays
        # (seed 3, at most 2M of them): the network overrides the plain order
        # only where it is at least that sure, and never where that costs
        # work on the training scene
        vidx = torch.arange(0, int(m.numel()), max(1, int(m.numel()) >> 21), device=dev)
        nv = int(vidx.numel())
        chosen = LR.choose_margin(model, bvh, o.view(-1, 3)[vidx].contiguous(), d.view(-1, 3)[vidx].contiguous(),
                                  m[vidx].contiguous())
        bvh = ctor.build(P.cuda_ftl(make(4)))
        if fam == "terrain":
            o, d, m = _frame_rays(lib, bvh, S.Camera((0.0, 0.6, 1.6), (0.0, 0.0, 0.0), w=3200, h=1800), 4, dev)
        else:
            o, d, m = _incoherent(1 << 23, 4, dev)
        nr = int(m.numel())
        hp, sp = LR.plain_trace(bvh, o, d, m, stats=True)
        hl, sl = model.trace(bvh, o, d, m, stats=True)
        _, si = LR.ideal_trace(bvh, o, d, m, hp, stats=True)
        sin = si.view(-1, 2).to(torch.float64).mean(0).cpu().numpy()
        a = hp.cpu().numpy().view(np.uint32).reshape(-1, 4)
        b = hl.cpu().numpy().view(np.uint32).reshape(-1, 4)
        hit = a[:, 0] != np.float32(3.4028235e38).view(np.uint32)
        same_hit = bool(np.array_equal(hit, b[:, 0] != np.float32(3.4028235e38).view(np.uint32)))
        t_other = int((a[:, 0] != b[:, 0]).sum())
        ta, tb = a[hit, 0].view(np.float32).astype(np.float64), b[hit, 0].view(np.float32).astype(np.float64)
        t_rel = float((np.abs(ta - tb) / np.abs(ta)).max(initial=0.0))
        ties = int((hit & (a[:, 3] != b[:, 3])).sum())
        spn = sp.view(-1, 2).to(torch.float64).mean(0).cpu().numpy()
        sln = sl.view(-1, 2).to(torch.float64).mean(0).cpu().numpy()

        def timed(fn, k=10):
            fn()
            ts = []
            for _ in range(k):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                fn()
                e1.record()
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            return statistics.median(ts)

        hbuf = torch.empty(4 * nr, dtype=torch.float32, device=dev)
        tp = timed(lambda: L.check(lib.rta_trace(C.byref(bvh.view), P._ptr(o), P._ptr(d), P._ptr(m), nr, None,
                                                 P._ptr(hbuf), L.TRACE_CIS, None, P._stream()), "trace"))
        tl = timed(lambda: L.check(lib.rta_trace_learned(C.byref(bvh.view), model.handle, P._ptr(o), P._ptr(d),
                                                         P._ptr(m), nr, None, P._ptr(hbuf), None, P._stream()),
                                   "trace_learned"))
        # the cost of asking the network at every overlapping decision (margin 0)
        kept_margin = model.margin()
        model.set_margin(0.0)
        tn = timed(lambda: L.check(lib.rta_trace_learned(C.byref(bvh.view), model.handle, P._ptr(o), P._ptr(d),
                                                         P._ptr(m), nr, None, P._ptr(hbuf), None, P._stream()),
                                   "trace_learned"))
        model.set_margin(kept_margin)
        work_p, work_l = float(spn.sum()), float(sln.sum())
        out[fam] = {
            "train_samples": samples, "train_loss_before": loss0, "train_loss_after": loss,
            "train_s": train_s, "sample_s": sample_s, "train_epochs": 4, "eval_rays": nr,
            "margin": chosen["margin"] if np.isfinite(chosen["margin"]) else "inf",
            "margin_selection": {"scene": "training seed 3, every k-th ray", "rays": nv,
                                 "plain_work_per_ray": chosen["plain_work_per_ray"],
                                 "work_per_ray_by_margin": chosen["tried"]},
            "plain": {"nodes_per_ray": float(spn[0]), "tris_per_ray": float(spn[1]), "ms": tp,
                      "mrays_s": nr / (tp * 1e-3) / 1e6},
            "learned": {"nodes_per_ray": float(sln[0]), "tris_per_ray": float(sln[1]), "ms": tl,
                        "mrays_s": nr / (tl * 1e-3) / 1e6,
                        "network_every_decision_mrays_s": nr / (tn * 1e-3) / 1e6},
            "ideal_order": {"nodes_per_ray": float(sin[0]), "tris_per_ray": float(sin[1]),
                            "work_reduction": 1.0 - float(sin.sum()) / work_p},
            "work_reduction": 1.0 - work_l / work_p,
            "same_rays_hit": same_hit, "rays_t_not_bit_identical": t_other, "t_max_rel_diff": t_rel,
            "rays_other_triangle": ties,
            "kept": work_l < work_p,
        }
    return out


# --------------------------------------------------------------------------- #
# incoherent large scene: 4M clustered triangles, 63-bit codes, 8M rays       #
# --------------------------------------------------------------------------- #

def incoherent_eval(args, dev):
    """Configuration 3: 4,194,304 triangles in 256 Gaussian clusters, 63-bit
    Morton codes (the build's bandwidth case: 1.5 GB of build traffic), and
    8,388,608 rays with origins uniform in [-12, 12]^3 and directions uniform
    on the sphere.  Build and trace are timed separately (CUDA events, L2
    flushed before each step); the per-ray work comes from one stats pass."""
    import torch
    from rta_gb300 import lib as L
    from rta_gb300 import plugin as P
    from rta_gb300 import scenes as S

    lib = L.load()
    tris = S.clusters(256, 16384, seed=SEED)
    n = tris.shape[0]
    ftl = P.cuda_ftl(tris)
    ctor = P.lbvh_constructor(morton_bits=63, keep_triangles=False)
    o, d, m = (torch.from_numpy(x).to(dev) for x in S.incoherent_rays(1 << 23, seed=SEED))
    nr = int(m.numel())
    hits = torch.empty(4 * nr, dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    sh = P._stream()

    def timed(fn, k):
        ts = []
        for _ in range(k):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    def build():
        L.check(lib.rta_lbvh_build(ctor.handle, P._ptr(ftl.triangle), n, 63, C.c_void_p(0), sh), "build")

    for _ in range(args.warmup):
        build()
    k = max(3, min(args.steps, 50))
    build_ms = timed(build, k)
    bvh = P.binary_lbvh(ctor, None)

    def trace(mode=L.TRACE_CIS, st=None):
        L.check(lib.rta_trace(C.byref(bvh.view), P._ptr(o), P._ptr(d), P._ptr(m), nr, C.c_void_p(0), P._ptr(hits),
                              mode, P._ptr(st), sh), "trace")

    for _ in range(max(1, args.warmup // 2)):
        trace()
    trace_ms = timed(trace, max(3, min(args.steps, 20)))
    st = torch.zeros(2 * nr, dtype=torch.int32, device=dev)
    trace(L.TRACE_CIS | L.TRACE_STATS, st)
    w = st.view(-1, 2).to(torch.float64).mean(0).cpu().numpy()
    torch.cuda.synchronize()
    hit_frac = float((hits.view(-1, 4)[:, 0] < 3.0e38).to(torch.float64).mean())
    alg = 504 * n   # build bytes per triangle with 63-bit keys (8 sort passes of 12-byte keys+ids)
    peak, peak_src = measured_peaks()
    # the trace's algorithmic bytes, as for the frame: 28 B ray + 16 B hit per
    # ray, 64 B per inner node visited (one two-child record), 48 B per
    # triangle tested
    trace_alg = nr * (28 + 16) + float(w[0]) * nr * 64 + float(w[1]) * nr * 48
    l2_peak = l2_copy_gbs(dev)
    traffic = None
    prof = os.path.join(ROOT, "profiles", "trace_traffic_incoherent.json")
    if os.path.exists(prof):
        with open(prof) as f:
            traffic = json.load(f).get("dram_bytes_per_launch")
    return {
        "triangles": n, "morton_bits": 63, "rays": nr, "hit_fraction": hit_frac,
        "build_ms": build_ms, "build_mtri_s": n / (build_ms * 1e-3) / 1e6,
        "build_algorithmic_bytes": alg, "build_gbs": alg / (build_ms * 1e-3) / 1e9,
        "build_frac_of_peak": alg / (build_ms * 1e-3) / 1e9 / peak,
        "trace_ms": trace_ms, "trace_mrays_s": nr / (trace_ms * 1e-3) / 1e6,
        "inner_visits_per_ray": float(w[0]), "tri_tests_per_ray": float(w[1]),
        "trace_roofline": {
            "bound": "hbm", "kernel": "k_trace<CIS> over the 63-bit cluster tree (80-entry stack)",
            "achieved": trace_alg / (trace_ms * 1e-3) / 1e9, "peak": peak, "peak_source": peak_src,
            "unit": "GB/s", "frac": trace_alg / (trace_ms * 1e-3) / 1e9 / peak,
            "algorithmic_bytes_per_launch": trace_alg, "traffic": traffic,
            "l2_copy_gbs": l2_peak, "frac_of_l2_copy": trace_alg / (trace_ms * 1e-3) / 1e9 / l2_peak,
            "note": "latency bound: the 456 MB tree does not fit the L2, so incoherent rays wait on DRAM; "
                    "traffic = DRAM bytes of one launch (ncu)"},
    }


# --------------------------------------------------------------------------- #
# batched multi-mesh: 512 meshes, one graph launch vs per-mesh launches       #
# --------------------------------------------------------------------------- #

def batch_eval(args, dev):
    """Configuration 5: 512 seeded meshes (terrains and cluster soups, 1k-200k
    triangles, about 25M in all) with 4k-1M rays each (about 50M in all, half
    primary from a per-mesh camera, half incoherent).  All trees are built
    and all rays traced by one CUDA graph launch with autotuned parameters;
    the comparison is the per-mesh path (one rta_lbvh_build + one rta_trace
    per mesh, launched back to back).  Inputs (2.6 GB of triangles, 1.4 GB of
    rays) are far larger than L2, so no flush is needed between steps."""
    import tempfile

    import torch
    from rta_gb300 import batch as BT
    from rta_gb300 import scenes as S

    t0 = time.perf_counter()
    work = BT.make_workload(S.batch_specs(512, seed=0))
    gen_s = time.perf_counter() - t0
    b = BT.Batch()
    b.set_meshes(work.tri_offsets, work.ray_offsets)
    nr = work.n_rays
    hits = torch.zeros(4 * nr, dtype=torch.float32, device=dev)
    cache = os.path.join(tempfile.gettempdir(), "rta_gb300_autotune.json")
    if os.path.exists(cache):
        os.remove(cache)   # tune afresh: the timing is part of what is reported
    t0 = time.perf_counter()
    chosen, tuned_ms = b.autotune(work.tris, work.orig, work.dirs, work.maxt, hits, cache_path=cache, reps=3)
    tune_s = time.perf_counter() - t0

    def timed(fn, k):
        ts = []
        for _ in range(k):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    steps = max(3, min(args.steps, 10))
    for _ in range(3):
        b.run(work.tris, work.orig, work.dirs, work.maxt, hits)
    graph_ms = timed(lambda: b.run(work.tris, work.orig, work.dirs, work.maxt, hits), steps)
    torch.cuda.synchronize()
    batch_hits = hits.clone()
    build_ms = timed(lambda: b.build(work.tris), steps)
    trace_ms = timed(lambda: b.trace(work.orig, work.dirs, work.maxt, hits), steps)
    seq_hits = torch.zeros_like(hits)
    ctor = BT.sequential(work, seq_hits)   # warm-up (allocates the largest mesh's buffers)
    seq_ms = timed(lambda: BT.sequential(work, seq_hits, ctor), max(3, steps // 3))
    torch.cuda.synchronize()
    same = bool(torch.equal(seq_hits.view(torch.int32), batch_hits.view(torch.int32)))
    return {
        "meshes": len(work.tri_offsets) - 1, "triangles": work.n_tris, "rays": nr,
        "graph_ms": graph_ms, "build_ms": build_ms, "trace_ms": trace_ms,
        "build_mtri_s": work.n_tris / (build_ms * 1e-3) / 1e6, "trace_mrays_s": nr / (trace_ms * 1e-3) / 1e6,
        "graph_mrays_s": nr / (graph_ms * 1e-3) / 1e6,
        "sequential_ms": seq_ms, "speedup_vs_sequential": seq_ms / graph_ms,
        "identical_hits_vs_sequential": same, "params": chosen, "autotune_s": tune_s,
        "autotune_best_ms": tuned_ms, "workload_gen_s": gen_s,
    }


# --------------------------------------------------------------------------- #
# GB300 arm                                                                   #
# --------------------------------------------------------------------------- #

def run_gb300(args):
    import torch

    from rta_gb300 import lib as L
    from rta_gb300 import plugin as P
    from rta_gb300 import scenes as S

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist

    lib = L.load()
    tris = S.terrain(1024, 512, seed=SEED)
    n = tris.shape[0]
    cam = S.terrain_camera()
    nrays = cam.w * cam.h
    ftl = P.cuda_ftl(tris)
    ctor = P.lbvh_constructor(morton_bits=30, keep_triangles=False)
    stream = torch.cuda.current_stream()
    sh = L.stream_handle(stream)

    # L2 flush buffer (larger than the 129 MB L2)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    # ---- build timing ----
    for _ in range(args.warmup):
        bvh = ctor.build(ftl)
    build_ms = []
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        L.check(lib.rta_lbvh_build(ctor.handle, P._ptr(ftl.triangle), n, 30, C.c_void_p(0), sh), "build")
        e1.record()
        e1.synchronize()
        build_ms.append(e0.elapsed_time(e1))
    bvh = P.binary_lbvh(ctor, None)
    assert bvh.status() & (L.DEV_SPIN_TIMEOUT | L.DEV_STACK_OVERFLOW) == 0

    # ---- rays, frame context ----
    rg = P.cam_ray_generator_shirley(cam.w, cam.h)
    rg.setup(cam.pos, cam.dir, cam.up, cam.fovy)
    rg.generate_rays()
    hits = torch.empty(nrays * 4, dtype=torch.float32, device=dev)
    fh = C.c_void_p()
    L.check(lib.rta_frame_create(C.byref(fh), nrays), "rta_frame_create")
    frame = L.FrameView()
    L.check(lib.rta_frame_get(fh, C.byref(frame)), "rta_frame_get")
    count_view = P.device_view(frame.count, 1, "<u4")

    def run_frame():
        L.check(lib.rta_frame_run(fh, C.byref(bvh.view), P._ptr(rg.gpu_origin), P._ptr(rg.gpu_direction),
                                  P._ptr(rg.gpu_maxt), nrays, P._ptr(hits), L.TRACE_CIS, SEED,
                                  np.float32(1e-4), sh), "rta_frame_run")

    clk = ClockSampler(local).__enter__()
    for _ in range(args.warmup):
        run_frame()
    torch.cuda.synchronize()
    nbounce = int(count_view.cpu().numpy().view(np.uint32)[0])
    rays_per_step = nrays + nbounce

    # per-ray work counts (one stats pass, outside the timed region)
    st = torch.zeros(2 * nrays, dtype=torch.int32, device=dev)
    tmp = torch.empty_like(hits)
    L.check(lib.rta_trace(C.byref(bvh.view), P._ptr(rg.gpu_origin), P._ptr(rg.gpu_direction),
                          P._ptr(rg.gpu_maxt), nrays, C.c_void_p(0), P._ptr(tmp),
                          L.TRACE_CIS | L.TRACE_STATS, P._ptr(st), sh), "stats")
    stp = st.view(-1, 2).to(torch.int64).sum(0).cpu().numpy()
    stb = torch.zeros(2 * nrays, dtype=torch.int32, device=dev)
    L.check(lib.rta_trace(C.byref(bvh.view), C.c_void_p(frame.orig), C.c_void_p(frame.dir),
                          C.c_void_p(frame.maxt), 0, C.c_void_p(frame.count), P._ptr(tmp),
                          L.TRACE_CIS | L.TRACE_STATS, P._ptr(stb), sh), "stats")
    stbs = stb.view(-1, 2).to(torch.int64).sum(0).cpu().numpy()
    inner_visits = int(stp[0] + stbs[0])
    tri_tests = int(stp[1] + stbs[1])

    # ---- timed frames (device-resident rays) ----
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    step_ms = []
    time.sleep(0.5)   # lets the clock sampler produce its first lines
    clk.mark(True)
    # the frame records CUDA events on its own stream around its trace launch
    # (rta_frame_set_timing), so the dominant kernel is timed in every step
    L.check(lib.rta_frame_set_timing(fh, 1), "rta_frame_set_timing")
    frame_trace_ms = []
    if True:
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run_frame()
            e1.record()
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            ft = C.c_float(0)
            L.check(lib.rta_frame_trace_ms(fh, C.byref(ft)), "rta_frame_trace_ms")
            frame_trace_ms.append(float(ft.value))
        torch.cuda.synchronize()
        L.check(lib.rta_frame_set_timing(fh, 0), "rta_frame_set_timing")
        # the primary rays alone, and the frame's bounce rays alone (rta_trace
        # over the frame's bounce buffers), for per-pass rates
        trace_ms, bounce_ms = [], []
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            L.check(lib.rta_trace(C.byref(bvh.view), P._ptr(rg.gpu_origin), P._ptr(rg.gpu_direction),
                                  P._ptr(rg.gpu_maxt), nrays, C.c_void_p(0), P._ptr(tmp), L.TRACE_CIS,
                                  C.c_void_p(0), sh), "trace")
            e1.record()
            e1.synchronize()
            trace_ms.append(e0.elapsed_time(e1))
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            L.check(lib.rta_trace(C.byref(bvh.view), C.c_void_p(frame.orig), C.c_void_p(frame.dir),
                                  C.c_void_p(frame.maxt), nbounce, C.c_void_p(0), P._ptr(tmp), L.TRACE_CIS,
                                  C.c_void_p(0), sh), "trace")
            e1.record()
            e1.synchronize()
            bounce_ms.append(e0.elapsed_time(e1))
    clk.mark(False)
    clk.__exit__(None, None, None)
    if pg:
        pg.barrier()
    total_ms = max_over_ranks(sum(step_ms), pg, dev)
    ms_per_step = total_ms / args.steps
    value = rays_per_step * world * args.steps / (total_ms * 1e-3) / 1e6

    # ---- e2e: host rays in, host hits out, through the C ABI ----
    h_orig = torch.empty(3 * nrays, dtype=torch.float32, pin_memory=True)
    h_dir = torch.empty(3 * nrays, dtype=torch.float32, pin_memory=True)
    h_maxt = torch.empty(nrays, dtype=torch.float32, pin_memory=True)
    h_orig.copy_(rg.gpu_origin)
    h_dir.copy_(rg.gpu_direction)
    h_maxt.copy_(rg.gpu_maxt)
    h_hits = torch.empty(nrays * 4, dtype=torch.float32, pin_memory=True)
    h_bhits = torch.empty(nrays * 4, dtype=torch.float32, pin_memory=True)
    h_bcount = torch.zeros(1, dtype=torch.int32, pin_memory=True)
    hf = P.host_frames(nrays)

    # One rta_host_frames_run per step: the step's rays are copied in, the
    # frame runs, and its primary hits, bounce hits and bounce count are
    # copied out, every step; the copies run on their own streams, so one
    # step's transfers overlap the neighbouring steps' traversal.
    def e2e_step():
        hf.run(bvh, h_orig, h_dir, h_maxt, h_hits, h_bhits, h_bcount, L.TRACE_CIS, SEED, 1e-4, nrays)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        e2e_step()
    e1.record()
    e1.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    h2d = (3 + 3 + 1) * 4 * nrays
    d2h = 16 * nrays + 16 * nrays + 4   # primary hits, all bounce slots, the bounce count
    e2e_value = rays_per_step * world / (e2e_ms * 1e-3) / 1e6
    # the zero-copy frame gives the same hits as the device-resident one
    torch.cuda.synchronize()
    ha, hb = h_hits.view(torch.int32).view(-1, 4), hits.cpu().view(torch.int32).view(-1, 4)
    hit_rows = ha[:, 0] != 0x7F7FFFFF   # t != FLT_MAX (a miss writes only t)
    ba = h_bhits[: 4 * nbounce].view(torch.int32).view(-1, 4)
    bb = P.device_view(frame.hits, 4 * nbounce).cpu().view(torch.int32).view(-1, 4)
    bhit_rows = ba[:, 0] != 0x7F7FFFFF
    e2e_same = bool(torch.equal(ha[:, 0], hb[:, 0]) and torch.equal(ha[hit_rows], hb[hit_rows])
                    and int(h_bcount.item()) == nbounce
                    and torch.equal(ba[:, 0], bb[:, 0]) and torch.equal(ba[bhit_rows], bb[bhit_rows]))

    # ---- roofline of the dominant kernel: the fused frame trace ----
    # algorithmic bytes of one launch: every ray (primary and bounce) read and
    # its hit written, 64 B per inner node visited, 48 B per triangle tested,
    # and each bounce ray's slot (ray 24 B + hit 16 B) plus one flag per pixel
    peak, peak_kind = measured_peaks()
    tr_ms = statistics.mean(trace_ms)
    ft_ms = statistics.mean(frame_trace_ms)
    bytes_per_launch = (44 * rays_per_step + 64 * (int(stp[0]) + int(stbs[0])) + 48 * (int(stp[1]) + int(stbs[1]))
                        + 40 * nbounce + 4 * nrays)
    achieved = bytes_per_launch / (ft_ms * 1e-3) / 1e9
    prim_bytes = 28 * nrays + 16 * nrays + 64 * int(stp[0]) + 48 * int(stp[1])
    traffic = None
    l2_peak = l2_copy_gbs(dev)
    prof = os.path.join(ROOT, "profiles", "trace_traffic.json")
    if os.path.exists(prof):
        with open(prof) as f:
            traffic = json.load(f).get("dram_bytes_per_launch")

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu_r = cpu_baseline(tris, rg.gpu_origin.cpu().numpy(), rg.gpu_direction.cpu().numpy(),
                             rg.gpu_maxt.cpu().numpy(), args.cpu_sample_rays)
        cpu = {"value": cpu_r["mrays_s"], "unit": UNIT, "cores": cpu_r["cores"], "kind": "port",
               "sample": f"{cpu_r['rays']} primary rays evenly strided over the 1920x1080 frame through "
                         f"the spatial-median bbvh of the same terrain (build {cpu_r['build_s']:.2f} s, untimed)"}

    incoherent = None
    if not args.no_incoherent:
        incoherent = incoherent_eval(args, dev)
    learned = None
    if not args.no_learned:
        learned = learned_eval(args, dev)
    batched = None
    if not args.no_batch:
        batched = batch_eval(args, dev)

    bmean = statistics.mean(build_ms)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "triangles": n, "primary_rays": nrays, "bounce_rays": nbounce,
                   "rays_per_step": rays_per_step, "morton_bits": 30,
                   "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "l2_copy_gbs": l2_peak, "frac_of_l2_copy": achieved / l2_peak,
                     "kernel": "k_trace<CIS,FUSE> frame: 1920x1080 primary rays + their bounce rays",
                     "algorithmic_bytes_per_launch": bytes_per_launch, "kernel_ms": ft_ms,
                     "share_of_frame": ft_ms / ms_per_step, "peak_source": peak_kind,
                     "note": "issue/latency bound; most of these bytes are served from L1/L2 "
                             "(traffic = DRAM bytes of one launch, ncu)"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms, "hits_equal_device_run": e2e_same,
                "how": "one rta_host_frames_run per step on pinned host buffers: rays copied in, frame, "
                       "primary hits, all bounce-hit slots and the bounce count copied out; copies on "
                       "their own streams overlap the neighbouring steps' traversal"},
        # per timed frame: the fused trace (primary + bounce rays) and the
        # bounce gather (the L2 flush between frames is a torch fill)
        "gpu_launches": 2 * args.steps,
        "clocks": clk.summary(),
        "build": {"ms": bmean, "ms_min": min(build_ms), "mtri_s": n / (bmean * 1e-3) / 1e6,
                  "algorithmic_bytes": 372 * n, "achieved_gbs": 372 * n / (bmean * 1e-3) / 1e9,
                  "frac_of_peak": 372 * n / (bmean * 1e-3) / 1e9 / peak},
        "trace": {"primary_ms": tr_ms, "primary_mrays_s": nrays / (tr_ms * 1e-3) / 1e6,
                  "bounce_ms": statistics.mean(bounce_ms),
                  "bounce_mrays_s": nbounce / (statistics.mean(bounce_ms) * 1e-3) / 1e6,
                  "combined_mrays_s": value,
                  "primary_algorithmic_gbs": prim_bytes / (tr_ms * 1e-3) / 1e9,
                  "inner_visits_per_ray": inner_visits / rays_per_step,
                  "tri_tests_per_ray": tri_tests / rays_per_step,
                  "inner_visits_per_primary_ray": int(stp[0]) / nrays,
                  "inner_visits_per_bounce_ray": int(stbs[0]) / max(nbounce, 1),
                  "tri_tests_per_primary_ray": int(stp[1]) / nrays,
                  "tri_tests_per_bounce_ray": int(stbs[1]) / max(nbounce, 1)},
        "incoherent": incoherent,
        "learned_order": learned,
        "batched": batched,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    L.check(lib.rta_frame_destroy(fh), "rta_frame_destroy")
    if pg:
        pg.destroy_process_group()


def run_section(args):
    """One workload alone (for profiling and quick checks): prints its object."""
    import torch
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    fn = {"incoherent": incoherent_eval, "learned": learned_eval, "batched": batch_eval}[args.section]
    print(json.dumps({args.section: fn(args, dev)}))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.section:
        run_section(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
