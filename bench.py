"""Benchmark of the N-BVH ray-query hot path on GB300.

Workload (N-BVH inference): a 65,536-triangle fBm-displaced sphere in the unit cube, its binned-SAH
BVH2 cut at depth 10 (1,024 neural leaves), 4 stratified points per leaf segment, hash grid of 16
levels x 2 FP16 features x 2^19 entries (resolution 16..2048), 64-wide 4-hidden-layer ReLU MLP in
FP16, 2^22 query rays (origins uniform in the 1.5x scene box, directions uniform on the sphere).
The network was trained on a GB300 by the library's own optimiser on classic-labelled rays (20,000
steps; the weights are committed under bench_data/, `--retrain` trains afresh before timing; weights
of the reference are not available). A step is one neural closest-hit query over
the 2^22 resident rays; the classic BVH kernel answers the same rays for the "vs classic" figure and
judges depth / visibility.

The roofline object is the dominant kernel, the wavefront encoder, timed per launch with CUDA
events inside the timed region. The same comparison is repeated on the 4,194,304-triangle sphere
(key "mesh_4m"), where the classic traversal is deeper while the neural query still works on a
1,024-leaf cut. The tcgen05 MLP kernel is also timed alone on 2^22 rows
("roofline_kernels.mlp_tc"), the network is trained in FP16, BF16 and FP8 from the same seed and
compared on held-out rays ("precision_sweep"), a fixed depth-10 cut is compared with a learned tree
cut ("learned_cut"), a 1920x1080 6-bounce hybrid path trace is timed on one model
("path_config4") and on 16 instances of three models ("scene_config4"), the serving loop runs a
Poisson load of render requests against 4 resident models, beside the same load on their classic
BLAS ("serving"), and the CPU restatements of the neural and classic queries run on the host cores
("cpu_baseline").

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--train-steps T]
                    [--mesh4m-train-steps T4 | -1] [--precision-sweep-steps T3 | 0] [--serve-seconds S | 0]
                    [--learned-cut-steps T5 | -1] [--scene-train-steps T6 | -1] [--log2-rays R]
                    [--mlp-only LOG2_ROWS]
"""

import argparse
import ctypes as C
import glob
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_RAYS = 1 << 22
SUBDIV = 7  # 4 * 4^7 = 65,536 triangles
# Weights of the headline network (trained on a GB300 by this library's own optimiser, 20,000
# steps of 2^18 rays; `--save-bench-data` regenerates the file) with the cut, the scene box and the
# configuration they belong to: both arms answer the same rays with the same FP16 weights.
BENCH_DATA = os.path.join(ROOT, "bench_data", "sphere65k_cut1024_trained.npz")
CUT_DEPTH = 10
FLOP_PER_SEGMENT = 43008  # 2 * (128*64 + 3*64*64 + 64*16)
# wavefront encoder, per segment: 4 points x 16 levels x 8 corners x 4 B gathered, the 256 B FP16
# feature row written, 52 B of list state read (origin/t, direction/mint, meta, sort order)
ENCODE_BYTES_PER_SEGMENT = 2048 + 256 + 52
WORKLOAD = "nbvh_inference_sphere65k_cut1024_rays4M"
METRIC = "neural vs classic Mrays/s at <=1% depth err on 1 GB300; p50/p99 batch latency"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--train-steps", type=int, default=20000)
    ap.add_argument("--cpu-sample", type=int, default=1 << 14)
    ap.add_argument("--mesh4m-train-steps", type=int, default=10000,
                    help="training steps for the 4M-triangle comparison; -1 skips it")
    ap.add_argument("--precision-sweep-steps", type=int, default=5000,
                    help="training steps per precision in the FP16/BF16/FP8 sweep; 0 skips it")
    ap.add_argument("--serve-seconds", type=float, default=3.0,
                    help="seconds of Poisson arrivals in the serving load; 0 skips it")
    ap.add_argument("--serve-train-steps", type=int, default=1500)
    ap.add_argument("--scene-train-steps", type=int, default=2000,
                    help="training steps per model of the instanced config-4 scene (-1 skips it)")
    ap.add_argument("--reference-default-steps", type=int, default=5000,
                    help="training steps of the reference's default grid (8 levels x 4 features x 2^18, 3 points) "
                         "on the headline scene before its query is timed (-1 skips it)")
    ap.add_argument("--learned-cut-steps", type=int, default=4000,
                    help="training steps of the fixed-cut vs learned-cut comparison (-1 skips it)")
    ap.add_argument("--log2-rays", type=int, default=22,
                    help="rays per step; smaller values are for profiling captures, not bench lines")
    ap.add_argument("--save-bench-data", default="",
                    help="train the headline network (--train-steps) and save its weights, cut and configuration "
                         "to this .npz, then exit")
    ap.add_argument("--retrain", action="store_true",
                    help="train the headline network on the device instead of loading the committed weights")
    ap.add_argument("--mlp-only", type=int, default=0, metavar="LOG2_ROWS",
                    help="time only the tcgen05 MLP on 2^LOG2_ROWS resident rows (inside the NVTX range "
                         "`mlp_roofline`), print its line and exit; for profiling captures")
    ap.add_argument("--query-only", action="store_true",
                    help="time only the neural and classic queries of the headline workload (--log2-rays rays, "
                         "committed weights), print their line and exit; for profiling captures")
    ap.add_argument("--train-only", type=int, default=0, metavar="STEPS",
                    help="run only the training roofline (STEPS profiled steps of 2^18 rays), print it and exit; "
                         "for profiling captures")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms during the timed region: start()
    returns once the first sample has arrived (nvidia-smi takes a while to come up), stop() waits for
    one more sample before ending the sampler, so the timed region lies between sampled lines."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self._wait_for(1, 5.0)
        except Exception:
            self.proc = None

    def _wait_for(self, count, seconds):
        t_end = time.perf_counter() + seconds
        while len(self.lines) < count and time.perf_counter() < t_end and self.proc.poll() is None:
            time.sleep(0.005)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self._wait_for(len(self.lines) + 1, 1.0)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def profiled_traffic(key="neural_query_dram_bytes_per_launch_full_workload"):
    """A DRAM-bytes figure (`key: value` line) from the committed ncu summaries, if any."""
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.txt")) + glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        with open(path) as f:
            for line in f:
                m = re.match(r"\s*%s:\s*([0-9.eE+]+)" % re.escape(key), line)
                if m:
                    return float(m.group(1))
    return None


def build_scene(nb, scenes, cfg, subdiv=SUBDIV):
    v, f = scenes.fbm_sphere(subdiv, seed=1)
    alb = scenes.palette_albedo(len(f), 1)
    h = nb.NBVH(cfg)
    h.set_mesh(v, f, alb)
    h.build_classic()
    h.build_neural_cut(CUT_DEPTH)
    return h, v, f, alb


def time_queries(h, rays, hits, chits, steps, warmup, nvtx_name, profile=None):
    """Device times (ms) of `steps` neural and classic queries over resident rays, L2 flushed
    between steps, CUDA events on the launching stream. With a `profile` list, the library also
    times each wavefront-encoder launch of every timed neural query (CUDA events on the query's
    stream) and one nbvh_kernel_profile per query is appended to it."""
    import torch
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    cev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for _ in range(warmup):
        h.query_closest_neural(rays, 1, hits)
        neural_launches = h.last_kernel_time()[1]
        h.query_closest_classic(rays, chits)
        classic_launches = h.last_kernel_time()[1]
    torch.cuda.synchronize()
    if profile is not None:
        h.set_kernel_profile(True)
    torch.cuda.nvtx.range_push(nvtx_name)  # ncu --nvtx --nvtx-include "timed/" selects these launches
    for i in range(steps):
        flush.zero_()
        ev[i][0].record(stream)
        h.query_closest_neural(rays, 1, hits)
        ev[i][1].record(stream)
        if profile is not None:
            profile.append(h.kernel_profile())  # waits for this query's encoder events
    for i in range(steps):
        flush.zero_()
        cev[i][0].record(stream)
        h.query_closest_classic(rays, chits)
        cev[i][1].record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    if profile is not None:
        h.set_kernel_profile(False)
    times = np.array([a.elapsed_time(b) for a, b in ev])
    ctimes = np.array([a.elapsed_time(b) for a, b in cev])
    return times, ctimes, neural_launches, classic_launches


def relative_depth_error(tn, tc):
    """Relative depth error of neural hit distances tn against classic ones tc (rays that hit in both)."""
    err = np.abs(tn - tc).astype(np.float64)
    rel = err / np.maximum(tc, 1e-6)
    # relative error is ill-conditioned for rays starting on the surface (t -> 0): the headline
    # mean floors the denominator at 1% of the unit scene; the raw mean is reported beside it
    any_ = bool(len(tn) > 0)
    return {"mean_rel_floor1pct": float(np.mean(err / np.maximum(tc, 1e-2))) if any_ else None,
            "mean_rel_raw": float(rel.mean()) if any_ else None,
            "median_rel": float(np.median(rel)) if any_ else None,
            "p90_rel": float(np.percentile(rel, 90)) if any_ else None,
            "p99_rel": float(np.percentile(rel, 99)) if any_ else None,
            "within_1pct": float(np.mean(rel <= 0.01)) if any_ else None}


def accuracy(hits, chits):
    """Visibility agreement and depth error of the neural hits against the classic kernel."""
    g = hits.cpu().numpy().view(np.uint32)
    c = chits.cpu().numpy().view(np.uint32)
    nvalid = (g[:, 8] & 1) != 0
    cvalid = c[:, 3] != 0xFFFFFFFF
    vis_agree = float(np.mean(nvalid == cvalid))
    both = nvalid & cvalid
    depth = relative_depth_error(g[both, 0].view(np.float32), c[both, 0].view(np.float32))
    return vis_agree, depth, float(g[:, 9].astype(np.float64).mean())


def depth_error_by_origin(hits, chits, rays, nn):
    """The depth error split by where a ray starts: inside a leaf box of the neural cut (next to
    the surface, where the classic hit distance tends to 0 and any miss of the network is a large
    relative error) or outside every leaf box (as camera rays do)."""
    import torch
    g = hits.cpu().numpy().view(np.uint32)
    c = chits.cpu().numpy().view(np.uint32)
    both = ((g[:, 8] & 1) != 0) & (c[:, 3] != 0xFFFFFFFF)
    nodes = torch.from_numpy(np.ascontiguousarray(nn).view(np.float32)).cuda()
    leaf = torch.from_numpy(np.ascontiguousarray(nn)[:, 3] != 0).cuda()
    lo, hi = nodes[leaf, 0:3], nodes[leaf, 4:7]
    o = rays[:, 0:3]
    inside = torch.zeros(o.shape[0], dtype=torch.bool, device=o.device)
    for k in range(0, o.shape[0], 1 << 15):
        oo = o[k:k + (1 << 15), None, :]
        inside[k:k + (1 << 15)] = ((oo >= lo[None]) & (oo <= hi[None])).all(dim=2).any(dim=1)
    inside = inside.cpu().numpy()
    tn, tc = g[:, 0].view(np.float32), c[:, 0].view(np.float32)
    out = {}
    for name, m in (("origin_outside_leaves", both & ~inside), ("origin_inside_leaves", both & inside)):
        d = relative_depth_error(tn[m], tc[m])
        d["rays"] = int(m.sum())
        out[name] = d
    return out


def mlp_roofline(h, peak, rows=1 << 22, reps=10):
    """The tcgen05 MLP kernel alone on `rows` FP16 input rows resident in HBM."""
    import torch
    feats = (torch.rand((rows, h.layout.n_inputs), device="cuda") * 0.2 - 0.1).half().contiguous()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(3):
        h.mlp_inference(feats)
    ks = []
    for _ in range(reps):
        flush.zero_()
        h.mlp_inference(feats)
        ks.append(h.last_kernel_time()[0])
    ms = float(np.median(ks))
    achieved = FLOP_PER_SEGMENT * rows / (ms * 1e-3) / 1e12
    return {"kernel": "k_mlp_tc", "bound": "tensor", "rows": rows, "ms": ms, "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak,
            "input_read_gbs": rows * h.layout.n_inputs * 2 / (ms * 1e-3) / 1e9}


def cpu_classic_baseline(h, v, f, rays, sample_all, sample_one):
    """The CPU restatement of CudaBVH2::intersect (closest hit, include/cuda/accel/bvh2.cuh:12-88)
    over the same BVH, at all host threads and at 1 thread, on the first rays of the batch."""
    from oracle.bindings import Oracle
    orc = Oracle()
    nodes, prims = h.classic_bvh()
    scene = orc.classic_scene(nodes, prims, v, f)
    threads = os.cpu_count() or 1
    out = {}
    for n_thr, n in ((threads, sample_all), (1, sample_one)):
        sub = rays[:n]
        orc.classic_query(scene, sub[:256], threads=n_thr)
        t0 = time.perf_counter()
        orc.classic_query(scene, sub, threads=n_thr)
        out[n_thr] = n / (time.perf_counter() - t0) / 1e6
    return {"kind": "port", "unit": "Mrays/s", "cores": threads, "value": out[threads], "single_thread": out[1],
            "sample": "%d rays (all threads) and %d rays (1 thread) of the batch" % (sample_all, sample_one)}


def cpu_neural_baseline(nb, cfg, h_or_none, v, f, rays, params, threads, sample):
    """The CPU restatement of the neural query on `sample` rays with `threads` host threads."""
    from oracle.bindings import Oracle
    orc = Oracle()
    if h_or_none is not None:
        nodes, prims = h_or_none.classic_bvh()
        nn, bbox = h_or_none.neural_bvh()
        layout = h_or_none.layout
    else:
        nodes, prims = nb.build_bvh2_host(v, f)
        nn = nb.build_neural_cut_host(nodes, CUT_DEPTH)
        mn, mx = nb.nodes_to_float(nodes[:1])
        bbox = np.concatenate([mn[0], mx[0]])
        layout = nb.param_layout(cfg)
    net = orc.network(cfg, layout, params)
    consts = orc.neural_consts(cfg)
    nscene = orc.neural_scene(nn, bbox)
    sub = rays[:sample]
    orc.neural_query(nscene, net, consts, sub[: min(256, sample)], threads=threads)  # warm
    t0 = time.perf_counter()
    hits = orc.neural_query(nscene, net, consts, sub, threads=threads)
    dt = time.perf_counter() - t0
    return len(sub) / dt / 1e6, hits


def load_bench_data():
    """The committed headline network: FP16 weights (as FP32 values), the neural cut, the scene box,
    the configuration and parameter layout (ctypes structs rebuilt from their bytes: no library call)."""
    from nbvh_gb300 import abi
    d = np.load(BENCH_DATA)
    cfg = abi.Config.from_buffer_copy(d["config"].tobytes())
    layout = abi.ParamLayout.from_buffer_copy(d["layout"].tobytes())
    params = d["params_f16"].view(np.float16).astype(np.float32)
    meta = json.loads(str(d["meta"]))
    return cfg, layout, params, d["neural"], d["bbox"], meta


def save_bench_data(path, h, cfg, nn, bbox, st, steps):
    params = h.params().astype(np.float16)
    meta = {"train_steps": steps, "train_batch": int(cfg.batch_size), "seed": int(cfg.seed),
            "last_loss": float(st.last_loss) if st else None, "mesh": "fbm_sphere(%d, seed=1)" % SUBDIV,
            "cut_depth": CUT_DEPTH}
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez_compressed(path, params_f16=params.view(np.uint16), neural=np.ascontiguousarray(nn, np.uint32),
                        bbox=np.asarray(bbox, np.float32), config=np.frombuffer(bytes(cfg), np.uint8),
                        layout=np.frombuffer(bytes(h.layout), np.uint8), meta=np.array(json.dumps(meta)))


def run_reference(args):
    """The reference path on the host cores: the CPU restatement of the neural closest-hit query
    (NeuralPathModule::neural_bvh_traversal and the tcnn network it calls; the reference itself
    cannot be built here) on a bounded sample of the same 2^22 rays, with the same weights, cut and
    configuration as the GPU arm (the committed bench data), all host threads. Loads no library of
    this repository but the oracle."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from nbvh_gb300 import scenes
    from oracle.bindings import Oracle
    from oracle.bindings import build as build_oracle
    build_oracle()
    cfg, layout, params, nn, bbox, meta = load_bench_data()
    rays = scenes.uniform_rays(N_RAYS, bbox[:3], bbox[3:], seed=2024)
    sample = rays[:args.cpu_sample]
    orc = Oracle()
    # the committed layout holds the level scales the GPU arm's handle encodes with (tcnn's
    # exp2f(l * log2f(s)) * base - 1 evaluated on the device); the oracle's own host evaluation must
    # give the same offsets, sizes and resolutions and scales within 2 ulp (CUDA's exp2f bound)
    hg = cfg.hashgrid
    off, size, res, scale, total = orc.grid_layout(hg.n_levels, hg.log2_hashmap_size, hg.base_resolution,
                                                   hg.per_level_scale)
    nl = hg.n_levels
    assert list(off) == list(layout.level_offset[:nl]) and list(size) == list(layout.level_size[:nl])
    assert list(res) == list(layout.level_resolution[:nl])
    committed = np.array(layout.level_scale[:nl], np.float32)
    assert np.abs(committed.view(np.int32).astype(np.int64) - np.asarray(scale, np.float32).view(np.int32)).max() <= 2
    net = orc.network(cfg, layout, params)
    consts = orc.neural_consts(cfg)
    nscene = orc.neural_scene(nn, bbox)
    threads = os.cpu_count() or 1
    orc.neural_query(nscene, net, consts, sample[:256], threads=threads)  # warm
    vals, segs = [], None
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        hits = orc.neural_query(nscene, net, consts, sample, threads=threads)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            vals.append(len(sample) / dt / 1e6)
        segs = float(hits[:, 9].astype(np.float64).mean())
    value = float(np.mean(vals))
    desc = ("%d of the 2^22 rays per step (the first ones of the GPU arm's batch), the GPU arm's trained FP16 "
            "weights (%d training steps), %d host threads" % (len(sample), meta["train_steps"], threads))
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value,
        "unit": "Mrays/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": len(sample) / (value * 1e6) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded mesh and rays; committed trained weights)",
        "config": {"workload": WORKLOAD, "rays_per_step": len(sample), "threads": threads, "same_weights": True,
                   "segments_per_ray": segs},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_ours(args):
    import torch

    import nbvh_gb300 as nb
    from nbvh_gb300 import scenes
    from nbvh_gb300.shard import max_over_ranks
    import __graft_entry__
    rank, world, local = dist_env()
    __graft_entry__.build()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    cfg = nb.default_config()
    h, v, f, alb = build_scene(nb, scenes, cfg)
    nn, bbox = h.neural_bvh()
    if args.train_only:
        peaks, _ = measured_peaks()
        h.close()
        if rank == 0:
            print(json.dumps({"train_roofline": run_train_roofline(nb, scenes, peaks, steps=args.train_only,
                                                                   warmup=3)}))
        return
    if args.mlp_only:
        peaks, peak_kind = measured_peaks()
        torch.cuda.nvtx.range_push("mlp_roofline")
        r = mlp_roofline(h, float(peaks.get("bf16_tflops", 1900.0)), rows=1 << args.mlp_only, reps=3)
        torch.cuda.nvtx.range_pop()
        if rank == 0:
            print(json.dumps({"mlp_tc": r, "peak_kind": peak_kind}))
        h.close()
        return
    # the headline network: the committed weights (trained by this library on a GB300), or trained
    # on the device here (outside the timed region)
    t0 = time.perf_counter()
    st, weights_from = None, "trained on the device in this run"
    use_file = (not args.retrain and not args.save_bench_data and os.path.exists(BENCH_DATA))
    if use_file:
        _, _, fparams, fnn, fbbox, fmeta = load_bench_data()
        if np.array_equal(fnn, nn) and np.array_equal(fbbox, bbox) and fparams.size == h.layout.n_params:
            h.set_params(fparams)
            weights_from = "committed weights (%d training steps on a GB300 by this library)" % fmeta["train_steps"]
        else:
            use_file = False
    if not use_file:
        st = h.run_optimisation(args.train_steps) if args.train_steps > 0 else None
    train_s = time.perf_counter() - t0
    if args.query_only:
        rays_np = scenes.uniform_rays(N_RAYS, bbox[:3], bbox[3:], seed=2024 + rank)
        rays = torch.from_numpy(rays_np).cuda()
        hits = torch.empty((N_RAYS, 12), dtype=torch.int32, device="cuda")
        chits = torch.empty((N_RAYS, 4), dtype=torch.int32, device="cuda")
        times, ctimes, nl, cl = time_queries(h, rays, hits, chits, args.steps, args.warmup, "timed")
        if rank == 0:
            print(json.dumps({"rays": N_RAYS, "neural_ms": float(times.mean()), "classic_ms": float(ctimes.mean()),
                              "neural_launches": nl, "classic_launches": cl, "weights": weights_from}))
        h.close()
        return
    if args.save_bench_data:
        if rank == 0:
            save_bench_data(args.save_bench_data, h, cfg, nn, bbox, st, args.train_steps)
            print(json.dumps({"saved": args.save_bench_data, "train_seconds": train_s,
                              "last_loss": st.last_loss if st else None}))
        h.close()
        return
    # the committed weights and the device have the same FP16 copy: the GPU arm uses exactly these
    params_used = h.params().astype(np.float16)
    # per-rank shard of rays (weak scaling: every rank answers its own 2^22 rays)
    rays_np = scenes.uniform_rays(N_RAYS, bbox[:3], bbox[3:], seed=2024 + rank)
    rays = torch.from_numpy(rays_np).cuda()
    hits = torch.empty((N_RAYS, 12), dtype=torch.int32, device="cuda")
    chits = torch.empty((N_RAYS, 4), dtype=torch.int32, device="cuda")

    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    enc_prof = []
    times, ctimes, neural_launches, classic_launches = time_queries(h, rays, hits, chits, args.steps, args.warmup,
                                                                     "timed", profile=enc_prof)
    barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    ms, cms = max_over_ranks([float(times.mean()), float(ctimes.mean())])
    stats = h.query_stats()
    vis_agree, depth_stats, segs_per_ray = accuracy(hits, chits)
    depth_by_origin = depth_error_by_origin(hits, chits, rays, nn)

    # e2e through the host-buffer C-ABI call: pinned host rays in, hits out, copies timed
    pin_in = torch.from_numpy(rays_np).pin_memory()
    pin_out = torch.empty((N_RAYS, 12), dtype=torch.int32).pin_memory()
    lib = h.lib
    e2e_times = []
    for i in range(args.warmup + max(3, args.steps // 4)):
        t0 = time.perf_counter()
        r = lib.nbvh_query_closest_neural_host(h.h, C.c_void_p(pin_in.data_ptr()), N_RAYS, 1,
                                               C.c_void_p(pin_out.data_ptr()))
        dt = time.perf_counter() - t0
        assert r == 0
        if i >= args.warmup:
            e2e_times.append(dt)
    e2e_ms = max_over_ranks([float(np.mean(e2e_times)) * 1e3])[0]

    peaks, peak_kind = measured_peaks()
    peak = float(peaks.get("bf16_tflops", 1900.0))
    flops = FLOP_PER_SEGMENT * stats.segments
    achieved = flops / (ms * 1e-3) / 1e12
    # dominant kernel: the wavefront encoder, timed per launch inside the timed region
    enc_launches = sum(p.encode_launches for p in enc_prof)
    enc_ms = sum(p.encode_ms for p in enc_prof)
    enc_bytes = ENCODE_BYTES_PER_SEGMENT * sum(p.encoded_segments for p in enc_prof)
    enc_gbs = enc_bytes / (enc_ms * 1e-3) / 1e9 if enc_ms > 0 else None
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    # DRAM bytes per launch: the encoder's DRAM bytes per encoded segment from its ncu capture
    # (profiles/k_wave_encode_sphere65k_rays1M.md) x the segments an average launch encodes here
    per_seg = profiled_traffic("encode_dram_bytes_per_segment")
    enc_traffic = (per_seg * sum(p.encoded_segments for p in enc_prof) / max(1, enc_launches)) if per_seg else None
    value = world * N_RAYS / (ms * 1e-3) / 1e6
    line = {
        "metric": METRIC,
        "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f16",
        "data": "synthetic (seeded mesh and rays); weights: " + weights_from,
        "config": {"workload": WORKLOAD, "rays_per_step": N_RAYS, "triangles": int(len(f)),
                   "neural_leaves": int((nn[:, 3] > 0).sum()), "points_per_segment": 4,
                   "grid": "16 levels x 2 x 2^19 FP16, res 16-2048", "mlp": "64x4 ReLU FP16",
                   "weights": weights_from, "train_batch": cfg.batch_size,
                   "l2": "flushed between timed steps (256 MB write); inputs 128 MB + outputs 192 MB",
                   "parallelism": "rays sharded per rank, no collective"},
        "classic_mrays": world * N_RAYS / (cms * 1e-3) / 1e6, "classic_ms_per_step": cms,
        "neural_over_classic": cms / ms,
        "p50_ms": float(np.percentile(times, 50)), "p99_ms": float(np.percentile(times, 99)),
        "depth_rel_err_mean": depth_stats["mean_rel_floor1pct"], "depth_error": depth_stats,
        "depth_error_by_origin": depth_by_origin,
        "visibility_agreement": vis_agree, "segments_per_ray": segs_per_ray,
        "train": {"steps": args.train_steps if st else 0, "seconds": train_s,
                  "last_loss": (st.last_loss if st else None), "ms_per_step": (st.ms_per_step if st else None)},
        "roofline": {"bound": "hbm", "achieved": enc_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": (enc_gbs / hbm_peak) if enc_gbs else None,
                     "peak_kind": peak_kind + " copy bandwidth (burst)",
                     "traffic": enc_traffic,
                     "kernel": "k_wave_encode (wavefront hash-grid encoder, %.0f%% of the query's device time)"
                               % (100.0 * enc_ms / max(1e-9, sum(times))),
                     "launches": enc_launches, "avg_launch_ms": enc_ms / max(1, enc_launches),
                     "algorithmic": "%d B per encoded segment (4 points x 16 levels x 8 corners x 4 B of table "
                                    "gathers + 256 B feature row + 52 B list state) x %d segments per launch"
                                    % (ENCODE_BYTES_PER_SEGMENT,
                                       sum(p.encoded_segments for p in enc_prof) // max(1, enc_launches)),
                     "note": "the 24 MB table is L2-resident: the gathers are served by L2 (DRAM traffic is "
                             "below the algorithmic bytes); the kernel is bound by the L1 miss path"},
        "e2e": {"value": world * N_RAYS / (e2e_ms * 1e-3) / 1e6, "unit": "Mrays/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": N_RAYS * 32, "d2h_bytes_per_step": N_RAYS * 48},
        "gpu_launches": args.steps * (neural_launches + classic_launches),
        "clocks": clk,
        "wall_s_timed": wall,
    }
    line["roofline_kernels"] = {
        "mlp_tc": mlp_roofline(h, peak),
        "whole_query_tensor": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                               "frac": achieved / peak, "traffic": None,
                               "algorithmic": "43,008 FLOP per inferred leaf segment x %d segments per query"
                                              % stats.segments},
    }
    if rank == 0:
        params = h.params()
        threads = os.cpu_count() or 1
        assert np.array_equal(params.astype(np.float16), params_used)
        mr, _ = cpu_neural_baseline(nb, cfg, h, v, f, rays_np, params, threads, args.cpu_sample)
        line["cpu_baseline"] = {"value": mr, "unit": "Mrays/s", "cores": threads, "kind": "port",
                                "sample": "%d of the 2^22 rays, the same weights, CPU restatement of the neural "
                                          "query" % args.cpu_sample}
        line["cpu_baseline"]["classic"] = cpu_classic_baseline(h, v, f, rays_np, 1 << 18, 1 << 16)
        line["classic_config1"] = run_classic_config1(h, v, f, bbox, scenes, args.steps, args.warmup, 1 << 17)
        line["path_config4"] = run_path_config4(h, nb, scenes, bbox)
    h.close()
    del rays, hits, chits, pin_in, pin_out
    torch.cuda.empty_cache()

    if args.mesh4m_train_steps >= 0:
        line["mesh_4m"] = run_mesh_4m(args, nb, scenes, cfg, max_over_ranks, rank)
    if rank == 0:
        line["train_roofline"] = run_train_roofline(nb, scenes, peaks)
    if args.precision_sweep_steps > 0:
        line["precision_sweep"] = run_precision_sweep(args, nb, scenes, args.precision_sweep_steps)
    if rank == 0 and args.reference_default_steps >= 0:
        line["config_reference_default"] = run_reference_default(args, nb, scenes, args.reference_default_steps)
    if rank == 0 and args.learned_cut_steps >= 0:
        line["learned_cut"] = run_learned_cut(args, nb, scenes, args.learned_cut_steps)
    if rank == 0 and args.scene_train_steps >= 0:
        line["scene_config4"] = run_scene_config4(args, nb, scenes)
    if args.serve_seconds > 0:
        line["serving"] = run_serving(args, nb, scenes)
    # the headline figures (throughputs, accuracy, latencies, rooflines), compact, at the end of the line
    line["summary"] = summary_of(line)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def summary_of(line):
    r = lambda x, k=1: None if x is None else round(float(x), k)
    cb = line.get("cpu_baseline", {}).get("classic", {})
    m4 = line.get("mesh_4m", {})
    de = line.get("depth_error", {})
    sv = line.get("serving", {}).get("neural", {}) if isinstance(line.get("serving"), dict) else {}
    b1m = sv.get("batch_1m", {})
    return {"neural_mrays": r(line["value"]), "classic_mrays": r(line.get("classic_mrays")),
            "neural_over_classic": r(line.get("neural_over_classic"), 3),
            "mesh4m_neural_over_classic": r(m4.get("neural_over_classic"), 3),
            "mesh4m_neural_mrays": r(m4.get("neural_mrays")), "mesh4m_classic_mrays": r(m4.get("classic_mrays")),
            "vis_agree": r(line.get("visibility_agreement"), 4), "depth_rel_mean_raw": r(de.get("mean_rel_raw"), 4),
            "depth_rel_mean_floor1pct": r(de.get("mean_rel_floor1pct"), 4),
            "depth_within_1pct": r(de.get("within_1pct"), 4),
            "depth_rel_mean_raw_origin_outside_leaves":
                r(line.get("depth_error_by_origin", {}).get("origin_outside_leaves", {}).get("mean_rel_raw"), 4),
            "cpu_classic_mrays_all": r(cb.get("value"), 2), "cpu_classic_mrays_1thr": r(cb.get("single_thread"), 3),
            "cpu_cores": cb.get("cores"),
            "serving_render_p99_ms_requests_0p5_to_2m_rays": r(sv.get("p99_ms_requests_0p5_to_2m_rays"), 2),
            "serving_1m_batch_p99_ms": r(b1m.get("p99_ms"), 2), "serving_1m_batch_p50_ms": r(b1m.get("p50_ms"), 2),
            "train_ms_per_step": r(line.get("train_roofline", {}).get("ms_per_step"), 3),
            "train_mlp_tc_frac": r(line.get("train_roofline", {}).get("mlp_tc", {}).get("frac"), 3),
            "mlp_tc_frac": r(line.get("roofline_kernels", {}).get("mlp_tc", {}).get("frac"), 3),
            "e2e_mrays": r(line.get("e2e", {}).get("value")),
            "refdefault_f4_mrays": r(line.get("config_reference_default", {}).get("query_mrays")),
            "refdefault_f4_vis_agree": r(line.get("config_reference_default", {}).get("visibility_agreement"), 4)}


def run_classic_config1(h, v, f, bbox, scenes, steps, warmup, cpu_sample):
    """Classic closest hit on 512x512 pinhole rays from a seeded orbit camera plus one cosine bounce
    per hit (the plain method's own workload): device time of the combined batch, bit-exact check
    of a sample against the CPU restatement, and that restatement's throughput on the host cores."""
    import torch
    from oracle.bindings import Oracle
    org, tgt, up = scenes.orbit_camera(bbox[:3], bbox[3:], seed=4)
    prim = scenes.camera_rays(512, 512, org, tgt, up, seed=4)
    prim_hits = h.query_closest_classic_host(prim)
    bounce = scenes.bounce_rays(prim, prim_hits.view(np.uint32).reshape(-1, 4), v, f, seed=4)
    rays_np = np.ascontiguousarray(np.concatenate([prim, bounce]), np.float32)
    n = len(rays_np)
    rays = torch.from_numpy(rays_np).cuda()
    out = torch.empty((n, 4), dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        h.query_closest_classic(rays, out)
    ts = []
    for _ in range(steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        h.query_closest_classic(rays, out)
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    ms = float(np.mean(ts))
    orc = Oracle()
    nodes, prims = h.classic_bvh()
    scene = orc.classic_scene(nodes, prims, v, f)
    idx = np.random.default_rng(5).choice(n, size=min(cpu_sample, n), replace=False)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref = orc.classic_query(scene, rays_np[idx], threads=threads)
    cpu_s = time.perf_counter() - t0
    got = out.cpu().numpy().view(np.uint32)[idx]
    return {"rays": n, "primary": len(prim), "bounce": len(bounce), "ms_per_step": ms,
            "mrays": n / (ms * 1e-3) / 1e6, "bit_exact_sample": bool(np.array_equal(got, ref)),
            "sample": len(idx), "cpu_mrays": len(idx) / cpu_s / 1e6, "cpu_threads": threads}


def run_scene_config4(args, nb, scenes, reps=3):
    """Config 4: hybrid path tracing at 1920 x 1080, 1 sample per pixel, 6 bounces over 16 instances
    of 3 neural BLAS (262,144-triangle fBm sphere, 1,048,576-triangle terrain, 4,194,304-triangle
    soup with 1e-3..1e-2 edges; each trained `args.scene_train_steps` steps) placed on a 4 x 4 grid
    with seeded rotations about y and scales 0.8-1.2, a classic ground plane and an analytic sky."""
    rng = np.random.default_rng(44)
    models, build_s, train_s = [], 0.0, 0.0
    for kind in ("sphere", "terrain", "soup"):
        t0 = time.perf_counter()
        if kind == "sphere":
            v, f = scenes.fbm_sphere(8, seed=21)
        elif kind == "terrain":
            v, f = scenes.terrain(1024, 512, seed=22)
        else:
            v, f = scenes.soup(4194304, seed=23)
        h = nb.NBVH(nb.default_config())
        h.set_mesh(v, f, scenes.palette_albedo(len(f), 24 + len(models)))
        h.build_classic()
        h.build_neural_cut(10)
        build_s += time.perf_counter() - t0
        t0 = time.perf_counter()
        h.run_optimisation(args.scene_train_steps)
        train_s += time.perf_counter() - t0
        models.append((h, len(f)))
    sc = nb.Scene()
    for k in range(16):
        h, _ = models[k % 3]
        ang = rng.uniform(0, 2 * np.pi)
        scl = rng.uniform(0.8, 1.2)
        c, s_ = np.cos(ang), np.sin(ang)
        A = scl * np.array([[c, 0, s_], [0, 1, 0], [-s_, 0, c]])
        centre = np.array([0.5, 0.0, 0.5])  # meshes live in the unit cube: rotate about its vertical axis
        gx, gz = k % 4, k // 4
        b = np.array([1.5 * gx, 0.0, 1.5 * gz]) - A @ centre
        sc.add_instance(h, np.hstack([A, b[:, None]]).astype(np.float32))
    lo, hi = np.array([-0.3, 0.0, -0.3]), np.array([5.3, 1.2, 5.3])
    cam = nb.render_request(1920, 1080, [2.5, 3.2, -2.8], [2.5, 0.2, 2.5], [0, 1, 0], 50.0)
    req = nb.path_request(cam, spp=1, max_bounces=6, seed=1, ground_height=-0.01, ground_albedo=(0.6, 0.6, 0.6))
    sc.render_path(req)  # warm
    ts, traced = [], 0
    for _ in range(reps):
        t0 = time.perf_counter()
        _, traced = sc.render_path(req)
        ts.append(time.perf_counter() - t0)
    t = float(np.median(ts))
    out = {"width": 1920, "height": 1080, "spp": 1, "bounces": 6, "instances": 16,
           "models_triangles": [m[1] for m in models], "train_steps_per_model": args.scene_train_steps,
           "build_seconds": build_s, "train_seconds": train_s, "rays_per_frame": int(traced),
           "ms_per_frame": t * 1e3, "mrays": traced / t / 1e6, "ground_plane": True}
    sc.close()
    for h, _ in models:
        h.close()
    del lo, hi
    return out


def run_path_config4(h, nb, scenes, bbox, reps=3):
    """Hybrid path tracing at 1920 x 1080, 1 sample per pixel, 6 bounces: one neural BLAS plus a
    classic ground plane under an analytic sky (the instanced form is run_scene_config4)."""
    org, tgt, up = scenes.orbit_camera(bbox[:3], bbox[3:], seed=12)
    cam = nb.render_request(1920, 1080, org, tgt, up, 45.0, sample_idx=0, sample_offset=0)
    req = nb.path_request(cam, spp=1, max_bounces=6, seed=1, ground_height=float(bbox[1]) - 0.01,
                          ground_albedo=(0.6, 0.6, 0.6))
    h.render_path(req)  # warm
    ts, traced = [], 0
    for _ in range(reps):
        t0 = time.perf_counter()
        _, traced = h.render_path(req)
        ts.append(time.perf_counter() - t0)
    t = float(np.median(ts))
    return {"width": 1920, "height": 1080, "spp": 1, "bounces": 6, "rays_per_frame": int(traced),
            "ms_per_frame": t * 1e3, "mrays": traced / t / 1e6, "ground_plane": True}


def run_serving(args, nb, scenes):
    """Serving: 4 resident models (65K / 262K / 1M / 4M-triangle spheres, config-2 network), 64
    open-loop clients with Poisson arrivals at 200 requests/s in total, each request a render of
    128^2..1024^2 pixels (log-uniform side), 1-8 samples and 0-4 bounces against a random model,
    served by 4 render slots, plus one query-lane slot (queries only, highest stream priority) that
    answers 1M-ray query batches submitted 20 times a second by a probing client. The same load then
    runs with every model answered by its classic BLAS (the classic-only loop)."""
    import threading
    models = []
    for subdiv in (7, 8, 9, 10):
        cfg = nb.default_config()
        h, v, f, _ = build_scene(nb, scenes, cfg, subdiv=subdiv)
        h.run_optimisation(args.serve_train_steps)
        models.append((h, h.neural_bvh()[1], len(f)))

    # 1M-ray query batches (rays through the model's scene box) submitted 20 times a second on top of
    # the render load: their latency is the p50 / p99 "per 1M-ray batch". The probing client keeps its
    # rays and a ring of hit buffers in page-locked memory, as a latency-bound client would.
    import torch
    n_probe, n_ring = 1 << 20, 4

    def pinned(n_words, dtype):
        return torch.empty(n_words, dtype=dtype).pin_memory().numpy()

    probe_rays = []
    for k, m in enumerate(models):
        buf = pinned(n_probe * 8, torch.float32).reshape(n_probe, 8)
        buf[:] = scenes.uniform_rays(n_probe, m[1][:3], m[1][3:], seed=900 + k)
        probe_rays.append(buf)
    probe_hits = [pinned(n_probe * 12, torch.int32).view(nb.NEURAL_HIT_DTYPE) for _ in range(n_ring)]

    def load(srv, ids, seconds, rate, clients, seed):
        done, lock = [], threading.Lock()
        probes, probe_queue = [], []

        def prober():
            rng = np.random.default_rng(seed + 77)
            tickets, t_end, n_sub = [], time.perf_counter() + seconds, 0
            t_next = time.perf_counter() + 0.05

            def finish(t):
                _, res = srv.wait(t, timeout_ms=600000)
                with lock:
                    probes.append(res.latency_ms)
                    probe_queue.append(res.queue_ms)

            while t_next < t_end:
                if len(tickets) >= n_ring:  # the ring's oldest hit buffer is reused next
                    finish(tickets.pop(0))
                delay = t_next - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                m = int(rng.integers(len(ids)))
                tickets.append(srv.submit_query(ids[m], probe_rays[m], 1, hits=probe_hits[n_sub % n_ring]))
                n_sub += 1
                t_next += 0.05
            for t in tickets:
                finish(t)

        def client(c):
            rng = np.random.default_rng(seed * 1000 + c)
            tickets, t_end = [], time.perf_counter() + seconds
            t_next = time.perf_counter() + rng.exponential(clients / rate)
            while t_next < t_end:
                delay = t_next - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                m = int(rng.integers(len(ids)))
                side = int(2 ** rng.uniform(7, 10))
                bbox = models[m][1]
                org, tgt, up = scenes.orbit_camera(bbox[:3], bbox[3:], seed=int(rng.integers(1 << 30)))
                cam = nb.render_request(side, side, org, tgt, up, 45.0, sample_idx=int(rng.integers(1000)))
                req = nb.path_request(cam, spp=int(rng.integers(1, 9)), max_bounces=int(rng.integers(0, 5)),
                                      seed=int(rng.integers(1 << 20)), ground_height=float(bbox[1]) - 0.01)
                tickets.append(srv.submit_render(ids[m], req))
                t_next += rng.exponential(clients / rate)
            for t in tickets:
                _, res = srv.wait(t, timeout_ms=600000)
                with lock:
                    done.append((res.latency_ms, res.rays_traced))

        threads = [threading.Thread(target=client, args=(c,)) for c in range(clients)]
        threads.append(threading.Thread(target=prober))
        t0 = time.perf_counter()
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        wall = time.perf_counter() - t0
        st = srv.stats()
        lat = np.array([d[0] for d in done]) if done else np.zeros(1)
        rays = np.array([max(d[1], 1) for d in done]) if done else np.ones(1)
        per_m = lat * 1e6 / rays                      # latency per 1M rays traced
        near_1m = lat[(rays >= 5e5) & (rays <= 2e6)]  # requests of 0.5M..2M rays
        return {"requests": st.requests_done, "p50_ms": st.p50_ms, "p99_ms": st.p99_ms, "mean_ms": st.mean_ms,
                "max_ms": st.max_ms, "rays_traced": st.rays_traced,
                "mrays": st.rays_traced / st.busy_seconds / 1e6 if st.busy_seconds > 0 else None,
                "busy_seconds": st.busy_seconds, "wall_seconds": wall, "batches": st.batches,
                # each render request's latency over its rays in millions: small renders (16K rays
                # in 10-20 ms) dominate the p99; the 1M-ray figures are batch_1m and the requests of
                # 0.5M-2M rays
                "ms_per_1m_rays_p50": float(np.percentile(per_m, 50)),
                "ms_per_1m_rays_p99": float(np.percentile(per_m, 99)),
                "requests_0p5_to_2m_rays": int(near_1m.size),
                "p99_ms_requests_0p5_to_2m_rays": float(np.percentile(near_1m, 99)) if near_1m.size else None,
                "mean_rays_per_request": float(rays.mean()),
                "batch_1m": {"count": len(probes), "p50_ms": float(np.percentile(probes, 50)) if probes else None,
                             "p99_ms": float(np.percentile(probes, 99)) if probes else None,
                             "max_ms": float(np.max(probes)) if probes else None,
                             "queue_p99_ms": float(np.percentile(probe_queue, 99)) if probes else None,
                             "what": "1,048,576-ray query batches from page-locked client buffers, 20 per "
                                     "second, under the render load, on the server's query lane (one slot of "
                                     "the device's highest stream priority)"}}

    out = {"models_triangles": [m[2] for m in models], "clients": 64, "rate_req_per_s": 200.0,
           "seconds_of_arrivals": args.serve_seconds, "hbm_budget_gb": 150, "render_slots": 4, "query_slots": 1,
           "slot_capacity_rays": 1 << 20}
    # Slots of 2^20 rays: a render's bounce batches (and so its kernels, which hold their SMs until
    # they end) stay short, so the query lane's kernels find SMs sooner. Measured on GB300 under this
    # load: 1M-batch p99 7.5 ms with 2^20-ray slots, 10.9 ms with 2^21, 12.4 ms with 2^22.
    srv = nb.Server(n_slots=5, query_slots=1, hbm_budget_gb=150.0, max_batch_rays=1 << 20)
    try:
        ids = [srv.add_model(m[0]) for m in models]
        out["neural"] = load(srv, ids, args.serve_seconds, 200.0, 64, 1)
        srv.reset_stats()
        for m in models:
            m[0].set_ignore_neural_blas(True)
        out["classic_only"] = load(srv, ids, args.serve_seconds, 200.0, 64, 1)
        for m in models:
            m[0].set_ignore_neural_blas(False)
    finally:
        srv.close()
        for m in models:
            m[0].close()
    return out


def run_reference_default(args, nb, scenes, steps):
    """The reference's own default encoding (include/cuda/neural/utils/tcnn_config.h:70-74: hash grid
    of 8 levels x 4 FP16 features x 2^18 entries, base resolution 8, level scale 2; 3 points per
    segment, 96 network inputs) on the headline scene and cut (65,536 triangles, depth-10 cut):
    `steps` training steps of 2^18 rays, then the neural and classic queries timed on the headline's
    2^22 rays and compared (visibility agreement, depth error). The reference default also learns
    its cut from the root; here the cut is the headline's fixed one, so that only the encoding
    differs from the headline."""
    import torch
    cfg = nb.reference_default_config()
    cfg.neural_bvh_max_depth = CUT_DEPTH
    h, v, f, _ = build_scene(nb, scenes, cfg)
    _, bbox = h.neural_bvh()
    t0 = time.perf_counter()
    st = h.run_optimisation(steps)
    train_s = time.perf_counter() - t0
    rays = torch.from_numpy(scenes.uniform_rays(N_RAYS, bbox[:3], bbox[3:], seed=2)).cuda()
    hits = torch.empty((N_RAYS, 12), dtype=torch.int32, device="cuda")
    chits = torch.empty((N_RAYS, 4), dtype=torch.int32, device="cuda")
    times, ctimes, _, _ = time_queries(h, rays, hits, chits, 5, 3, "reference_default")
    vis, depth, segs = accuracy(hits, chits)
    L = nb.param_layout(cfg)
    out = {"grid": "8 levels x 4 FP16 features x 2^18, res 8-1024 (scale 2)", "points_per_segment": 3,
           "network_inputs": 96, "params": int(L.n_params), "cut": "fixed depth 10 (1,024 leaves)",
           "train_steps": steps, "train_ms_per_step": st.ms_per_step, "train_seconds": train_s,
           "last_loss": st.last_loss, "rays": N_RAYS, "query_ms": float(times.mean()),
           "query_mrays": N_RAYS / (float(times.mean()) * 1e-3) / 1e6,
           "classic_mrays": N_RAYS / (float(ctimes.mean()) * 1e-3) / 1e6,
           "visibility_agreement": vis, "depth_error": depth, "segments_per_ray": segs}
    out["neural_over_classic"] = out["query_mrays"] / out["classic_mrays"]
    h.close()
    return out


def run_precision_sweep(args, nb, scenes, steps):
    """Config 3: the same network trained from the same seed in each MLP precision (FP16, BF16,
    FP8-E4M3 hidden layers) for
    `steps` steps of 2^18 device-labelled rays, then evaluated against the classic kernel on 2^20
    held-out rays (visibility agreement, depth error) and timed as a query."""
    import torch
    out = {}
    for name, prec in (("fp16", 0), ("bf16", 1), ("fp8", 2)):
        cfg = nb.default_config(**{"network.precision": prec})
        h, v, f, _ = build_scene(nb, scenes, cfg)
        nn, bbox = h.neural_bvh()
        t0 = time.perf_counter()
        st = h.run_optimisation(steps)
        train_s = time.perf_counter() - t0
        n = 1 << 20
        rays = torch.from_numpy(scenes.uniform_rays(n, bbox[:3], bbox[3:], seed=777)).cuda()
        hits = torch.empty((n, 12), dtype=torch.int32, device="cuda")
        chits = torch.empty((n, 4), dtype=torch.int32, device="cuda")
        times, _, _, _ = time_queries(h, rays, hits, chits, 5, 3, "sweep")
        vis, depth, segs = accuracy(hits, chits)
        out[name] = {"train_steps": steps, "train_ms_per_step": st.ms_per_step, "train_seconds": train_s,
                     "last_loss": st.last_loss, "heldout_rays": n, "visibility_agreement": vis,
                     "depth_error": depth, "query_ms": float(times.mean()),
                     "query_mrays": n / (float(times.mean()) * 1e-3) / 1e6}
        h.close()
    return out


def run_learned_cut(args, nb, scenes, steps):
    """The learned tree cut against the fixed depth-10 cut: the same network trained for `steps`
    steps either on the fixed cut or with tree-cut learning from the root on the schedule of the
    reference's shipped chess cut (split interval 40, scaling 2.5, last split at 3000: 25,249
    nodes), node survival on; then held-out accuracy and query time on 2^20 rays."""
    import torch
    out = {}
    sched = dict(splitting_interval=40, split_scaling=2.5, last_split_iteration=3000)
    for name in ("fixed_depth10", "learned"):
        cfg = nb.default_config()
        h, v, f, _ = build_scene(nb, scenes, cfg)
        if name == "learned":
            h.begin_tree_cut(nb.tree_cut_options(**sched), 0)
        t0 = time.perf_counter()
        st = h.run_optimisation(steps)
        train_s = time.perf_counter() - t0
        nn, bbox = h.neural_bvh()
        n = 1 << 20
        rays = torch.from_numpy(scenes.uniform_rays(n, bbox[:3], bbox[3:], seed=778)).cuda()
        hits = torch.empty((n, 12), dtype=torch.int32, device="cuda")
        chits = torch.empty((n, 4), dtype=torch.int32, device="cuda")
        times, _, _, _ = time_queries(h, rays, hits, chits, 5, 3, "learned_cut")
        vis, depth, segs = accuracy(hits, chits)
        row = {"train_steps": steps, "train_ms_per_step": st.ms_per_step, "train_seconds": train_s,
               "last_loss": st.last_loss, "cut_nodes": int(len(nn)), "heldout_rays": n,
               "visibility_agreement": vis, "depth_error": depth, "segments_per_ray": segs,
               "query_ms": float(times.mean()), "query_mrays": n / (float(times.mean()) * 1e-3) / 1e6}
        if name == "learned":
            info = h.tree_cut_info()
            row.update({"schedule": sched, "expected_nodes": int(info.expected_nodes),
                        "total_splits": int(info.total_splits), "max_depth": int(info.max_depth)})
        out[name] = row
        h.close()
    return out


def run_train_roofline(nb, scenes, peaks, steps=50, warmup=5):
    """Config 3's training step (2^18 rays per step on the 65,536-triangle sphere, FP16): device time
    of each phase of a step (kernel profile of the last step of each call), the tensor-core
    training kernel against the sustained dense peak, Adam against the copy bandwidth."""
    cfg = nb.default_config()
    h, v, f, alb = build_scene(nb, scenes, cfg)
    try:
        h.run_optimisation(warmup)
        h.set_kernel_profile(True)
        st = h.run_optimisation(steps)
        p = h.kernel_profile()
        h.set_kernel_profile(False)
        rows = int(p.train_rows)
        L = h.layout
        flop = 3.0 * FLOP_PER_SEGMENT * rows  # forward, data gradients, weight gradients
        tc_tflops = flop / (p.train_mlp_ms * 1e-3) / 1e12
        sustained = float(peaks.get("bf16_tflops_sustained", 1700.0))
        # Adam per parameter: FP32 master, m, v and gradient read; master, m, v and the 16-bit copy written
        adam_bytes = 30.0 * L.n_params
        adam_gbs = adam_bytes / (p.train_adam_ms * 1e-3) / 1e9
        hbm = float(peaks.get("hbm_gbs", 6800.0))
        gathers = rows * cfg.module.input_segment_points * cfg.hashgrid.n_levels * 8
        return {"rows_per_step": rows, "ms_per_step": st.ms_per_step, "steps": steps,
                "phases_ms": {"sample": p.train_sample_ms, "encode": p.train_encode_ms, "mlp_tc": p.train_mlp_ms,
                              "grid_scatter": p.train_scatter_ms, "adam": p.train_adam_ms},
                "mlp_tc": {"kernel": "k_train_tc", "bound": "tensor", "achieved": tc_tflops, "peak": sustained,
                           "unit": "TFLOP/s", "frac": tc_tflops / sustained,
                           "algorithmic": "3 x 43,008 FLOP per row (forward, data and weight gradients)"},
                "adam": {"kernel": "k_adam", "bound": "hbm", "achieved": adam_gbs, "peak": hbm, "unit": "GB/s",
                         "frac": adam_gbs / hbm, "algorithmic": "30 B per parameter x %d parameters" % L.n_params},
                "grid_scatter": {"atomics_per_s": gathers / (p.train_scatter_ms * 1e-3),
                                 "algorithmic": "one 8-byte vector atomic per (row, point, level, corner)"}}
    finally:
        h.close()


def run_mesh_4m(args, nb, scenes, cfg, max_over_ranks, rank):
    """The same query on the 4,194,304-triangle fBm sphere: the neural cost depends on the cut
    (1,024 leaves), not on the triangle count, while the classic traversal deepens."""
    import torch
    t0 = time.perf_counter()
    h, v, f, _ = build_scene(nb, scenes, cfg, subdiv=10)
    build_s = time.perf_counter() - t0
    nn, bbox = h.neural_bvh()
    t0 = time.perf_counter()
    st = h.run_optimisation(args.mesh4m_train_steps) if args.mesh4m_train_steps > 0 else None
    train_s = time.perf_counter() - t0
    rays_np = scenes.uniform_rays(N_RAYS, bbox[:3], bbox[3:], seed=4048 + rank)
    rays = torch.from_numpy(rays_np).cuda()
    hits = torch.empty((N_RAYS, 12), dtype=torch.int32, device="cuda")
    chits = torch.empty((N_RAYS, 4), dtype=torch.int32, device="cuda")
    times, ctimes, _, _ = time_queries(h, rays, hits, chits, args.steps, args.warmup, "timed_4m")
    ms, cms = max_over_ranks([float(times.mean()), float(ctimes.mean())])
    vis_agree, depth_stats, segs_per_ray = accuracy(hits, chits)
    out = {"triangles": int(len(f)), "classic_nodes": int(len(h.classic_bvh()[0])), "rays_per_step": N_RAYS,
           "neural_mrays": N_RAYS / (ms * 1e-3) / 1e6, "neural_ms_per_step": ms,
           "classic_mrays": N_RAYS / (cms * 1e-3) / 1e6, "classic_ms_per_step": cms,
           "neural_over_classic": cms / ms, "p50_ms": float(np.percentile(times, 50)),
           "p99_ms": float(np.percentile(times, 99)), "visibility_agreement": vis_agree,
           "depth_error": depth_stats, "segments_per_ray": segs_per_ray,
           "train": {"steps": args.mesh4m_train_steps, "seconds": train_s,
                     "last_loss": (st.last_loss if st else None)},
           "build_seconds": build_s}
    h.close()
    return out


def main():
    global N_RAYS
    args = parse()
    N_RAYS = 1 << args.log2_rays
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
