"""Generates tests/golden/golden.npz: golden vectors of the N-BVH ray-query path computed by the
independent pure-Python restatement in pyref.py (not by the C oracle), on small seeded inputs.

    python tests/golden/make_golden.py

The BVH topologies fed to both restatements come from the library's host builder (its output is an
input here; the traversal results are what the vectors pin).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import pyref  # noqa: E402
import nbvh_gb300 as nb  # noqa: E402
from nbvh_gb300 import scenes  # noqa: E402

F = np.float32


def main():
    out = {}
    # RNG streams: get_lcg_rng(index, frame, linear) then 6 draws
    seeds = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [7 * 262144, 0, 12345], [3, 2, 99999],
                      [0xFFFFFFFF, 5, 77]], np.uint64)
    streams = []
    for s in seeds:
        r = pyref.Rng(pyref.lcg_seed(int(s[0]) & 0xFFFFFFFF, int(s[1]), int(s[2])))
        streams.append([r.f() for _ in range(6)])
    out["rng_seeds"] = seeds.astype(np.uint32)
    out["rng_streams"] = np.array(streams, np.float32)
    # sin/cos of 2 pi u
    us = np.concatenate([np.linspace(0, 1, 97, dtype=np.float32), np.array([1e-7, 0.124999, 0.875001], F)])
    out["sincos_u"] = us
    out["sincos"] = np.array([pyref.sincos_turns(u) for u in us], np.float32)

    # classic traversal on a 1,024-triangle sphere
    v, f = scenes.fbm_sphere(4, seed=9)
    nodes, prims = nb.build_bvh2_host(v, f)
    mn, mx = nb.nodes_to_float(nodes[:1])
    rays = scenes.uniform_rays(200, mn[0], mx[0], seed=9)
    rays[:5, 3] = np.array([-0.5, 0.0, 1e-4, 0.3, 0.6], F)
    rays[5:10, 7] = np.array([0.1, 0.2, 0.5, 1.0, 2.0], F)
    hits = np.zeros((len(rays), 4), np.uint32)
    any_hits = np.zeros((len(rays), 4), np.uint32)
    for i, r in enumerate(rays):
        for arr, flag in ((hits, False), (any_hits, True)):
            t, u, vv, p = pyref.classic_intersect(nodes, prims, v, f, r, flag)
            arr[i] = [F(t).view(np.uint32), F(u).view(np.uint32), F(vv).view(np.uint32), p]
    out.update(mesh_v=v, mesh_f=f, bvh_nodes=nodes, bvh_prims=prims, classic_rays=rays, classic_hits=hits,
               any_hits=any_hits)

    # neural segments with the cut at depth 4 (inference epsilons and dilation)
    neural = nb.build_neural_cut_host(nodes, 4)
    nrays = rays[:120].copy()
    nrays[:, 3] = F(1e-4)
    segs = np.zeros((len(nrays), 32, 4), np.uint32)
    counts = np.zeros(len(nrays), np.uint32)
    for i, r in enumerate(nrays):
        ss = pyref.neural_segments(neural, r, F(1e-5), F(1e-4), F(1e-3))
        counts[i] = len(ss)
        for k, (a, b, nd) in enumerate(ss[:32]):
            segs[i, k] = [F(a).view(np.uint32), F(b).view(np.uint32), nd, 0]
    out.update(neural_nodes=neural, neural_rays=nrays, neural_segments=segs, neural_counts=counts)

    # hash-grid levels: 4 levels, 2^8 entries, base 4, scale 2 (two dense, two hashed)
    offs, sizes, res, scl = [], [], [], []
    o, p = 0, 1.0
    for level in range(4):
        s = F(4.0 * p - 1.0)
        rr = int(np.ceil(s)) + 1
        dense = rr ** 3
        sz = min((dense + 7) // 8 * 8, 256)
        offs.append(o)
        sizes.append(sz)
        res.append(rr)
        scl.append(s)
        o += sz
        p *= 2.0
    rng = np.random.default_rng(5)
    grid = rng.uniform(-1, 1, (o, 2)).astype(np.float16).astype(np.float32)
    pts = rng.uniform(-0.01, 1.01, (60, 3)).astype(np.float32)
    feats = np.array([[pyref.encode_level(grid, offs[lv], sizes[lv], res[lv], scl[lv], q) for lv in range(4)]
                      for q in pts], np.float32).reshape(60, 8)
    out.update(grid_offsets=np.array(offs, np.uint32), grid_sizes=np.array(sizes, np.uint32),
               grid_res=np.array(res, np.uint32), grid_scale=np.array(scl, np.float32), grid_values=grid,
               grid_points=pts, grid_features=feats)

    # LocalT depth decode
    cases = rng.uniform(0, 1, (50, 3)).astype(np.float32)
    dec = []
    for k, (u, a, b) in enumerate(cases):
        mint = F(a - 0.5) if k % 2 else F(a)
        maxt = F(mint + F(b * 0.5) + F(0.01))
        dec.append([u, mint, maxt, pyref.decode_local_t(u, mint, maxt, mint < 0)])
    out["decode"] = np.array(dec, np.float32)

    # losses: (kind, target, prediction) -> (loss, gradient)
    kinds = ["L1", "L2", "RelativeL2", "BinaryCrossEntropy"]
    lrows = []
    for ki, kind in enumerate(kinds):
        for t, pr in rng.uniform(0, 1, (25, 2)).astype(np.float32):
            l, g = pyref.loss_and_gradient(kind, t, pr)
            lrows.append([ki, t, pr, l, g])
    out["losses"] = np.array(lrows, np.float32)

    # hash-grid levels with 4 and 8 features per entry (the reference's default encoding has 4):
    # the same 4-level geometry, own values and points (a generator of its own, so the vectors
    # above do not move)
    wide = np.random.default_rng(11)
    for nf in (4, 8):
        gridw = wide.uniform(-1, 1, (o, nf)).astype(np.float16).astype(np.float32)
        ptsw = wide.uniform(-0.01, 1.01, (40, 3)).astype(np.float32)
        featw = np.array([[pyref.encode_level(gridw, offs[lv], sizes[lv], res[lv], scl[lv], q) for lv in range(4)]
                          for q in ptsw], np.float32).reshape(40, 4 * nf)
        out["grid_values_f%d" % nf] = gridw
        out["grid_points_f%d" % nf] = ptsw
        out["grid_features_f%d" % nf] = featw
    # the network: 4 levels x 2 features of one point (8 inputs), 2 hidden layers of 64, FP16 weights
    netr = np.random.default_rng(12)
    n_w = 64 * 8 + 64 * 64 + 16 * 64
    wts = (netr.standard_normal(n_w) * 0.3).astype(np.float16)
    pts_n = netr.uniform(0.0, 1.0, (40, 3)).astype(np.float32)
    mlp_out = []
    for q in pts_n:
        x = [v for lv in range(4) for v in pyref.encode_level(grid, offs[lv], sizes[lv], res[lv], scl[lv], q)]
        mlp_out.append(pyref.mlp_forward(wts.astype(np.float32), 8, 2, x))
    out["mlp_weights"] = wts.view(np.uint16)
    out["mlp_points"] = pts_n
    out["mlp_outputs"] = np.array(mlp_out, np.float32)

    # Adam: 3 steps from step 9 with the decay starting at step 10, every step (so the first step
    # has the full rate and the next two halve it), L2 term on
    adr = np.random.default_rng(13)
    p0 = adr.standard_normal(64).astype(np.float32)
    grads = (adr.standard_normal((3, 64)) * 0.1).astype(np.float32)
    pa, ma, va = list(p0), [F(0)] * 64, [F(0)] * 64
    hyper = dict(lr=F(1e-2), beta1=F(0.9), beta2=F(0.999), eps=F(1e-8), l2_reg=F(1e-3), decay_start=10,
                 decay_interval=1, decay_base=F(0.5))
    for k in range(3):
        pyref.adam_step(pa, ma, va, grads[k], 9 + k, **hyper)
    out["adam_params0"] = p0
    out["adam_grads"] = grads
    out["adam_params3"] = np.array(pa, np.float32)
    out["adam_m3"] = np.array(ma, np.float32)
    out["adam_v3"] = np.array(va, np.float32)
    # the neural closest-hit query on the depth-4 cut: 2 points per segment over the 4-level grid
    # (16 inputs), 2 hidden layers, the library's default constants; the scene box is the cut's root
    qr = np.random.default_rng(14)
    wq = (qr.standard_normal(64 * 16 + 64 * 64 + 16 * 64) * 0.3).astype(np.float16)
    rmn, rmx = nb.nodes_to_float(neural[:1])
    consts = dict(node_extent_dilation=1e-4, fixed_node_dilation=1e-5, mint_eps=1e-4, maxt_eps=1e-3, points=2,
                  distribution=0, threshold=0.5, depth_epsilon=0.2, fixed_depth_epsilon=1e-5, max_steps=1000)
    levels = list(zip(offs, sizes, res, scl))
    qhits = np.array([pyref.neural_query(neural, r, rmn[0], rmx[0], grid, levels, wq.astype(np.float32), 2, consts)
                      for r in nrays], np.uint32)
    out["query_weights"] = wq.view(np.uint16)
    out["query_scene_box"] = np.concatenate([rmn[0], rmx[0]]).astype(np.float32)
    out["query_hits"] = qhits
    # training rays on the same cut and mesh (step 3 of batches of 4,096, 4 points per segment,
    # per-triangle albedo), with leaf-boundary sampling off and always on
    alb = np.random.default_rng(15).uniform(0, 1, (len(f), 3)).astype(np.float32)
    tcon = dict(node_extent_dilation=1e-4, fixed_node_dilation=1e-5, learning_mint_eps=1e-3, learning_maxt_eps=1e-3,
                sampling_bbox_scaling=1.5, points=4, distribution=0)
    for name, ratio in (("train0", 0.0), ("train1", 1.0)):
        rows = [pyref.training_sample(i, 3, 4096, neural, rmn[0], rmx[0], nodes, prims, v, f, alb,
                                      dict(tcon, leaf_boundary_sampling_ratio=ratio)) for i in range(96)]
        out[name + "_points"] = np.array([r[0] for r in rows], np.float32)
        out[name + "_targets"] = np.array([r[1] for r in rows], np.float32)
        out[name + "_nodes"] = np.array([r[2] for r in rows], np.uint32)
    out["train_albedo"] = alb

    # a path-traced 8 x 6 frame, 2 samples per pixel, 2 bounces, ground plane and sky, on the
    # query's network and cut
    pp = dict(origin=[0.5, 0.45, -1.2], du=[0.7, 0.0, 0.0], dv=[0.0, -0.55, 0.0], tl=[-0.35, 0.275, 1.0], width=8,
              height=6, spp=2, sample_base=4, sample_offset=1, seed=7, max_bounces=2, has_ground=1, ground_y=0.1,
              ground_albedo=[0.5, 0.4, 0.3], sky_zenith=[0.3, 0.5, 0.9], sky_horizon=[0.9, 0.9, 0.8])
    img, traced = pyref.path_trace(neural, rmn[0], rmx[0], grid, levels, wq.astype(np.float32), 2, consts, pp)
    out["path_params"] = np.array(pp["origin"] + pp["du"] + pp["dv"] + pp["tl"] + [pp["ground_y"]] +
                                  pp["ground_albedo"] + pp["sky_zenith"] + pp["sky_horizon"], np.float32)
    out["path_image"] = img
    out["path_traced"] = np.array([traced], np.uint64)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", os.path.join(HERE, "golden.npz"))


if __name__ == "__main__":
    main()
