"""Shared scene setup and comparison helpers for the tests."""

import os

import numpy as np

import nbvh_gb300 as nb
from nbvh_gb300 import scenes

_MESHES = {}


def mesh(kind="sphere65k", seed=1):
    key = (kind, seed)
    if key not in _MESHES:
        if kind == "sphere65k":
            _MESHES[key] = scenes.fbm_sphere(7, seed=seed)
        elif kind == "sphere4k":
            _MESHES[key] = scenes.fbm_sphere(5, seed=seed)
        elif kind == "sphere1k":
            _MESHES[key] = scenes.fbm_sphere(4, seed=seed)
        elif kind == "soup64k":
            _MESHES[key] = scenes.soup(65536, seed=seed)
        elif kind == "terrain32k":
            _MESHES[key] = scenes.terrain(128, 128, seed=seed)
        else:
            raise KeyError(kind)
    return _MESHES[key]


def handle(cfg=None, kind="sphere65k", seed=1, depth=None, albedo=False):
    """A built NBVH handle over a synthetic mesh plus host copies of its BVHs."""
    v, f = mesh(kind, seed)
    cfg = cfg if cfg is not None else nb.default_config()
    h = nb.NBVH(cfg)
    alb = scenes.palette_albedo(len(f), seed) if albedo else None
    h.set_mesh(v, f, alb)
    h.build_classic()
    h.build_neural_cut(depth)
    nodes, prims = h.classic_bvh()
    nn, bbox = h.neural_bvh()
    return h, dict(v=v, f=f, albedo=alb, nodes=nodes, prims=prims, neural=nn, bbox=bbox)


def as_u32(t):
    return t.cpu().numpy().view(np.uint32)


def float_view(a):
    return np.ascontiguousarray(a).view(np.float32)


def reference_root():
    """Root of the reference source tree when it is present on this machine (NBVH_REFERENCE
    overrides the default); tests that read its shipped data files skip without it."""
    return os.environ.get("NBVH_REFERENCE", "/root/reference")


def gradient_blocks(h):
    """[start, end) of every network matrix in the parameter vector, then the hash grid."""
    off, blocks = 0, []
    H = h.cfg.network.n_hidden_layers
    for m in range(H + 1):
        rows = 16 if m == H else 64
        cols = h.layout.n_inputs if m == 0 else 64
        blocks.append((off, off + rows * cols))
        off += rows * cols
    blocks.append((h.layout.n_network_params, h.layout.n_params))
    return blocks


def check_gradients(oracle, h, params, pos, tgt, g, rg, base_tol):
    """GPU gradient g against the oracle's rg, block by block. The gradient summed over a batch
    cancels strongly, so its relative error is set by the 16-bit rounding of a few activations that
    lands on the other side of a rounding or ReLU boundary (the GPU sums in another order): the
    oracle's own gradient moves by a few percent when the positions move by one float ulp. Each
    block's bound is the larger of base_tol and 2.5 x the largest such movement over two nudges
    (positions one ulp up, one ulp down), measured here; a wrong backward pass is off by far more."""
    import numpy as np
    net = oracle.network(h.cfg, h.layout, params)
    moved = []
    for toward in (np.float32(2), np.float32(-1)):
        pos_n = np.nextafter(pos, toward).astype(np.float32)
        rg_n, _ = oracle.compute_gradients(net, oracle.loss_consts(h.cfg), pos_n, tgt, h.layout.n_params,
                                           loss_scale=h.cfg.optimizer.loss_scale)
        moved.append(rg_n.astype(np.float64))
    for a, b in gradient_blocks(h):
        den = max(np.linalg.norm(rg[a:b]), 1e-30)
        noise = max(np.linalg.norm(m[a:b] - rg[a:b]) / den for m in moved)
        err = np.linalg.norm(g[a:b] - rg[a:b]) / den
        assert err < max(base_tol, 2.5 * noise), (a, b, err, noise)
