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
