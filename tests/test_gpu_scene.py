"""Instanced scenes (nbvh_scene_*) on the GPU.

* One instance with the identity transform answers every ray exactly as its model does (every
  word of the record but the instance id).
* A scaled and translated instance answers the world rays like its model answers the same rays in
  object space: hit decisions equal except on a few borderline rays (the object-space rays are
  rounded differently, which moves the FP16 network's outputs slightly), distances scaled by the
  transform within 1e-4 relative and normals within 2e-3 on 99% of the rays.
* Two instances side by side: every ray keeps the closer of the two models' answers and names the
  instance that gave it.
* The path tracer renders a scene of three instances with a finite image.
"""

import numpy as np
import pytest
import torch

import nbvh_gb300 as nb
from helpers import handle
from nbvh_gb300 import scenes

pytestmark = pytest.mark.gpu

FLT_MAX = np.float32(3.4028235e38)


@pytest.fixture(scope="module")
def model(built):
    h, s = handle(kind="sphere4k", seed=4, depth=6)
    h.run_optimisation(300)
    yield h, s
    h.close()


def _words(t):
    return t.cpu().numpy().view(np.uint32).reshape(-1, 12)


def _object_rays(rays, A, b):
    """World rays -> object rays as the scene does (o' = A^-1 (o - b), d' = A^-1 d normalised)."""
    inv = np.linalg.inv(A.astype(np.float64))
    o = (rays[:, 0:3].astype(np.float64) - b) @ inv.T
    d = rays[:, 4:7].astype(np.float64) @ inv.T
    s = np.linalg.norm(d, axis=1)
    out = rays.copy()
    out[:, 0:3] = o.astype(np.float32)
    out[:, 4:7] = (d / s[:, None]).astype(np.float32)
    return out, s


def test_identity_instance_is_the_model(model):
    h, s = model
    sc = nb.Scene()
    assert sc.add_instance(h) == 0
    rays = scenes.uniform_rays(1 << 16, s["bbox"][:3], s["bbox"][3:], seed=8)
    dev = torch.from_numpy(rays).cuda()
    ref = _words(h.query_closest_neural(dev))
    got = _words(sc.query_closest(dev))
    assert np.array_equal(got[:, :11], ref[:, :11])
    hit = (ref[:, 8] & 1) != 0
    assert hit.sum() > 1000
    assert np.all(got[hit, 11] == 0) and np.all(got[~hit, 11] == 0xFFFFFFFF)
    sc.close()


def test_transformed_instance(model):
    h, s = model
    A = np.diag([2.0, 2.0, 2.0]).astype(np.float32)
    b = np.array([3.0, -1.0, 0.5], np.float32)
    sc = nb.Scene()
    sc.add_instance(h, np.hstack([A, b[:, None]]))
    lo, hi = s["bbox"][:3] * 2 + b, s["bbox"][3:] * 2 + b
    world = scenes.uniform_rays(1 << 16, lo, hi, seed=9)
    obj, scale = _object_rays(world, A, b)
    ref = _words(h.query_closest_neural(torch.from_numpy(obj).cuda()))
    got = _words(sc.query_closest(torch.from_numpy(world).cuda()))
    hr, hg = (ref[:, 8] & 1) != 0, (got[:, 8] & 1) != 0
    assert hr.sum() > 1000
    assert np.mean(hr != hg) < 5e-3
    both = hr & hg
    tr = ref[both, 0].view(np.float32) / scale[both]
    tg = got[both, 0].view(np.float32)
    assert np.mean(np.abs(tg - tr) <= 1e-4 * np.abs(tr)) > 0.99
    nr = ref[both, 1:4].view(np.float32)
    ng = got[both, 1:4].view(np.float32)
    assert np.mean(np.all(np.abs(ng - nr) < 2e-3, axis=1)) > 0.99
    sc.close()


def test_two_instances_keep_the_closer_hit(model):
    h, s = model
    ext = s["bbox"][3:] - s["bbox"][:3]
    I = np.eye(3, dtype=np.float32)
    b0 = np.zeros(3, np.float32)
    b1 = np.array([1.5 * ext[0], 0.0, 0.0], np.float32)
    sc = nb.Scene()
    sc.add_instance(h, np.hstack([I, b0[:, None]]))
    sc.add_instance(h, np.hstack([I, b1[:, None]]))
    lo = s["bbox"][:3]
    hi = s["bbox"][3:] + b1
    world = scenes.uniform_rays(1 << 16, lo, hi, seed=10)
    got = _words(sc.query_closest(torch.from_numpy(world).cuda()))
    ref0 = _words(h.query_closest_neural(torch.from_numpy(_object_rays(world, I, b0)[0]).cuda()))
    ref1 = _words(h.query_closest_neural(torch.from_numpy(_object_rays(world, I, b1)[0]).cuda()))
    t0 = np.where((ref0[:, 8] & 1) != 0, ref0[:, 0].view(np.float32), FLT_MAX)
    t1 = np.where((ref1[:, 8] & 1) != 0, ref1[:, 0].view(np.float32), FLT_MAX)
    tg = np.where((got[:, 8] & 1) != 0, got[:, 0].view(np.float32), FLT_MAX)
    want = np.minimum(t0, t1)
    which = np.where(t0 <= t1, 0, 1)
    hits = want < FLT_MAX
    assert hits.sum() > 1000 and (which[hits] == 1).sum() > 100
    agree = np.isclose(tg, want, rtol=1e-5) | (tg == want)
    assert np.mean(agree) > 0.995
    ok = hits & agree & (t0 != t1)
    assert np.mean(got[ok, 11] == which[ok]) > 0.999
    sc.close()


def test_scene_path_render(built, model):
    h, s = model
    h2, s2 = handle(kind="terrain32k", seed=5, depth=6)
    h2.run_optimisation(200)
    sc = nb.Scene()
    sc.add_instance(h)
    sc.add_instance(h, np.hstack([np.eye(3, dtype=np.float32) * 0.5, np.array([[1.2], [0.0], [0.0]], np.float32)]))
    sc.add_instance(h2, np.hstack([np.eye(3, dtype=np.float32), np.array([[-1.2], [0.0], [0.0]], np.float32)]))
    cam = nb.render_request(96, 64, [0.5, 0.6, 3.0], [0.5, 0.4, 0.5], [0, 1, 0], 60.0)
    req = nb.path_request(cam, spp=2, max_bounces=3, seed=7, ground_height=-0.2)
    img, traced = sc.render_path(req)
    img = img.cpu().numpy()
    assert np.all(np.isfinite(img)) and img[:, :3].max() > 0
    assert traced > 96 * 64 * 2
    sc.close()
    h2.close()
