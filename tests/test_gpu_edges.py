"""Edge cases of the neural query on the GPU: empty, ragged and single-ray batches, and rays at
the edges of the input domain, through device buffers and pageable and page-locked host buffers
(the no-alloc entry point has its own tests).

* A batch of 0 rays returns NBVH_OK and an empty result, on every route.
* A ray's record does not depend on the other rays of its batch: every ragged sub-batch (1, 2, 31,
  32, 33, 127, 1,000 and 4,097 rays at odd offsets) gives the same record words as the ray got in
  the whole batch, and a batch large enough for the leaf sort gives the words of the same rays
  queried in batches below the sort's threshold.
* Rays at the domain's edges (an empty interval tmin > tmax, a zero-length interval, rays far
  outside pointing away, axis-aligned rays from the scene centre, rays with a huge tmax, rays whose
  direction is not of unit length, rays starting on the scene box's corner) answer like the
  oracle's restatement, within the full-query tolerance of test_gpu_neural.py.
"""

import numpy as np
import pytest
import torch

import nbvh_gb300 as nb
from helpers import as_u32, handle
from nbvh_gb300 import scenes
from test_gpu_neural import _borderline, _compare_queries, _cuda, _spread_params

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(built):
    h, s = handle(kind="sphere65k", seed=5, albedo=True)
    s["params"] = _spread_params(h, seed=3)
    yield h, s
    h.close()


def _edge_rays(bbox, rng):
    lo, hi = np.asarray(bbox[:3], np.float32), np.asarray(bbox[3:], np.float32)
    c, ext = 0.5 * (lo + hi), hi - lo
    out = []

    def ray(o, d, tmin=0.0, tmax=3.4e38):
        out.append(np.concatenate([np.asarray(o, np.float32), [tmin], np.asarray(d, np.float32), [tmax]]))

    for k in range(8):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        ray(c + 0.1 * k * ext / 8, d, tmin=1.0, tmax=0.5)        # empty interval
        ray(c, d, tmin=0.25, tmax=0.25)                          # zero-length interval
        ray(c + 10.0 * ext * np.sign(d), np.sign(d) * np.abs(d))  # far outside, pointing away
        ray(c, 3.0 * d)                                          # not unit length
        ray(c, 0.01 * d)
        ray(lo if k % 2 == 0 else hi, -d if k % 2 else d)        # from a corner of the box
    for axis in range(3):
        for sgn in (-1.0, 1.0):
            d = np.zeros(3, np.float32)
            d[axis] = sgn
            ray(c, d)                                            # axis-aligned from the centre
            ray(c + 0.3 * ext, d, tmin=1e-4)
    return np.stack(out).astype(np.float32)


def test_empty_batches(scene):
    h, _ = scene
    empty = torch.empty((0, 8), dtype=torch.float32, device="cuda")
    assert h.query_closest_neural(empty).shape[0] == 0
    assert h.query_visibility_neural(empty).shape[0] == 0
    assert h.query_closest_classic(empty).shape[0] == 0
    segs, counts = h.query_segments(empty, 4)
    assert segs.shape[0] == 0 and counts.shape[0] == 0
    h.query_closest_neural(empty)
    st = h.query_stats()  # the statistics cover exactly this (empty) call
    assert st.segments == 0 and st.step_capped == 0
    assert h.network_inference(torch.empty((0, 3), dtype=torch.float32, device="cuda")).shape[0] == 0
    assert len(h.query_closest_neural_host(np.empty((0, 8), np.float32))) == 0
    assert len(h.query_closest_neural_host(nb.pinned_copy(np.empty((0, 8), np.float32)))) == 0


def test_ragged_batches_match_the_whole_batch(scene):
    h, s = scene
    rays = scenes.uniform_rays(6000, s["bbox"][:3], s["bbox"][3:], seed=77)
    whole = as_u32(h.query_closest_neural(_cuda(rays)))
    vis_whole = as_u32(h.query_visibility_neural(_cuda(rays)))
    offsets = [0, 5, 999, 1234, 1900]
    for k, n in enumerate([1, 2, 31, 32, 33, 127, 1000, 4097]):
        o = offsets[k % len(offsets)]
        part = as_u32(h.query_closest_neural(_cuda(rays[o:o + n])))
        assert np.array_equal(part, whole[o:o + n]), n
        vis = as_u32(h.query_visibility_neural(_cuda(rays[o:o + n])))
        assert np.array_equal(vis, vis_whole[o:o + n]), n
    # host buffers, pageable and page-locked, ragged
    for n, o in ((37, 11), (4097, 1500)):
        got = h.query_closest_neural_host(rays[o:o + n]).view(np.uint32).reshape(n, 12)
        assert np.array_equal(got, whole[o:o + n])
        pin = h.query_closest_neural_host(nb.pinned_copy(rays[o:o + n])).view(np.uint32).reshape(n, 12)
        assert np.array_equal(pin, whole[o:o + n])


def test_edge_rays_match_oracle(scene, oracle):
    h, s = scene
    rng = np.random.default_rng(9)
    edge = _edge_rays(s["bbox"], rng)
    rays = np.concatenate([scenes.uniform_rays(4096, s["bbox"][:3], s["bbox"][3:], seed=78), edge])
    got = as_u32(h.query_closest_neural(_cuda(rays)))
    net = oracle.network(h.cfg, h.layout, s["params"])
    consts = oracle.neural_consts(h.cfg)
    nscene = oracle.neural_scene(s["neural"], s["bbox"])
    ref = oracle.neural_query(nscene, net, consts, rays, threads=8)
    border = _borderline(h, oracle, s, rays)
    _compare_queries(got, ref, border)
    e = slice(4096, None)
    # every edge ray: the same hit decision as the oracle unless it was borderline there
    assert np.all(((got[e, 8] & 1) == (ref[e, 8] & 1)) | border[e])
    # rays pointing away from far outside the scene never hit
    away = np.zeros(len(edge), bool)
    away[2:48:6] = True
    assert np.all((got[e, 8][away] & 1) == 0)
    st = h.query_stats()
    assert st.step_capped == 0 and st.stack_overflow == 0


def test_sorted_and_unsorted_batches_agree(scene):
    """A batch large enough for the leaf sort (2^17 rays: rows grouped by leaf and by the octant of
    their segment midpoint before the encoder) and the same rays in batches below the sort's
    threshold (walked in list order) give the same record words."""
    h, s = scene
    rays = scenes.uniform_rays(1 << 17, s["bbox"][:3], s["bbox"][3:], seed=79)
    whole = as_u32(h.query_closest_neural(_cuda(rays)))
    parts = [as_u32(h.query_closest_neural(_cuda(rays[k:k + (1 << 15)]))) for k in range(0, 1 << 17, 1 << 15)]
    assert np.array_equal(whole, np.concatenate(parts))
