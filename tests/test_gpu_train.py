"""run-optimisation on the GPU against the CPU oracle.

* Training rays (granular_sample_bvh_network_input_data, src/cuda/neural/neural_bvh_module_kernels.cu:
  119-264, with the reference RNG): positions and classic-kernel labels bit-identical.
* Gradients of the composite loss (pt_composite_loss.cuh:18-123) w.r.t. every parameter block
  against the FP64 oracle that rounds the same tensors to FP16: relative L2 error below 2e-2, or
  below 2.5x the oracle's own change when the positions move by one float ulp where that is larger
  (the batch sum cancels, so a few activations rounded across a boundary move it by percents).
* Adam + ExponentialDecay: bit-identical to the restatement.
* Parameters through a tcnn trainer JSON file (the reference's save / load_network_model format):
  export, import into a second handle, same parameters and query records.
* The optimisation loop lowers the loss, and the trained network beats the untrained one against
  the classic judge.
"""

import numpy as np
import pytest
import torch

import nbvh_gb300 as nb
from helpers import as_u32, check_gradients, handle
from nbvh_gb300 import scenes

pytestmark = pytest.mark.gpu


def _cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def scene(built):
    cfg = nb.default_config(batch_size=1 << 14)
    h, s = handle(cfg, kind="sphere65k", seed=1, albedo=True)
    yield h, s
    h.close()


@pytest.mark.parametrize("ratio", [0.0, 1.0])
def test_training_batch_bit_exact(built, oracle, ratio):
    cfg = nb.default_config(batch_size=1 << 14, **{"bvh.leaf_boundary_sampling_ratio": ratio})
    h, s = handle(cfg, kind="sphere65k", seed=1, albedo=True)
    try:
        pos, tgt, nodes = h.generate_training_batch(7, 1 << 14)
        nscene = oracle.neural_scene(s["neural"], s["bbox"])
        cs = oracle.classic_scene(s["nodes"], s["prims"], s["v"], s["f"])
        rpos, rtgt, rnodes = oracle.training_batch(nscene, cs, s["albedo"], oracle.neural_consts(cfg), 7,
                                                   cfg.batch_size, 1 << 14)
        assert np.array_equal(nodes.cpu().numpy().view(np.uint32), rnodes)
        assert np.array_equal(pos.cpu().numpy().view(np.uint32), rpos.view(np.uint32))
        assert np.array_equal(tgt.cpu().numpy().view(np.uint32), rtgt.view(np.uint32))
        vis = rtgt[:, 0]
        assert 0.05 < vis.mean() < 0.95
        hit = vis > 0.5
        assert np.all((rtgt[hit, 1] >= 0) & (rtgt[hit, 1] <= 1))
    finally:
        h.close()


def test_gradients_match_oracle(scene, oracle):
    h, s = scene
    rng = np.random.default_rng(1)
    p = h.params()
    nn = h.layout.n_network_params
    p[:nn] *= 2.0
    p[nn:] = rng.uniform(-0.5, 0.5, p.size - nn).astype(np.float32)
    h.set_params(p)
    pos, tgt, _ = h.generate_training_batch(3, 2048)
    g, loss = h.compute_gradients(pos, tgt)
    g = g.cpu().numpy().astype(np.float64)
    net = oracle.network(h.cfg, h.layout, p)
    rg, rloss = oracle.compute_gradients(net, oracle.loss_consts(h.cfg), pos.cpu().numpy(), tgt.cpu().numpy(),
                                         h.layout.n_params, loss_scale=h.cfg.optimizer.loss_scale)
    assert abs(loss - rloss) <= 1e-3 * abs(rloss) + 1e-6
    check_gradients(oracle, h, p, pos.cpu().numpy(), tgt.cpu().numpy(), g, rg.astype(np.float64), 2e-2)


def test_adam_bit_exact(scene, oracle):
    h, s = scene
    rng = np.random.default_rng(2)
    p0 = h.params()
    h.set_params(p0)  # resets the moments and the step
    m = np.zeros_like(p0)
    v = np.zeros_like(p0)
    p = p0.copy()
    for step in range(3):
        grad = (rng.standard_normal(p0.size) * 1e-3).astype(np.float32)
        h.adam_step(_cuda(grad))
        oracle.adam_step(p, m, v, grad, step, h.cfg)
    torch.cuda.synchronize()
    assert np.array_equal(h.params().view(np.uint32), p.view(np.uint32))


def test_optimisation_lowers_loss_and_beats_untrained(built, oracle):
    cfg = nb.default_config(batch_size=1 << 16, **{"bvh.leaf_boundary_sampling_ratio": 0.0})
    h, s = handle(cfg, kind="sphere65k", seed=1, albedo=True)
    try:
        rays = scenes.uniform_rays(1 << 16, s["bbox"][:3], s["bbox"][3:], seed=41)
        cs = oracle.classic_scene(s["nodes"], s["prims"], s["v"], s["f"])
        ref = oracle.classic_query(cs, rays, threads=8)
        ref_hit = ref[:, 3] != 0xFFFFFFFF

        def agreement():
            got = as_u32(h.query_closest_neural(_cuda(rays)))
            return np.mean(((got[:, 8] & 1) != 0) == ref_hit), got

        before, _ = agreement()
        first = h.run_optimisation(20)
        last = h.run_optimisation(300)
        after, got = agreement()
        assert np.isfinite(last.last_loss)
        assert last.mean_loss < first.mean_loss
        assert after > before + 0.05, (before, after)
        assert h.training_step == 320
    finally:
        h.close()


def test_checkpoint_round_trip(scene, tmp_path):
    h, s = scene
    h.run_optimisation(2)
    path = str(tmp_path / "ck.nbvh")
    h.save(path)
    rays = scenes.uniform_rays(4096, s["bbox"][:3], s["bbox"][3:], seed=42)
    a = as_u32(h.query_closest_neural(_cuda(rays)))
    with nb.NBVH(nb.default_config()) as h2:
        h2.load(path)
        assert h2.training_step == h.training_step
        assert np.array_equal(h2.params(), h.params())
        b = as_u32(h2.query_closest_neural(_cuda(rays)))
    assert np.array_equal(a, b)
    with open(path, "r+b") as f:
        f.write(b"XXXX")
    with nb.NBVH(nb.default_config()) as h3:
        with pytest.raises(nb.NBVHError) as e:
            h3.load(path)
        assert e.value.status == nb.abi.NBVH_EIO


def test_tcnn_weights_round_trip(scene, tmp_path):
    """The handle's parameters exported as a tcnn trainer JSON file and imported into a second
    handle of the same configuration and scene: the same FP32 master parameters and the same query
    records; a file with another parameter count is refused with NBVH_EINVAL."""
    h, s = scene
    path = str(tmp_path / "weights.json")
    h.export_tcnn_weights(path)
    rays = scenes.uniform_rays(4096, s["bbox"][:3], s["bbox"][3:], seed=43)
    a = as_u32(h.query_closest_neural(_cuda(rays)))
    h2, _ = handle(h.cfg, kind="sphere65k", seed=1, albedo=True)
    try:
        h2.import_tcnn_weights(path)
        assert np.array_equal(h2.params().view(np.uint32), h.params().view(np.uint32))
        assert np.array_equal(as_u32(h2.query_closest_neural(_cuda(rays))), a)
        short = str(tmp_path / "short.json")
        nb.write_tcnn_params(short, h.params()[:-8])
        with pytest.raises(nb.NBVHError) as e:
            h2.import_tcnn_weights(short)
        assert e.value.status == nb.abi.NBVH_EINVAL
    finally:
        h2.close()


def test_training_step_profile(scene):
    """With kernel profiling on, the last step of a run-optimisation call reports its phases."""
    h, s = scene
    h.set_kernel_profile(True)
    try:
        h.run_optimisation(2)
        p = h.kernel_profile()
    finally:
        h.set_kernel_profile(False)
    assert p.train_rows == h.cfg.batch_size
    for f in ("train_sample_ms", "train_encode_ms", "train_mlp_ms", "train_scatter_ms", "train_adam_ms"):
        assert getattr(p, f) > 0, f
