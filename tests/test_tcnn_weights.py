"""tcnn trainer weights as the reference saves and loads them (NeuralBVHRenderer::save_network_model /
load_network_model, src/cuda/neural/neural_bvh_renderer_init.cu:385-404: the JSON text of
trainer->serialize(false), whose binary value nlohmann writes as {"bytes": [...], "subtype": null}).
No tcnn weights ship with the reference, so the reader is checked on files written the way that
serializer writes them, on the CPU:

* FP32 parameters written and read back bit for bit (negative zero, subnormals, infinities);
* an FP16 ("__half") file with other keys around it (an optimizer object, another key order,
  whitespace) widened exactly to FP32;
* a byte count that does not match n_params, a params_type that contradicts it, a missing key and a
  missing file are NBVH_EIO.
"""

import json

import numpy as np
import pytest

import nbvh_gb300 as nb
from nbvh_gb300 import abi


def _tcnn_text(values, type_name, extra_first=False):
    raw = np.ascontiguousarray(values).tobytes()
    body = {"n_params": int(len(values)), "params_type": type_name,
            "params_binary": {"bytes": list(raw), "subtype": None}}
    if extra_first:  # another key order, a nested object before the parameters
        body = {"optimizer": {"otype": "Adam", "state": {"m": [1, 2, [3]], "note": "a } b"}},
                "params_binary": body["params_binary"], "params_type": type_name, "n_params": body["n_params"]}
    return json.dumps(body, indent=1)


def test_fp32_round_trip(built, tmp_path):
    rng = np.random.default_rng(0)
    p = rng.standard_normal(10007).astype(np.float32)
    p[:4] = [np.float32(-0.0), np.float32(1e-42), np.float32(np.inf), np.float32(-np.inf)]
    path = tmp_path / "w.json"
    nb.write_tcnn_params(path, p)
    got = nb.read_tcnn_params(path)
    assert got.dtype == np.float32 and np.array_equal(got.view(np.uint32), p.view(np.uint32))
    text = path.read_text()
    js = json.loads(text)
    assert js["n_params"] == p.size and js["params_type"] == "float"
    assert bytes(js["params_binary"]["bytes"]) == p.tobytes() and js["params_binary"]["subtype"] is None


def test_fp16_file_in_tcnn_text_form(built, tmp_path):
    rng = np.random.default_rng(1)
    h = rng.standard_normal(4099).astype(np.float16)
    h[:5] = [np.float16(-0.0), np.float16(6e-8), np.float16(3e-5), np.float16(65504), np.float16(-np.inf)]
    for extra in (False, True):
        path = tmp_path / ("h%d.json" % extra)
        path.write_text(_tcnn_text(h, "__half", extra_first=extra))
        got = nb.read_tcnn_params(path)
        assert np.array_equal(got.view(np.uint32), h.astype(np.float32).view(np.uint32))
    # a bare byte array is read too
    path = tmp_path / "bare.json"
    path.write_text(json.dumps({"n_params": 3, "params_binary": list(np.float32([1, 2, 3]).tobytes())}))
    assert np.array_equal(nb.read_tcnn_params(path), np.float32([1, 2, 3]))


def test_malformed_files_are_eio(built, tmp_path):
    p = np.arange(8, dtype=np.float32)
    cases = {
        "count": {"n_params": 9, "params_type": "float", "params_binary": {"bytes": list(p.tobytes())}},
        "type": {"n_params": 8, "params_type": "__half", "params_binary": {"bytes": list(p.tobytes())}},
        "missing": {"n_params": 8, "params_type": "float"},
        "notbytes": {"n_params": 8, "params_binary": {"bytes": [1, 2, 300]}},
    }
    for name, body in cases.items():
        path = tmp_path / (name + ".json")
        path.write_text(json.dumps(body))
        with pytest.raises(nb.NBVHError) as e:
            nb.read_tcnn_params(path)
        assert e.value.status == abi.NBVH_EIO, name
    with pytest.raises(nb.NBVHError) as e:
        nb.read_tcnn_params(tmp_path / "absent.json")
    assert e.value.status == abi.NBVH_EIO
