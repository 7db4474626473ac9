"""The reference's .nbvh neural-cut file (NeuralBVHRenderer::save_neural_bvh / load_neural_bvh,
src/cuda/neural/neural_bvh_renderer_accel.cpp:170-254).

Pinned against the cut file the reference ships (tests/golden/make_nbvh_golden.py decodes it with
numpy alone): the reader gives the same nodes, the writer gives the same bytes, and malformed files
are refused with NBVH_EIO. The GPU case checks that an exported-then-imported cut answers neural
queries bit-identically.
"""

import hashlib
import json
import os
import struct

import numpy as np
import pytest

import nbvh_gb300 as nb
from helpers import reference_root
from nbvh_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOP5 = os.path.join(GOLDEN, "nbvh_chess_top5.nbvh")
REFERENCE_FILE = os.path.join(reference_root(), "scene_data/scenes_path_tracing/chess/nbvhs/"
                              "nodes_32940_hash_18_lvl_8_tsteps_10000.nbvh")


def _decode(raw):
    """Independent numpy decode of a .nbvh file into the library's 8-word node layout."""
    n = struct.unpack_from("<Q", raw, 0)[0]
    rec = np.frombuffer(raw[16:16 + 40 * n], [("box", "<f4", 6), ("first", "<u8"), ("count", "<u8")])
    box = rec["box"].reshape(-1, 3, 2)
    out = np.zeros((n, 8), np.uint32)
    out[:, 0:3] = box[:, :, 0].view(np.uint32)
    out[:, 4:7] = box[:, :, 1].view(np.uint32)
    out[:, 3] = rec["count"]
    out[:, 7] = rec["first"]
    return out


def test_reads_golden_cut(built):
    raw = open(TOP5, "rb").read()
    got = nb.read_nbvh(TOP5)
    assert got.shape == (63, 8)
    assert np.array_equal(got, _decode(raw))
    leaves = got[:, 3] > 0
    assert np.all(got[leaves, 7] == 0xFFFFFFFF) and leaves.sum() == 32


def test_write_is_byte_identical(built, tmp_path):
    raw = open(TOP5, "rb").read()
    out = tmp_path / "copy.nbvh"
    nb.write_nbvh(out, nb.read_nbvh(TOP5))
    assert out.read_bytes() == raw


def test_layout_of_written_cut(built, tmp_path):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    f = np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]], np.uint32)
    nodes, _ = nb.build_bvh2_host(v, f)
    cut = nb.build_neural_cut_host(nodes, 1)
    out = tmp_path / "cut.nbvh"
    nb.write_nbvh(out, cut)
    raw = out.read_bytes()
    n = len(cut)
    assert len(raw) == 16 + 40 * n + 8
    assert struct.unpack_from("<QQ", raw, 0) == (n, 1)
    assert struct.unpack_from("<Q", raw, len(raw) - 8)[0] == 0
    mn, mx = nb.nodes_to_float(cut)
    for i in range(n):
        fields = struct.unpack_from("<6fQQ", raw, 16 + 40 * i)
        assert fields[0:6:2] == tuple(mn[i]) and fields[1:6:2] == tuple(mx[i])
        assert fields[6] == cut[i, 7] and fields[7] == cut[i, 3]


@pytest.mark.skipif(not os.path.exists(REFERENCE_FILE), reason="reference checkout not present")
def test_reference_file_matches_summary(built, tmp_path):
    summary = json.load(open(os.path.join(GOLDEN, "nbvh_chess_summary.json")))
    raw = open(REFERENCE_FILE, "rb").read()
    assert hashlib.sha256(raw).hexdigest() == summary["sha256"]
    got = nb.read_nbvh(REFERENCE_FILE)
    assert len(got) == summary["nodes"]
    assert hashlib.sha256(got.tobytes()).hexdigest() == summary["words_sha256"]
    cnt, hist = np.unique(got[:, 3], return_counts=True)
    assert {str(int(c)): int(k) for c, k in zip(cnt, hist)} == summary["prim_count_histogram"]
    out = tmp_path / "chess.nbvh"
    nb.write_nbvh(out, got)
    assert out.read_bytes() == raw


def _corrupt(raw, offset, fmt, value):
    b = bytearray(raw)
    struct.pack_into(fmt, b, offset, value)
    return bytes(b)


def _record(i, field):
    return 16 + 40 * i + {"min_x": 0, "max_x": 4, "first": 24, "count": 32}[field]


@pytest.mark.parametrize("case", ["short", "count", "header", "trailer", "child_range", "leaf_child",
                                  "leaf_count", "box_order", "shared_child", "truncated"])
def test_malformed_files_are_refused(built, tmp_path, case):
    raw = open(TOP5, "rb").read()
    nodes = _decode(raw)
    first_leaf = int(np.where(nodes[:, 3] > 0)[0][0])
    bad = {
        "short": raw[:20],
        "count": _corrupt(raw, 0, "<Q", 64),
        "header": _corrupt(raw, 8, "<Q", 2),
        "trailer": _corrupt(raw, len(raw) - 8, "<Q", 7),
        "child_range": _corrupt(raw, _record(0, "first"), "<Q", 62),
        "leaf_child": _corrupt(raw, _record(first_leaf, "first"), "<Q", 3),
        "leaf_count": _corrupt(raw, _record(first_leaf, "count"), "<Q", 9),
        "box_order": _corrupt(raw, _record(5, "min_x"), "<f", 10.0),
        # node 1's children made equal to node 2's: two parents, unreachable nodes
        "shared_child": _corrupt(raw, _record(1, "first"), "<Q", int(nodes[2, 7])),
        "truncated": raw[:-40],
    }[case]
    path = tmp_path / "bad.nbvh"
    path.write_bytes(bad)
    with pytest.raises(nb.NBVHError) as e:
        nb.read_nbvh(path)
    assert e.value.status == abi.NBVH_EIO


def test_missing_file_and_invalid_nodes(built, tmp_path):
    with pytest.raises(nb.NBVHError) as e:
        nb.read_nbvh(tmp_path / "absent.nbvh")
    assert e.value.status == abi.NBVH_EIO
    nodes = nb.read_nbvh(TOP5)
    nodes[0, 7] = 1000  # child out of range
    with pytest.raises(nb.NBVHError) as e:
        nb.write_nbvh(tmp_path / "x.nbvh", nodes)
    assert e.value.status == abi.NBVH_EINVAL


@pytest.mark.gpu
def test_imported_cut_answers_identically(built, tmp_path):
    import torch

    from helpers import as_u32, handle
    from nbvh_gb300 import scenes

    h, s = handle(depth=8)
    rays = torch.from_numpy(scenes.uniform_rays(1 << 16, s["bbox"][:3], s["bbox"][3:], seed=5)).cuda()
    before = as_u32(h.query_closest_neural(rays))
    path = tmp_path / "cut.nbvh"
    h.export_neural_cut(path)
    assert np.array_equal(nb.read_nbvh(path), s["neural"])

    h.build_neural_cut(3)  # a different cut in between
    h.import_neural_cut(path)
    nn, _ = h.neural_bvh()
    assert np.array_equal(nn, s["neural"])
    assert np.array_equal(as_u32(h.query_closest_neural(rays)), before)

    # a second handle over the same mesh and parameters, cut loaded from the file
    h2, _ = handle(depth=2)
    h2.set_params(h.params())
    h2.import_neural_cut(path)
    assert np.array_equal(as_u32(h2.query_closest_neural(rays)), before)
    h.close()
    h2.close()
