"""Generates the .nbvh golden fixtures from the neural-cut file the reference ships
(scene_data/scenes_path_tracing/chess/nbvhs/nodes_32940_hash_18_lvl_8_tsteps_10000.nbvh, written by
NeuralBVHRenderer::save_neural_bvh, src/cuda/neural/neural_bvh_renderer_accel.cpp:170-199).

Decoding here uses numpy alone (not the library's reader), so the fixtures pin the reader and
writer independently:

* nbvh_chess_summary.json -- size, sha256, node count, prim_count histogram, root box and the first
  and last records of the reference file, plus the sha256 of its nodes in the library's 8-word
  layout (f32 min.xyz, u32 prim_count, f32 max.xyz, u32 first_id).
* nbvh_chess_topology.npz -- the reference cut's topology without boxes (prim_count and first_id
  per node): the learned tree cut's split order is checked against it.
* nbvh_chess_top5.nbvh -- the reference cut's top five levels, renumbered breadth-first (children
  adjacent) with depth-5 interior nodes turned into LoD leaves (first_id 0xFFFFFFFF, prim_count
  8), written in the same byte layout. A small, valid cut that travels with the tests.

Run: python tests/golden/make_nbvh_golden.py [path-to-reference-checkout]
"""

import hashlib
import json
import os
import sys

import numpy as np

REL = "scene_data/scenes_path_tracing/chess/nbvhs/nodes_32940_hash_18_lvl_8_tsteps_10000.nbvh"
RECORD = np.dtype([("box", "<f4", 6), ("first", "<u8"), ("count", "<u8")])
HERE = os.path.dirname(os.path.abspath(__file__))


def decode(raw):
    n, one = np.frombuffer(raw[:16], "<u8")
    assert one == 1 and len(raw) == 16 + 40 * int(n) + 8
    assert np.frombuffer(raw[-8:], "<u8")[0] == 0
    return np.frombuffer(raw[16:16 + 40 * int(n)], RECORD)


def encode(rec):
    return (np.array([len(rec), 1], "<u8").tobytes() + np.ascontiguousarray(rec, RECORD).tobytes()
            + np.array([0], "<u8").tobytes())


def to_words(rec):
    """Records in the library's node layout (8 x u32 per node)."""
    box = rec["box"].reshape(-1, 3, 2)  # (min, max) per axis
    out = np.zeros((len(rec), 8), np.uint32)
    out[:, 0:3] = box[:, :, 0].view(np.uint32)
    out[:, 4:7] = box[:, :, 1].view(np.uint32)
    out[:, 3] = rec["count"].astype(np.uint32)
    out[:, 7] = rec["first"].astype(np.uint32)
    return out


def top_levels(rec, depth):
    """Breadth-first copy of the tree down to `depth`: the children of the k-th interior node of
    the copy sit at 1 + 2k and 2 + 2k."""
    order = [(0, 0)]  # (source node, depth), appended breadth-first
    nodes = []
    k = 0
    for src, d in order:
        r = rec[src].copy()
        if r["count"] == 0:
            if d == depth:
                r["first"], r["count"] = 0xFFFFFFFF, 8
            else:
                c = int(rec[src]["first"])
                order.extend([(c, d + 1), (c + 1, d + 1)])
                r["first"] = 1 + 2 * k
                k += 1
        nodes.append(r)
    return np.array(nodes, RECORD)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    raw = open(os.path.join(ref, REL), "rb").read()
    rec = decode(raw)
    words = to_words(rec)
    cnt, hist = np.unique(rec["count"], return_counts=True)
    box = rec["box"][0].reshape(3, 2)
    summary = {
        "source": REL,
        "bytes": len(raw),
        "sha256": hashlib.sha256(raw).hexdigest(),
        "nodes": int(len(rec)),
        "prim_count_histogram": {str(int(c)): int(k) for c, k in zip(cnt, hist)},
        "root_min": [float(x) for x in box[:, 0]],
        "root_max": [float(x) for x in box[:, 1]],
        "first_words": words[:4].tolist(),
        "last_words": words[-4:].tolist(),
        "words_sha256": hashlib.sha256(words.tobytes()).hexdigest(),
    }
    with open(os.path.join(HERE, "nbvh_chess_summary.json"), "w") as f:
        json.dump(summary, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "nbvh_chess_topology.npz"),
                        prim_count=rec["count"].astype(np.uint8), first=rec["first"].astype(np.uint32))
    top = top_levels(rec, 5)
    with open(os.path.join(HERE, "nbvh_chess_top5.nbvh"), "wb") as f:
        f.write(encode(top))
    print("nodes", len(rec), "top5", len(top))


if __name__ == "__main__":
    main()
