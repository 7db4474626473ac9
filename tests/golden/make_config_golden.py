"""Generates tests/golden/chess_config_hash18.json from the configuration file the reference ships
for its chess scene (scene_data/scenes_path_tracing/chess/configs/
nodes_32940_hash_18_lvl_8_tsteps_10000_neural.json, the configuration of the shipped .nbvh cut).

Only the keys the renderer's N-BVH module reads (src/cuda/neural/neural_bvh_renderer_init.cu:690-712:
the neural module's output, module, network, optimiser and encoding options, the batch size, the
BVH constants, the split scheduler and the tree-cut switch) are kept, unchanged, under the same
nesting, so that GPU tests can create a handle from the reference's own configuration on a machine
without the reference tree.

Run: python tests/golden/make_config_golden.py [path-to-reference-checkout]
"""

import json
import os
import sys

REL = "scene_data/scenes_path_tracing/chess/configs/nodes_32940_hash_18_lvl_8_tsteps_10000_neural.json"
HERE = os.path.dirname(os.path.abspath(__file__))
MODULE_KEYS = ("pt_output_constants", "bvh_module_constants", "network", "optimizer", "segment_encoding")
RENDERER_KEYS = ("batch_size", "neural_bvh_min_depth", "bvh_constants", "bvh_split_scheduler", "tree_cut_learning")


def main(root):
    with open(os.path.join(root, REL)) as f:
        js = json.load(f)
    r = js["neural_bvh_renderer"]
    out = {k: r[k] for k in RENDERER_KEYS if k in r}
    out["neural_module"] = {k: r["neural_module"][k] for k in MODULE_KEYS if k in r["neural_module"]}
    with open(os.path.join(HERE, "chess_config_hash18.json"), "w") as f:
        json.dump({"source": REL, "neural_bvh_renderer": out}, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
