"""The reference's scene-file property names (construct_list_of_attributes,
scene/beta_model.py:286-296), evaluated by the reference's own method for
6-D and 7-D models, stored as ply_attributes.json next to this script.

Usage:  python tests/golden/make_ply_golden.py /path/to/reference
"""
import json
import os
import sys

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_mcmc_golden as mm  # noqa: E402  (its stubbed loader of BetaModel)


def main():
    BetaModel = mm.load_beta_model()
    out = {}
    for D in (6, 7):
        m = object.__new__(BetaModel)
        m.input_dim = D
        m._beta = torch.zeros(2, D - 2)
        m._scale = torch.zeros(2, D)
        m._l_triangle = torch.zeros(2, D * (D - 1) // 2)
        out["d%d" % D] = m.construct_list_of_attributes()
    with open(os.path.join(HERE, "ply_attributes.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote ply_attributes.json", {k: len(v) for k, v in out.items()})


if __name__ == "__main__":
    main()
