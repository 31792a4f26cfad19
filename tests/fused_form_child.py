"""Child process of the fused-form test: runs one 2D TMz scene on the FP32 fused path with the
kernel form chosen by OMX_FUSED_KERNEL and saves the fields and the detector trace.

usage: fused_form_child.py nx ny bx by src steps out.npz
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for _p in (HERE, os.path.join(ROOT, "one-mxll-to-rule-them-all_gb300"), ROOT):
    sys.path.insert(0, _p)

import omx  # noqa: E402
from omx import decks  # noqa: E402
from gpu_harness import tmz_variant_deck  # noqa: E402


def main(argv):
    nx, ny, bx, by = (int(a) for a in argv[:4])
    src, steps, out = argv[4], int(argv[5]), argv[6]
    d = tmz_variant_deck(nx, ny, bx, by, src=src)
    g = omx.TMxll(d["dimensions"], d["grid_Ndims"], d["npml"], d["boundaries"], d["dt"], d["dr"], mode=d["mode"],
                  precision="fp32")
    decks.apply_deck(g, d, omx, decks.media_map(d, omx.media_map_from_voxels))
    for det in d["detectors"]:
        g.add_detector(det["type"], det["field"], det["idx"])
    g.run(1, steps, d["n_skip"], d["t_det_print"], use_graph=True)
    _, trace = g.drain_detectors()
    fields = {f"f{f}": g.read_field(f) for f in (3, 4, 5)}
    np.savez(out, trace=np.asarray(trace), **fields)
    g.kill()


if __name__ == "__main__":
    main(sys.argv[1:])
