"""The network's layer table is stated three times: the library's (csrc/sf_unet.cu, the UNet constructor), the
oracle's (oracle/unet_ref.py) and the trainer's weight initialisation (train.py).  They agree layer for layer
(input channels, output channels, level, taps), so the parameter vector means the same in all three (CPU only)."""
import importlib
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _library_table():
    src = open(os.path.join(ROOT, "simferrofluid-cuda_gb300", "csrc", "sf_unet.cu")).read()
    body = src[src.index("const S spec[] = {"):]
    body = body[:body.index("};")]
    return [tuple(int(v) for v in m) for m in re.findall(r"\{(\d+),\s*(\d+),\s*(\d+),\s*(\d+)\}", body)]


def test_layer_tables_agree():
    from oracle import unet_ref as ref
    train = importlib.import_module("simferrofluid-cuda_gb300.train")
    lib = _library_table()
    orc = [(ci, co, lv, k ** 3) for _, ci, co, lv, k in ref.layer_specs(16)]
    assert lib == orc
    assert [(ci, co, taps) for ci, co, _, taps in lib] == [tuple(t) for t in train._layer_table()]
    # parameter count: weights then biases per layer, as the library lays them out
    n = sum(taps * co * ci + co for ci, co, _, taps in lib)
    assert n == ref.flatten(ref.init_params(16, seed=0)).size
