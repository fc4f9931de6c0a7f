"""TSDF storage precision (the 1024^3 study's method at a reduced size):
FP32, FP16 and int16 storage on the GPU against a full-FP64 oracle run of the
same frames.  Bounds: the TSDF field within 1e-3 (FP32), 2e-3 (FP16) and
1e-3 (int16) of the FP64 field on average, in units of the truncation; the
camera positions within 2 mm of the FP64 oracle's."""
import dataclasses
import importlib
import sys

import pytest

pytestmark = pytest.mark.gpu


def test_storage_precision_against_fp64_oracle(cuda):
    from conftest import ROOT
    sys.path.insert(0, str(ROOT / "tests"))
    ps = importlib.import_module("precision_study")
    syn = importlib.import_module("3deye_gb300.synth")
    base = syn.small_config("c4", frames=12, cols=160, rows=120, voxels=128)
    cfg = dataclasses.replace(base, volume_m=4.0, trunc_m=3 * 4.0 / 128)
    res = ps.study(cfg, 0, log=lambda *_: None)
    bounds = {"fp32": 1e-3, "fp16": 2e-3, "int16": 1e-3}
    for name, b in bounds.items():
        r = res[name]
        assert r["tsdf_voxels_compared"] > 10000, name
        assert r["tsdf_abs_err_mean"] < b, (name, r)
        assert r["pose_err_max_mm"] < 2.0, (name, r)
        assert r["raycast_hit_agreement"] > 0.99, (name, r)
