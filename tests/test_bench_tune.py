"""bench.apply_tune hands an FP32 tuning to either form: the pair-reduced P2G (modes 5, 6) and the staged pass 2
(gather 2) exist in the FP32 form only, so an FP64 engine takes the cell-run P2G and the one-corner gathers."""
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
import bench  # noqa: E402
from code_mpm_gb300 import engine  # noqa: E402


class FakeEngine:
    def __init__(self, form):
        self.form = form
        self.opts = {}

    def set_option(self, key, value):
        self.opts[key] = value


TUNE = {"p2g_reduce": 6, "p2g_block": 128, "pass_block": 128, "gather_batch": 2, "pass1_corners": 2,
        "pass1_block": 128}


def test_fp32_engine_takes_the_tuning_as_is():
    e = FakeEngine(engine.FORM_FP32)
    bench.apply_tune(e, TUNE)
    assert e.opts[engine.OPT_P2G_REDUCE] == 6 and e.opts[engine.OPT_GATHER] == 2


def test_fp64_engine_maps_the_fp32_only_modes():
    e = FakeEngine(engine.FORM_FP64)
    bench.apply_tune(e, TUNE)
    assert e.opts[engine.OPT_P2G_REDUCE] == 3 and e.opts[engine.OPT_GATHER] == 0
    assert e.opts[engine.OPT_P2G_BLOCK] == 128 and e.opts[engine.OPT_PASS1_CORNERS] == 2


def test_no_tuning_sets_nothing():
    e = FakeEngine(engine.FORM_FP64)
    bench.apply_tune(e, None)
    assert e.opts == {}
