"""The forms of the FP32 zebra half-sweep compute the same update.

The mixed V-cycle's smoother relaxes the y-lines of one colour per half-sweep.
The set-up autotuner chooses per level between two kernels (residual, then
line solves), one kernel (residual straight into shared memory), either with 8
or with 4 lines per tile, and one kernel whose tiles are staged by TMA bulk
tensor copies in chunks of 4, 8 or 16 row pairs (cvb_zebra_half_f32 runs a
named form).  On levels without cross-derivative terms all seven must give the
same x: checked here against the
two-kernel form, within 1e-5 of the size of the update (FP32 sums whose
multiply-adds the compiler may contract differently per kernel), on a periodic
channel (mx = 2 mod 4), a walled box (mx = 0 mod 4) and the finest level of
the 256x128x128 channel, for both colours, on two successive half-sweeps.
"""
import numpy as np
import pytest

from curvib_old_gb300._lib import CVB_BAD_INPUT, CvbError

pytestmark = pytest.mark.gpu

FORMS = ["fused", "split4", "fused4", "tma4", "tma8", "tma16"]


def _problems():
    from curvib_old_gb300 import workload as W
    return {
        "channel18x10x10": W.make_problem((16, 8, 8), (2.0, 1.0, 1.0), 2.5, False, (True, False, True), [],
                                          nlevels=2),
        "box20x16x12": W.make_problem((18, 14, 10), (1.0, 1.0, 1.0), 2.0, False, (False, False, False),
                                      [(0.5, 0.5, 0.5, 0.25)], nlevels=2),
        "channel258x130x130": W.config1_problem(),
        # lines of 198 rows (8 per lane): with 4-line tiles the factors sit in registers
        "tall18x200x12": W.make_problem((16, 198, 10), (1.0, 2.0, 1.0), 2.0, False, (False, False, False),
                                        [(0.5, 1.0, 0.5, 0.25)], nlevels=2),
        "tall18x200x12_distorted": W.make_problem((16, 198, 10), (1.0, 2.0, 1.0), 2.0, True, (False, False, False),
                                                  [], nlevels=2),
    }


@pytest.fixture(scope="module")
def ctxs():
    from curvib_old_gb300.solver import PoissonContext
    out = {}
    for name, P in _problems().items():
        out[name] = PoissonContext().setup(P)
    yield out
    for c in out.values():
        c.close()


@pytest.mark.parametrize("name", ["channel18x10x10", "box20x16x12", "channel258x130x130", "tall18x200x12",
                                  "tall18x200x12_distorted"])
def test_zebra_forms_agree(ctxs, name):
    ctx = ctxs[name]
    levels = [ctx.nlevels - 1] if name.startswith("channel258") else range(ctx.nlevels)
    ran = 0
    for l in levels:
        # with cross terms only the two-kernel forms update in place
        forms = ["split4"] if ctx.level_cross(l)[0] else FORMS
        rng = np.random.default_rng(17 + l)
        b = rng.standard_normal(ctx.shapes[l]).astype(np.float32)
        x0 = rng.standard_normal(ctx.shapes[l]).astype(np.float32)
        ref = x0
        for color in (0, 1):
            ref = ctx.zebra_half_f32(l, "split", color, b, ref)
        for form in forms:
            x = x0
            try:
                for color in (0, 1):
                    x = ctx.zebra_half_f32(l, form, color, b, x)
            except CvbError as e:
                assert e.status == CVB_BAD_INPUT
                continue
            scale = float(np.abs(ref.astype(np.float64) - x0).max())
            err = float(np.abs(x.astype(np.float64) - ref).max())
            assert err <= 1e-5 * scale, (name, l, form, err, scale)
            ran += 1
    assert ran > 0
