"""The zebra sweep in plane slabs gives the whole-level sweep's result.

The set-up autotuner may run a level's zebra sweep (colour 0, then colour 1)
as the one-kernel half-sweep launched slab by slab, colour 1 one plane behind
colour 0, so that colour 1 reads what colour 0's launch left in L2.  Every line
then sees the same neighbour values as in the two whole-level half-sweeps, and
the kernel and its arithmetic are the same, so the results must agree bit for
bit: checked for 1 to 8 slabs against two whole-level one-kernel half-sweeps,
in FP32 and FP64, on a periodic channel (the first and last interior planes
are neighbours in z), a walled box, and the finest level of the 256x128x128
channel, on two sweeps in a row.
"""
import numpy as np
import pytest

from curvib_old_gb300._lib import CVB_BAD_INPUT, CvbError

pytestmark = pytest.mark.gpu


def _problems():
    from curvib_old_gb300 import workload as W
    return {
        "channel18x10x14": W.make_problem((16, 8, 12), (2.0, 1.0, 1.0), 2.5, False, (True, False, True), [],
                                          nlevels=2),
        "box20x16x18": W.make_problem((18, 14, 16), (1.0, 1.0, 1.0), 2.0, False, (False, False, False),
                                      [(0.5, 0.5, 0.5, 0.25)], nlevels=2),
        "channel258x130x130": W.config1_problem(),
    }


@pytest.fixture(scope="module")
def ctxs():
    from curvib_old_gb300.solver import PoissonContext
    out = {name: PoissonContext().setup(P) for name, P in _problems().items()}
    yield out
    for c in out.values():
        c.close()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("name", ["channel18x10x14", "box20x16x18", "channel258x130x130"])
def test_slab_sweep_matches_whole_level_sweep(ctxs, name, precision):
    ctx = ctxs[name]
    dt = np.float32 if precision == "mixed" else np.float64
    l = ctx.nlevels - 1
    assert not ctx.level_cross(l)[0]
    rng = np.random.default_rng(29)
    b = rng.standard_normal(ctx.shapes[l]).astype(dt)
    x0 = rng.standard_normal(ctx.shapes[l]).astype(dt)
    ref = x0
    for _ in range(2):
        ref = ctx.zebra_sweep_slabs(l, 1, b, ref, precision)
    if precision == "mixed":
        # slabs = 1 is the two whole-level one-kernel half-sweeps
        y = x0
        for _ in range(2):
            for color in (0, 1):
                y = ctx.zebra_half_f32(l, "fused", color, b, y)
        assert np.array_equal(y, ref)
    assert float(np.abs(ref.astype(np.float64) - x0).max()) > 0
    for slabs in (2, 3, 4, 8):
        try:
            x = x0
            for _ in range(2):
                x = ctx.zebra_sweep_slabs(l, slabs, b, x, precision)
        except CvbError as e:  # too few planes for that many slabs is still a valid call
            pytest.fail(f"{name} slabs={slabs}: {e}")
        assert np.array_equal(x, ref), (name, precision, slabs, float(np.abs(x - ref).max()))


def test_slab_sweep_refuses_levels_with_cross_terms(ctxs):
    from curvib_old_gb300 import workload as W
    from curvib_old_gb300.solver import PoissonContext
    P = W.make_problem((12, 10, 12), (1.0, 1.0, 1.0), 2.0, True, (False, False, False), [], nlevels=2)
    ctx = PoissonContext().setup(P)
    try:
        l = ctx.nlevels - 1
        assert ctx.level_cross(l)[0]
        z = np.zeros(ctx.shapes[l], dtype=np.float32)
        with pytest.raises(CvbError) as e:
            ctx.zebra_sweep_slabs(l, 2, z, z)
        assert e.value.status == CVB_BAD_INPUT
    finally:
        ctx.close()
