"""Orthogonal grids: the operator kernels drop the cross-derivative terms.

On a grid without distortion the cross-derivative coefficients and the 12 edge
weights of every row are exactly zero; the set-up detects that per level and
the FP32 and FP64 operator kernels then read the seven face points only.  Bars:
the flags are 0 on such grids and set on a distorted one; the FP64 apply stays
within 1e-12 relative of the reference operator's CSR and the FP32 apply within
the FP32 bar; the converged pressure, mean removed, is within 1e-8 relative L2
of a direct FP64 solve in both precisions.
"""
import types

import numpy as np
import pytest

from cases import seeded
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DT, ST = 1e-3, 1.0

# name -> (cells, lengths, y-stretch, periodic, spheres, levels)
ORTHO = {
    "channel_sphere": ((16, 8, 8), (2.0, 1.0, 1.0), 2.5, (True, False, True), [(0.4, 0.5, 0.5, 0.25)], 2),
    "box_sphere": ((12, 12, 12), (1.0, 1.0, 1.0), 2.0, (False, False, False), [(0.5, 0.45, 0.55, 0.3)], 3),
    # odd mx with a periodic x seam: the colours meet across the seam, so the
    # in-place one-kernel zebra form is not allowed on the finest level
    "odd_periodic": ((15, 8, 8), (1.5, 1.0, 1.0), 2.0, (True, False, False), [(0.5, 0.5, 0.5, 0.2)], 2),
}


def _problem(name):
    from curvib_old_gb300 import workload as W
    cells, lengths, beta, per, spheres, nl = ORTHO[name]
    return W.make_problem(cells, lengths, beta, False, per, spheres, nlevels=nl)


def _levels(P):
    nl = len(P.metrics)
    Ls = [None] * nl
    Ls[-1] = O.OLevel(P.metrics[-1], P.nvert, P.bctype, P.semi)
    for l in range(nl - 2, -1, -1):
        nvc = O.nvert_restrict(Ls[l + 1], P.metrics[l]["Aj"].shape, l == 0, P.semi)
        Ls[l] = O.OLevel(P.metrics[l], nvc, P.bctype, P.semi)
    return Ls


@pytest.fixture(scope="module")
def ctxs():
    from curvib_old_gb300.solver import PoissonContext
    out = {}
    for name in ORTHO:
        P = _problem(name)
        out[name] = (PoissonContext().setup(P), P, _levels(P))
    yield out
    for c, _, _ in out.values():
        c.close()


@pytest.mark.parametrize("name", sorted(ORTHO))
def test_flags_and_apply(ctxs, name):
    ctx, P, Ls = ctxs[name]
    for l in range(ctx.nlevels):
        assert ctx.level_cross(l) == (0, 0), l
        A = O.lhs_csr(Ls[l])
        x = seeded(ctx.shapes[l], 30 + l)
        y_ref = (A @ x.ravel()).reshape(x.shape)
        y = ctx.apply(l, x)
        assert np.abs(y - y_ref).max() <= 1e-12 * np.abs(y_ref).max()
        y32 = ctx.apply_f32(l, x.astype(np.float32)).astype(np.float64)
        y_ref32 = (A @ x.astype(np.float32).astype(np.float64).ravel()).reshape(x.shape)
        assert np.abs(y32 - y_ref32).max() <= 2e-6 * np.abs(A).max() * np.abs(x).max() * 4


def test_odd_periodic_level_is_not_fused_in_place(ctxs):
    ctx, P, Ls = ctxs["odd_periodic"]
    assert ctx.shapes[-1][2] % 2 == 1  # mx odd
    fine = ctx.tuning()["line_sweep"][-1]
    assert fine["level"] == ctx.nlevels - 1
    # whichever form the autotuner kept, the solve below must match the direct solve


def test_distorted_grid_keeps_cross_terms():
    from curvib_old_gb300 import workload as W
    from curvib_old_gb300.solver import PoissonContext
    P = W.make_problem((12, 12, 12), (1.0, 1.0, 1.0), 2.0, True, (False, False, False), [], nlevels=2)
    ctx = PoissonContext().setup(P)
    try:
        assert ctx.level_cross(ctx.nlevels - 1) == (1, 1)
    finally:
        ctx.close()


@pytest.mark.parametrize("name", sorted(ORTHO))
@pytest.mark.parametrize("precision", [0, 1])
def test_solve_matches_direct(ctxs, name, precision):
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    from curvib_old_gb300 import workload as W
    ctx, P, Ls = ctxs[name]
    L = Ls[-1]
    uc, _, _ = O.volume_flux_rev(L, P.ucont, 0.0, 1)
    b, _ = O.poisson_rhs(L, uc, DT, ST)
    b = W.noisy_rhs(b, L.nvert, P.metrics[-1]["Aj"], DT, seed=12)
    A = O.lhs_csr(L).tocsr()
    fl = np.zeros(b.shape, dtype=bool)
    fl[1:-1, 1:-1, 1:-1] = L.nvert[1:-1, 1:-1, 1:-1] < 0.1
    idx = np.flatnonzero(fl.ravel())
    Af = A[idx][:, idx]
    one = sp.csr_matrix(np.ones((1, idx.size)))
    sol = sla.spsolve(sp.bmat([[Af, one.T], [one, None]]).tocsc(), np.concatenate([b.ravel()[idx], [0.0]]))
    x_ref = np.zeros(b.size)
    x_ref[idx] = sol[:-1]
    x_ref = x_ref.reshape(b.shape)
    phi, st = ctx.solve(b, precision=precision, rtol=1e-10, max_it=100)
    assert st["status"] == 0 and st["rel_residual"] <= 1e-10
    r = b.ravel() - A @ phi.ravel()
    assert np.linalg.norm(r) <= 1.5e-10 * np.linalg.norm(b)
    d = phi[fl] - phi[fl].mean() - (x_ref[fl] - x_ref[fl].mean())
    assert np.linalg.norm(d) <= 1e-8 * np.linalg.norm(x_ref[fl] - x_ref[fl].mean())
