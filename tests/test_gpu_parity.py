"""GPU path (libcvb.so through its C ABI) against the CPU oracle.

Bars: masks, index maps, assembled rows, transfers, RHS, pressure update and
projection bit-exact; the FP64 operator apply within 1e-12 relative (a
matrix-free sum in another order); the FP32 apply within 2e-6 relative; sums
that the GPU reduces in a tree (compatibility sum, IB flux) within 1e-12 of
their scale; the converged pressure, mean removed, within 1e-8 relative L2 of a
direct FP64 solve.
"""
import types

import numpy as np
import pytest

from cases import SCENARIOS, build, seeded
from oracle import oracle as O
from parity_util import weights_to_csr as _weights_to_csr

pytestmark = pytest.mark.gpu

DT, ST = 1e-3, 1.0


def _problem(name):
    c = build(name)
    return types.SimpleNamespace(metrics=c["metrics"], nvert=c["nvert"], ucont=c["ucont"],
                                 bctype=c["bctype"], semi=c["semi"], per=c["per"], nl=c["nl"])


def _oracle_levels(P):
    Ls = [None] * P.nl
    Ls[-1] = O.OLevel(P.metrics[-1], P.nvert, P.bctype, P.semi)
    for l in range(P.nl - 2, -1, -1):
        nvc = O.nvert_restrict(Ls[l + 1], P.metrics[l]["Aj"].shape, l == 0, P.semi)
        Ls[l] = O.OLevel(P.metrics[l], nvc, P.bctype, P.semi)
    return Ls


@pytest.fixture(scope="module")
def ctxs():
    from curvib_old_gb300.solver import PoissonContext
    out = {}
    for name in SCENARIOS:
        P = _problem(name)
        out[name] = (PoissonContext().setup(P), P, _oracle_levels(P))
    yield out
    for c, _, _ in out.values():
        c.close()


@pytest.mark.parametrize("name", sorted(SCENARIOS))
def test_masks_and_rows_bit_exact(ctxs, name):
    ctx, P, Ls = ctxs[name]
    for l in range(P.nl):
        nv, mns = ctx.get_nvert(l)
        assert np.array_equal(nv, Ls[l].nvert), ("nvert", l)
        A = O.lhs_csr(Ls[l])
        W = ctx.weights(l)
        B = _weights_to_csr(W, ctx.shapes[l], P.bctype)
        d = (A - B)
        d.eliminate_zeros()
        assert d.nnz == 0, ("rows differ", l, abs(d).max())
    assert mns == O.fully_blocked(Ls[0])[0]


@pytest.mark.parametrize("name", sorted(SCENARIOS))
def test_operator_apply(ctxs, name):
    ctx, P, Ls = ctxs[name]
    for l in range(P.nl):
        A = O.lhs_csr(Ls[l])
        x = seeded(ctx.shapes[l], 7 + l)
        y_ref = (A @ x.ravel()).reshape(x.shape)
        y = ctx.apply(l, x)
        scale = np.abs(y_ref).max()
        assert np.abs(y - y_ref).max() <= 1e-12 * scale
        y32 = ctx.apply_f32(l, x.astype(np.float32)).astype(np.float64)
        y_ref32 = (A @ x.astype(np.float32).astype(np.float64).ravel()).reshape(x.shape)
        assert np.abs(y32 - y_ref32).max() <= 2e-6 * np.abs(A).max() * np.abs(x).max() * 4


@pytest.mark.parametrize("name", sorted(SCENARIOS))
def test_transfers_and_nullspace(ctxs, name):
    ctx, P, Ls = ctxs[name]
    for l in range(1, P.nl):
        xf = seeded(ctx.shapes[l], 100 + l)
        assert np.array_equal(ctx.restrict(l - 1, xf), O.restrict(Ls[l], Ls[l - 1], xf))
        xc = seeded(ctx.shapes[l - 1], 200 + l)
        assert np.array_equal(ctx.interpolate(l, xc), O.interpolate(Ls[l - 1], Ls[l], xc))
    for l in range(1, P.nl):  # single-region levels
        x = seeded(ctx.shapes[l], 300 + l)
        y = O.nullspace(Ls[l], x, False)
        assert np.abs(ctx.nullspace(l, x) - y).max() <= 1e-13 * np.abs(x).max()


@pytest.mark.parametrize("name", sorted(SCENARIOS))
def test_rhs_flux_update_projection(ctxs, name):
    ctx, P, Ls = ctxs[name]
    L = Ls[-1]
    uc_g, f_g, a_g = ctx.volume_flux_rev(P.ucont, 0.0, 1)
    uc_o, f_o, a_o = O.volume_flux_rev(L, P.ucont, 0.0, 1)
    assert np.abs(uc_g - uc_o).max() <= 1e-13 * max(np.abs(uc_o).max(), 1e-300)
    assert abs(a_g - a_o) <= 1e-12 * max(a_o, 1.0)
    assert abs(f_g - f_o) <= 1e-12 * max(np.abs(uc_o).max(), 1.0)
    b_g, s_g = ctx.poisson_rhs(uc_o, DT, ST)
    b_o, s_o = O.poisson_rhs(L, uc_o, DT, ST)
    assert np.array_equal(b_g, b_o)
    aj = P.metrics[-1]["Aj"]
    assert abs(s_g - s_o) <= 1e-12 * np.abs(b_o / aj).sum() * DT
    fine = ctx.shapes[-1]
    p, phi = seeded(fine, 400), seeded(fine, 401)
    p_g, phi_g = ctx.update_pressure(p, phi)
    p_o, phi_o, uc2_o = O.update_and_project(L, p, phi, uc_o, DT, ST)
    assert np.array_equal(p_g, p_o) and np.array_equal(phi_g, phi_o)
    uc2_g = ctx.projection(phi_g, DT, ST, uc_o)
    assert np.array_equal(uc2_g, uc2_o)


def _direct_solution(A, b, nvert):
    """FP64 direct solve of the singular system on fluid cells with the fluid mean pinned."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    fl = np.zeros(nvert.shape, dtype=bool)
    fl[1:-1, 1:-1, 1:-1] = nvert[1:-1, 1:-1, 1:-1] < 0.1
    idx = np.flatnonzero(fl.ravel())
    Af = A.tocsr()[idx][:, idx]
    one = sp.csr_matrix(np.ones((1, len(idx))))
    K = sp.bmat([[Af, one.T], [one, None]]).tocsc()
    sol = sla.spsolve(K, np.concatenate([b.ravel()[idx], [0.0]]))
    x = np.zeros(b.size)
    x[idx] = sol[:-1]
    return x.reshape(b.shape), fl


@pytest.mark.parametrize("name", ["box_sphere", "channel_periodic", "ksemi_sphere", "triply_periodic"])
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("smoother", [0, 1])
def test_solve_matches_direct(ctxs, name, precision, smoother):
    from curvib_old_gb300 import workload as W
    ctx, P, Ls = ctxs[name]
    L = Ls[-1]
    uc, _, _ = O.volume_flux_rev(L, P.ucont, 0.0, 1)
    b, _ = O.poisson_rhs(L, uc, DT, ST)
    b = W.noisy_rhs(b, L.nvert, P.metrics[-1]["Aj"], DT, seed=11)
    A = O.lhs_csr(L)
    x_ref, fl = _direct_solution(A, b, L.nvert)
    phi, st = ctx.solve(b, precision=precision, rtol=1e-10, max_it=100, smoother=smoother,
                        omega=0.9 if smoother == 0 else 1.0)
    assert st["status"] == 0 and st["rel_residual"] <= 1e-10
    r = b.ravel() - A @ phi.ravel()
    assert np.linalg.norm(r) <= 1.5e-10 * np.linalg.norm(b)
    d = phi[fl] - phi[fl].mean() - (x_ref[fl] - x_ref[fl].mean())
    assert np.linalg.norm(d) <= 1e-8 * np.linalg.norm(x_ref[fl] - x_ref[fl].mean())
    assert np.all(phi[~fl] == 0.0)


def test_ghosted_inputs_match_box_inputs():
    """Local (ghosted) arrays as a periodic DMDA holds them give the same operator."""
    from curvib_old_gb300.solver import PoissonContext
    P = _problem("channel_periodic")
    s = 3
    ghosted = []
    box_shapes = []
    for m in P.metrics:
        g = {}
        for k, a in m.items():
            pad = [(s, s) if P.per[2] else (0, 0), (s, s) if P.per[1] else (0, 0),
                   (s, s) if P.per[0] else (0, 0)] + ([(0, 0)] if a.ndim == 4 else [])
            g[k] = np.pad(a, pad, mode="wrap")
        ghosted.append(g)
        box_shapes.append(m["Aj"].shape)
    nvpad = [(s, s) if P.per[2] else (0, 0), (s, s) if P.per[1] else (0, 0), (s, s) if P.per[0] else (0, 0)]
    G = types.SimpleNamespace(metrics=ghosted, nvert=np.pad(P.nvert, nvpad, mode="wrap"), bctype=P.bctype,
                              semi=P.semi, box_shapes=box_shapes)
    gh = [(-s if P.per[0] else 0, -s if P.per[1] else 0, -s if P.per[2] else 0)] * len(P.metrics)
    a = PoissonContext().setup(P)
    b = PoissonContext().setup(G, ghosts=gh)
    for l in range(len(P.metrics)):
        assert np.array_equal(a.weights(l), b.weights(l))
    a.close()
    b.close()
