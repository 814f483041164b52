"""Synthetic CURVIB inputs: curvilinear grids, per-level metrics, IB flags, fluxes.

This module builds, on the host, what the reference's set-up produces before the
pressure-projection path runs:

* node coordinates (the reference reads them from grid.dat, init.c:606-744) and
  their injection onto the multigrid levels (init.c:786-828);
* the level sizes of MGDACreate (init.c:78-107): IM_c = (IM+1)/2 unless that
  direction is semi-coarsened; the DMDA box is (IM+1) x (JM+1) x (KM+1);
* the curvilinear metrics of FormMetrics (metrics.c:4-1229) -- cell-centre
  Csi/Eta/Zet/Aj with their boundary copies, and the I/J/K face metrics built
  from face-centre differences -- followed by Update_Metrics_PBC
  (implicitsolver.c:2174-2573), which copies the periodic images into the ring;
* nvert flags for spheres (0 fluid, 1 immersed-boundary layer, 3 solid) with
  the 27-neighbour IB layer rule of ibm_search_advanced (ibm.c:4407-4438),
  classified on cell centres;
* contravariant face fluxes of an analytic or seeded velocity field.

Every array uses the reference's DMDA global layout: shape (mz, my, mx) or
(mz, my, mx, 3), index [k][j][i], i fastest, including the boundary ring.  The
arithmetic mirrors the reference expression by expression (same operand order,
no fused multiply-add), so on the same inputs the metrics agree with the
reference bit for bit.
"""
from __future__ import annotations

import math
import numpy as np

COEF_TIME_ACCURACY = 1.5  # variables.h:421

METRIC_NAMES = ("Csi", "Eta", "Zet", "ICsi", "IEta", "IZet", "JCsi", "JEta", "JZet",
                "KCsi", "KEta", "KZet")
JACOBIAN_NAMES = ("Aj", "IAj", "JAj", "KAj")


# --------------------------------------------------------------------------- grids
def level_dims(IM: int, JM: int, KM: int, nlevels: int, semi=(0, 0, 0)):
    """Node counts per level, coarsest first (MGDACreate, init.c:78-107)."""
    dims = [(IM, JM, KM)]
    for _ in range(nlevels - 1):
        im, jm, km = dims[0]
        dims.insert(0, (im if semi[0] else (im + 1) // 2,
                        jm if semi[1] else (jm + 1) // 2,
                        km if semi[2] else (km + 1) // 2))
    return dims


def stretched(n_nodes: int, beta: float) -> np.ndarray:
    """tanh clustering toward both ends of [0,1]: 0.5*(1 + tanh(beta*(2e-1))/tanh(beta))."""
    eta = np.arange(n_nodes, dtype=np.float64) / (n_nodes - 1)
    if beta == 0.0:
        return eta
    return 0.5 * (1.0 + np.tanh(beta * (2.0 * eta - 1.0)) / math.tanh(beta))


def box_nodes(cells, lengths=(1.0, 1.0, 1.0), beta_y: float = 0.0, distort: bool = False):
    """Node coordinates (KM, JM, IM, 3) of a box with tanh stretching in y.

    With ``distort`` every node moves by x += 0.05 sin(2 pi y), z += 0.03 sin(2 pi x),
    both evaluated at the undistorted (unit-scaled) position.
    """
    nx, ny, nz = cells
    x = np.arange(nx + 1, dtype=np.float64) / nx
    y = stretched(ny + 1, beta_y)
    z = np.arange(nz + 1, dtype=np.float64) / nz
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    if distort:
        Xd = X + 0.05 * np.sin(2.0 * np.pi * Y)
        Zd = Z + 0.03 * np.sin(2.0 * np.pi * X)
    else:
        Xd, Zd = X, Z
    out = np.empty(X.shape + (3,), dtype=np.float64)
    out[..., 0] = Xd * lengths[0]
    out[..., 1] = Y * lengths[1]
    out[..., 2] = Zd * lengths[2]
    return out


def level_coordinates(nodes: np.ndarray, nlevels: int, semi=(0, 0, 0)):
    """Coordinate vectors in DMDA layout (mz, my, mx, 3) per level, coarsest first.

    Finest: nodes in [0,KM)x[0,JM)x[0,IM), zero elsewhere (init.c:655-744).
    Coarser: the DMDA's uniform coordinates with the injected fine nodes written
    over [0,mx-1)x[0,my-1)x[0,mz-1) (init.c:786-828).
    """
    KM, JM, IM = nodes.shape[:3]
    dims = level_dims(IM, JM, KM, nlevels, semi)
    out = [None] * nlevels
    fine = np.zeros((KM + 1, JM + 1, IM + 1, 3))
    fine[:KM, :JM, :IM] = nodes
    out[-1] = fine
    for l in range(nlevels - 2, -1, -1):
        im, jm, km = dims[l]
        mx, my, mz = im + 1, jm + 1, km + 1
        c = np.empty((mz, my, mx, 3))
        c[..., 0] = (np.arange(mx) / (mx - 1))[None, None, :]
        c[..., 1] = (np.arange(my) / (my - 1))[None, :, None]
        c[..., 2] = (np.arange(mz) / (mz - 1))[:, None, None]
        sk = 1 if semi[2] else 2
        sj = 1 if semi[1] else 2
        si = 1 if semi[0] else 2
        h = out[l + 1]
        c[:mz - 1, :my - 1, :mx - 1] = h[0:sk * (mz - 1):sk, 0:sj * (my - 1):sj, 0:si * (mx - 1):si]
        out[l] = c
    return out


# ---------------------------------------------------------------- ghosted arrays
class _Local:
    """A DMDA local (ghosted) array addressed by global indices [k][j][i].

    One rank: a periodic direction has ``s`` ghost layers each side that wrap, a
    non-periodic one has none.
    """

    def __init__(self, shape, per, s, dof):
        self.shape = shape  # (mz, my, mx)
        self.o = tuple(s if p else 0 for p in per)  # offsets (z, y, x)
        full = tuple(n + 2 * o for n, o in zip(shape, self.o))
        self.a = np.zeros(full + ((dof,) if dof > 1 else ()))

    @classmethod
    def from_global(cls, g, per, s):
        dof = g.shape[3] if g.ndim == 4 else 1
        L = cls(g.shape[:3], per, s, dof)
        idx = [np.arange(-o, n + o) % n for n, o in zip(g.shape[:3], L.o)]
        L.a[...] = g[np.ix_(*idx)]
        return L

    def __call__(self, k0, k1, j0, j1, i0, i1):
        oz, oy, ox = self.o
        return self.a[k0 + oz:k1 + oz, j0 + oy:j1 + oy, i0 + ox:i1 + ox]

    def to_global(self):
        oz, oy, ox = self.o
        mz, my, mx = self.shape
        return self.a[oz:oz + mz, oy:oy + my, ox:ox + mx].copy()


def _cross_metrics(dxdc, dydc, dzdc, dxde, dyde, dzde, dxdz, dydz, dzdz):
    csi = np.stack([dyde * dzdz - dzde * dydz, -dxde * dzdz + dzde * dxdz,
                    dxde * dydz - dyde * dxdz], -1)
    eta = np.stack([dydz * dzdc - dzdz * dydc, -dxdz * dzdc + dzdz * dxdc,
                    dxdz * dydc - dydz * dxdc], -1)
    zet = np.stack([dydc * dzde - dzdc * dyde, -dxdc * dzde + dzdc * dxde,
                    dxdc * dyde - dydc * dxde], -1)
    det = (dxdc * (dyde * dzdz - dzde * dydz) - dydc * (dxde * dzdz - dzde * dxdz)
           + dzdc * (dxde * dydz - dyde * dxdz))
    return csi, eta, zet, 1.0 / det


def form_metrics(coor: np.ndarray, per=(False, False, False)):
    """FormMetrics (metrics.c:4-1229) + Update_Metrics_PBC (implicitsolver.c:2174).

    ``coor``: (mz, my, mx, 3) coordinates of one level in DMDA layout.  ``per`` is
    (x, y, z) periodicity.  Returns a dict of global-layout arrays: the twelve
    Cmpnts metric fields (…, 3), Aj/IAj/JAj/KAj and the cell centres Cent.
    """
    mz, my, mx = coor.shape[:3]
    perz = (per[2], per[1], per[0])
    s = 3 if any(per) else 2
    IM, JM, KM = mx - 1, my - 1, mz - 1
    c = _Local.from_global(coor, perz, s)
    X = lambda k0, k1, j0, j1, i0, i1: c(k0, k1, j0, j1, i0, i1)

    csi = np.zeros((mz, my, mx, 3)); eta = np.zeros_like(csi); zet = np.zeros_like(csi)
    aj = np.zeros((mz, my, mx))
    # csi: k,j interior, i in [0, mx-1)    (metrics.c:80-104)
    a, b = X(1, mz - 1, 1, my - 1, 0, mx - 1), X(0, mz - 2, 1, my - 1, 0, mx - 1)
    cm, d = X(1, mz - 1, 0, my - 2, 0, mx - 1), X(0, mz - 2, 0, my - 2, 0, mx - 1)
    de = 0.5 * (a + b - cm - d)          # d/deta:  [k][j]+[k-1][j]-[k][j-1]-[k-1][j-1]
    dz = 0.5 * (cm + a - d - b)          # d/dzeta: [k][j-1]+[k][j]-[k-1][j-1]-[k-1][j]
    csi[1:mz - 1, 1:my - 1, 0:mx - 1] = np.stack(
        [de[..., 1] * dz[..., 2] - de[..., 2] * dz[..., 1],
         -de[..., 0] * dz[..., 2] + de[..., 2] * dz[..., 0],
         de[..., 0] * dz[..., 1] - de[..., 1] * dz[..., 0]], -1)
    # eta: k,j,i interior   (metrics.c:107-132)
    a, b = X(1, mz - 1, 1, my - 1, 1, mx - 1), X(0, mz - 2, 1, my - 1, 1, mx - 1)
    cm, d = X(1, mz - 1, 1, my - 1, 0, mx - 2), X(0, mz - 2, 1, my - 1, 0, mx - 2)
    dc = 0.5 * (a + b - cm - d)          # [k][j][i]+[k-1][j][i]-[k][j][i-1]-[k-1][j][i-1]
    dz = 0.5 * (a + cm - b - d)          # [k][j][i]+[k][j][i-1]-[k-1][j][i]-[k-1][j][i-1]
    eta[1:mz - 1, 1:my - 1, 1:mx - 1] = np.stack(
        [dz[..., 1] * dc[..., 2] - dz[..., 2] * dc[..., 1],
         -dz[..., 0] * dc[..., 2] + dz[..., 2] * dc[..., 0],
         dz[..., 0] * dc[..., 1] - dz[..., 1] * dc[..., 0]], -1)
    # zet: k in [0, mz-1), j,i interior   (metrics.c:135-158)
    a, b = X(0, mz - 1, 1, my - 1, 1, mx - 1), X(0, mz - 1, 0, my - 2, 1, mx - 1)
    cm, d = X(0, mz - 1, 1, my - 1, 0, mx - 2), X(0, mz - 1, 0, my - 2, 0, mx - 2)
    dc = 0.5 * (a + b - cm - d)          # [j][i]+[j-1][i]-[j][i-1]-[j-1][i-1]
    de = 0.5 * (a + cm - b - d)          # [j][i]+[j][i-1]-[j-1][i]-[j-1][i-1]
    zet[0:mz - 1, 1:my - 1, 1:mx - 1] = np.stack(
        [dc[..., 1] * de[..., 2] - dc[..., 2] * de[..., 1],
         -dc[..., 0] * de[..., 2] + dc[..., 2] * de[..., 0],
         dc[..., 0] * de[..., 1] - dc[..., 1] * de[..., 0]], -1)
    # Jacobian (metrics.c:161-212)
    p000 = X(1, mz - 1, 1, my - 1, 1, mx - 1)        # [k][j][i]
    p010 = X(1, mz - 1, 0, my - 2, 1, mx - 1)        # [k][j-1][i]
    p100 = X(0, mz - 2, 1, my - 1, 1, mx - 1)        # [k-1][j][i]
    p110 = X(0, mz - 2, 0, my - 2, 1, mx - 1)        # [k-1][j-1][i]
    p001 = X(1, mz - 1, 1, my - 1, 0, mx - 2)        # [k][j][i-1]
    p011 = X(1, mz - 1, 0, my - 2, 0, mx - 2)        # [k][j-1][i-1]
    p101 = X(0, mz - 2, 1, my - 1, 0, mx - 2)        # [k-1][j][i-1]
    p111 = X(0, mz - 2, 0, my - 2, 0, mx - 2)        # [k-1][j-1][i-1]
    dc = 0.25 * (p000 + p010 + p100 + p110 - p001 - p011 - p101 - p111)
    de = 0.25 * (p000 + p001 + p100 + p101 - p010 - p011 - p110 - p111)
    dz = 0.25 * (p000 + p010 + p001 + p011 - p100 - p110 - p101 - p111)
    det = (dc[..., 0] * (de[..., 1] * dz[..., 2] - de[..., 2] * dz[..., 1])
           - dc[..., 1] * (de[..., 0] * dz[..., 2] - de[..., 2] * dz[..., 0])
           + dc[..., 2] * (de[..., 0] * dz[..., 1] - de[..., 1] * dz[..., 0]))
    aj[1:mz - 1, 1:my - 1, 1:mx - 1] = 1.0 / det
    # boundary copies, in the reference's order (metrics.c:214-322)
    eta[:, :, 0] = eta[:, :, 1]; zet[:, :, 0] = zet[:, :, 1]; aj[:, :, 0] = aj[:, :, 1]
    eta[:, :, mx - 1] = eta[:, :, mx - 2]; zet[:, :, mx - 1] = zet[:, :, mx - 2]
    aj[:, :, mx - 1] = aj[:, :, mx - 2]
    csi[:, 0] = csi[:, 1]; zet[:, 0] = zet[:, 1]; aj[:, 0] = aj[:, 1]
    csi[:, my - 1] = csi[:, my - 2]; zet[:, my - 1] = zet[:, my - 2]; aj[:, my - 1] = aj[:, my - 2]
    eta[0] = eta[1]; csi[0] = csi[1]; aj[0] = aj[1]
    eta[mz - 1] = eta[mz - 2]; csi[mz - 1] = csi[mz - 2]; aj[mz - 1] = aj[mz - 2]

    # cell centres and grid spacing (metrics.c:332-425)
    cent = np.zeros((mz, my, mx, 3))
    cent[1:mz - 1, 1:my - 1, 1:mx - 1] = 0.125 * (p000 + p010 + p100 + p110 + p001 + p011 + p101 + p111)
    gs = np.zeros((mz, my, mx, 3))
    q = lambda a_, b_, c_, d_: 0.25 * (a_ + b_ + c_ + d_)
    p_ = q(p000, p010, p110, p100); m_ = q(p001, p011, p111, p101)
    gs[1:mz - 1, 1:my - 1, 1:mx - 1, 0] = np.sqrt(_sq3(p_ - m_))
    p_ = q(p000, p001, p100, p101); m_ = q(p010, p011, p110, p111)
    gs[1:mz - 1, 1:my - 1, 1:mx - 1, 1] = np.sqrt(_sq3(p_ - m_))
    p_ = q(p000, p001, p010, p011); m_ = q(p100, p101, p110, p111)
    gs[1:mz - 1, 1:my - 1, 1:mx - 1, 2] = np.sqrt(_sq3(p_ - m_))
    lgs = _Local.from_global(gs, perz, s)

    # face-centre coordinates (metrics.c:629-662, 800-830, 946-1000)
    centx = _Local((mz, my, mx), perz, s, 3)
    centx(1, mz, 1, my, 0, mx)[...] = (X(1, mz, 1, my, 0, mx) + X(0, mz - 1, 1, my, 0, mx)
                                       + X(1, mz, 0, my - 1, 0, mx) + X(0, mz - 1, 0, my - 1, 0, mx)) * 0.25
    centy = _Local((mz, my, mx), perz, s, 3)
    centy(1, mz, 0, my, 1, mx)[...] = (X(1, mz, 0, my, 1, mx) + X(0, mz - 1, 0, my, 1, mx)
                                       + X(1, mz, 0, my, 0, mx - 1) + X(0, mz - 1, 0, my, 0, mx - 1)) * 0.25
    centz = _Local((mz, my, mx), perz, s, 3)
    centz(0, mz, 1, my, 1, mx)[...] = (X(0, mz, 1, my, 1, mx) + X(0, mz, 0, my - 1, 1, mx)
                                       + X(0, mz, 1, my, 0, mx - 1) + X(0, mz, 0, my - 1, 0, mx - 1)) * 0.25
    # periodic extensions of the face centres (cgrid == 0 branches)
    if per[0]:
        oz, oy = centx.o[0], centx.o[1]
        k0, k1 = -oz + 1, mz + oz
        j0, j1 = -oy + 1, my + oy
        lo = centx(k0, k1, j0, j1, -1, 0); c0 = centx(k0, k1, j0, j1, 0, 1)
        lo[...] = c0
        lo[..., 0] = c0[..., 0] - lgs(k0, k1, j0, j1, -2, -1)[..., 0]
        hi = centx(k0, k1, j0, j1, mx - 1, mx); cm1 = centx(k0, k1, j0, j1, mx - 2, mx - 1)
        hi[...] = cm1
        hi[..., 0] = cm1[..., 0] + lgs(k0, k1, j0, j1, mx + 1, mx + 2)[..., 0]
    if per[1]:
        oz, ox = centy.o[0], centy.o[2]
        k0, k1 = -oz + 1, mz + oz
        i0, i1 = -ox + 1, mx + ox
        lo = centy(k0, k1, -1, 0, i0, i1); c0 = centy(k0, k1, 0, 1, i0, i1)
        lo[...] = c0
        lo[..., 1] = c0[..., 1] - lgs(k0, k1, -2, -1, i0, i1)[..., 1]
        hi = centy(k0, k1, my - 1, my, i0, i1); cm1 = centy(k0, k1, my - 2, my - 1, i0, i1)
        hi[...] = cm1
        hi[..., 1] = cm1[..., 1] + lgs(k0, k1, my + 1, my + 2, i0, i1)[..., 1]
    if per[2]:
        oy, ox = centz.o[1], centz.o[2]
        j0, j1 = -oy + 1, my + oy
        i0, i1 = -ox + 1, mx + ox
        lo = centz(-1, 0, j0, j1, i0, i1); c0 = centz(0, 1, j0, j1, i0, i1)
        lo[...] = c0
        lo[..., 2] = c0[..., 2] - lgs(-2, -1, j0, j1, i0, i1)[..., 2]
        hi = centz(mz - 1, mz, j0, j1, i0, i1); cm1 = centz(mz - 2, mz - 1, j0, j1, i0, i1)
        hi[...] = cm1
        hi[..., 2] = cm1[..., 2] + lgs(mz + 1, mz + 2, j0, j1, i0, i1)[..., 2]

    out = {"Csi": csi, "Eta": eta, "Zet": zet, "Aj": aj, "Cent": cent,
           "Centx": centx.to_global(), "Centy": centy.to_global(), "Centz": centz.to_global()}
    # I faces: k,j interior, i in [0, mx-1)  (metrics.c:713-788)
    out.update(_face_metrics("I", centx, (mz, my, mx), per))
    out.update(_face_metrics("J", centy, (mz, my, mx), per))
    out.update(_face_metrics("K", centz, (mz, my, mx), per))
    if any(per):
        _update_metrics_pbc(out, per)
    return out


def _sq3(v):
    return v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1] + v[..., 2] * v[..., 2]


def _diff_kind(lo, hi, axis_len, own_axis, periodic):
    """0 central, 1 forward, 2 backward for indices lo..hi-1 of one axis."""
    idx = np.arange(lo, hi)
    kind = np.zeros(idx.shape, dtype=np.int8)
    if own_axis:
        if not periodic:
            kind[idx == 0] = 1
            kind[idx == axis_len - 2] = 2
    else:
        kind[:] = -1
        kind[(idx > 1) & (idx < axis_len - 2)] = 0
        kind[(idx == 1) & (kind == -1)] = 1
        kind[(idx == axis_len - 2) & (kind == -1)] = 2
    return idx, kind


def _derivative(cf, axis, k, j, i, kind):
    """d(cf)/d(axis) at global index arrays (k, j, i) with per-point difference kind."""
    def at(dk, dj, di):
        oz, oy, ox = cf.o
        return cf.a[k + dk + oz, j + dj + oy, i + di + ox]
    e = [(1, 0, 0), (0, 1, 0), (0, 0, 1)][axis]
    p, m, c0 = at(*e), at(-e[0], -e[1], -e[2]), at(0, 0, 0)
    cen = (p - m) * 0.5
    fwd = p - c0
    bwd = c0 - m
    kind = kind[..., None]
    return np.where(kind == 0, cen, np.where(kind == 1, fwd, bwd))


def _face_metrics(which, cf, shape, per):
    mz, my, mx = shape
    if which == "I":
        kr, jr, ir = (1, mz - 1), (1, my - 1), (0, mx - 1)
        own = 2
    elif which == "J":
        kr, jr, ir = (1, mz - 1), (0, my - 1), (1, mx - 1)
        own = 1
    else:
        kr, jr, ir = (0, mz - 1), (1, my - 1), (1, mx - 1)
        own = 0
    lens = (mz, my, mx)
    pz = (per[2], per[1], per[0])
    ranges = (kr, jr, ir)
    kinds = []
    idxs = []
    for ax in range(3):
        idx, kind = _diff_kind(ranges[ax][0], ranges[ax][1], lens[ax], ax == own, pz[ax])
        idxs.append(idx)
        kinds.append(kind)
    K, J, I = np.meshgrid(*idxs, indexing="ij")
    KK, KJ, KI = np.meshgrid(*kinds, indexing="ij")
    d_c = _derivative(cf, 2, K, J, I, KI)   # d/dxi  (i)
    d_e = _derivative(cf, 1, K, J, I, KJ)   # d/deta (j)
    d_z = _derivative(cf, 0, K, J, I, KK)   # d/dzeta(k)
    csi, eta, zet, ajf = _cross_metrics(d_c[..., 0], d_c[..., 1], d_c[..., 2],
                                        d_e[..., 0], d_e[..., 1], d_e[..., 2],
                                        d_z[..., 0], d_z[..., 1], d_z[..., 2])
    res = {}
    for nm, arr in ((which + "Csi", csi), (which + "Eta", eta), (which + "Zet", zet)):
        full = np.zeros((mz, my, mx, 3))
        full[kr[0]:kr[1], jr[0]:jr[1], ir[0]:ir[1]] = arr
        res[nm] = full
    full = np.zeros((mz, my, mx))
    full[kr[0]:kr[1], jr[0]:jr[1], ir[0]:ir[1]] = ajf
    res[which + "Aj"] = full
    return res


def _update_metrics_pbc(m, per):
    """Update_Metrics_PBC (implicitsolver.c:2174): ring <- periodic image, per direction."""
    names = METRIC_NAMES + JACOBIAN_NAMES
    for ax, p in ((2, per[0]), (1, per[1]), (0, per[2])):
        if not p:
            continue
        for nm in names:
            a = m[nm]
            n = a.shape[ax]
            sl_lo = [slice(None)] * a.ndim; sl_lo[ax] = 0
            src_lo = [slice(None)] * a.ndim; src_lo[ax] = n - 2
            sl_hi = [slice(None)] * a.ndim; sl_hi[ax] = n - 1
            src_hi = [slice(None)] * a.ndim; src_hi[ax] = 1
            a[tuple(sl_lo)] = a[tuple(src_lo)]
            a[tuple(sl_hi)] = a[tuple(src_hi)]


# ------------------------------------------------------------------ IB flags
IB_CODE = 1.4     # ibm_search_advanced_rev's immersed-boundary layer (ibm.c:1072-1081)
SOLID_CODE = 3.4  # ... and its solid cells


def sphere_nvert(cent: np.ndarray, spheres, ib_code: float = IB_CODE,
                 solid_code: float = SOLID_CODE) -> np.ndarray:
    """nvert of cell centres for a union of spheres [(cx, cy, cz, r), ...].

    Interior cells inside a sphere are solid; fluid interior cells with a solid
    cell among their 26 neighbours form the IB layer (ibm.c:4407-4438);
    everything else, the boundary ring included, is fluid (0).  The default
    codes 1.4 / 3.4 are the ones ibm_search_advanced_rev leaves -- the search
    the reference's main.c runs (main.c:1020) and whose IB layer VolumeFlux_rev
    corrects (nvert in (1.1, 1.5), poisson.c:3753).  All bodies share one code
    (the per-body +ibi/1000 of ibm.c:4651 is not used).  A fluid cell left with
    no fluid face neighbour is marked IB too.  Boxes with periodic directions
    count links across the seam as absent (a conservative choice).
    """
    mz, my, mx = cent.shape[:3]
    solid = np.zeros((mz, my, mx), dtype=bool)
    c = cent[1:-1, 1:-1, 1:-1]
    for (cx, cy, cz, r) in spheres:
        d2 = (c[..., 0] - cx) ** 2 + (c[..., 1] - cy) ** 2 + (c[..., 2] - cz) ** 2
        solid[1:-1, 1:-1, 1:-1] |= d2 < r * r
    near = np.zeros_like(solid)
    for dk in (-1, 0, 1):
        for dj in (-1, 0, 1):
            for di in (-1, 0, 1):
                near[1:-1, 1:-1, 1:-1] |= solid[1 + dk:mz - 1 + dk, 1 + dj:my - 1 + dj, 1 + di:mx - 1 + di]
    nv = np.zeros((mz, my, mx))
    nv[near & ~solid] = ib_code
    nv[solid] = solid_code
    nv[0, :, :] = nv[-1, :, :] = 0.0
    nv[:, 0, :] = nv[:, -1, :] = 0.0
    nv[:, :, 0] = nv[:, :, -1] = 0.0
    # A fluid cell enclosed on all six faces by IB cells (a gap between two
    # bodies narrower than a cell) would have an empty pressure row: mark it IB.
    while True:
        fl = np.zeros((mz, my, mx), dtype=bool)
        fl[1:-1, 1:-1, 1:-1] = nv[1:-1, 1:-1, 1:-1] < 0.1
        c = fl[1:-1, 1:-1, 1:-1]
        links = (fl[2:, 1:-1, 1:-1].astype(int) + fl[:-2, 1:-1, 1:-1] + fl[1:-1, 2:, 1:-1] + fl[1:-1, :-2, 1:-1]
                 + fl[1:-1, 1:-1, 2:] + fl[1:-1, 1:-1, :-2])
        lone = c & (links == 0)
        if not lone.any():
            return nv
        nv[1:-1, 1:-1, 1:-1][lone] = ib_code


# ------------------------------------------------------------------- fluxes
def ucont_from_velocity(m: dict, vel, per=(False, False, False)) -> np.ndarray:
    """Contravariant fluxes Ucont (mz, my, mx, 3) of a Cartesian velocity field.

    ``vel(xyz) -> (…, 3)`` is evaluated at the face centres (Centx/Centy/Centz)
    and dotted with the face area vectors Csi/Eta/Zet: Ucont.x[k][j][i] is the
    flux through the face between cells i and i+1.  Wall faces carry zero flux;
    on a periodic seam both copies of the face carry the same flux.
    """
    csi, eta, zet = m["Csi"], m["Eta"], m["Zet"]
    mz, my, mx = csi.shape[:3]
    uc = np.zeros((mz, my, mx, 3))
    for comp, (area, fc) in enumerate(((csi, m["Centx"]), (eta, m["Centy"]), (zet, m["Centz"]))):
        v = vel(fc)
        flux = v[..., 0] * area[..., 0] + v[..., 1] * area[..., 1] + v[..., 2] * area[..., 2]
        sl = [slice(1, mz - 1), slice(1, my - 1), slice(1, mx - 1)]
        ax = 2 - comp                       # comp 0 -> i axis (2), 1 -> j (1), 2 -> k (0)
        sl[ax] = slice(0, (mz, my, mx)[ax] - 1)
        uc[tuple(sl) + (comp,)] = flux[tuple(sl)]
        n = (mz, my, mx)[ax]
        lo = [slice(None)] * 3; lo[ax] = 0
        hi = [slice(None)] * 3; hi[ax] = n - 2
        p = per[comp]
        if p:
            uc[tuple(lo) + (comp,)] = uc[tuple(hi) + (comp,)]
        else:
            uc[tuple(lo) + (comp,)] = 0.0
            uc[tuple(hi) + (comp,)] = 0.0
    return uc


def taylor_green(xyz: np.ndarray) -> np.ndarray:
    """u* = (sin(pi x) cos(pi y), -cos(pi x) sin(pi y), 0)."""
    x, y = xyz[..., 0], xyz[..., 1]
    out = np.zeros(xyz.shape)
    out[..., 0] = np.sin(np.pi * x) * np.cos(np.pi * y)
    out[..., 1] = -np.cos(np.pi * x) * np.sin(np.pi * y)
    return out


def smoothed_noise_ucont(m: dict, per, sigma: float, passes: int, rng) -> np.ndarray:
    """Fluxes of a seeded Gaussian cell-centre velocity smoothed by damped-Jacobi passes.

    Each pass is v <- v + (2/3)(mean of the six neighbours - v); periodic
    directions wrap, wall directions repeat the edge value.  Face velocities are
    the average of the two adjacent cells; wall faces carry zero flux.
    """
    mz, my, mx = m["Aj"].shape
    v = rng.normal(0.0, sigma, size=(mz - 2, my - 2, mx - 2, 3))
    for _ in range(passes):
        pad = np.pad(v, [(1, 1), (1, 1), (1, 1), (0, 0)],
                     mode="edge")
        if per[2]:
            pad[0], pad[-1] = pad[-2].copy(), pad[1].copy()
        if per[1]:
            pad[:, 0], pad[:, -1] = pad[:, -2].copy(), pad[:, 1].copy()
        if per[0]:
            pad[:, :, 0], pad[:, :, -1] = pad[:, :, -2].copy(), pad[:, :, 1].copy()
        nb = (pad[2:, 1:-1, 1:-1] + pad[:-2, 1:-1, 1:-1] + pad[1:-1, 2:, 1:-1] + pad[1:-1, :-2, 1:-1]
              + pad[1:-1, 1:-1, 2:] + pad[1:-1, 1:-1, :-2]) / 6.0
        v = v + (2.0 / 3.0) * (nb - v)
    full = np.zeros((mz, my, mx, 3))
    full[1:-1, 1:-1, 1:-1] = v
    for ax, p in ((2, per[0]), (1, per[1]), (0, per[2])):
        n = full.shape[ax]
        lo = [slice(None)] * 4; lo[ax] = 0
        hi = [slice(None)] * 4; hi[ax] = n - 1
        s1 = [slice(None)] * 4; s1[ax] = 1
        s2 = [slice(None)] * 4; s2[ax] = n - 2
        if p:
            full[tuple(lo)] = full[tuple(s2)]
            full[tuple(hi)] = full[tuple(s1)]
        else:
            full[tuple(lo)] = full[tuple(s1)]
            full[tuple(hi)] = full[tuple(s2)]
    uc = np.zeros((mz, my, mx, 3))
    areas = (m["Csi"], m["Eta"], m["Zet"])
    for comp in range(3):
        ax = 2 - comp
        n = full.shape[ax]
        a = [slice(None)] * 4; a[ax] = slice(0, n - 1)
        b = [slice(None)] * 4; b[ax] = slice(1, n)
        face_v = np.zeros_like(full)
        face_v[tuple(a)] = 0.5 * (full[tuple(a)] + full[tuple(b)])
        ar = areas[comp]
        flux = (face_v[..., 0] * ar[..., 0] + face_v[..., 1] * ar[..., 1]
                + face_v[..., 2] * ar[..., 2])
        sl = [slice(1, mz - 1), slice(1, my - 1), slice(1, mx - 1)]
        sl[ax] = slice(0, n - 1)
        uc[tuple(sl) + (comp,)] = flux[tuple(sl)]
        lo = [slice(None)] * 3; lo[ax] = 0
        hi = [slice(None)] * 3; hi[ax] = n - 2
        if per[comp]:
            uc[tuple(lo) + (comp,)] = uc[tuple(hi) + (comp,)]
        else:
            uc[tuple(lo) + (comp,)] = 0.0
            uc[tuple(hi) + (comp,)] = 0.0
    return uc


def compatible(b: np.ndarray, aj: np.ndarray, nvert: np.ndarray) -> np.ndarray:
    """Project b onto the range of the singular Neumann operator.

    The operator's left null vector is 1/aj on fluid cells (its rows are
    flux differences scaled by -aj), so b is made to satisfy sum(b/aj) = 0 over
    fluid cells: b -= aj * mean_fluid(b/aj).  Non-fluid and ring cells stay 0.
    """
    mz, my, mx = b.shape
    fl = np.zeros(b.shape, dtype=bool)
    fl[1:-1, 1:-1, 1:-1] = nvert[1:-1, 1:-1, 1:-1] < 0.1
    c = (b[fl] / aj[fl]).mean()
    out = b.copy()
    out[fl] -= aj[fl] * c
    return out


# ------------------------------------------------------------------ problems
class Problem:
    """One block's inputs for the path: per-level metrics (coarsest first), the
    finest level's nvert and fluxes, boundary types and semi-coarsening flags."""

    def __init__(self, metrics, nvert, ucont, bctype, semi=(0, 0, 0), per=(False, False, False), name=""):
        self.metrics = metrics
        self.nvert = nvert
        self.ucont = ucont
        self.bctype = list(bctype)
        self.semi = tuple(semi)
        self.per = tuple(per)
        self.name = name
        self.b = None

    @property
    def shape(self):
        return self.nvert.shape

    @property
    def unknowns(self):
        mz, my, mx = self.shape
        return (mx - 2) * (my - 2) * (mz - 2)


def auto_levels(cells, per=(False, False, False), semi=(0, 0, 0), max_coarse_box=600):
    """Number of levels: halve while every halved direction stays even-divisible,
    keeps >= 2 cells (>= 3 when periodic) and the coarsest box (ring included)
    is still larger than ``max_coarse_box``."""
    c = list(cells)
    levels = 1
    while True:
        nxt = [ci if s else ci // 2 for ci, s in zip(c, semi)]
        ok = all(s or (ci % 2 == 0 and ci // 2 >= (3 if p else 2)) for ci, p, s in zip(c, per, semi))
        if not ok or (c[0] + 2) * (c[1] + 2) * (c[2] + 2) <= max_coarse_box:
            return levels
        c = nxt
        levels += 1


def make_problem(cells, lengths=(1.0, 1.0, 1.0), beta_y=0.0, distort=False, per=(False, False, False),
                 spheres=(), nlevels=None, semi=(0, 0, 0), velocity="taylor_green", seed=0, name=""):
    per = tuple(bool(p) for p in per)
    if nlevels is None:
        nlevels = auto_levels(cells, per, semi)
    nodes = box_nodes(cells, lengths, beta_y, distort)
    coords = level_coordinates(nodes, nlevels, semi)
    mets = [form_metrics(c, per) for c in coords]
    nv = sphere_nvert(mets[-1]["Cent"], list(spheres))
    if velocity == "taylor_green":
        uc = ucont_from_velocity(mets[-1], taylor_green, per)
    else:
        uc = smoothed_noise_ucont(mets[-1], per, 0.1, 3, np.random.default_rng(seed))
    bct = [7 if per[0] else 1] * 2 + [7 if per[1] else 1] * 2 + [7 if per[2] else 1] * 2
    return Problem(mets, nv, uc, bct, semi, per, name)


def config0_problem(n=64, nlevels=3):
    """64^3 box on [0,1]^3, tanh stretching 2.0 in y, sin distortion, sphere
    r=0.15 at the centre; 3 multigrid levels (64, 32, 16 cells) as the
    workload states (None: as many as auto_levels allows)."""
    return make_problem((n, n, n), (1.0, 1.0, 1.0), 2.0, True, (False, False, False),
                        [(0.5, 0.5, 0.5, 0.15)], nlevels=nlevels, name=f"box{n}^3-sphere")


def config1_problem(cells=(256, 128, 128), nlevels=5):
    """Channel: periodic x and z, walls in y with tanh stretching 2.5, no body.
    The box is 2pi x 2 x pi (a standard minimal-channel size; the grid and the
    stretching are the fixed part of the workload).  5 multigrid levels as the
    workload states (None: as many as auto_levels allows)."""
    if nlevels is not None:
        nlevels = min(nlevels, auto_levels(cells, (True, False, True), max_coarse_box=0))
    return make_problem(cells, (2 * np.pi, 2.0, np.pi), 2.5, False, (True, False, True), [],
                        velocity="noise", seed=1, nlevels=nlevels, name="channel%dx%dx%d" % tuple(cells))


CONFIG3_SIZES = ((32, 32, 32), (48, 48, 48), (64, 64, 96), (96, 96, 96), (128, 64, 64))


def box_geometry(cells, nlevels=None):
    """Metrics of every level and the Taylor-Green fluxes of a [0,1]^3 box with
    the box-with-sphere geometry rules (tanh stretching 2.0 in y, sin
    distortion, walls everywhere); shared by every problem of that size."""
    per = (False, False, False)
    if nlevels is None:
        nlevels = auto_levels(cells, per)
    nodes = box_nodes(cells, (1.0, 1.0, 1.0), 2.0, True)
    coords = level_coordinates(nodes, nlevels, (0, 0, 0))
    mets = [form_metrics(c, per) for c in coords]
    uc = ucont_from_velocity(mets[-1], taylor_green, per)
    return mets, uc


def config3_problems(count=64, seed=3):
    """Batched uneven solves: sizes drawn uniformly from CONFIG3_SIZES (cells in
    x, y, z), each a [0,1]^3 box with the box-with-sphere geometry rules
    (tanh stretching 2.0 in y, sin distortion) and one sphere of radius
    U[0.1, 0.2] centred in U[0.3, 0.7]^3.  Returns [(problem, rhs seed)]; the
    metrics of equal sizes are shared."""
    rng = np.random.default_rng(seed)
    geo = {}
    out = []
    for q in range(count):
        cells = CONFIG3_SIZES[int(rng.integers(len(CONFIG3_SIZES)))]
        r = float(rng.uniform(0.1, 0.2))
        c = rng.uniform(0.3, 0.7, size=3)
        if cells not in geo:
            geo[cells] = box_geometry(cells)
        mets, uc = geo[cells]
        nv = sphere_nvert(mets[-1]["Cent"], [(float(c[0]), float(c[1]), float(c[2]), r)])
        P = Problem(mets, nv, uc, [1] * 6, (0, 0, 0), (False, False, False),
                    "batch%d-%dx%dx%d" % ((q,) + tuple(cells)))
        out.append((P, int(rng.integers(1 << 30))))
    return out


def noisy_rhs(b, nvert, aj, dt, seed, amp=1e-2):
    """Add seeded uniform noise in [-amp, amp], scaled by 1/dt, on fluid cells, then
    make the result compatible with the Neumann operator."""
    rng = np.random.default_rng(seed)
    fl = np.zeros(b.shape, dtype=bool)
    fl[1:-1, 1:-1, 1:-1] = nvert[1:-1, 1:-1, 1:-1] < 0.1
    out = b.copy()
    out[fl] += rng.uniform(-amp, amp, size=int(fl.sum())) / dt
    return compatible(out, aj, nvert)


def sphere_mesh(center, radius: float, subdivisions: int = 3):
    """A closed triangulated sphere, as the immersed-body meshes ibm_search_advanced
    (ibm.c:4197) classifies cells against: an icosahedron whose faces are split
    in four `subdivisions` times, nodes pushed out to the sphere.  Returns
    (xyz [n_v, 3], tri [n_elmt, 3] int32 node indices, nf [n_elmt, 3] unit
    normals pointing out of the body)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    for _ in range(subdivisions):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mid[key] = len(verts) - 1
            return mid[key]

        nf_ = []
        for (a, b, c) in f:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf_ += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf_
    xyz = np.array(verts) * radius + np.asarray(center, dtype=np.float64)
    tri = np.array(f, dtype=np.int32)
    e1 = xyz[tri[:, 1]] - xyz[tri[:, 0]]
    e2 = xyz[tri[:, 2]] - xyz[tri[:, 0]]
    n = np.cross(e1, e2)
    n /= np.linalg.norm(n, axis=1)[:, None]
    out = (xyz[tri].mean(axis=1) - np.asarray(center)) @ np.eye(3)
    flip = np.einsum("ij,ij->i", n, out) < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    n[flip] = -n[flip]
    return xyz, tri, n
