"""Helpers shared by the GPU parity tests: the library's stored rows as a sparse
matrix in the reference's column order, fluid masks, mean-removed errors and a
direct solve of the singular all-Neumann system."""
from __future__ import annotations

import numpy as np

SLOTS = ["CP", "EP", "WP", "NP", "SP", "TP", "BP", "NE", "SE", "NW", "SW", "TN", "BN", "TS", "BS", "TE", "BE",
         "TW", "BW"]


def weights_to_csr(w, shape, bctype):
    """The stored rows ([19][mz][my][mx]) as a sparse matrix, columns wrapped as
    the reference's periodic DMDA wraps them (poisson.c:576-594 slot order)."""
    import scipy.sparse as sp
    mz, my, mx = shape
    px, py, pz = bctype[0] == 7, bctype[2] == 7, bctype[4] == 7
    K, J, I = np.meshgrid(np.arange(mz), np.arange(my), np.arange(mx), indexing="ij")

    def up(a, m, p):
        return np.where(p & (a == m - 2), 1, a + 1)

    def dn(a, m, p):
        return np.where(p & (a == 1), m - 2, a - 1)
    iu, id_, ju, jd, ku, kd = up(I, mx, px), dn(I, mx, px), up(J, my, py), dn(J, my, py), up(K, mz, pz), dn(K, mz, pz)
    off = {"CP": (I, J, K), "EP": (iu, J, K), "WP": (id_, J, K), "NP": (I, ju, K), "SP": (I, jd, K),
           "TP": (I, J, ku), "BP": (I, J, kd), "NE": (iu, ju, K), "SE": (iu, jd, K), "NW": (id_, ju, K),
           "SW": (id_, jd, K), "TN": (I, ju, ku), "BN": (I, ju, kd), "TS": (I, jd, ku), "BS": (I, jd, kd),
           "TE": (iu, J, ku), "BE": (iu, J, kd), "TW": (id_, J, ku), "BW": (id_, J, kd)}
    rows, cols, vals = [], [], []
    n = mx * my * mz
    for s, nm in enumerate(SLOTS):
        a, b, c = off[nm]
        ok = (a >= 0) & (a < mx) & (b >= 0) & (b < my) & (c >= 0) & (c < mz) & (w[s] != 0)
        r = np.arange(n).reshape(shape)[ok]
        cc = (c * my + b) * mx + a
        rows.append(r)
        cols.append(cc[ok])
        vals.append(w[s][ok])
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))


def fluid_mask(nvert):
    """Interior cells with nvert < 0.1: the reference's null-space mask (poisson.c:411-430)."""
    fl = np.zeros(nvert.shape, dtype=bool)
    fl[1:-1, 1:-1, 1:-1] = nvert[1:-1, 1:-1, 1:-1] < 0.1
    return fl


def mean_removed_error(phi, ref, regions):
    """||(phi - ref) with each region's mean removed|| / ||ref with each region's mean removed||."""
    num, den = 0.0, 0.0
    for m in regions:
        d = (phi[m] - phi[m].mean()) - (ref[m] - ref[m].mean())
        r = ref[m] - ref[m].mean()
        num += float(d @ d)
        den += float(r @ r)
    return (num / den) ** 0.5


def direct_solution(A, b, regions):
    """FP64 direct solve of the singular system on the fluid cells, the mean of
    each fluid region pinned to zero by a bordering row."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    fl = np.zeros(b.shape, dtype=bool)
    for m in regions:
        fl |= m
    idx = np.flatnonzero(fl.ravel())
    Af = A.tocsr()[idx][:, idx]
    pos = np.full(b.size, -1)
    pos[idx] = np.arange(len(idx))
    C = sp.lil_matrix((len(regions), len(idx)))
    for r, m in enumerate(regions):
        C[r, pos[np.flatnonzero(m.ravel())]] = 1.0
    C = C.tocsr()
    K = sp.bmat([[Af, C.T], [C, None]]).tocsc()
    sol = sla.spsolve(K, np.concatenate([b.ravel()[idx], np.zeros(len(regions))]))
    x = np.zeros(b.size)
    x[idx] = sol[:len(idx)]
    return x.reshape(b.shape)
