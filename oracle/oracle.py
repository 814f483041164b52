"""TEST INFRASTRUCTURE ONLY: ctypes front-end of the CPU oracle (cvb_oracle.c).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker; the product library never imports it.  ``build()`` compiles the C
restatement into oracle/_build/; ``build_reference()`` compiles the reference's
own sources against the API shim into oracle/_ref/ when a reference checkout is
present (oracle/build_ref.sh).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libcvboracle.so"
REF_LIB = HERE / "_ref" / "libcvbref.so"
# The reference checkout: CVB_REFERENCE_DIR, else the directory the last
# build_reference() compiled from (recorded in oracle/_ref/), else none.
_REF_RECORD = HERE / "_ref" / "REFERENCE_DIR"


def _reference_dir() -> Path:
    if os.environ.get("CVB_REFERENCE_DIR"):
        return Path(os.environ["CVB_REFERENCE_DIR"])
    if _REF_RECORD.exists():
        return Path(_REF_RECORD.read_text().strip())
    return HERE / "_ref" / "no-reference-checkout"


REF_DIR = _reference_dir()

_lib = None
_ref = None


def build(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = [s for s in (HERE / "cvb_oracle.c", HERE / "cvb_solver.c") if s.exists()]
    if force or not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in srcs):
        cmd = ["gcc", "-std=gnu99", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-o", str(LIB)] + [str(s) for s in srcs] + ["-lm"]
        subprocess.run(cmd, check=True)
    return LIB


def build_reference(ref_dir=None) -> Path | None:
    """Compile the reference's sources in ``ref_dir`` (default: CVB_REFERENCE_DIR,
    else the checkout recorded by the last build) against the API shim into
    oracle/_ref/; None when there is no checkout or it holds no poisson.c."""
    global REF_DIR
    if ref_dir is None:
        ref_dir = os.environ.get("CVB_REFERENCE_DIR") or _reference_dir()
    if not ref_dir or not (Path(ref_dir) / "poisson.c").exists():
        # no checkout here: rebuild from the preprocessed units an earlier
        # build left in oracle/_ref/src/ (they travel with the repository)
        pre = HERE / "_ref" / "src"
        if not (pre / "poisson.i").exists():
            return None
        units = list(pre.glob("*.i")) + [pre / "ref_stubs.c"]
        if not REF_LIB.exists() or any(u.stat().st_mtime > REF_LIB.stat().st_mtime for u in units):
            subprocess.run(["bash", str(HERE / "build_ref.sh"), "--preprocessed"], check=True,
                           stdout=subprocess.DEVNULL)
        return REF_LIB
    ref_dir = Path(ref_dir).resolve()
    subprocess.run(["bash", str(HERE / "build_ref.sh"), str(ref_dir)], check=True,
                   stdout=subprocess.DEVNULL)
    _REF_RECORD.write_text(str(ref_dir) + "\n")
    REF_DIR = ref_dir
    return REF_LIB


class Level(ctypes.Structure):
    _fields_ = [("mx", ctypes.c_int), ("my", ctypes.c_int), ("mz", ctypes.c_int),
                ("bctype", ctypes.c_int * 6),
                ("isc", ctypes.c_int), ("jsc", ctypes.c_int), ("ksc", ctypes.c_int)] + [
        (n, ctypes.c_void_p) for n in ("icsi", "ieta", "izet", "jcsi", "jeta", "jzet",
                                       "kcsi", "keta", "kzet", "iaj", "jaj", "kaj", "aj",
                                       "csi", "eta", "zet", "nvert")]


_FIELD_OF = {"icsi": "ICsi", "ieta": "IEta", "izet": "IZet", "jcsi": "JCsi", "jeta": "JEta",
             "jzet": "JZet", "kcsi": "KCsi", "keta": "KEta", "kzet": "KZet", "iaj": "IAj",
             "jaj": "JAj", "kaj": "KAj", "aj": "Aj", "csi": "Csi", "eta": "Eta", "zet": "Zet"}


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build()))
        P = ctypes.c_void_p
        L = ctypes.POINTER(Level)
        _lib.orc_lhs_csr.argtypes = [L, P, P, P, ctypes.c_int]
        _lib.orc_csr_mult.argtypes = [ctypes.c_int, P, P, P, P, P]
        _lib.orc_poisson_rhs.argtypes = [L, P, ctypes.c_double, ctypes.c_double, P]
        _lib.orc_poisson_rhs.restype = ctypes.c_double
        _lib.orc_volume_flux_rev.argtypes = [L, P, ctypes.c_double, ctypes.c_int, P, P]
        _lib.orc_nvert_restrict.argtypes = [L] + [ctypes.c_int] * 7 + [P]
        _lib.orc_fully_blocked.argtypes = [L, P]
        _lib.orc_restrict.argtypes = [L, L, P, P]
        _lib.orc_interpolate.argtypes = [L, L, P, P]
        _lib.orc_nullspace.argtypes = [L, ctypes.c_int, P, P]
        _lib.orc_update_pressure.argtypes = [L, P, P]
        _lib.orc_projection.argtypes = [L, P, ctypes.c_double, ctypes.c_double, P]
        _lib.orc_contra2cart.argtypes = [L, P, P]
        _lib.orc_ghost_node_velocity.argtypes = [L, P, P]
        _lib.orc_ghost_node_velocity.restype = ctypes.c_int
        _lib.orc_ghost_node_velocity_ext.argtypes = [L, P, P, P, ctypes.c_double]
        _lib.orc_ghost_node_velocity_ext.restype = ctypes.c_int
        _lib.orc_ibm_search.argtypes = [ctypes.c_int] * 3 + [P, ctypes.c_int, P, ctypes.c_int, P, P] + \
            [ctypes.c_int] * 2 + [P, P, ctypes.c_int]
        _lib.orc_ibm_search.restype = ctypes.c_int
        _lib.orc_ibm_ray_offsets.argtypes = [ctypes.c_int, P]
        _lib.orc_divergence.argtypes = [L, P, P, P]
        _lib.orc_metrics_divergence.argtypes = [L, P, P]
        _lib.orc_convection.argtypes = [L, P, P, ctypes.c_int, P]
        D, I = ctypes.c_double, ctypes.c_int
        _lib.orc_viscous.argtypes = [L, P, D, P]
        _lib.orc_form_function1.argtypes = [L, P, P, P, D, I, P]
        _lib.orc_calc_rhs.argtypes = [L, P, P, P, P, P, D, D, I, I, I, P]
        _lib.orc_inflow_flux.argtypes = [L, P, P, I, P]
        _lib.orc_inflow_flux.restype = I
        _lib.orc_inflow_flux_ext.argtypes = [L, P, P, I, P, P, P]
        _lib.orc_inflow_flux_ext.restype = I
        _lib.orc_set_inlet_nodes.argtypes = [P, P]
        _lib.orc_set_inlet_nodes.restype = None
        _lib.orc_set_inlet_globals.argtypes = [ctypes.c_double, I]
        _lib.orc_set_inlet_globals.restype = None
        _lib.orc_set_inlet_table.argtypes = [P]
        _lib.orc_set_inlet_table.restype = None
        _lib.orc_form_bcs.argtypes = [L, P, P, P, P, D, D]
        _lib.orc_form_bcs.restype = I
        _lib.orc_imp_rk.argtypes = [L, P, P, P, P, P, P, D, D, D, D, I, I, I, D, D, I, I, D, P]
        _lib.orc_imp_rk.restype = I
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OLevel:
    """One multigrid level handed to the oracle (keeps its arrays alive)."""

    def __init__(self, metrics: dict, nvert: np.ndarray, bctype, semi=(0, 0, 0)):
        self.keep = {}
        mz, my, mx = nvert.shape
        self.s = Level()
        self.s.mx, self.s.my, self.s.mz = mx, my, mz
        for q in range(6):
            self.s.bctype[q] = int(bctype[q])
        self.s.isc, self.s.jsc, self.s.ksc = (int(v) for v in semi)
        for f, name in _FIELD_OF.items():
            a = np.ascontiguousarray(metrics[name], dtype=np.float64)
            self.keep[f] = a
            setattr(self.s, f, _p(a))
        self.set_nvert(nvert)
        self.shape = (mz, my, mx)

    def set_nvert(self, nvert):
        a = np.ascontiguousarray(nvert, dtype=np.float64)
        self.keep["nvert"] = a
        self.s.nvert = _p(a)

    @property
    def nvert(self):
        return self.keep["nvert"]

    def ref(self):
        return ctypes.byref(self.s)


def lhs_csr(L: OLevel):
    import scipy.sparse as sp
    n = int(np.prod(L.shape))
    cap = 19 * n + 16
    rp = np.zeros(n + 1, np.int32)
    cols = np.zeros(cap, np.int32)
    vals = np.zeros(cap)
    nnz = lib().orc_lhs_csr(L.ref(), _p(rp), _p(cols), _p(vals), cap)
    if nnz < 0:
        raise RuntimeError("orc_lhs_csr: capacity")
    return sp.csr_matrix((vals[:nnz].copy(), cols[:nnz].copy(), rp.copy()), shape=(n, n))


def poisson_rhs(L: OLevel, ucont, dt, st):
    b = np.zeros(L.shape)
    uc = np.ascontiguousarray(ucont, dtype=np.float64)
    s = lib().orc_poisson_rhs(L.ref(), _p(uc), dt, st, _p(b))
    return b, s


def volume_flux_rev(L: OLevel, ucont, flux_intp_sum=0.0, flg=1):
    uc = np.array(ucont, dtype=np.float64, copy=True, order="C")
    f = ctypes.c_double()
    a = ctypes.c_double()
    lib().orc_volume_flux_rev(L.ref(), _p(uc), flux_intp_sum, flg, ctypes.byref(f), ctypes.byref(a))
    return uc, f.value, a.value


def nvert_restrict(F: OLevel, coarse_shape, coarse_is_level0, semi=(0, 0, 0)):
    mz, my, mx = coarse_shape
    out = np.zeros(coarse_shape)
    lib().orc_nvert_restrict(F.ref(), mx, my, mz, int(coarse_is_level0), *[int(v) for v in semi], _p(out))
    return out


def fully_blocked(L: OLevel):
    mz, my, mx = L.shape
    k = np.zeros(2 * mx * my, np.int32)
    mns = lib().orc_fully_blocked(L.ref(), _p(k))
    return bool(mns), k


def restrict(F: OLevel, C: OLevel, xf):
    x = np.ascontiguousarray(xf, dtype=np.float64)
    out = np.zeros(C.shape)
    lib().orc_restrict(F.ref(), C.ref(), _p(x), _p(out))
    return out


def interpolate(C: OLevel, F: OLevel, xc):
    x = np.ascontiguousarray(xc, dtype=np.float64)
    out = np.zeros(F.shape)
    lib().orc_interpolate(C.ref(), F.ref(), _p(x), _p(out))
    return out


def nullspace(L: OLevel, x, mns=False, kske=None):
    y = np.array(x, dtype=np.float64, copy=True, order="C")
    k = np.zeros(2, np.int32) if kske is None else np.ascontiguousarray(kske, dtype=np.int32)
    lib().orc_nullspace(L.ref(), int(mns), _p(k), _p(y))
    return y


def update_and_project(L: OLevel, p, phi, ucont, dt, st):
    pp = np.array(p, dtype=np.float64, copy=True, order="C")
    ph = np.array(phi, dtype=np.float64, copy=True, order="C")
    uc = np.array(ucont, dtype=np.float64, copy=True, order="C")
    lib().orc_update_pressure(L.ref(), _p(pp), _p(ph))
    lib().orc_projection(L.ref(), _p(ph), dt, st, _p(uc))
    return pp, ph, uc


def contra2cart(L: OLevel, ucont, ucat):
    """Contra2Cart (rhs.c:25-143): returns the new ucat ([mz][my][mx][3])."""
    uc = np.ascontiguousarray(ucont, dtype=np.float64)
    out = np.array(ucat, dtype=np.float64, copy=True, order="C")
    lib().orc_contra2cart(L.ref(), _p(uc), _p(out))
    return out


def ghost_node_velocity(L: OLevel, ubcs, ucat, cent=None, u_bc=0.0):
    """GhostNodeVelocity (bcs.c:3645-4435): returns (status, ubcs, ucat).
    cent: the cell centres an annulus face (bctype[2] 11) needs; u_bc: the
    rheology plates' velocity (bctype 13)."""
    ub = np.array(ubcs, dtype=np.float64, copy=True, order="C")
    u = np.array(ucat, dtype=np.float64, copy=True, order="C")
    if cent is None:
        rc = lib().orc_ghost_node_velocity_ext(L.ref(), _p(ub), _p(u), None, float(u_bc))
    else:
        c = np.ascontiguousarray(cent, dtype=np.float64)
        rc = lib().orc_ghost_node_velocity_ext(L.ref(), _p(ub), _p(u), _p(c), float(u_bc))
    return rc, ub, u


def divergence(L: OLevel, ucont):
    """Divergence (main.c:469-593): (max |div|, its index in the box)."""
    uc = np.ascontiguousarray(ucont, dtype=np.float64)
    m, at = ctypes.c_double(), ctypes.c_longlong()
    lib().orc_divergence(L.ref(), _p(uc), ctypes.byref(m), ctypes.byref(at))
    return m.value, at.value


def convection(L: OLevel, ucont, ucat, central=0):
    """Convection (rhs.c:1463-1946): (status, conv); status -1 for a periodic
    face, with conv zero."""
    uc = np.ascontiguousarray(ucont, dtype=np.float64)
    u = np.ascontiguousarray(ucat, dtype=np.float64)
    out = np.zeros_like(u)
    rc = lib().orc_convection(L.ref(), _p(uc), _p(u), int(central), _p(out))
    return rc, out


def viscous(L: OLevel, ucat, ren):
    """Viscous (rhs.c:1947-2566), laminar: visc with nu = 1/ren, 0 on the ring."""
    u = np.ascontiguousarray(ucat, dtype=np.float64)
    out = np.zeros_like(u)
    lib().orc_viscous(L.ref(), _p(u), float(ren), _p(out))
    return out


def form_function1(L: OLevel, ucont, ucat, p, ren, central=0, rhs=None):
    """FormFunction1 (rhs.c:2567-3351), walled boxes: (status, rhs, ucat after
    its Contra2Cart); rhs's ring is what was passed (zeros by default)."""
    uc = np.ascontiguousarray(ucont, dtype=np.float64)
    u = np.array(ucat, dtype=np.float64, copy=True, order="C")
    pp = np.ascontiguousarray(p, dtype=np.float64)
    out = np.zeros_like(uc) if rhs is None else np.array(rhs, dtype=np.float64, copy=True, order="C")
    rc = lib().orc_form_function1(L.ref(), _p(uc), _p(u), _p(pp), float(ren), int(central), _p(out))
    return rc, out, u


def calc_rhs(L: OLevel, ucont, ucont_o, ucont_rm1, ucat, p, ren, dt, ti, tistart, central=0, rhs=None):
    """CalcRHS (implicitsolver.c:6449-6713), walled boxes: (status, rhs, ucat)."""
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (ucont, ucont_o, ucont_rm1)]
    u = np.array(ucat, dtype=np.float64, copy=True, order="C")
    pp = np.ascontiguousarray(p, dtype=np.float64)
    out = np.zeros_like(a[0]) if rhs is None else np.array(rhs, dtype=np.float64, copy=True, order="C")
    rc = lib().orc_calc_rhs(L.ref(), *[_p(x) for x in a], _p(u), _p(pp), float(ren), float(dt), int(ti),
                            int(tistart), int(central), _p(out))
    return rc, out, u


class ImpRKStats(ctypes.Structure):
    _fields_ = [("pseudo_iterations", ctypes.c_int), ("rejected", ctypes.c_int), ("norm_du", ctypes.c_double),
                ("rel_du", ctypes.c_double), ("norm_f", ctypes.c_double), ("rel_f", ctypes.c_double),
                ("lambda_", ctypes.c_double)]


def set_inlet_globals(flux_in, ti):
    """Flux_in and ti, which the uniform inlet profiles 3, 6 and 8 read."""
    lib().orc_set_inlet_globals(float(flux_in), int(ti))


_TABLE = None


def set_inlet_table(uinr):
    """The inlet table [101][1001] of the profiles 0 and 5 (None: none); kept
    here while the oracle holds it."""
    global _TABLE
    _TABLE = None if uinr is None else np.ascontiguousarray(uinr, dtype=np.float64).reshape(101, 1001)
    lib().orc_set_inlet_table(None if _TABLE is None else _p(_TABLE))


def inflow_flux(L: OLevel, ucont, ubcs, inletprofile, flux_in_sum=0.0, coor=None, cm=(0.0, 0.0, 0.0)):
    """InflowFlux (bcs.c:99-400), inlet on k = 0, a constant profile or (with
    the node coordinates coor, box layout, and cm = CMx_c, CMy_c, CMz_c) a
    shaped one: (status, ucont, ubcs, FluxInSum)."""
    uc = np.array(ucont, dtype=np.float64, copy=True, order="C")
    ub = np.array(ubcs, dtype=np.float64, copy=True, order="C")
    f = ctypes.c_double(flux_in_sum)
    cmv = np.array(cm, dtype=np.float64)
    co = None if coor is None else np.ascontiguousarray(coor, dtype=np.float64)
    rc = lib().orc_inflow_flux_ext(L.ref(), _p(uc), _p(ub), int(inletprofile), None if co is None else _p(co),
                                   _p(cmv), ctypes.byref(f))
    return rc, uc, ub, f.value


def form_bcs(L: OLevel, ucont, ubcs, ucat, p, flux_in_sum=0.0, flux_intp_sum=0.0):
    """FormBCS (bcs.c:4436-5889): (status, ucont, ubcs, ucat, p)."""
    uc, ub, u, pp = [np.array(x, dtype=np.float64, copy=True, order="C") for x in (ucont, ubcs, ucat, p)]
    rc = lib().orc_form_bcs(L.ref(), _p(uc), _p(ub), _p(u), _p(pp), float(flux_in_sum), float(flux_intp_sum))
    return rc, uc, ub, u, pp


def imp_rk(L: OLevel, ucont, ucont_o, ucont_rm1, ucat, p, ubcs, ren, dt, st, cfl, ti, tistart, central=0,
           atol=1e-7, rtol=1e-4, max_it=50, inletprofile=1, flux_intp_sum=0.0, coor=None, cm=(0.0, 0.0, 0.0)):
    """ImpRK (implicitsolver.c:7094-7257), no immersed body (coor, cm: the
    k = 0 node plane and centre of a shaped inlet profile): (status, ucont,
    ucat, p, stats, ubcs)."""
    co = None if coor is None else np.ascontiguousarray(coor, dtype=np.float64)
    cmv = np.array(cm, dtype=np.float64)
    lib().orc_set_inlet_nodes(None if co is None else _p(co), _p(cmv))
    try:
        return _imp_rk(L, ucont, ucont_o, ucont_rm1, ucat, p, ubcs, ren, dt, st, cfl, ti, tistart, central, atol, rtol,
                       max_it, inletprofile, flux_intp_sum)
    finally:
        lib().orc_set_inlet_nodes(None, None)


def _imp_rk(L, ucont, ucont_o, ucont_rm1, ucat, p, ubcs, ren, dt, st, cfl, ti, tistart, central, atol, rtol, max_it,
            inletprofile, flux_intp_sum):
    uc = np.array(ucont, dtype=np.float64, copy=True, order="C")
    uo, urm = [np.ascontiguousarray(x, dtype=np.float64) for x in (ucont_o, ucont_rm1)]
    ub = np.array(ubcs, dtype=np.float64, copy=True, order="C")
    u = np.array(ucat, dtype=np.float64, copy=True, order="C")
    pp = np.array(p, dtype=np.float64, copy=True, order="C")
    st_ = ImpRKStats()
    rc = lib().orc_imp_rk(L.ref(), _p(uc), _p(uo), _p(urm), _p(u), _p(pp), _p(ub), float(ren), float(dt), float(st),
                          float(cfl), int(ti), int(tistart), int(central), float(atol), float(rtol), int(max_it),
                          int(inletprofile), float(flux_intp_sum), ctypes.byref(st_))
    return rc, uc, u, pp, st_, ub


def metrics_divergence(L: OLevel):
    """MetricsDivergence (metrics.c:1551-1625): (max |div of the metrics|, its
    index in the box)."""
    m, at = ctypes.c_double(), ctypes.c_longlong()
    lib().orc_metrics_divergence(L.ref(), ctypes.byref(m), ctypes.byref(at))
    return m.value, at.value


def ibm_search(cent, xyz, tri, nf, ibi, nbodies, nvert_o, nvert, max_tries=64):
    """The nvert classification of ibm_search_advanced (ibm.c:4197-4740):
    returns (status, nvert); status -1 if some cell found no clean ray."""
    mz, my, mx = cent.shape[:3]
    c = np.ascontiguousarray(cent, dtype=np.float64)
    x = np.ascontiguousarray(xyz, dtype=np.float64)
    t = np.ascontiguousarray(tri, dtype=np.int32)
    n = np.ascontiguousarray(nf, dtype=np.float64)
    no = np.ascontiguousarray(nvert_o, dtype=np.float64)
    out = np.array(nvert, dtype=np.float64, copy=True, order="C")
    rc = lib().orc_ibm_search(mx, my, mz, _p(c), len(x), _p(x), len(t), _p(t), _p(n), ibi, nbodies, _p(no),
                              _p(out), max_tries)
    return rc, out


# ------------------------------------------------------------------ reference
class Reference:
    """The reference's own routines, compiled against the API shim (oracle/_ref/)."""

    def __init__(self, nodes, nlevels, bctype, semi=(0, 0, 0)):
        global _ref
        if _ref is None:
            path = build_reference()
            if path is None:
                raise FileNotFoundError("reference checkout not present")
            _ref = ctypes.CDLL(str(path))
        self.L = _ref
        KM, JM, IM = nodes.shape[:3]
        bc = (ctypes.c_int * 6)(*[int(v) for v in bctype])
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        rc = self.L.ref_init(nlevels, IM, JM, KM, bc, *[int(v) for v in semi], _p(self.nodes))
        if rc:
            raise RuntimeError("ref_init failed")
        self.nlevels = nlevels

    def shape(self, level):
        mx, my, mz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.L.ref_dims(level, ctypes.byref(mx), ctypes.byref(my), ctypes.byref(mz))
        return (mz.value, my.value, mx.value)

    def field(self, level, name, dof=1):
        sh = self.shape(level) + ((3,) if dof == 3 else ())
        out = np.zeros(sh)
        if self.L.ref_get_field(level, name.encode(), _p(out)):
            raise KeyError(name)
        return out

    def set_nvert(self, level, nv):
        a = np.ascontiguousarray(nv, dtype=np.float64)
        self.L.ref_set_nvert(level, _p(a))

    def set_ucont(self, uc):
        a = np.ascontiguousarray(uc, dtype=np.float64)
        self.L.ref_set_ucont(_p(a))

    def restart_write(self, directory, ti, block, nvert, ucont, ucat, p):
        """Ucont_P_Binary_Output (main.c:285) of the finest level's fields into directory."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (nvert, ucont, ucat, p)]
        rc = self.L.ref_restart_write(str(directory).encode(), ti, block, *[_p(a) for a in arrs])
        if rc:
            raise RuntimeError(f"ref_restart_write failed: {rc}")

    def restart_read(self, directory, ti, block):
        """Ucont_P_Binary_Input (main.c:75): (Ucont, P, Nvert_o) as the reference reads them."""
        sh = self.shape(self.nlevels - 1)
        uc, p, nv = np.zeros(sh + (3,)), np.zeros(sh), np.zeros(sh)
        rc = self.L.ref_restart_read(str(directory).encode(), ti, block, _p(uc), _p(p), _p(nv))
        if rc:
            raise RuntimeError(f"ref_restart_read failed: {rc}")
        return uc, p, nv

    def nvert_restrict(self):
        mz, my, mx = self.shape(0)
        mns = ctypes.c_int()
        k = np.zeros(2 * mx * my, np.int32)
        self.L.ref_nvert_restrict(ctypes.byref(mns), _p(k))
        return bool(mns.value), k

    def lhs_csr(self, level):
        import scipy.sparse as sp
        n = int(np.prod(self.shape(level)))
        cap = 19 * n + 16
        rp = np.zeros(n + 1, np.int32)
        cols = np.zeros(cap, np.int32)
        vals = np.zeros(cap)
        nnz = self.L.ref_lhs(level, _p(rp), _p(cols), _p(vals), cap)
        return sp.csr_matrix((vals[:nnz].copy(), cols[:nnz].copy(), rp.copy()), shape=(n, n))

    def volume_flux(self, ucont, flux_intp_sum=0.0, flg=1):
        uc = np.array(ucont, dtype=np.float64, copy=True, order="C")
        f, a = ctypes.c_double(), ctypes.c_double()
        self.L.ref_volume_flux(ctypes.c_double(flux_intp_sum), flg, _p(uc), ctypes.byref(f), ctypes.byref(a))
        return uc, f.value, a.value

    def rhs(self, dt, st):
        b = np.zeros(self.shape(self.nlevels - 1))
        s = ctypes.c_double()
        self.L.ref_rhs(ctypes.c_double(dt), ctypes.c_double(st), _p(b), ctypes.byref(s))
        return b, s.value

    def restrict(self, coarse, xf):
        x = np.ascontiguousarray(xf, dtype=np.float64)
        out = np.zeros(self.shape(coarse))
        self.L.ref_restrict(coarse, _p(x), _p(out))
        return out

    def interpolate(self, fine, xc):
        x = np.ascontiguousarray(xc, dtype=np.float64)
        out = np.zeros(self.shape(fine))
        self.L.ref_interpolate(fine, _p(x), _p(out))
        return out

    def nullspace(self, level, x):
        y = np.array(x, dtype=np.float64, copy=True, order="C")
        self.L.ref_nullspace(level, _p(y))
        return y

    def update_and_project(self, p, phi, ucont, dt, st):
        pp = np.array(p, dtype=np.float64, copy=True, order="C")
        ph = np.array(phi, dtype=np.float64, copy=True, order="C")
        uc = np.array(ucont, dtype=np.float64, copy=True, order="C")
        self.L.ref_update_and_project(ctypes.c_double(dt), ctypes.c_double(st), _p(pp), _p(ph), _p(uc))
        return pp, ph, uc


    def contra2cart(self, ucont, ucat):
        uc = np.ascontiguousarray(ucont, dtype=np.float64)
        out = np.array(ucat, dtype=np.float64, copy=True, order="C")
        self.L.ref_contra2cart(_p(uc), _p(out))
        return out

    def ghost_node_velocity(self, ubcs, ucat, u_bc=0.0):
        """The reference's own GhostNodeVelocity; u_bc is bcs.c's U_bc (the
        rheology plates' velocity), the cell centres its FormMetrics' Cent."""
        ub = np.array(ubcs, dtype=np.float64, copy=True, order="C")
        u = np.array(ucat, dtype=np.float64, copy=True, order="C")
        self.L.ref_set_u_bc(ctypes.c_double(u_bc))
        self.L.ref_ghost_node_velocity(_p(ub), _p(u))
        return ub, u


    def divergence(self, ucont):
        uc = np.ascontiguousarray(ucont, dtype=np.float64)
        m, at = ctypes.c_double(), ctypes.c_int()
        if self.L.ref_divergence(_p(uc), ctypes.byref(m), ctypes.byref(at)):
            raise RuntimeError("ref_divergence failed")
        return m.value, at.value

    def convection(self, ucont, ucat, central=0):
        uc = np.ascontiguousarray(ucont, dtype=np.float64)
        u = np.ascontiguousarray(ucat, dtype=np.float64)
        out = np.zeros_like(u)
        if self.L.ref_convection(_p(uc), _p(u), int(central), _p(out)):
            raise RuntimeError("ref_convection failed")
        return out

    def viscous(self, ucat, ren):
        u = np.ascontiguousarray(ucat, dtype=np.float64)
        out = np.zeros_like(u)
        if self.L.ref_viscous(_p(u), ctypes.c_double(ren), _p(out)):
            raise RuntimeError("ref_viscous failed")
        return out

    def form_function1(self, ucont, ucat, p, ren, central=0, rhs=None):
        uc = np.ascontiguousarray(ucont, dtype=np.float64)
        u = np.array(ucat, dtype=np.float64, copy=True, order="C")
        pp = np.ascontiguousarray(p, dtype=np.float64)
        out = np.zeros_like(uc) if rhs is None else np.array(rhs, dtype=np.float64, copy=True, order="C")
        if self.L.ref_form_function1(_p(uc), _p(u), _p(pp), ctypes.c_double(ren), int(central), _p(out)):
            raise RuntimeError("ref_form_function1 failed")
        return out, u

    def calc_rhs(self, ucont, ucont_o, ucont_rm1, ucat, p, ren, dt, ti, tistart, central=0, rhs=None):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (ucont, ucont_o, ucont_rm1)]
        u = np.array(ucat, dtype=np.float64, copy=True, order="C")
        pp = np.ascontiguousarray(p, dtype=np.float64)
        out = np.zeros_like(a[0]) if rhs is None else np.array(rhs, dtype=np.float64, copy=True, order="C")
        if self.L.ref_calc_rhs(*[_p(x) for x in a], _p(u), _p(pp), ctypes.c_double(ren), ctypes.c_double(dt),
                               int(ti), int(tistart), int(central), _p(out)):
            raise RuntimeError("ref_calc_rhs failed")
        return out, u

    def set_inlet_table(self, uinr):
        """The finest level's InletRead table (r = 0.005 i, uinr [101][1001])."""
        t = np.ascontiguousarray(uinr, dtype=np.float64)
        self.L.ref_set_inlet_table(_p(t))

    def set_inlet_globals(self, flux_in, ti):
        """The reference's Flux_in and ti globals."""
        self.L.ref_set_inlet_globals(ctypes.c_double(flux_in), int(ti))

    def inflow_flux(self, ucont, ubcs, inletprofile, flux_in_sum=0.0, cm=(0.0, 0.0, 0.0)):
        uc, ub = [np.array(x, dtype=np.float64, copy=True, order="C") for x in (ucont, ubcs)]
        f = ctypes.c_double(flux_in_sum)
        self.L.ref_set_cm(ctypes.c_double(cm[0]), ctypes.c_double(cm[1]), ctypes.c_double(cm[2]))
        if self.L.ref_inflow_flux(_p(uc), _p(ub), int(inletprofile), ctypes.byref(f)):
            raise RuntimeError("ref_inflow_flux failed")
        return uc, ub, f.value

    def form_bcs(self, ucont, ubcs, ucat, p, flux_in_sum=0.0, flux_intp_sum=0.0):
        uc, ub, u, pp = [np.array(x, dtype=np.float64, copy=True, order="C") for x in (ucont, ubcs, ucat, p)]
        if self.L.ref_form_bcs(_p(uc), _p(ub), _p(u), _p(pp), ctypes.c_double(flux_in_sum),
                               ctypes.c_double(flux_intp_sum)):
            raise RuntimeError("ref_form_bcs failed")
        return uc, ub, u, pp

    def imp_rk(self, ucont, ucont_o, ucont_rm1, ucat, p, ubcs, ren, dt, st, cfl, ti, tistart, central=0,
               atol=1e-7, rtol=1e-4, max_it=50, inletprofile=1, flux_intp_sum=0.0, cm=(0.0, 0.0, 0.0)):
        """ImpRK through the reference's own routine (cm: CMx_c, CMy_c, CMz_c):
        (ucont, ucat, p, ubcs); it appends to Converge_dU0 in the working
        directory."""
        self.L.ref_set_cm(ctypes.c_double(cm[0]), ctypes.c_double(cm[1]), ctypes.c_double(cm[2]))
        uc = np.array(ucont, dtype=np.float64, copy=True, order="C")
        uo, urm = [np.ascontiguousarray(x, dtype=np.float64) for x in (ucont_o, ucont_rm1)]
        ub = np.array(ubcs, dtype=np.float64, copy=True, order="C")
        u = np.array(ucat, dtype=np.float64, copy=True, order="C")
        pp = np.array(p, dtype=np.float64, copy=True, order="C")
        D = ctypes.c_double
        if self.L.ref_imp_rk(_p(uc), _p(uo), _p(urm), _p(u), _p(pp), _p(ub), D(ren), D(dt), D(st), D(cfl), int(ti),
                             int(tistart), int(central), D(atol), D(rtol), int(max_it), int(inletprofile),
                             D(flux_intp_sum)):
            raise RuntimeError("ref_imp_rk failed")
        return uc, u, pp, ub

    def metrics_divergence(self):
        m, at = ctypes.c_double(), ctypes.c_int()
        if self.L.ref_metrics_divergence(ctypes.byref(m), ctypes.byref(at)):
            raise RuntimeError("ref_metrics_divergence failed")
        return m.value, at.value

    def ibm_search(self, xyz, tri, nf, ibi, nbodies, nvert_o, nvert):
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        t = np.ascontiguousarray(tri, dtype=np.int32)
        n = np.ascontiguousarray(nf, dtype=np.float64)
        no = np.ascontiguousarray(nvert_o, dtype=np.float64)
        out = np.array(nvert, dtype=np.float64, copy=True, order="C")
        rc = self.L.ref_ibm_search(len(x), _p(x), len(t), _p(t), _p(n), ibi, nbodies, _p(no), _p(out))
        if rc:
            raise RuntimeError(f"ref_ibm_search failed: {rc}")
        return out


def solve_mg(levels, b, rtol=1e-8, max_it=500, restart=30, nu=2, threads=0):
    """The reference's solver algorithm on the CPU (cvb_solver.c): FGMRES + PCMG
    with Richardson / block-Jacobi ILU(0).  levels: OLevel list, coarsest first.
    Returns (x, iterations, relres, setup_seconds, solve_seconds)."""
    L = lib()
    f = L.orc_solve_mg
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                  ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p]
    arr = (ctypes.POINTER(Level) * len(levels))(*[ctypes.pointer(l.s) for l in levels])
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(bb.shape)
    rr, ts, tv = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    its = f(len(levels), arr, _p(bb), _p(x), rtol, max_it, restart, nu, threads, ctypes.byref(rr),
            ctypes.byref(ts), ctypes.byref(tv))
    return x, its, rr.value, ts.value, tv.value


def levels_for(problem, nlevels=None):
    """OLevel hierarchy of a workload.Problem, the coarsest ``nlevels`` dropped
    from the top when fewer levels are asked for (the reference's -mg_level)."""
    mets = problem.metrics
    if nlevels is not None:
        mets = mets[len(mets) - nlevels:]
    nl = len(mets)
    Ls = [None] * nl
    Ls[-1] = OLevel(mets[-1], problem.nvert, problem.bctype, problem.semi)
    for l in range(nl - 2, -1, -1):
        Ls[l] = OLevel(mets[l], nvert_restrict(Ls[l + 1], mets[l]["Aj"].shape, l == 0, problem.semi),
                       problem.bctype, problem.semi)
    return Ls
