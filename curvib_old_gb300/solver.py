"""Python front-end of the cvb C ABI, named after the reference routines it replaces.

    ctx = PoissonContext()
    ctx.setup(problem)                       # MG_Initial's hierarchy -> device (once)
    phi, stats = ctx.poisson_solver_mg(ucont, dt, st)   # PoissonSolver_MG (poisson.c:1775)
    ctx.update_pressure(p, phi)              # UpdatePressure (poisson.c:2908)
    ctx.projection(phi, dt, st, ucont)       # Projection (poisson.c:2281)

Every call goes through libcvb.so; errors raise CvbError with the library's message.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import CvbError, LevelDesc, default_opts, ptr

_FIELDS = {"icsi": "ICsi", "ieta": "IEta", "izet": "IZet", "jcsi": "JCsi", "jeta": "JEta", "jzet": "JZet",
           "kcsi": "KCsi", "keta": "KEta", "kzet": "KZet", "iaj": "IAj", "jaj": "JAj", "kaj": "KAj",
           "aj": "Aj", "csi": "Csi", "eta": "Eta", "zet": "Zet"}


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class PoissonContext:
    """One CURVIB block's pressure-projection path resident on one GPU."""

    def __init__(self, device: int = 0, stream=None):
        L = _lib.lib()
        self._L = L
        self._ctx = ctypes.c_void_p()
        o = _lib.Options()
        o.device = device
        o.stream = stream
        rc = L.cvb_init(ctypes.byref(self._ctx), ctypes.byref(o))
        if rc:
            msg = L.cvb_last_error(self._ctx).decode()
            L.cvb_destroy(self._ctx)
            self._ctx = None
            raise CvbError(rc, msg)
        self._keep = []
        self.shapes = []

    def close(self):
        if getattr(self, "_ctx", None):
            self._L.cvb_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise CvbError(rc, self._L.cvb_last_error(self._ctx).decode())

    # ------------------------------------------------------------------ setup
    def _descs(self, problem, ghosts):
        levels = problem.metrics
        n = len(levels)
        descs = (LevelDesc * n)()
        keep = []
        for l, m in enumerate(levels):
            d = descs[l]
            mz, my, mx = m["Aj"].shape[:3] if ghosts is None else problem.box_shapes[l]
            d.mx, d.my, d.mz = mx, my, mz
            if ghosts is None:
                d.gxs = d.gys = d.gzs = 0
                d.gxm, d.gym, d.gzm = mx, my, mz
            else:
                gx, gy, gz = ghosts[l]
                d.gxs, d.gys, d.gzs = gx, gy, gz
                sh = m["Aj"].shape
                d.gzm, d.gym, d.gxm = sh[0], sh[1], sh[2]
            for q in range(6):
                d.bctype[q] = int(problem.bctype[q])
            d.isc, d.jsc, d.ksc = (int(v) for v in problem.semi)
            for f, nm in _FIELDS.items():
                if nm in m and (nm not in ("Csi", "Eta", "Zet") or l == n - 1):
                    a = _c64(m[nm])
                    keep.append(a)
                    setattr(d, f, ptr(a))
        return n, descs, keep

    def _dims(self, n):
        self.shapes = []
        for l in range(n):
            a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            self._L.cvb_level_dims(self._ctx, l, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
            self.shapes.append((c.value, b.value, a.value))
        self.nlevels = n

    def setup_geometry(self, problem, ghosts=None):
        """Upload a grid's metrics only (a donor for setup_like; cannot solve)."""
        n, descs, keep = self._descs(problem, ghosts)
        self._check(self._L.cvb_setup_geometry(self._ctx, n, descs))
        self.shapes = [tuple(m["Aj"].shape[:3]) for m in problem.metrics] if ghosts is None else \
            list(problem.box_shapes)
        self.nlevels = n
        return self

    def setup(self, problem, ghosts=None):
        """Upload the hierarchy of a workload.Problem (levels coarsest first).

        ``ghosts``: optional per-level (gxs, gys, gzs) offsets; the arrays of the
        problem are then expected to be ghosted local arrays of that box.
        """
        n, descs, keep = self._descs(problem, ghosts)
        nv = _c64(problem.nvert)
        keep.append(nv)
        self._check(self._L.cvb_setup_hierarchy(self._ctx, n, descs, ptr(nv)))
        self._dims(n)
        return self

    def set_nvert(self, nvert):
        a = _c64(nvert)
        self._check(self._L.cvb_set_nvert(self._ctx, ptr(a)))

    def get_nvert(self, level):
        out = np.zeros(self.shapes[level])
        mns = ctypes.c_int()
        self._check(self._L.cvb_get_nvert(self._ctx, level, ptr(out), ctypes.byref(mns)))
        return out, bool(mns.value)

    # --------------------------------------------------------------- the path
    def volume_flux_rev(self, ucont, flux_intp_sum=0.0, flg=1):
        uc = np.array(ucont, dtype=np.float64, order="C", copy=True)
        f, a = ctypes.c_double(), ctypes.c_double()
        self._check(self._L.cvb_volume_flux_rev(self._ctx, ptr(uc), flux_intp_sum, flg, ctypes.byref(f),
                                                ctypes.byref(a)))
        return uc, f.value, a.value

    def poisson_rhs(self, ucont, dt, st):
        uc = _c64(ucont)
        b = np.zeros(self.shapes[-1])
        s = ctypes.c_double()
        self._check(self._L.cvb_poisson_rhs(self._ctx, ptr(uc), dt, st, ptr(b), ctypes.byref(s)))
        return b, s.value

    def solve(self, b, phi0=None, check=True, **opts):
        o = default_opts(**opts)
        bb = _c64(b)
        phi = np.zeros(self.shapes[-1]) if phi0 is None else np.array(phi0, dtype=np.float64, order="C", copy=True)
        if phi0 is not None:
            o.warm_start = 1
        st = _lib.SolveStats()
        rc = self._L.cvb_poisson_solve(self._ctx, ptr(bb), ptr(phi), ctypes.byref(o), ctypes.byref(st))
        if check and rc not in (0,):
            raise CvbError(rc, self._L.cvb_last_error(self._ctx).decode())
        return phi, st.as_dict()

    def poisson_solver_mg(self, ucont, dt, st, immersed=1, flux_intp_sum=0.0, **opts):
        """PoissonSolver_MG: VolumeFlux_rev, PoissonRHS and the solve.  Returns
        (phi, corrected ucont, stats)."""
        o = default_opts(**opts)
        uc = np.array(ucont, dtype=np.float64, order="C", copy=True)
        phi = np.zeros(self.shapes[-1])
        s = _lib.SolveStats()
        self._check(self._L.cvb_poisson_solver_mg(self._ctx, ptr(uc), flux_intp_sum, immersed, dt, st, ptr(phi),
                                                  ctypes.byref(o), ctypes.byref(s)))
        return phi, uc, s.as_dict()

    def update_pressure(self, p, phi):
        pp = np.array(p, dtype=np.float64, order="C", copy=True)
        ph = np.array(phi, dtype=np.float64, order="C", copy=True)
        self._check(self._L.cvb_update_pressure(self._ctx, ptr(pp), ptr(ph)))
        return pp, ph

    def projection(self, phi, dt, st, ucont):
        uc = np.array(ucont, dtype=np.float64, order="C", copy=True)
        self._check(self._L.cvb_projection(self._ctx, ptr(_c64(phi)), dt, st, ptr(uc)))
        return uc

    def contra2cart(self, ucont, ucat):
        """Contra2Cart (rhs.c:25): returns the new ucat ([mz][my][mx][3])."""
        out = np.array(ucat, dtype=np.float64, order="C", copy=True)
        self._check(self._L.cvb_contra2cart(self._ctx, ptr(_c64(ucont)), ptr(out)))
        return out

    def ghost_node_velocity(self, ubcs, ucat):
        """GhostNodeVelocity (bcs.c:3645): returns (ubcs, ucat)."""
        ub = np.array(ubcs, dtype=np.float64, order="C", copy=True)
        u = np.array(ucat, dtype=np.float64, order="C", copy=True)
        self._check(self._L.cvb_ghost_node_velocity(self._ctx, ptr(ub), ptr(u)))
        return ub, u

    def divergence(self, ucont=None):
        """Divergence (main.c:469): (max |div|, its index in the box); ucont None
        uses the device copy the last projection left."""
        m, at = ctypes.c_double(), ctypes.c_longlong()
        self._check(self._L.cvb_divergence(self._ctx, None if ucont is None else ptr(_c64(ucont)), ctypes.byref(m),
                                           ctypes.byref(at)))
        return m.value, at.value

    def convection(self, ucont=None, ucat=None, central=False):
        """Convection (rhs.c:1463): the convective term at the cell centres,
        [mz][my][mx][3]; None for ucont / ucat uses the device copies the last
        projection left."""
        shape = tuple(self.shapes[-1]) + (3,)
        out = np.empty(shape, dtype=np.float64)
        self._check(self._L.cvb_convection(self._ctx, None if ucont is None else ptr(_c64(ucont)),
                                           None if ucat is None else ptr(_c64(ucat)), int(bool(central)), ptr(out)))
        return out

    def viscous(self, ucat, ren):
        """Viscous (rhs.c:1947), laminar: visc [mz][my][mx][3]."""
        u = None if ucat is None else _c64(ucat)
        out = np.zeros(self.shapes[-1] + (3,))
        self._check(self._L.cvb_viscous(self._ctx, None if u is None else ptr(u), float(ren), ptr(out)))
        return out

    def form_function1(self, ucont, ucat, p, ren, central=False, rhs=None):
        """FormFunction1 (rhs.c:2567): (rhs, ucat after its Contra2Cart)."""
        uc = _c64(ucont)
        u = np.array(ucat, dtype=np.float64, copy=True, order="C")
        out = np.zeros(uc.shape) if rhs is None else np.array(rhs, dtype=np.float64, copy=True, order="C")
        self._check(self._L.cvb_form_function1(self._ctx, ptr(uc), ptr(u), ptr(_c64(p)), float(ren), int(central),
                                               ptr(out)))
        return out, u

    def calc_rhs(self, ucont, ucont_o, ucont_rm1, ucat, p, ren, dt, ti, tistart, central=False, rhs=None):
        """CalcRHS (implicitsolver.c:6449): (rhs, ucat after its Contra2Cart)."""
        uc, uo, urm = _c64(ucont), _c64(ucont_o), _c64(ucont_rm1)
        u = np.array(ucat, dtype=np.float64, copy=True, order="C")
        out = np.zeros(uc.shape) if rhs is None else np.array(rhs, dtype=np.float64, copy=True, order="C")
        self._check(self._L.cvb_calc_rhs(self._ctx, ptr(uc), ptr(uo), ptr(urm), ptr(u), ptr(_c64(p)), float(ren),
                                         float(dt), int(ti), int(tistart), int(central), ptr(out)))
        return out, u

    def set_cell_centres(self, cent):
        """The finest level's cell centres, for an annulus face (bctype[2] 11)."""
        self._check(self._L.cvb_set_cell_centres(self._ctx, ptr(_c64(cent))))

    def set_plate_velocity(self, u_bc):
        """The rheology plates' velocity (bctype 13), bcs.c's U_bc."""
        self._check(self._L.cvb_set_plate_velocity(self._ctx, float(u_bc)))

    def set_inlet_nodes(self, coor0, cm=(0.0, 0.0, 0.0)):
        """The k = 0 node plane ([my][mx][3]) and CMx_c, CMy_c, CMz_c for the
        shaped inlet profiles 2, 4, 7 and 10 (bcs.c:152-195)."""
        c = np.ascontiguousarray(coor0, dtype=np.float64)
        self._check(self._L.cvb_set_inlet_nodes(self._ctx, ptr(c), float(cm[0]), float(cm[1]), float(cm[2])))

    def set_inlet_flux(self, flux_in, ti):
        """Flux_in and ti for the uniform inlet profiles 3, 6 and 8
        (bcs.c:67-82)."""
        self._check(self._L.cvb_set_inlet_flux(self._ctx, float(flux_in), int(ti)))

    def set_inlet_table(self, uinr):
        """InletRead's table uinr [101][1001] for the inlet profiles 0 and 5
        (bcs.c:40-96)."""
        t = np.ascontiguousarray(uinr, dtype=np.float64)
        if t.size != 101 * 1001:
            raise ValueError("uinr must hold 101 x 1001 values")
        self._check(self._L.cvb_set_inlet_table(self._ctx, ptr(t)))

    def inlet_flux_in(self):
        """Flux_in as the last InflowFlux left it (profile 8 sets it)."""
        return self._L.cvb_inlet_flux_in(self._ctx)

    def inflow_flux(self, ucont, ubcs, inletprofile, flux_in_sum=0.0):
        """InflowFlux (bcs.c:99): (ucont, ubcs, FluxInSum)."""
        uc, ub = [np.array(x, dtype=np.float64, copy=True, order="C") for x in (ucont, ubcs)]
        f = ctypes.c_double(flux_in_sum)
        self._check(self._L.cvb_inflow_flux(self._ctx, ptr(uc), ptr(ub), int(inletprofile), ctypes.byref(f)))
        return uc, ub, f.value

    def form_bcs(self, ucont, ubcs, ucat, p, flux_in_sum=0.0, flux_intp_sum=0.0):
        """FormBCS (bcs.c:4436): (ucont, ubcs, ucat, p)."""
        uc, ub, u, pp = [np.array(x, dtype=np.float64, copy=True, order="C") for x in (ucont, ubcs, ucat, p)]
        self._check(self._L.cvb_form_bcs(self._ctx, ptr(uc), ptr(ub), ptr(u), ptr(pp), float(flux_in_sum),
                                         float(flux_intp_sum)))
        return uc, ub, u, pp

    def imp_rk(self, ucont, ucont_o, ucont_rm1, ucat, p, ubcs, ren, dt, st, cfl, ti, tistart, central=False,
               atol=1e-7, rtol=1e-4, max_it=50, inletprofile=1, flux_intp_sum=0.0):
        """ImpRK (implicitsolver.c:7094) with no immersed body: (ucont, ucat, p,
        stats dict, ubcs)."""
        uc, u, pp, ub = [np.array(x, dtype=np.float64, copy=True, order="C") for x in (ucont, ucat, p, ubcs)]
        o = _lib.imp_rk_opts(ren=float(ren), dt=float(dt), st=float(st), cfl=float(cfl), ti=int(ti),
                             tistart=int(tistart), central=int(central), imp_atol=float(atol), imp_rtol=float(rtol),
                             imp_max_it=int(max_it), inletprofile=int(inletprofile),
                             flux_intp_sum=float(flux_intp_sum))
        st_ = _lib.ImpRKStats()
        self._check(self._L.cvb_imp_rk(self._ctx, ptr(uc), ptr(_c64(ucont_o)), ptr(_c64(ucont_rm1)), ptr(u), ptr(pp),
                                       ptr(ub), ctypes.byref(o), ctypes.byref(st_)))
        return uc, u, pp, st_.as_dict(), ub

    def metrics_divergence(self):
        """MetricsDivergence (metrics.c:1551): (max |div of the metrics|, its
        index in the box) on the finest level."""
        m, at = ctypes.c_double(), ctypes.c_longlong()
        self._check(self._L.cvb_metrics_divergence(self._ctx, ctypes.byref(m), ctypes.byref(at)))
        return m.value, at.value

    def ibm_search(self, cent, xyz, tri, nf, ibi, nbodies, nvert_o, nvert):
        """ibm_search_advanced's nvert classification (ibm.c:4197): returns the
        new nvert ([mz][my][mx]) of body ibi of nbodies.  cent None reuses the
        cell centres of an earlier call."""
        out = np.array(nvert, dtype=np.float64, order="C", copy=True)
        x = _c64(xyz)
        t = np.ascontiguousarray(tri, dtype=np.int32)
        c = None if cent is None else _c64(cent)
        self._check(self._L.cvb_ibm_search(self._ctx, None if c is None else ptr(c), len(x), ptr(x), len(t), ptr(t),
                                           ptr(_c64(nf)),
                                           ibi, nbodies, ptr(_c64(nvert_o)), ptr(out)))
        return out

    def projection_cart(self, phi, dt, st, ucont, ubcs, ucat):
        """Projection, Contra2Cart and GhostNodeVelocity in one call: returns
        (ucont, ubcs, ucat)."""
        uc = np.array(ucont, dtype=np.float64, order="C", copy=True)
        ub = np.array(ubcs, dtype=np.float64, order="C", copy=True)
        u = np.array(ucat, dtype=np.float64, order="C", copy=True)
        self._check(self._L.cvb_projection_cart(self._ctx, ptr(_c64(phi)), dt, st, ptr(uc), ptr(ub), ptr(u)))
        return uc, ub, u

    # ------------------------------------------------------- resident solves
    def device_rhs(self):
        return self._L.cvb_device_rhs(self._ctx)

    def device_phi(self):
        return self._L.cvb_device_phi(self._ctx)

    def stream(self):
        return self._L.cvb_stream(self._ctx)

    def solve_resident(self, check=True, **opts):
        o = default_opts(**opts)
        st = _lib.SolveStats()
        rc = self._L.cvb_solve_resident(self._ctx, ctypes.byref(o), ctypes.byref(st))
        if check and rc:
            raise CvbError(rc, self._L.cvb_last_error(self._ctx).decode())
        return st.as_dict()

    def set_rhs(self, b):
        """Copy a host right-hand side into the resident rhs."""
        self._check(self._L.cvb_set_rhs(self._ctx, ptr(_c64(b))))

    def set_phi(self, phi):
        """Copy a host pressure into the resident phi (a warm start's initial guess)."""
        self._check(self._L.cvb_set_phi(self._ctx, ptr(_c64(phi))))

    def get_phi(self):
        """The resident solution, copied to the host."""
        phi = np.zeros(self.shapes[-1])
        self._check(self._L.cvb_get_phi(self._ctx, ptr(phi)))
        return phi

    def setup_like(self, donor, nvert):
        """Set up on the grid of a set-up donor context (its resident metrics are
        shared) with this problem's finest-level nvert."""
        nv = _c64(nvert)
        self._check(self._L.cvb_setup_like(self._ctx, donor._ctx, ptr(nv)))
        self.shapes = list(donor.shapes)
        self.nlevels = donor.nlevels
        return self

    def device_bytes(self):
        """Device memory held by this context alone."""
        v = ctypes.c_ulonglong()
        self._check(self._L.cvb_device_bytes(self._ctx, ctypes.byref(v)))
        return int(v.value)

    def geometry_bytes(self):
        """(bytes, id) of the grid metrics this context shares."""
        v, i = ctypes.c_ulonglong(), ctypes.c_ulonglong()
        self._check(self._L.cvb_geometry_bytes(self._ctx, ctypes.byref(v), ctypes.byref(i)))
        return int(v.value), int(i.value)

    def tuning(self):
        """The set-up autotuner's measurements and choices (dict)."""
        import json
        buf = ctypes.create_string_buffer(1 << 16)
        self._check(self._L.cvb_tuning_report(self._ctx, buf, len(buf)))
        return json.loads(buf.value.decode())

    def time_kernel(self, name, level=-1, reps=20):
        """(average ms per launch, algorithmic bytes per launch) of one kernel."""
        lvl = level % self.nlevels
        ms, by = ctypes.c_double(), ctypes.c_double()
        self._check(self._L.cvb_time_kernel(self._ctx, _lib.KERNELS[name], lvl, reps, ctypes.byref(ms),
                                            ctypes.byref(by)))
        return ms.value, by.value

    # ---------------------------------------------------------- parity hooks
    def apply(self, level, x):
        xx = _c64(x)
        y = np.zeros(self.shapes[level])
        self._check(self._L.cvb_apply_operator(self._ctx, level, ptr(xx), ptr(y)))
        return y

    def apply_f32(self, level, x):
        xx = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros(self.shapes[level], dtype=np.float32)
        self._check(self._L.cvb_apply_operator_f32(self._ctx, level, ptr(xx), ptr(y)))
        return y

    def set_device_limit(self, nbytes):
        """Cap the device memory this context may allocate (0: no cap)."""
        self._check(self._L.cvb_set_device_limit(self._ctx, int(nbytes)))

    def level_cross(self, level):
        """(FP32, FP64) flags: the level's operator has cross-derivative terms."""
        a, b = ctypes.c_int(), ctypes.c_int()
        self._check(self._L.cvb_level_cross(self._ctx, level, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    ZEBRA_FORMS = {"split": 0, "fused": 1, "split4": 2, "fused4": 3, "tma4": 4, "tma8": 8, "tma16": 16}

    def zebra_half_f32(self, level, form, color, b, x, omega=1.3):
        """One FP32 zebra half-sweep of x (returned) in the named form."""
        xb = np.ascontiguousarray(x, dtype=np.float32).copy()
        bb = np.ascontiguousarray(b, dtype=np.float32)
        rc = self._L.cvb_zebra_half_f32(self._ctx, level, self.ZEBRA_FORMS[form], color, omega, ptr(bb), ptr(xb))
        if rc:
            raise CvbError(rc, self._L.cvb_last_error(self._ctx).decode())
        return xb

    def setup_times(self):
        """Milliseconds of the last set-up by phase: metrics upload, level
        arrays, operators, autotuner, coarsest solver."""
        v = np.zeros(5)
        self._check(self._L.cvb_setup_times(self._ctx, ptr(v)))
        return dict(zip(("metrics_upload", "level_arrays", "operators", "autotuner", "coarse_solver"),
                        (float(x) for x in v)))

    def weights(self, level):
        w = np.zeros((19,) + self.shapes[level])
        self._check(self._L.cvb_get_weights(self._ctx, level, ptr(w)))
        return w

    def restrict(self, coarse, xf):
        out = np.zeros(self.shapes[coarse])
        self._check(self._L.cvb_restrict(self._ctx, coarse, ptr(_c64(xf)), ptr(out)))
        return out

    def interpolate(self, fine, xc):
        out = np.zeros(self.shapes[fine])
        self._check(self._L.cvb_interpolate(self._ctx, fine, ptr(_c64(xc)), ptr(out)))
        return out

    def nullspace(self, level, x):
        y = np.array(x, dtype=np.float64, order="C", copy=True)
        self._check(self._L.cvb_nullspace(self._ctx, level, ptr(y)))
        return y


class SolveBatch:
    """Many solves at once on set-up PoissonContexts (cvb_batch_*).

    ``solve(ctxs)`` runs a fixed set to completion; ``submit`` / ``step`` /
    ``poll`` run a stream of solves with continuous batching.  Precision,
    restart, sweeps and omega are batch-wide (``opts``); tolerances per solve.
    """

    def __init__(self, device: int = 0, stream=None, **opts):
        L = _lib.lib()
        self._L = L
        self._b = ctypes.c_void_p()
        o = _lib.Options()
        o.device = device
        o.stream = stream
        self.opts = default_opts(**opts)
        rc = L.cvb_batch_create(ctypes.byref(self._b), ctypes.byref(o), ctypes.byref(self.opts))
        if rc:
            raise CvbError(rc, "cvb_batch_create failed")
        self._ctx_of = {}
        self._keep = {}

    def close(self):
        if getattr(self, "_b", None):
            self._L.cvb_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise CvbError(rc, self._L.cvb_batch_last_error(self._b).decode())

    def submit(self, ctx, b=None, rtol=None, atol=None, max_it=None, warm_start=False, project_rhs=True):
        """Queue a solve of ``ctx``'s resident rhs (or of ``b``); returns its ticket."""
        t = ctypes.c_int()
        bb = None if b is None else _c64(b)
        self._check(self._L.cvb_batch_submit(
            self._b, ctx._ctx, None if bb is None else ptr(bb),
            self.opts.rtol if rtol is None else rtol, self.opts.atol if atol is None else atol,
            self.opts.max_it if max_it is None else max_it, int(warm_start), int(project_rhs), ctypes.byref(t)))
        self._ctx_of[t.value] = ctx
        if bb is not None:
            self._keep[t.value] = bb
        return t.value

    def step(self):
        """Admit queued solves and issue one round; returns the solves still in flight."""
        n = ctypes.c_int()
        self._check(self._L.cvb_batch_step(self._b, ctypes.byref(n)))
        return n.value

    def poll(self):
        """[(ticket, stats dict), ...] of the solves that finished so far."""
        out = []
        while True:
            t = ctypes.c_int()
            st = _lib.SolveStats()
            self._check(self._L.cvb_batch_poll(self._b, ctypes.byref(t), ctypes.byref(st)))
            if t.value < 0:
                return out
            self._keep.pop(t.value, None)
            self._ctx_of.pop(t.value, None)
            out.append((t.value, st.as_dict()))

    def read_phi(self, ctx):
        phi = np.zeros(ctx.shapes[-1])
        self._check(self._L.cvb_batch_read_phi(self._b, ctx._ctx, ptr(phi)))
        return phi

    def set_round_limit(self, rounds):
        """Bound ``solve``'s loop to ``rounds`` rounds (0: the default); past it
        ``solve`` raises CVB_TIMEOUT with the unfinished solves still in flight."""
        self._check(self._L.cvb_batch_set_round_limit(self._b, int(rounds)))

    def set_graphs(self, on):
        """Replay the mixed rounds' V-cycles from CUDA graphs (on by default)."""
        self._check(self._L.cvb_batch_set_graphs(self._b, 1 if on else 0))

    def graph_stats(self):
        """{"captures", "updates", "replays"} of the V-cycle graphs so far."""
        v = [ctypes.c_longlong() for _ in range(3)]
        self._check(self._L.cvb_batch_graph_stats(self._b, *[ctypes.byref(q) for q in v]))
        return {"captures": v[0].value, "updates": v[1].value, "replays": v[2].value}

    def solve(self, ctxs):
        """Solve every context's resident rhs; returns their stats in order."""
        n = len(ctxs)
        arr = (ctypes.c_void_p * n)(*[c._ctx.value for c in ctxs])
        sts = (_lib.SolveStats * n)()
        rc = self._L.cvb_batch_solve(self._b, n, arr, sts)
        out = [s.as_dict() for s in sts]
        if rc:
            raise CvbError(rc, self._L.cvb_batch_last_error(self._b).decode())
        return out

