"""Device-resident multigrid and model steppers (Python side of the engine).

``Gmg``   -- core/gmg/hierarchy.py's Gmg: ``twoVcycle(x, b)`` and
             ``solve(x, b, param)`` on CUDA tensors, same names and argument
             meaning (x updated in place).
``Model`` -- an Euler / Boussinesq / QG model whose state lives on the GPU,
             with the reference's model API: ``var.state``, ``get(name)``,
             ``step(t, dt)``, ``diagnostics(var, t)``, ``diags``,
             ``set_psi_from_vorticity()``.  ``run(nsteps)`` chains the loop
             body of core/fluid2d.py:237-268 (set_dt, step, diagnostics) with
             no host synchronisation, optionally replaying a CUDA graph.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from . import workloads

MODEL_KIND = {"euler": 0, "boussinesq": 1, "quasigeostrophic": 2}


class _DevArray(object):
    """__cuda_array_interface__ view of library-owned device memory."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3,
                                         "strides": None}


def device_view(ptr, shape, dtype=torch.float64):
    ts = {torch.float64: "<f8", torch.int8: "|i1", torch.float32: "<f4"}[dtype]
    return torch.as_tensor(_DevArray(ptr, shape, ts), device="cuda")


def _stream():
    return torch.cuda.current_stream().cuda_stream


class Gmg(object):
    """Geometric multigrid of core/gmg/hierarchy.py on the GPU.

    ``mskp`` is the corner mask (core/operators.py:59-67), int8 (ny+6, nx+6)."""

    def __init__(self, mskp, nx, ny, dx, dy, hydroepsilon=1., qgoperator=False, Rd=1.,
                 variant="product"):
        self.variant = variant
        self.L = _lib.lib(variant)
        m = np.ascontiguousarray(np.asarray(mskp).astype(np.int8))
        h = ctypes.c_void_p()
        self._call("f2d_gmg_create", m.ctypes.data, int(nx), int(ny), float(dx), float(dy),
                   float(hydroepsilon), int(bool(qgoperator)), float(Rd), ctypes.byref(h))
        self.h = h
        nlev, cs = ctypes.c_int(), ctypes.c_int()
        mv = (ctypes.c_int * 32)()
        nv = (ctypes.c_int * 32)()
        self._call("f2d_gmg_levels", self.h, ctypes.byref(nlev), mv, nv, ctypes.byref(cs))
        self.nlevs = nlev.value
        self.coarse_level = cs.value
        self.shapes = [(mv[k], nv[k]) for k in range(self.nlevs)]

    def _call(self, name, *args):
        _lib.call(name, *args, variant=self.variant)

    def level_array(self, lev, which):
        ptr = self.L.f2d_gmg_level_ptr(self.h, lev, which.encode())
        if not ptr:
            raise KeyError(which)
        mv, nv = self.shapes[lev]
        if which == "msk":
            return device_view(ptr, (mv, nv), torch.int8)
        if which == "A":
            return device_view(ptr, (6, mv, nv))
        return device_view(ptr, (mv, nv))

    def twoVcycle(self, x, b, param=None):
        """core/gmg/hierarchy.py:207-218; x (warm start) updated in place."""
        self._call("f2d_gmg_twovcycle", self.h, x.data_ptr(), b.data_ptr(), _stream())
        return 1, 0.

    def solve(self, x, b, param=None):
        """core/gmg/hierarchy.py:154-192; returns (nite, res) (synchronises)."""
        param = param or {"maxite": 4, "tol": 1e-11}
        self._call("f2d_gmg_solve", self.h, x.data_ptr(), b.data_ptr(), int(param["maxite"]),
                   float(param["tol"]), _stream())
        torch.cuda.current_stream().synchronize()
        nite, res, st = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
        self._call("f2d_gmg_solve_stats", self.h, ctypes.byref(nite), ctypes.byref(res),
                   ctypes.byref(st))
        if st.value:
            raise _lib.F2DError("solve", st.value, "solver is not converging")
        return nite.value, res.value

    def Vcycle(self, lev1):
        self._call("f2d_gmg_vcycle", self.h, int(lev1), _stream())

    def Fcycle(self, lev1):
        self._call("f2d_gmg_fcycle", self.h, int(lev1), _stream())

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.L.f2d_gmg_destroy(self.h)
        except Exception:
            pass


# status word bits (include/fluid2d_gb300.h F2D_STATUS_*)
STATUS_NAMES = {1: "non-finite values", 2: "blow-up (maxspeed > 1e3)",
                4: "multigrid solve diverged", 8: "bad time step"}


def status_text(bits):
    return ", ".join(v for k, v in sorted(STATUS_NAMES.items()) if bits & k) or "ok"


def statuses(models, clear=False):
    """The status words of many models, read with one synchronisation."""
    if not models:
        return []
    arr = (ctypes.c_void_p * len(models))(*[m.h.value for m in models])
    out = (ctypes.c_int * len(models))()
    _lib.call("f2d_models_status", arr, len(models), int(bool(clear)), out, _stream(),
              variant=models[0].variant)
    return list(out)


class _Var(object):
    def __init__(self, state, names):
        self.state = state
        self.varname_list = names

    def get(self, name):
        return self.state[self.varname_list.index(name)]


class Model(object):
    """A Fluid2d model (Euler, Boussinesq or QG) stepped on the GPU."""

    def __init__(self, modelname="euler", nx=128, ny=128, Lx=1., Ly=1., geometry="closed",
                 msk=None, order=5, flux_splitting_method="parabolic", aparab=0.05,
                 gravity=1., Rd=1., beta=0., hydroepsilon=1., adaptable_dt=False, dt=0.1,
                 cfl=0.5, dtmax=5., precision="fp64", variant="product", diffusion=False,
                 Kdiff=0., noslip=False, msknoslip=None):
        self.variant = variant
        self.L = _lib.lib(variant)
        self.modelname = modelname
        if msk is None:
            msk = workloads.base_mask(nx, ny, geometry)
        self.msk = np.ascontiguousarray(msk, dtype=np.int8)
        d = _lib.ModelDesc()
        d.model = MODEL_KIND[modelname]
        d.nx, d.ny, d.Lx, d.Ly = int(nx), int(ny), float(Lx), float(Ly)
        d.perio = int(geometry == "perio")
        d.order = int(order)
        d.flux_method = 0 if flux_splitting_method == "minmax" else 1
        d.aparab, d.gravity, d.Rd, d.beta = float(aparab), float(gravity), float(Rd), float(beta)
        d.hydroepsilon = float(hydroepsilon)
        d.adaptable_dt = int(bool(adaptable_dt))
        d.dt, d.cfl, d.dtmax = float(dt), float(cfl), float(dtmax)
        d.precision = {"fp64": 0, "mixed": 1}[precision]
        # Kdiff: one value for every tracer, or {tracer: value}
        # (core/operators.py:146-152)
        d.diffusion = int(bool(diffusion))
        tracers = {"euler": ["vorticity"], "boussinesq": ["vorticity", "buoyancy"],
                   "quasigeostrophic": ["pv"]}[modelname]
        for q, tr in enumerate(tracers):
            d.Kdiff[q] = float(Kdiff[tr] if isinstance(Kdiff, dict) else Kdiff)
        self.desc = d
        h = ctypes.c_void_p()
        self._call("f2d_model_create", ctypes.byref(d), self.msk.ctypes.data, ctypes.byref(h))
        self.h = h
        nvar, mv, nv, nlev, cs = (ctypes.c_int() for _ in range(5))
        st, dg = ctypes.POINTER(ctypes.c_double)(), ctypes.POINTER(ctypes.c_double)()
        self._call("f2d_model_info", self.h, ctypes.byref(nvar), ctypes.byref(mv),
                   ctypes.byref(nv), ctypes.byref(nlev), ctypes.byref(cs), ctypes.byref(st),
                   ctypes.byref(dg))
        self.nvar, self.nyl, self.nxl = nvar.value, mv.value, nv.value
        self.nlevs, self.coarse_level = nlev.value, cs.value
        names = [self.L.f2d_model_varname(self.h, k).decode() for k in range(self.nvar)]
        self.var = _Var(device_view(ctypes.cast(st, ctypes.c_void_p).value,
                                    (self.nvar, self.nyl, self.nxl)), names)
        self.diag_names = []
        k = 0
        while True:
            nm = self.L.f2d_model_diagname(self.h, k)
            if nm is None:
                break
            self.diag_names.append(nm.decode())
            k += 1
        self._diag = device_view(ctypes.cast(dg, ctypes.c_void_p).value, (8,))
        self.diags = {}
        self.dx, self.dy = d.Lx / d.nx, d.Ly / d.ny
        if noslip:
            # the no-slip walls: the geometry's mask before islands are carved
            # (core/grid.py:101), unless given
            mns = workloads.base_mask(nx, ny, geometry) if msknoslip is None else msknoslip
            self.msknoslip = np.ascontiguousarray(mns, dtype=np.int8)
            self._call("f2d_model_noslip", self.h, self.msknoslip.ctypes.data, _stream())

    def _call(self, name, *args):
        _lib.call(name, *args, variant=self.variant)

    def buffer(self, which):
        ptr = self.L.f2d_model_buffer(self.h, which.encode())
        if which in ("state", "dx0", "dx1", "dx2"):
            return device_view(ptr, (self.nvar, self.nyl, self.nxl))
        if which == "work":
            return device_view(ptr, (self.nyl, self.nxl))
        return device_view(ptr, (8,))

    def get(self, name):
        return self.var.get(name)

    def set_psi_from_vorticity(self):
        self._call("f2d_model_set_psi", self.h, _stream())

    set_psi_from_pv = set_psi_from_vorticity

    def diagnostics(self, var=None, t=0.):
        self._call("f2d_model_diagnostics", self.h, _stream())
        return self.read_diags()

    def read_diags(self):
        vals = self._diag.cpu().numpy()
        self.diags = {n: float(vals[k]) for k, n in enumerate(self.diag_names)}
        return self.diags

    def set_dt(self, dt):
        self._call("f2d_model_set_dt", self.h, float(dt))

    def step(self, t=0., dt=None):
        """One iteration of the Fluid2d loop body: set_dt (dt fixed unless
        adaptable_dt), the RK3 step, the diagnostics (kept on the device)."""
        if dt is not None and dt != self.desc.dt:
            self.desc.dt = dt
            self.set_dt(dt)
        self._call("f2d_model_step", self.h, 1, _stream())

    def run(self, nsteps, graph=False):
        if graph:
            self._call("f2d_model_step_graph", self.h, int(nsteps), _stream())
        else:
            self._call("f2d_model_step", self.h, int(nsteps), _stream())

    def run_host(self, nsteps, state_host):
        """nsteps steps with the state in host memory: ``state_host`` (a
        page-locked float64 tensor shaped like ``var.state``) is uploaded,
        stepped and read back every step, as one captured graph replayed on
        the current (non-default) stream.  Asynchronous."""
        if (state_host.device.type != "cpu" or state_host.dtype != torch.float64
                or tuple(state_host.shape) != tuple(self.var.state.shape)
                or not state_host.is_contiguous() or not state_host.is_pinned()):
            raise ValueError("run_host: needs a page-locked contiguous float64 host tensor "
                             "shaped like var.state")
        self._call("f2d_model_step_host", self.h, int(nsteps), state_host.data_ptr(), _stream())

    def probe(self, enable=None):
        """Enable/disable the finest-level smoother probe, or (enable=None)
        return (count, mean ms) over the probed calls of the last step."""
        c, ms = ctypes.c_int(), ctypes.c_double()
        if enable is None:
            self._call("f2d_model_probe", self.h, -1, ctypes.byref(c), ctypes.byref(ms))
            return c.value, ms.value
        self._call("f2d_model_probe", self.h, int(bool(enable)), None, None)

    def graph_kernels(self):
        n = ctypes.c_int()
        self._call("f2d_model_graph_kernels", self.h, ctypes.byref(n))
        return n.value

    def nbytes(self):
        """Device memory held by the model."""
        b = ctypes.c_size_t()
        self._call("f2d_model_bytes", self.h, ctypes.byref(b))
        return b.value

    @property
    def cells(self):
        return self.desc.nx * self.desc.ny

    def status(self, clear=False):
        """The device status word (STATUS_* bits; 0 = healthy), read
        synchronously on the current stream; cleared afterwards if asked."""
        v = ctypes.c_int()
        self._call("f2d_model_status", self.h, int(bool(clear)), ctypes.byref(v), _stream())
        return v.value

    def solve_stats(self):
        nite, res, st = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
        self._call("f2d_model_solve_stats", self.h, ctypes.byref(nite), ctypes.byref(res),
                   ctypes.byref(st))
        return nite.value, res.value, st.value

    def coarse_switch(self, level=None):
        """Query (level=None) or set the level from which the multigrid runs in
        one CTA; returns (current, first allowed, number of levels)."""
        cur, first, nlev = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._call("f2d_model_coarse_level", self.h, -1 if level is None else int(level),
                   ctypes.byref(cur), ctypes.byref(first), ctypes.byref(nlev))
        self.coarse_level = cur.value
        return cur.value, first.value, nlev.value

    def reset_graphs(self):
        """Drop the captured graphs; the next graph run captures again with
        the launch settings then current."""
        self._call("f2d_model_reset_graphs", self.h)

    def coarse_operator(self, enable=None):
        """Query (enable=None) or switch the coarse part of the multigrid as a
        precomputed linear map (product build); returns its size (0: none)."""
        n = ctypes.c_int()
        self._call("f2d_model_coarse_op", self.h, -1 if enable is None else int(bool(enable)),
                   ctypes.byref(n))
        return n.value

    def cluster_level(self):
        """The float level from which the mixed form's small-level cycles run
        as one thread-block-cluster launch (-1: none)."""
        lev = ctypes.c_int()
        self._call("f2d_model_cluster_level", self.h, ctypes.byref(lev))
        return lev.value

    def set_islands(self, rhsp, psi):
        """Islands with a prescribed streamfunction: the rhsp and psi arrays of
        core/island.py (``fluid2d_gb300.island.Island.finalize``)."""
        r = np.ascontiguousarray(rhsp, dtype=np.float64)
        p = np.ascontiguousarray(psi, dtype=np.float64)
        if r.shape != (self.nyl, self.nxl) or p.shape != (self.nyl, self.nxl):
            raise ValueError("island arrays must be (ny+6, nx+6)")
        self._call("f2d_model_islands", self.h, r.ctypes.data, p.ctypes.data, _stream())

    # ---- flux diagnostic: core/fluxes.py:100-213
    def flux_setup(self):
        self._call("f2d_model_flux_setup", self.h, _stream())
        n, ptr = ctypes.c_int(), ctypes.POINTER(ctypes.c_double)()
        self._call("f2d_model_flux_info", self.h, ctypes.byref(n), ctypes.byref(ptr))
        self.flx = device_view(ctypes.cast(ptr, ctypes.c_void_p).value,
                               (n.value, self.nyl, self.nxl))
        self.fullflx_list = [self.L.f2d_model_flux_name(self.h, k).decode()
                             for k in range(n.value)]

    def diag_fluxes(self, x=None, t=0., dt=None):
        """Fluxes.diag_fluxes with the model's current dt and umax: the rev/irr
        flux planes land in ``self.flx`` (device, order ``fullflx_list``)."""
        if not hasattr(self, "flx"):
            self.flux_setup()
        self._call("f2d_model_diag_fluxes", self.h, _stream())
        return self.flx

    # ---- device time loop: core/fluid2d.py:190-330 with core/output.py:62-94
    LOOP_STATUS = {0: "running", 1: "tend", 2: "blowup", 3: "bad_dt"}

    def loop_setup(self, tend, freq_his=1., freq_diag=1., var_to_save=("vorticity",),
                   exacthistime=True, rescaledtime="none", his_cap=8, diag_cap=1024, t=0.,
                   kt=0, tnexthis=0., tnextdiag=0., diag_fluxes=False):
        """Set the device clock and the record rings.  t, kt, tnexthis and
        tnextdiag are a restart's values (0 for a new run)."""
        if isinstance(var_to_save, str):
            var_to_save = (list(self.var.varname_list) if var_to_save == "all"
                           else [var_to_save])
        for v in var_to_save:
            if v not in self.var.varname_list:
                raise ValueError("%s is not a model variable => modify param.var_to_save" % v)
        if rescaledtime not in ("none", "enstrophy"):
            raise ValueError("rescaledtime must be 'none' or 'enstrophy'")
        d = _lib.LoopDesc()
        d.tend, d.freq_his, d.freq_diag = float(tend), float(freq_his), float(freq_diag)
        d.exacthistime = int(bool(exacthistime))
        d.rescaledtime = int(rescaledtime == "enstrophy")
        d.nsave = len(var_to_save)
        for q, v in enumerate(var_to_save):
            d.save[q] = self.var.varname_list.index(v)
        d.his_cap, d.diag_cap = int(his_cap), int(diag_cap)
        d.t, d.tnexthis, d.tnextdiag, d.kt = float(t), float(tnexthis), float(tnextdiag), int(kt)
        d.diag_fluxes = int(bool(diag_fluxes))
        self._call("f2d_model_loop_setup", self.h, ctypes.byref(d), _stream())
        self._loop = d
        self.var_to_save = list(var_to_save)
        if diag_fluxes:
            self.flux_setup()

    def loop_start(self):
        """Diagnostics and Output.do at the clock's time (the loop's start)."""
        self._call("f2d_model_loop_start", self.h, _stream())

    def loop_run(self, max_steps):
        """Launch the loop graph: steps until tend, a blow-up, a full ring or
        max_steps steps (asynchronous)."""
        self._call("f2d_model_loop_run", self.h, int(max_steps), _stream())

    def loop_state(self):
        s = _lib.LoopState()
        self._call("f2d_model_loop_state", self.h, ctypes.byref(s), _stream())
        return {"t": s.t, "dt": s.dt, "kt": s.kt, "tnexthis": s.tnexthis,
                "tnextdiag": s.tnextdiag, "status": self.LOOP_STATUS.get(s.status, s.status),
                "nhis": s.nhis, "ndiag": s.ndiag}

    def loop_drain(self):
        """The records waiting in the rings, as (t, kt, {var: float32 array})
        history records (with the flux planes when the loop runs the flux
        diagnostic) and (t, kt, {diag: value}) diagnostic rows; empties the
        rings."""
        d = self._loop
        ny, nx = self.desc.ny, self.desc.nx
        his = np.empty((d.his_cap, max(1, d.nsave), ny, nx), np.float32)
        fl = self.fullflx_list if d.diag_fluxes else []
        flx = np.empty((d.his_cap, max(1, len(fl)), ny, nx), np.float32)
        ht = np.empty(d.his_cap, np.float64)
        hk = np.empty(d.his_cap, np.int32)
        names = self.diag_names + ["dkedt", "dvdt"]
        rows = np.empty((d.diag_cap, len(names) + 2), np.float64)
        nh, nd = ctypes.c_int(), ctypes.c_int()
        self._call("f2d_model_loop_drain", self.h, his.ctypes.data,
                   flx.ctypes.data if fl else None, ht.ctypes.data, hk.ctypes.data,
                   rows.ctypes.data, ctypes.byref(nh), ctypes.byref(nd), _stream())
        recs = []
        for k in range(nh.value):
            f = {v: his[k, q].copy() for q, v in enumerate(self.var_to_save)}
            f.update({"flx:" + v: flx[k, q].copy() for q, v in enumerate(fl)})
            recs.append((float(ht[k]), int(hk[k]), f))
        diag = [(float(rows[k, 0]), int(rows[k, 1]),
                 {n: float(rows[k, 2 + q]) for q, n in enumerate(names)})
                for k in range(nd.value)]
        return recs, diag

    def loop(self, tend, output=None, max_steps=None, start=True, **setup):
        """Fluid2d.loop on the device: run to tend (or max_steps steps),
        handing history records and diagnostic rows to ``output``
        (``write_his(t, kt, fields)``, ``write_diag(t, kt, diags)``) each
        time the rings are drained, or collecting them when output is None.
        Returns the final clock (loop_state) with the collected records."""
        self.loop_setup(tend, **setup)
        his, diag = [], []

        def hand(recs, rows):
            if output is None:
                his.extend(recs)
                diag.extend(rows)
                return
            for t, kt, f in recs:
                output.write_his(t, kt, {k: v for k, v in f.items() if not k.startswith("flx:")})
                fl = {k[4:]: v for k, v in f.items() if k.startswith("flx:")}
                if fl:
                    output.write_flx(t, kt, fl)
            for t, kt, dg in rows:
                output.write_diag(t, kt, dg)

        kt0 = self._loop.kt
        if start:
            self.loop_start()
        while True:
            left = 2 ** 31 - 1
            if max_steps is not None:
                left = int(max_steps) - (self.loop_state()["kt"] - kt0)
                if left <= 0:
                    break
            self.loop_run(left)
            st = self.loop_state()
            hand(*self.loop_drain())
            if st["status"] != "running":
                break
        st = self.loop_state()
        hand(*self.loop_drain())
        self.read_diags()
        st["his"], st["diag"] = his, diag
        return st

    def write_restart(self, path, tend):
        """core/restart.py:120-143: the clock and the float64 state with halo."""
        from .output import Restart
        st = self.loop_state()
        Restart.write(path, tend, st["t"], st["dt"], st["kt"], st["tnextdiag"], st["tnexthis"],
                      self.var.state.cpu().numpy(), self.var.varname_list)

    def read_restart(self, path):
        """core/restart.py:145-163 and Fluid2d.relaunch (core/fluid2d.py:356-368):
        loads the state, returns the clock to pass to ``loop`` (t, kt,
        tnexthis, tnextdiag) and the stored tend."""
        from .output import Restart
        clock, state = Restart.read(path, self.var.varname_list)
        self.var.state.copy_(torch.from_numpy(state).to(self.var.state.device))
        return clock

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.L.f2d_model_destroy(self.h)
        except Exception:
            pass


def from_workload(wl, variant="product", precision="fp64", **kw):
    """A Model initialised from a workloads.* dict (fields uploaded, psi set)."""
    m = Model(wl["model"], wl["nx"], wl["ny"], wl["Lx"], wl["Ly"], wl["geometry"],
              msk=wl["msk"], gravity=wl.get("gravity", 1.), variant=variant,
              precision=precision, **kw)
    for name, f in wl["fields"].items():
        m.get(name).copy_(torch.from_numpy(np.ascontiguousarray(f)).cuda())
    return m


class Ensemble(object):
    """Independent simulations advanced together on one GPU.

    Every instance keeps its own device state and captured step graph; the
    graphs are replayed on `nstreams` CUDA streams (instance i on stream
    i mod nstreams), so the many small, latency-bound kernels of different
    instances overlap on the device.  Instances never share data, so each one
    evolves exactly as it would alone.  For more than 8 concurrent streams set
    CUDA_DEVICE_MAX_CONNECTIONS (up to 32) before CUDA is initialised.
    """

    def __init__(self, models, nstreams=32, batched=False, groups=1, policy=1):
        self.models = list(models)
        self.streams = [torch.cuda.Stream() for _ in range(max(1, nstreams))]
        self.batch = None
        self.failed = []  # (model, status bits) of retired instances
        if batched:
            self.build_batch(groups, policy)

    def build_batch(self, groups=1, policy=1, balanced=False):
        """Batched steps: the instances, sorted by size, are split into
        `groups` groups (consecutive runs of the sorted list, or, balanced,
        dealt round-robin so that every group holds a share of the large
        instances); one step of every instance of a group is merged into
        launches that each run one kernel for the whole group
        (f2d_batch_create), captured as one graph per group, and the groups'
        graphs run on their own streams."""
        self.free_batch()
        self._batch_args = (groups, policy, balanced)
        L = self.models[0].L
        order = sorted(range(len(self.models)), key=lambda k: self.models[k].cells)
        groups = max(1, min(int(groups), len(order)))
        self.batch = []
        for g in range(groups):
            if balanced:
                idx = order[g::groups]
            else:
                idx = order[g * len(order) // groups:(g + 1) * len(order) // groups]
            arr = (ctypes.c_void_p * len(idx))(*[self.models[k].h.value for k in idx])
            h = ctypes.c_void_p()
            _lib.call("f2d_batch_create", arr, len(idx), int(policy), ctypes.byref(h),
                      variant=self.models[0].variant)
            self.batch.append(h)
        self._L = L

    def coarse_offset(self, d):
        """Put every instance's coarse switch at its first allowed level + d
        (clamped to the number of levels): each step larger means a quarter of
        the coarse operator's points (and a sixteenth of its bytes) per
        instance.  A built batch is rebuilt."""
        args = getattr(self, "_batch_args", None) if self.batch is not None else None
        self.free_batch()
        for m in self.models:
            cur, first, nlev = m.coarse_switch()
            m.coarse_switch(min(first + int(d), nlev))
        if args is not None:
            self.build_batch(*args)

    def batch_info(self):
        """(launches per step, operations recorded) summed over the groups"""
        tot = [0, 0]
        for h in self.batch:
            n, ops = ctypes.c_int(), ctypes.c_int()
            _lib.call("f2d_batch_info", h, ctypes.byref(n), ctypes.byref(ops),
                      variant=self.models[0].variant)
            tot[0] += n.value
            tot[1] += ops.value
        return tuple(tot)

    def free_batch(self):
        for h in getattr(self, "batch", None) or []:
            self._L.f2d_batch_destroy(h)
        self.batch = None

    def __del__(self):
        try:
            self.free_batch()
        except Exception:
            pass

    @property
    def cells(self):
        return sum(m.cells for m in self.models)

    def retire_failed(self):
        """Read every instance's status word (synchronous).  Instances whose
        run failed -- a non-finite value, a blow-up (maxspeed > 1e3,
        core/fluid2d.py:309-314), a diverged solve -- leave the ensemble:
        their graphs no longer run (batched launches are merged again without
        them) and they go to ``failed`` with their status bits.  The other
        instances never shared data with them and go on unchanged.  Returns
        the instances retired now."""
        now = list(zip(self.models, statuses(self.models)))
        bad = [(m, st) for m, st in now if st]
        if not bad:
            return []
        self.failed.extend(bad)
        gone = set(id(m) for m, _ in bad)
        self.models = [m for m in self.models if id(m) not in gone]
        if self.batch is not None:
            args = getattr(self, "_batch_args", (1, 1, False))
            self.free_batch()
            if self.models:
                self.build_batch(*args)
        return bad

    def run(self, nsteps, lockstep=False, check=False):
        """Advance every instance by nsteps (asynchronous unless ``check``:
        then the instances that failed are retired, see retire_failed, and
        returned)."""
        self._run(nsteps, lockstep)
        return self.retire_failed() if check else []

    def _run(self, nsteps, lockstep=False):
        if not self.models:
            return
        cur = torch.cuda.current_stream()
        if self.batch is not None:
            streams = self.streams[:len(self.batch)]
            for s in streams:
                s.wait_stream(cur)
            for h, s in zip(self.batch, streams):
                _lib.call("f2d_batch_step", h, int(nsteps), s.cuda_stream,
                          variant=self.models[0].variant)
            for s in streams:
                cur.wait_stream(s)
            return
        for s in self.streams:
            s.wait_stream(cur)
        if lockstep:
            for _ in range(nsteps):
                for i, m in enumerate(self.models):
                    with torch.cuda.stream(self.streams[i % len(self.streams)]):
                        m.run(1, graph=True)
        else:
            for i, m in enumerate(self.models):
                with torch.cuda.stream(self.streams[i % len(self.streams)]):
                    m.run(nsteps, graph=True)
        for s in self.streams:
            cur.wait_stream(s)

    def capture(self):
        """Capture every instance's step graph (one step each)."""
        self.run(1)


def ensemble_from_workloads(wls, precision="fp64", variant="product", nstreams=32, batched=False,
                            groups=1, policy=1, **kw):
    """An Ensemble of initialised models (psi set, diagnostics, fixed dt from
    CFL 0.8 on each instance's initial max|u|); batched: one merged graph of
    batched launches instead of per-instance graphs on streams."""
    models = []
    for wl in wls:
        m = from_workload(wl, precision=precision, variant=variant, **kw)
        m.set_psi_from_vorticity()
        d = m.diagnostics()
        if d["maxspeed"] > 0:
            m.set_dt(0.8 * min(m.dx, m.dy) / d["maxspeed"])
        models.append(m)
    return Ensemble(models, nstreams=nstreams, batched=batched, groups=groups, policy=policy)
