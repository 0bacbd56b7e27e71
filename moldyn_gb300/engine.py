"""Engine: a persistent handle on one GB300 holding one system (or an
ensemble of independent replicas) resident in HBM.

This is the performance interface; ``moldyn_gb300.solver`` mirrors the
reference's functional API (``update_force``, ``Integrator.calculate``) on top
of it.  Every method calls libmdgb.so; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import check, load


@dataclass
class StepCoupling:
    """Thermostat / barostat settings for one engine step call."""
    thermostat: object | None = None   # initializer.Thermostat
    target_temperature: float = 0.0
    barostat: object | None = None     # initializer.Barostat
    target_pressure: float = 0.0


@dataclass
class Stats:
    steps: int = 0
    rebuilds: int = 0
    kernel_launches: int = 0
    graph_launches: int = 0
    neighbor_capacity: int = 0
    max_neighbors: int = 0
    threads_per_atom: int = 0
    retries: int = 0
    force_ms: float = 0.0
    force_launches: int = 0
    integrate_ms: float = 0.0
    integrate_launches: int = 0
    class_threads_per_atom: tuple = (0, 0, 0)
    class_replicas: tuple = (0, 0, 0)
    class_skin: tuple = (0.0, 0.0, 0.0)
    direct_list_builds: int = 0
    extra: dict = field(default_factory=dict)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


class Engine:
    """One libmdgb handle.

    precision: "fp64" (plain path, the reference's arithmetic), "mixed"
    (FP32 pair maths, 64-bit fixed-point force sums, FP64 drift/reductions) or
    "fp32_naive" (the precision study's variant: force sums in plain FP32).
    reference_order: FP64 only -- reproduce the reference's summation order so
    forces and trajectories are bit-identical to its FP64 CPU results.
    direct_list: build every neighbour list directly (each cell against all
    27 neighbour cells) rather than testing each pair of cells once; the same
    lists, for comparison.
    """

    def __init__(self, precision: str = "mixed", skin: float = 0.0, rebuild_every: int = 0,
                 threads_per_atom: int = 0, graph_steps: int = 0, neighbor_capacity: int = 0,
                 device: int = 0, reference_order: bool = False, profile: bool = False,
                 persistent: bool = False, trace: bool = False, direct_list: bool = False):
        L = load()
        cfg = _lib.Config()
        check(L.mdgb_config_default(C.byref(cfg)))
        cfg.precision = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED,
                         "fp32_naive": _lib.PRECISION_FP32_NAIVE}[precision]
        cfg.skin = float(skin)
        cfg.rebuild_every = int(rebuild_every)
        cfg.threads_per_atom = int(threads_per_atom)
        cfg.graph_steps = int(graph_steps)
        cfg.neighbor_capacity = int(neighbor_capacity)
        cfg.device = int(device)
        cfg.flags = ((_lib.FLAG_REFERENCE_ORDER if reference_order else 0)
                     | (_lib.FLAG_PROFILE if profile else 0)
                     | (_lib.FLAG_PERSISTENT if persistent else 0)
                     | (_lib.FLAG_TRACE if trace else 0)
                     | (_lib.FLAG_DIRECT_LIST if direct_list else 0))
        h = C.c_void_p()
        st = L.mdgb_create(C.byref(cfg), C.byref(h))
        if st != _lib.MDGB_OK:
            raise _lib.MdgbError(st, "mdgb_create failed (no usable CUDA device, or the library "
                                     "was not built for this GPU)")
        self._h = h
        self._L = L
        self.precision = precision
        self.reference_order = reference_order
        self.n = 0
        self.nrep = 0
        self.ntypes = 0
        # macro parameters per type, kept until the state changes: the
        # reference's getters (one per quantity) then cost one reduction
        self._macro_cache = {}

    # -- lifecycle ------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.mdgb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    @property
    def stream_ptr(self) -> int:
        return int(self._L.mdgb_stream(self._h) or 0)

    def _check(self, st):
        check(st, self._h)

    # -- potentials -----------------------------------------------------
    def set_potential(self, t0: int, t1: int, sigma: float, eps: float):
        self._macro_cache.clear()
        self._check(self._L.mdgb_set_potential(self._h, t0, t1, sigma, eps))

    def set_potential_raw(self, t0: int, t1: int, sigma: float, eps: float, r_cut: float, u_cut: float):
        self._macro_cache.clear()
        self._check(self._L.mdgb_set_potential_raw(self._h, t0, t1, sigma, eps, r_cut, u_cut))

    # -- state ----------------------------------------------------------
    def upload(self, types, pos, vel, mass_per_type, box):
        self._macro_cache.clear()
        types = np.ascontiguousarray(types, dtype=np.uint16)
        n = len(types)
        pos = _f64(pos, (n, 3))
        vel = None if vel is None else _f64(vel, (n, 3))
        mass = _f64(mass_per_type).reshape(-1)
        box = _f64(box).reshape(3)
        self._check(self._L.mdgb_upload_state(self._h, n, types, pos.reshape(-1), _lib.as_ptr(vel), mass,
                                              len(mass), box))
        self.n, self.nrep, self.ntypes = n, 1, len(mass)

    def upload_ensemble(self, offsets, types, pos, vel, mass_per_type, boxes):
        self._macro_cache.clear()
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        types = np.ascontiguousarray(types, dtype=np.uint16)
        n = len(types)
        pos = _f64(pos, (n, 3))
        vel = None if vel is None else _f64(vel, (n, 3))
        mass = _f64(mass_per_type).reshape(-1)
        boxes = _f64(boxes).reshape(-1, 3)
        nrep = len(offsets) - 1
        self._check(self._L.mdgb_ensemble_upload(self._h, nrep, offsets, types, pos.reshape(-1),
                                                 _lib.as_ptr(vel), mass, len(mass), boxes.reshape(-1)))
        self.n, self.nrep, self.ntypes = n, nrep, len(mass)

    def upload_forces(self, force=None, potential=None, temp=None):
        self._macro_cache.clear()
        n = self.n
        f = None if force is None else _f64(force, (n, 3))
        p = None if potential is None else _f64(potential).reshape(n)
        t = None if temp is None else _f64(temp).reshape(n)
        self._check(self._L.mdgb_upload_forces(self._h, _lib.as_ptr(f), _lib.as_ptr(p), _lib.as_ptr(t)))

    def interacting_pairs(self, capacity: int | None = None):
        """(i, j) caller-index pairs with reference-rule distance <= r_cut, from the list."""
        cnt = C.c_int64()
        self._check(self._L.mdgb_interacting_pairs(self._h, 0, None, None, C.byref(cnt)))
        cap = int(cnt.value) if capacity is None else int(capacity)
        ii = np.zeros(max(cap, 1), dtype=np.int32)
        jj = np.zeros(max(cap, 1), dtype=np.int32)
        self._check(self._L.mdgb_interacting_pairs(
            self._h, cap, ii.ctypes.data_as(C.POINTER(C.c_int32)), jj.ctypes.data_as(C.POINTER(C.c_int32)),
            C.byref(cnt)))
        k = min(cap, int(cnt.value))
        return ii[:k], jj[:k]

    def compute_forces(self):
        self._macro_cache.clear()
        self._check(self._L.mdgb_compute_forces(self._h))

    def step(self, nsteps: int, dt: float, thermostat=None, target_temperature: float = 0.0,
             barostat=None, target_pressure: float = 0.0):
        """Integrator::VerletMethod.calculate `nsteps` times.  thermostat /
        barostat are initializer.Thermostat / Barostat objects whose coupling
        state (lambda, psi, myu) is updated in place."""
        self._macro_cache.clear()
        th = ba = None
        if thermostat is not None:
            th = _lib.CThermostat(thermostat.kind_id, thermostat.tau, target_temperature,
                                  thermostat.lambda_, thermostat.psi)
        if barostat is not None:
            ba = _lib.CBarostat(barostat.beta, barostat.tau, target_pressure, barostat.myu)
        self._check(self._L.mdgb_step(self._h, int(nsteps), float(dt),
                                      C.byref(th) if th is not None else None,
                                      C.byref(ba) if ba is not None else None))
        if thermostat is not None:
            thermostat.lambda_ = th.lambda_
            thermostat.psi = th.psi
        if barostat is not None:
            barostat.myu = ba.myu

    def prepare_step(self, nsteps: int, dt: float, thermostat=None, barostat=None):
        """Capture the CUDA graphs a later step(nsteps, dt, ...) with these
        coupling kinds replays, without taking a step (graph_steps > 1)."""
        th = ba = None
        if thermostat is not None:
            th = _lib.CThermostat(thermostat.kind_id, thermostat.tau, 0.0, thermostat.lambda_, thermostat.psi)
        if barostat is not None:
            ba = _lib.CBarostat(barostat.beta, barostat.tau, 0.0, barostat.myu)
        if self.nrep > 1:
            self._check(self._L.mdgb_ensemble_prepare(self._h, int(nsteps), float(dt)))
        else:
            self._check(self._L.mdgb_prepare_step(self._h, int(nsteps), float(dt),
                                                  C.byref(th) if th is not None else None,
                                                  C.byref(ba) if ba is not None else None))

    def test_barrier_timeout(self, hold_block: int, wait_cycles: int):
        """Arm the bounded-barrier failure test for the next step call."""
        self._check(self._L.mdgb_test_barrier_timeout(self._h, int(hold_block), int(wait_cycles)))

    def download(self, out: dict | None = None, fields=("pos", "vel", "force", "potential", "temp")):
        """The state in the caller's atom order.  `out` may hold arrays to fill
        (reused across calls); only `fields` are copied from the device."""
        n = self.n
        shapes = {"pos": (n, 3), "vel": (n, 3), "force": (n, 3), "potential": (n,), "temp": (n,)}
        res = {} if out is None else out
        for k in fields:
            a = res.get(k)
            if a is None or a.shape != shapes[k] or a.dtype != np.float64 or not a.flags.c_contiguous:
                res[k] = np.empty(shapes[k])
        box = np.empty(3 * max(self.nrep, 1))
        fn = self._L.mdgb_download_state if self.nrep == 1 else self._L.mdgb_ensemble_download
        ptr = {k: (_lib.as_ptr(res[k]) if k in fields else None) for k in shapes}
        self._check(fn(self._h, ptr["pos"], ptr["vel"], ptr["force"], ptr["potential"], ptr["temp"],
                       _lib.as_ptr(box)))
        res["box"] = box[:3].copy() if self.nrep == 1 else box.reshape(-1, 3)
        return res

    def macro(self, type_id: int = 0):
        key = int(type_id)
        if key in self._macro_cache:
            hit = self._macro_cache[key]
            return ({k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in hit.items()} if self.nrep == 1
                    else [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in x.items()} for x in hit])
        m = (_lib.CMacro * max(self.nrep, 1))()
        fn = self._L.mdgb_macro_parameters if self.nrep == 1 else self._L.mdgb_ensemble_macro
        self._check(fn(self._h, int(type_id), m))
        res = [dict(kinetic_energy=x.kinetic_energy, potential_energy=x.potential_energy,
                    thermal_energy=x.thermal_energy, temperature=x.temperature,
                    pressure=x.pressure, com_velocity=np.array(list(x.com_velocity)),
                    momentum=np.array(list(x.momentum)), count=int(x.count)) for x in m]
        out = res[0] if self.nrep == 1 else res
        self._macro_cache[key] = out
        return self.macro(key)

    # -- ensembles --------------------------------------------------------
    def ensemble_set_coupling(self, thermostats=None, target_temperatures=None, barostats=None,
                              target_pressures=None):
        nrep = self.nrep
        th = ba = None
        if thermostats is not None:
            th = (_lib.CThermostat * nrep)()
            for r in range(nrep):
                t = thermostats[r]
                th[r] = _lib.CThermostat(t.kind_id, t.tau, float(target_temperatures[r]), t.lambda_, t.psi)
        if barostats is not None:
            ba = (_lib.CBarostat * nrep)()
            for r in range(nrep):
                b = barostats[r]
                ba[r] = _lib.CBarostat(b.beta, b.tau, float(target_pressures[r]), b.myu)
        self._check(self._L.mdgb_ensemble_set_coupling(self._h, th, ba))
        self._coupling = (thermostats, th, barostats, ba)

    def ensemble_step(self, nsteps: int, dt: float):
        self._macro_cache.clear()
        self._check(self._L.mdgb_ensemble_step(self._h, int(nsteps), float(dt)))

    def ensemble_get_coupling(self):
        thermostats, th, barostats, ba = getattr(self, "_coupling", (None, None, None, None))
        self._check(self._L.mdgb_ensemble_get_coupling(self._h, th, ba))
        if thermostats is not None:
            for r, t in enumerate(thermostats):
                t.lambda_ = th[r].lambda_
                t.psi = th[r].psi
        if barostats is not None:
            for r, b in enumerate(barostats):
                b.myu = ba[r].myu

    # -- diagnostics ------------------------------------------------------
    def stats(self) -> Stats:
        s = _lib.CStats()
        self._check(self._L.mdgb_get_stats(self._h, C.byref(s)))
        vals = {}
        for f, _ in _lib.CStats._fields_:
            v = getattr(s, f)
            vals[f] = tuple(v) if f.startswith("class_") else v
        return Stats(**vals)

    def trace_phases(self) -> dict:
        """Per-phase microseconds of the step kernel since the last call (trace=True)."""
        out = np.zeros(len(_lib.TRACE_PHASES))
        self._check(self._L.mdgb_trace_phases(self._h, out, len(out)))
        return dict(zip(_lib.TRACE_PHASES, out.tolist()))

    def reset_stats(self):
        self._check(self._L.mdgb_reset_stats(self._h))

    def synchronize(self):
        self._check(self._L.mdgb_synchronize(self._h))
