"""Host-side mirror of the reference's per-step interface over the C ABI.

`GpuSolver` plays the roles the reference splits over Factory::getSolver + ISolver::create/integrate
(core/timestepping/ISolver.h:20-67), ITimeStepping::step (core/timestepping/TimeStepping.cpp:34-75) and
IGravity (core/gravity/IGravity.h:16-62): the particle state lives on the GPU between calls and is
transferred with set_quantity / get_quantity (Storage::getValue / getDt / getD2t).

There is no CPU fallback: constructing a GpuSolver without the built libsphgpu.so or without a CUDA device
raises.
"""
import ctypes
import os

import numpy as np

from . import abi

_F8P = ctypes.POINTER(ctypes.c_double)
_U4P = ctypes.POINTER(ctypes.c_uint32)
_LIB = None


class SphGpuError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"sphgpu error {code}: {message}")
        self.code = code


def measure_fp32_peak(ms_target=200.0):
    """The device's FP32 FMA rate in TFLOP/s (an FMA-chain kernel on every SM timed with CUDA events)."""
    out = np.zeros(1)
    rc = library().sphgpu_measure_fp32_peak(float(ms_target), out.ctypes.data_as(_F8P))
    if rc != abi.OK:
        raise SphGpuError(rc, "sphgpu_measure_fp32_peak failed")
    return float(out[0])


def library():
    """Loads libsphgpu.so (built in-tree by opensph_gb300.build); raises if it is missing."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(abi.LIBRARY_PATH):
        raise RuntimeError(f"{abi.LIBRARY_PATH} is not built; run `python -m opensph_gb300.build`")
    lib = ctypes.CDLL(abi.LIBRARY_PATH)
    h = ctypes.c_void_p
    lib.sphgpu_abi_version.restype = ctypes.c_int
    lib.sphgpu_create.argtypes = [ctypes.POINTER(abi.Config), ctypes.POINTER(h)]
    lib.sphgpu_destroy.argtypes = [h]
    lib.sphgpu_last_error.argtypes = [h]
    lib.sphgpu_last_error.restype = ctypes.c_char_p
    lib.sphgpu_stream.argtypes = [h]
    lib.sphgpu_stream.restype = ctypes.c_void_p
    lib.sphgpu_synchronize.argtypes = [h]
    lib.sphgpu_set_quantity.argtypes = [h, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_uint64]
    lib.sphgpu_get_quantity.argtypes = [h, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_uint64]
    lib.sphgpu_build_neighbors.argtypes = [h]
    lib.sphgpu_get_pairs.argtypes = [h, _U4P, _U4P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
    lib.sphgpu_gravity_build.argtypes = [h]
    lib.sphgpu_gravity_eval.argtypes = [h, _F8P, ctypes.c_uint64]
    lib.sphgpu_gravity_eval_points.argtypes = [h, _F8P, ctypes.c_uint64, _F8P]
    lib.sphgpu_gravity_direct.argtypes = [h, _U4P, ctypes.c_uint64, _F8P]
    lib.sphgpu_get_radius_pairs.argtypes = [h, _U4P, _U4P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
    lib.sphgpu_find_neighbors.argtypes = [h, _F8P, ctypes.c_double, _U4P, _F8P, ctypes.c_uint64,
                                          ctypes.POINTER(ctypes.c_uint64)]
    lib.sphgpu_gravity_attractors.argtypes = [h, _F8P, ctypes.c_uint64, _F8P, _F8P, ctypes.c_uint64]
    lib.sphgpu_measure_fp32_peak.argtypes = [ctypes.c_double, _F8P]
    lib.sphgpu_gravity_stats.argtypes = [h, ctypes.POINTER(ctypes.c_uint64)]
    lib.sphgpu_gravity_interactions.argtypes = [h, ctypes.POINTER(ctypes.c_uint64)]
    lib.sphgpu_integrate.argtypes = [h]
    lib.sphgpu_step.argtypes = [h, ctypes.c_uint32]
    lib.sphgpu_get_timestep.argtypes = [h, _F8P]
    lib.sphgpu_get_time.argtypes = [h, _F8P]
    lib.sphgpu_set_time.argtypes = [h, ctypes.c_double]
    lib.sphgpu_set_timestep.argtypes = [h, ctypes.c_double]
    lib.sphgpu_totals.argtypes = [h, _F8P]
    lib.sphgpu_totals_frame.argtypes = [h, ctypes.c_double, _F8P]
    lib.sphgpu_check_finite.argtypes = [h, ctypes.POINTER(ctypes.c_uint64)]
    lib.sphgpu_set_profiling.argtypes = [h, ctypes.c_int32]
    lib.sphgpu_phase_times.argtypes = [h, _F8P, ctypes.POINTER(ctypes.c_uint64)]
    lib.sphgpu_adjoint_forward.argtypes = [h, ctypes.POINTER(abi.AdjointConfig), _F8P]
    lib.sphgpu_adjoint_backward.argtypes = [h, ctypes.c_double, _F8P, _F8P, _F8P, _F8P, _F8P]
    lib.sphgpu_collide.argtypes = [h, ctypes.c_double]
    lib.sphgpu_particle_count.argtypes = [h, ctypes.POINTER(ctypes.c_uint64)]
    lib.sphgpu_collision_stats.argtypes = [h, ctypes.POINTER(ctypes.c_uint64)]
    lib.sphgpu_collision_profile.argtypes = [h, ctypes.POINTER(ctypes.c_uint64)]
    lib.sphgpu_take_removed.argtypes = [h, _U4P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
    _LIB = lib
    return lib


# (field name of the state dictionaries) -> (quantity id, derivative order)
STATE_QUANTITIES = {
    "r": (abi.Q_POSITION, 0), "v": (abi.Q_POSITION, 1), "dv": (abi.Q_POSITION, 2),
    "m": (abi.Q_MASS, 0), "rho": (abi.Q_DENSITY, 0), "drho": (abi.Q_DENSITY, 1),
    "u": (abi.Q_ENERGY, 0), "du": (abi.Q_ENERGY, 1), "p": (abi.Q_PRESSURE, 0), "cs": (abi.Q_SOUND_SPEED, 0),
    "divv": (abi.Q_VELOCITY_DIVERGENCE, 0), "ncnt": (abi.Q_NEIGHBOR_CNT, 0), "flag": (abi.Q_FLAG, 0),
    "mat": (abi.Q_MATERIAL_ID, 0), "S": (abi.Q_DEVIATORIC_STRESS, 0), "dS": (abi.Q_DEVIATORIC_STRESS, 1),
    "gradv": (abi.Q_VELOCITY_GRADIENT, 0), "reduce": (abi.Q_STRESS_REDUCING, 0), "D": (abi.Q_DAMAGE, 0),
    "dD": (abi.Q_DAMAGE, 1), "eps_min": (abi.Q_EPS_MIN, 0), "m_zero": (abi.Q_M_ZERO, 0),
    "growth": (abi.Q_EXPLICIT_GROWTH, 0), "n_flaws": (abi.Q_N_FLAWS, 0),
    "corr": (abi.Q_STRAIN_RATE_CORRECTION_TENSOR, 0),
    "w": (abi.Q_ANGULAR_FREQUENCY, 0),
}
# the state of the N-body solver (HardSphereSolver): r (radius as h), v, dv, m, angular frequency
NBODY_FIELDS = ["r", "v", "dv", "m", "w"]
# inputs of a run (the outputs are recomputed by integrate/step)
INPUT_FIELDS = ["r", "v", "dv", "m", "rho", "drho", "u", "du", "flag", "mat", "S", "dS", "reduce", "D", "dD",
                "eps_min", "m_zero", "growth", "n_flaws", "p", "cs"]


class GpuSolver:
    def __init__(self, config, keepalive=None):
        self._lib = library()
        self._keep = keepalive
        self.config = config
        self.n = int(config.particle_count)
        self._h = ctypes.c_void_p()
        rc = self._lib.sphgpu_create(ctypes.byref(config), ctypes.byref(self._h))
        if rc:
            raise SphGpuError(rc, self._lib.sphgpu_last_error(None).decode())
        self.solid = bool(config.forces & abi.FORCE_SOLID_STRESS)
        self.nbody = config.solver_type == abi.SOLVER_NBODY_HARD_SPHERE

    def close(self):
        if self._h:
            self._lib.sphgpu_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc:
            raise SphGpuError(rc, self._lib.sphgpu_last_error(self._h).decode())

    @property
    def stream(self):
        return self._lib.sphgpu_stream(self._h)

    def synchronize(self):
        self._check(self._lib.sphgpu_synchronize(self._h))

    def set_quantity(self, qid, order, values):
        comps, dt = abi.QUANTITY_LAYOUT[qid]
        a = np.ascontiguousarray(values, dtype=dt)
        if a.size != comps * self.n:
            raise ValueError(f"quantity {qid}: {a.size} values for {self.n} particles x {comps}")
        self._check(self._lib.sphgpu_set_quantity(self._h, qid, order, a.ctypes.data, self.n))

    def get_quantity(self, qid, order=0):
        comps, dt = abi.QUANTITY_LAYOUT[qid]
        a = np.zeros(comps * self.n, dtype=dt)
        self._check(self._lib.sphgpu_get_quantity(self._h, qid, order, a.ctypes.data, self.n))
        return a

    def set_state(self, st):
        if self.nbody:
            for name in NBODY_FIELDS:
                if name in st and st[name] is not None:
                    qid, order = STATE_QUANTITIES[name]
                    self.set_quantity(qid, order, st[name])
            return
        for name in INPUT_FIELDS:
            if name in st and st[name] is not None:
                qid, order = STATE_QUANTITIES[name]
                if not self.solid and name in ("S", "dS", "reduce", "gradv"):
                    continue
                if not self._has_damage() and name in ("D", "dD", "eps_min", "m_zero", "growth", "n_flaws"):
                    continue
                self.set_quantity(qid, order, st[name])

    def _has_damage(self):
        if not self.solid:
            return False
        mats = [self.config.materials[k] for k in range(self.config.material_count)]
        return any(m.yielding != abi.YIELDING_NONE and m.damage != abi.DAMAGE_NONE for m in mats)

    def get_state(self, fields=None):
        out = {}
        for name, (qid, order) in STATE_QUANTITIES.items():
            if fields is not None and name not in fields:
                continue
            if (self.nbody and name not in NBODY_FIELDS) or (not self.nbody and name == "w"):
                continue
            if not self.solid and name in ("S", "dS", "reduce", "gradv"):
                continue
            if not self._has_damage() and name in ("D", "dD", "eps_min", "m_zero", "growth", "n_flaws"):
                continue
            if name == "corr" and not self.config.correction_tensor:
                continue
            out[name] = self.get_quantity(qid, order)
        return out

    def integrate(self):
        self._check(self._lib.sphgpu_integrate(self._h))

    def step(self, nsteps=1):
        self._check(self._lib.sphgpu_step(self._h, nsteps))
        self._refresh_count()

    def _refresh_count(self):
        cnt = ctypes.c_uint64(0)
        self._check(self._lib.sphgpu_particle_count(self._h, ctypes.byref(cnt)))
        self.n = int(cnt.value)

    def collide(self, dt):
        """HardSphereSolver::collide over [0, dt) (N-body solver); merged particles are removed."""
        self._check(self._lib.sphgpu_collide(self._h, float(dt)))
        self._refresh_count()

    def take_removed(self):
        """Indices (numbering of the previous call or of the last position upload) removed by merging since."""
        cnt = ctypes.c_uint64(0)
        rc = self._lib.sphgpu_take_removed(self._h, None, 0, ctypes.byref(cnt))
        if rc not in (abi.OK, abi.ERR_CAPACITY):
            self._check(rc)
        out = np.zeros(cnt.value, dtype="u4")
        if cnt.value:
            self._check(self._lib.sphgpu_take_removed(self._h, out.ctypes.data_as(_U4P), cnt.value,
                                                      ctypes.byref(cnt)))
        return out

    def collision_profile(self):
        """Records processed by the collision loop and its SM cycles (serial part, re-searches, insertions)."""
        out = (ctypes.c_uint64 * 4)()
        self._check(self._lib.sphgpu_collision_profile(self._h, out))
        return list(out)

    def collision_stats(self):
        """Collisions, mergers, bounces and overlaps summed over all collide calls of this handle."""
        out = (ctypes.c_uint64 * 4)()
        self._check(self._lib.sphgpu_collision_stats(self._h, out))
        return list(out)

    @property
    def timestep(self):
        v = ctypes.c_double()
        self._check(self._lib.sphgpu_get_timestep(self._h, ctypes.byref(v)))
        return v.value

    @timestep.setter
    def timestep(self, dt):
        self._check(self._lib.sphgpu_set_timestep(self._h, float(dt)))

    @property
    def time(self):
        v = ctypes.c_double()
        self._check(self._lib.sphgpu_get_time(self._h, ctypes.byref(v)))
        return v.value

    @time.setter
    def time(self, t):
        self._check(self._lib.sphgpu_set_time(self._h, float(t)))

    def pairs(self):
        cnt = ctypes.c_uint64(0)
        rc = self._lib.sphgpu_get_pairs(self._h, None, None, 0, ctypes.byref(cnt))
        if rc not in (abi.OK, abi.ERR_CAPACITY):
            self._check(rc)
        pi = np.zeros(cnt.value, dtype="u4")
        pj = np.zeros(cnt.value, dtype="u4")
        self._check(self._lib.sphgpu_get_pairs(self._h, pi.ctypes.data_as(_U4P), pj.ctypes.data_as(_U4P),
                                               cnt.value, ctypes.byref(cnt)))
        return pi, pj

    def gravity(self):
        """IGravity::build + evalSelfGravity: the self-gravity accelerations (4 doubles per particle)."""
        self._check(self._lib.sphgpu_gravity_build(self._h))
        dv = np.zeros(4 * self.n)
        self._check(self._lib.sphgpu_gravity_eval(self._h, dv.ctypes.data_as(_F8P), self.n))
        return dv

    def gravity_points(self, points):
        pts = np.ascontiguousarray(points, dtype="f8")
        acc = np.zeros_like(pts)
        self._check(self._lib.sphgpu_gravity_eval_points(self._h, pts.ctypes.data_as(_F8P), pts.size // 4,
                                                         acc.ctypes.data_as(_F8P)))
        return acc

    def radius_pairs(self):
        """The directed pairs (i, j), j != i, |r_j - r_i| < 2 h_i of every particle, sorted by i then j."""
        cnt = ctypes.c_uint64(0)
        rc = self._lib.sphgpu_get_radius_pairs(self._h, None, None, 0, ctypes.byref(cnt))
        if rc not in (abi.OK, abi.ERR_CAPACITY):
            self._check(rc)
        pi = np.zeros(cnt.value, dtype="u4")
        pj = np.zeros(cnt.value, dtype="u4")
        if cnt.value:
            self._check(self._lib.sphgpu_get_radius_pairs(self._h, pi.ctypes.data_as(_U4P), pj.ctypes.data_as(_U4P),
                                                          cnt.value, ctypes.byref(cnt)))
        return pi, pj

    def find_neighbors(self, pos, radius):
        """Particles within radius of pos (ascending index) and their squared distances, on the grid of the last
        neighbour build."""
        p = np.ascontiguousarray(pos[:3], dtype="f8")
        cap = 1024
        while True:
            idx = np.zeros(cap, dtype="u4")
            d2 = np.zeros(cap)
            cnt = ctypes.c_uint64(0)
            rc = self._lib.sphgpu_find_neighbors(self._h, p.ctypes.data_as(_F8P), float(radius),
                                                 idx.ctypes.data_as(_U4P), d2.ctypes.data_as(_F8P), cap,
                                                 ctypes.byref(cnt))
            if rc == abi.ERR_CAPACITY:
                cap = int(cnt.value)
                continue
            self._check(rc)
            return idx[:cnt.value], d2[:cnt.value]

    def gravity_direct(self, targets):
        """BruteForceGravity's FP64 direct sum for the particles listed in targets (4 doubles per target)."""
        t = np.ascontiguousarray(targets, dtype="u4")
        acc = np.zeros(4 * t.size)
        self._check(self._lib.sphgpu_gravity_direct(self._h, t.ctypes.data_as(_U4P), t.size,
                                                    acc.ctypes.data_as(_F8P)))
        return acc

    def gravity_attractors(self, attractors, dv, attractor_acc):
        """IGravity::evalAttractors: attractors (count x 5: x, y, z, radius, mass); dv (4 per particle) and
        attractor_acc (3 per attractor) are updated in place and returned."""
        att = np.ascontiguousarray(attractors, dtype="f8").ravel()
        dv = np.ascontiguousarray(dv, dtype="f8")
        acc = np.ascontiguousarray(attractor_acc, dtype="f8")
        self._check(self._lib.sphgpu_gravity_attractors(self._h, att.ctypes.data_as(_F8P), att.size // 5,
                                                        acc.ctypes.data_as(_F8P), dv.ctypes.data_as(_F8P),
                                                        dv.size // 4))
        return dv, acc

    def gravity_stats(self):
        out = (ctypes.c_uint64 * 3)()
        self._check(self._lib.sphgpu_gravity_stats(self._h, out))
        return list(out)

    def gravity_interactions(self):
        out = (ctypes.c_uint64 * 2)()
        self._check(self._lib.sphgpu_gravity_interactions(self._h, out))
        return list(out)

    def totals(self, frame_frequency=None):
        """Momentum (3), angular momentum (3), kinetic and internal energy and mass; with a frame frequency the
        momenta of the frame rotating about z (TotalMomentum / TotalAngularMomentum(omega))."""
        out = np.zeros(9)
        if frame_frequency is None:
            self._check(self._lib.sphgpu_totals(self._h, out.ctypes.data_as(_F8P)))
        else:
            self._check(self._lib.sphgpu_totals_frame(self._h, float(frame_frequency), out.ctypes.data_as(_F8P)))
        return out

    PHASES = ["predict", "gravity_build", "gravity_eval", "neighbors", "sph_eval", "correct", "collide",
              "walk_evaluation"]

    def set_profiling(self, enabled=True):
        self._check(self._lib.sphgpu_set_profiling(self._h, 1 if enabled else 0))

    def phase_times(self):
        """(dict phase -> device ms, own kernel launches) accumulated since the previous call."""
        out = np.zeros(len(self.PHASES))
        launches = ctypes.c_uint64(0)
        self._check(self._lib.sphgpu_phase_times(self._h, out.ctypes.data_as(_F8P), ctypes.byref(launches)))
        return dict(zip(self.PHASES, out.tolist())), launches.value

    def adjoint_forward(self, cfg):
        """Loss of the frozen-list hydrodynamic model run from the current state (which stays unchanged)."""
        loss = ctypes.c_double(0.0)
        self._check(self._lib.sphgpu_adjoint_forward(self._h, ctypes.byref(cfg), ctypes.byref(loss)))
        return loss.value

    def adjoint_backward(self, loss_bar=1.0):
        """loss_bar x gradient of the last adjoint_forward's loss: dict r, v (4 per particle), rho, u, alpha."""
        g = {"r": np.zeros(4 * self.n), "v": np.zeros(4 * self.n), "rho": np.zeros(self.n), "u": np.zeros(self.n)}
        alpha = ctypes.c_double(0.0)
        self._check(self._lib.sphgpu_adjoint_backward(
            self._h, float(loss_bar), g["r"].ctypes.data_as(_F8P), g["v"].ctypes.data_as(_F8P),
            g["rho"].ctypes.data_as(_F8P), g["u"].ctypes.data_as(_F8P), ctypes.byref(alpha)))
        g["alpha"] = alpha.value
        return g

    def check_finite(self):
        bad = ctypes.c_uint64(0)
        rc = self._lib.sphgpu_check_finite(self._h, ctypes.byref(bad))
        return rc, bad.value
