"""ctypes wrapper of the CPU oracle (oracle/liboracle.so). TEST INFRASTRUCTURE, NOT THE PRODUCT.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, as the checker and the
timed CPU baseline. State dictionaries use the field names of ora_state (oracle/sph_oracle.h).
"""
import ctypes
import os
import subprocess

import numpy as np

from opensph_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_F8 = ctypes.POINTER(ctypes.c_double)
_U4 = ctypes.POINTER(ctypes.c_uint32)

FIELDS = [
    ("n", ctypes.c_uint32, None, None),
    ("r", _F8, 4, "f8"), ("v", _F8, 4, "f8"), ("dv", _F8, 4, "f8"),
    ("m", _F8, 1, "f8"), ("rho", _F8, 1, "f8"), ("drho", _F8, 1, "f8"),
    ("u", _F8, 1, "f8"), ("du", _F8, 1, "f8"), ("p", _F8, 1, "f8"), ("cs", _F8, 1, "f8"),
    ("divv", _F8, 1, "f8"), ("ncnt", _U4, 1, "u4"), ("flag", _U4, 1, "u4"), ("mat", _U4, 1, "u4"),
    ("S", _F8, 5, "f8"), ("dS", _F8, 5, "f8"), ("gradv", _F8, 6, "f8"), ("reduce", _F8, 1, "f8"),
    ("D", _F8, 1, "f8"), ("dD", _F8, 1, "f8"), ("eps_min", _F8, 1, "f8"), ("m_zero", _F8, 1, "f8"),
    ("growth", _F8, 1, "f8"), ("n_flaws", _U4, 1, "u4"), ("corr", _F8, 6, "f8"),
]
REQUIRED = ["r", "v", "dv", "m", "rho", "drho", "u", "du", "p", "cs", "divv", "ncnt", "flag", "mat"]
SOLID = ["S", "dS", "gradv", "reduce"]
DAMAGE = ["D", "dD", "eps_min", "m_zero", "growth", "n_flaws"]


class OraState(ctypes.Structure):
    _fields_ = [(name, ctype) for name, ctype, _, _ in FIELDS]


def build():
    """Compile liboracle.so from oracle/sph_oracle.cpp (plain g++, no reference sources needed)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def _lib():
    global _LIB
    try:
        return _LIB
    except NameError:
        pass
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    lib.ora_sph_kernel_value.restype = ctypes.c_double
    lib.ora_sph_kernel_value.argtypes = [ctypes.c_double]
    lib.ora_sph_kernel_grad.restype = ctypes.c_double
    lib.ora_sph_kernel_grad.argtypes = [ctypes.c_double]
    lib.ora_gravity_kernel_grad.restype = ctypes.c_double
    lib.ora_gravity_kernel_grad.argtypes = [ctypes.c_double]
    lib.ora_set_threads.argtypes = [ctypes.c_int]
    _LIB = lib
    return lib


def set_threads(n):
    _lib().ora_set_threads(int(n))


def new_state(n, solid=False, damage=False):
    st = {}
    for name, _, comps, dt in FIELDS[1:]:
        if name in REQUIRED or (solid and name in SOLID) or (damage and name in DAMAGE):
            st[name] = np.zeros(n * comps, dtype=dt)
    return st


def _pack(st):
    n = len(st["m"])
    s = OraState()
    s.n = n
    keep = []
    for name, ctype, comps, dt in FIELDS[1:]:
        a = st.get(name)
        if a is None:
            continue
        a = np.ascontiguousarray(a, dtype=dt)
        if a.size != n * comps:
            raise ValueError(f"{name}: expected {n * comps} values, got {a.size}")
        st[name] = a
        keep.append(a)
        setattr(s, name, a.ctypes.data_as(ctype))
    return s, keep


def integrate(cfg, st):
    s, keep = _pack(st)
    rc = _lib().ora_integrate(ctypes.byref(cfg), ctypes.byref(s))
    if rc:
        raise RuntimeError(f"ora_integrate failed: {rc}")
    return st


def run(cfg, st, steps, dt):
    s, keep = _pack(st)
    dtv = ctypes.c_double(dt)
    dts = np.zeros(max(steps, 1))
    rc = _lib().ora_run(ctypes.byref(cfg), ctypes.byref(s), ctypes.c_uint32(steps), ctypes.byref(dtv),
                        dts.ctypes.data_as(_F8))
    if rc:
        raise RuntimeError(f"ora_run failed: {rc}")
    return dtv.value, dts[:steps]


def totals(st):
    s, keep = _pack(st)
    out = np.zeros(9)
    _lib().ora_totals(ctypes.byref(s), out.ctypes.data_as(_F8))
    return out


def eos(material, rho, u):
    rho = np.ascontiguousarray(rho, dtype="f8")
    u = np.ascontiguousarray(u, dtype="f8")
    p = np.zeros_like(rho)
    cs = np.zeros_like(rho)
    rc = _lib().ora_eos(ctypes.byref(material), ctypes.c_uint64(rho.size), rho.ctypes.data_as(_F8),
                        u.ctypes.data_as(_F8), p.ctypes.data_as(_F8), cs.ctypes.data_as(_F8))
    if rc:
        raise RuntimeError(f"ora_eos failed: {rc}")
    return p, cs


def pairs(r):
    r = np.ascontiguousarray(r, dtype="f8")
    n = r.size // 4
    cnt = ctypes.c_uint64(0)
    _lib().ora_pairs(ctypes.c_uint64(n), r.ctypes.data_as(_F8), None, None, ctypes.c_uint64(0),
                     ctypes.byref(cnt))
    pi = np.zeros(cnt.value, dtype="u4")
    pj = np.zeros(cnt.value, dtype="u4")
    rc = _lib().ora_pairs(ctypes.c_uint64(n), r.ctypes.data_as(_F8), pi.ctypes.data_as(_U4),
                          pj.ctypes.data_as(_U4), ctypes.c_uint64(cnt.value), ctypes.byref(cnt))
    if rc:
        raise RuntimeError(f"ora_pairs failed: {rc}")
    return pi, pj


def gravity_bh(r, m, G=1.0, theta=0.5, order=3, leaf_size=25, kernel_radius=2):
    r = np.ascontiguousarray(r, dtype="f8")
    m = np.ascontiguousarray(m, dtype="f8")
    n = m.size
    dv = np.zeros(4 * n)
    stats = (ctypes.c_uint64 * 3)()
    rc = _lib().ora_gravity_bh(ctypes.c_uint64(n), r.ctypes.data_as(_F8), m.ctypes.data_as(_F8),
                               ctypes.c_double(G), ctypes.c_double(theta), ctypes.c_int(order),
                               ctypes.c_uint32(leaf_size), ctypes.c_int(kernel_radius),
                               dv.ctypes.data_as(_F8), stats)
    if rc:
        raise RuntimeError(f"ora_gravity_bh failed: {rc}")
    return dv, list(stats)


def gravity_points(r, m, points, G=1.0, theta=0.5, order=3, leaf_size=25, kernel_radius=2):
    r = np.ascontiguousarray(r, dtype="f8")
    m = np.ascontiguousarray(m, dtype="f8")
    points = np.ascontiguousarray(points, dtype="f8")
    acc = np.zeros_like(points)
    rc = _lib().ora_gravity_points(ctypes.c_uint64(m.size), r.ctypes.data_as(_F8), m.ctypes.data_as(_F8),
                                   ctypes.c_double(G), ctypes.c_double(theta), ctypes.c_int(order),
                                   ctypes.c_uint32(leaf_size), ctypes.c_int(kernel_radius),
                                   ctypes.c_uint64(points.size // 4), points.ctypes.data_as(_F8),
                                   acc.ctypes.data_as(_F8))
    if rc:
        raise RuntimeError(f"ora_gravity_points failed: {rc}")
    return acc


def gravity_direct(r, m, G=1.0, kernel_radius=2, targets=None):
    r = np.ascontiguousarray(r, dtype="f8")
    m = np.ascontiguousarray(m, dtype="f8")
    n = m.size
    if targets is None:
        idx = None
        nt = n
    else:
        targets = np.ascontiguousarray(targets, dtype="u4")
        idx = targets.ctypes.data_as(_U4)
        nt = targets.size
    acc = np.zeros(4 * nt)
    rc = _lib().ora_gravity_direct(ctypes.c_uint64(n), r.ctypes.data_as(_F8), m.ctypes.data_as(_F8),
                                   ctypes.c_double(G), ctypes.c_int(kernel_radius), ctypes.c_uint64(nt),
                                   idx, acc.ctypes.data_as(_F8))
    if rc:
        raise RuntimeError(f"ora_gravity_direct failed: {rc}")
    return acc


def gravity_attractors(r, m, attractors, dv, acc, G=1.0, kernel_radius=2):
    """BarnesHut::evalAttractors: attractors (count x 5: x, y, z, radius, mass); dv (4 per particle) and acc
    (3 per attractor) are updated in place and returned."""
    r = np.ascontiguousarray(r, dtype="f8")
    m = np.ascontiguousarray(m, dtype="f8")
    att = np.ascontiguousarray(attractors, dtype="f8").ravel()
    dv = np.ascontiguousarray(dv, dtype="f8")
    acc = np.ascontiguousarray(acc, dtype="f8")
    rc = _lib().ora_gravity_attractors(ctypes.c_uint64(m.size), r.ctypes.data_as(_F8), m.ctypes.data_as(_F8),
                                       ctypes.c_double(G), ctypes.c_int(kernel_radius), ctypes.c_uint64(att.size // 5),
                                       att.ctypes.data_as(_F8), dv.ctypes.data_as(_F8), acc.ctypes.data_as(_F8))
    if rc:
        raise RuntimeError(f"ora_gravity_attractors failed: {rc}")
    return dv, acc


def kernel_values(qsqr):
    lib = _lib()
    return (np.array([lib.ora_sph_kernel_value(float(q)) for q in qsqr]),
            np.array([lib.ora_sph_kernel_grad(float(q)) for q in qsqr]),
            np.array([lib.ora_gravity_kernel_grad(float(q)) for q in qsqr]))


class FrozenParams(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_uint32), ("rebuild_every", ctypes.c_uint32), ("n_target", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("dt", ctypes.c_double), ("gamma", ctypes.c_double),
                ("alpha", ctypes.c_double), ("beta", ctypes.c_double)]


def frozen_loss(r, v, m, rho, u, steps, dt, n_target, rebuild_every=10, gamma=5.0 / 3.0, alpha=1.5, beta=3.0,
                tangent=None):
    """Loss of the frozen-list model (ora_frozen_loss) and, with tangent = dict of optional r, v (4 per
    particle), rho, u arrays and an alpha float, its directional derivative. Returns (loss, dloss)."""
    prm = FrozenParams(steps, rebuild_every, n_target, 0, dt, gamma, alpha, beta)
    arrs = [np.ascontiguousarray(a, dtype="f8") for a in (r, v, m, rho, u)]
    n = arrs[2].size
    tan = tangent or {}
    tarr = []
    for name, comps in (("r", 4), ("v", 4), ("rho", 1), ("u", 1)):
        t = tan.get(name)
        if t is None:
            tarr.append(None)
            continue
        t = np.ascontiguousarray(t, dtype="f8")
        if t.size != comps * n:
            raise ValueError(f"tangent {name}: expected {comps * n} values")
        tarr.append(t)
    ptr = [a.ctypes.data_as(_F8) for a in arrs]
    tptr = [None if t is None else t.ctypes.data_as(_F8) for t in tarr]
    loss = ctypes.c_double(0.0)
    dloss = ctypes.c_double(0.0)
    rc = _lib().ora_frozen_loss(ctypes.byref(prm), ctypes.c_uint64(n), *ptr, *tptr,
                                ctypes.c_double(float(tan.get("alpha", 0.0))), ctypes.byref(loss),
                                ctypes.byref(dloss))
    if rc:
        raise RuntimeError(f"ora_frozen_loss failed: {rc}")
    return loss.value, dloss.value


# ---- HardSphereSolver (ora_nbody_*) ----------------------------------------------------------------------

class OraNbodyState(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("r", _F8), ("v", _F8), ("dv", _F8), ("m", _F8), ("w", _F8)]


def _pack_nbody(st):
    n = len(st["m"])
    for name in ("r", "v", "dv", "w"):
        if st.get(name) is None:
            st[name] = np.zeros(4 * n)
        st[name] = np.ascontiguousarray(st[name], dtype="f8").reshape(-1).copy()
    st["m"] = np.ascontiguousarray(st["m"], dtype="f8").copy()
    s = OraNbodyState()
    s.n = n
    for name in ("r", "v", "dv", "m", "w"):
        setattr(s, name, st[name].ctypes.data_as(_F8))
    return s


def _unpack_nbody(st, n):
    for name in ("r", "v", "dv", "w"):
        st[name] = st[name][:4 * n].copy()
    st["m"] = st["m"][:n].copy()


def nbody_collide(cfg, st, dt, origin=False, prev_removed=None):
    """HardSphereSolver::collide over [0, dt) on the state dict (r, v, dv, m, w; shrunk in place).
    Returns (stats[4], ambiguous) and, with origin, the index before the call of each kept particle.
    prev_removed: a list holding the indices removed by the previous call (updated in place)."""
    s = _pack_nbody(st)
    stats = np.zeros(4, dtype=np.uint64)
    amb = ctypes.c_uint64(0)
    org = np.zeros(max(s.n, 1), dtype=np.uint32)
    prev = np.zeros(max(s.n, 1), dtype=np.uint32)
    cnt = ctypes.c_uint32(0)
    if prev_removed is not None:
        cnt.value = len(prev_removed)
        prev[:len(prev_removed)] = prev_removed
    rc = _lib().ora_nbody_collide(ctypes.byref(cfg), ctypes.byref(s), ctypes.c_double(dt),
                                  stats.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), ctypes.byref(amb),
                                  org.ctypes.data_as(_U4), prev.ctypes.data_as(_U4), ctypes.byref(cnt))
    if prev_removed is not None:
        prev_removed[:] = prev[:cnt.value].tolist()
    if rc:
        raise RuntimeError(f"ora_nbody_collide failed: {rc}")
    _unpack_nbody(st, s.n)
    if origin:
        return stats, amb.value, org[:s.n].copy()
    return stats, amb.value


def nbody_integrate(cfg, st):
    s = _pack_nbody(st)
    rc = _lib().ora_nbody_integrate(ctypes.byref(cfg), ctypes.byref(s))
    if rc:
        raise RuntimeError(f"ora_nbody_integrate failed: {rc}")
    _unpack_nbody(st, s.n)
    return st


def nbody_run(cfg, st, steps, dt):
    """steps leap-frog steps of the N-body solver. Returns (next dt, dts, counts, stats[4], ambiguous)."""
    s = _pack_nbody(st)
    dtv = ctypes.c_double(dt)
    dts = np.zeros(max(steps, 1))
    counts = np.zeros(max(steps, 1), dtype=np.uint32)
    stats = np.zeros(4, dtype=np.uint64)
    amb = ctypes.c_uint64(0)
    rc = _lib().ora_nbody_run(ctypes.byref(cfg), ctypes.byref(s), ctypes.c_uint32(steps), ctypes.byref(dtv),
                              dts.ctypes.data_as(_F8), stats.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                              ctypes.byref(amb), counts.ctypes.data_as(_U4))
    if rc:
        raise RuntimeError(f"ora_nbody_run failed: {rc}")
    _unpack_nbody(st, s.n)
    return dtv.value, dts[:steps], counts[:steps], stats, amb.value
