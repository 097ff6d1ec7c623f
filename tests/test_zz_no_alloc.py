"""sphgpu_totals_noalloc — the allocation-free variant of the conserved totals — against sphgpu_totals.

Callers that cannot call cudaMalloc (an application that owns the device memory budget, a per-step hook that
must not allocate) pass their own device buffers; the entry point keeps its scratch in a fixed array inside
the library. The tests run two calls in a row on the same output buffer (the shared scratch must not carry
state between calls) on states that fill one and several scratch rows, an empty set (zeros), the largest
accepted set (every row; compared with numpy's pairwise sums, and with no change of the device's free memory
across the call), and check the size limit. This file is collected last so that a failure here does not hide
the other GPU tests.
"""
import ctypes

import numpy as np
import pytest

import cases
from opensph_gb300 import abi
from opensph_gb300.solver import GpuSolver, library

pytestmark = pytest.mark.gpu

MAX_PARTICLES = 4194304


def _entry():
    lib = library()
    f = lib.sphgpu_totals_noalloc
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _reference_and_scale(state, cfg, keep):
    with GpuSolver(cfg, keep) as g:
        g.set_state(state)
        ref = g.totals()
    r = state["r"].reshape(-1, 4)[:, :3]
    v = state["v"].reshape(-1, 4)[:, :3]
    m = state["m"]
    terms = np.concatenate([m[:, None] * v, m[:, None] * np.cross(r, v), (0.5 * m * np.sum(v * v, 1))[:, None],
                            (m * state["u"])[:, None], m[:, None]], 1)
    return ref, np.sum(np.abs(terms), 0)


def _states():
    fx = cases.load("sphere_n1000")
    cfg, keep = cases.config_of(fx)
    yield cases.state_of(fx, "s0_"), cfg, keep
    rng = np.random.default_rng(9)
    n = 50000
    st = {"r": rng.normal(size=4 * n), "v": rng.normal(size=4 * n), "m": rng.random(n) + 0.5,
          "rho": np.ones(n), "u": rng.random(n), "dv": np.zeros(4 * n), "drho": np.zeros(n), "du": np.zeros(n),
          "flag": np.zeros(n, "u4"), "mat": np.zeros(n, "u4")}
    st["r"].reshape(-1, 4)[:, 3] = 0.1
    cfg2, keep2 = abi.make_config(n, [abi.ideal_gas()], forces=abi.FORCE_PRESSURE)
    yield st, cfg2, keep2


def test_totals_noalloc_matches_totals_twice():
    torch = pytest.importorskip("torch")
    f = _entry()
    for st, cfg, keep in _states():
        ref, scale = _reference_and_scale(st, cfg, keep)
        n = len(st["m"])
        dev = {k: torch.tensor(st[k], dtype=torch.float64, device="cuda") for k in ("r", "v", "m", "u")}
        out = torch.empty(9, dtype=torch.float64, device="cuda")
        for _ in range(2):
            out.fill_(float("nan"))
            torch.cuda.synchronize()
            rc = f(dev["r"].data_ptr(), dev["v"].data_ptr(), dev["m"].data_ptr(), dev["u"].data_ptr(), n,
                   out.data_ptr(), None)
            torch.cuda.synchronize()
            assert rc == abi.OK
            got = out.cpu().numpy()
            assert np.all(np.abs(got - ref) <= 1e-13 * scale + 1e-300), (got, ref)


def test_totals_noalloc_empty_input_gives_zeros():
    torch = pytest.importorskip("torch")
    f = _entry()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    out = torch.full((9,), float("nan"), dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    assert f(p, p, p, p, 0, out.data_ptr(), None) == abi.OK
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), np.zeros(9))


def test_totals_noalloc_at_its_limit_allocates_nothing():
    # the largest accepted set fills every row of the scratch array; the call changes no device memory
    # reservation (a first call may load device code, so the comparison brackets the second)
    torch = pytest.importorskip("torch")
    f = _entry()
    n = MAX_PARTICLES
    rng = np.random.default_rng(21)
    st = {"r": rng.normal(size=4 * n), "v": rng.normal(size=4 * n), "m": rng.random(n) + 0.5, "u": rng.random(n)}
    r = st["r"].reshape(-1, 4)[:, :3]
    v = st["v"].reshape(-1, 4)[:, :3]
    terms = np.concatenate([st["m"][:, None] * v, st["m"][:, None] * np.cross(r, v),
                            (0.5 * st["m"] * np.sum(v * v, 1))[:, None], (st["m"] * st["u"])[:, None],
                            st["m"][:, None]], 1)
    # numpy's pairwise summation along contiguous rows (a reduction along axis 0 would add row after row)
    ref = np.sum(np.ascontiguousarray(terms.T), axis=1)
    scale = np.sum(np.abs(terms), 0)
    dev = {k: torch.tensor(st[k], dtype=torch.float64, device="cuda") for k in ("r", "v", "m", "u")}
    out = torch.empty(9, dtype=torch.float64, device="cuda")
    args = (dev["r"].data_ptr(), dev["v"].data_ptr(), dev["m"].data_ptr(), dev["u"].data_ptr(), n, out.data_ptr(),
            None)
    assert f(*args) == abi.OK
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    assert f(*args) == abi.OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    got = out.cpu().numpy()
    assert np.all(np.abs(got - ref) <= 1e-13 * scale), (got, ref)


def test_totals_noalloc_rejects_oversized_input():
    torch = pytest.importorskip("torch")
    f = _entry()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    assert f(p, p, p, p, MAX_PARTICLES + 1, p, None) == abi.ERR_CAPACITY
    assert f(None, p, p, p, 10, p, None) == abi.ERR_ARGUMENT
