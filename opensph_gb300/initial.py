"""Host-side initial conditions for the benchmark workloads (numpy).

The drop-in receives an already initialised particle state, exactly as the reference's solver receives the
Storage built by InitialConditions; these helpers build such states for the benchmark configurations:

* hcp_sphere   — HexagonalPacking::generate (core/sph/initial/Distribution.cpp:126-205) in a spherical
                 domain, with InitialConditions::setQuantities (core/sph/initial/Initial.cpp:290-330):
                 h = eta * (V/N)^(1/3), equal masses rho0 * V / N, centre of mass moved to the domain centre.
* impact_state — two bodies placed like CollisionGeometrySetupJob (core/run/jobs/ParticleJobs.cpp:531-573):
                 target at the origin, impactor at ((R_t+R_i) cos phi + 4 h, (R_t+R_i) sin phi, 0) moving with
                 (-v, 0, 0); FLAG 0 / 1; flaws of ScalarGradyKippModel::setFlaws
                 (core/physics/Damage.cpp:17-126) drawn from a seeded numpy generator.
* gas_impact   — ideal-gas sphere (rho 1, p 1) hit by a small ideal-gas impactor at a given Mach number: the
                 workload of the adjoint (the target's particles come first).
* plummer      — equal-mass Plummer sphere (gravity-only workload; the reference has no Plummer generator).
"""
import math

import numpy as np

from . import abi

W0 = 1.0 / math.pi  # LutKernel<3>(CubicSpline<3>).valueImpl(0)


def hcp_sphere(n, radius, center=(0.0, 0.0, 0.0), eta=1.3):
    """Returns positions (N x 4: x, y, z, h) of an HCP lattice filling a sphere, as HexagonalPacking."""
    volume = 4.0 / 3.0 * math.pi * radius ** 3
    h = 1.0 / (n / volume) ** (1.0 / 3.0)
    dx = 1.1 * h
    dy = math.sqrt(3.0) * 0.5 * dx
    dz = math.sqrt(6.0) / 3.0 * dx
    c = np.asarray(center, dtype="f8")
    lo = c - radius + 0.5 * np.array([dx, dy, dz])
    hi = c + radius
    nx = int(math.floor((hi[0] - lo[0]) / dx)) + 1
    ny = int(math.floor((hi[1] - lo[1]) / dy)) + 1
    nz = int(math.floor((hi[2] - lo[2]) / dz)) + 1
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    x = lo[0] + i * dx
    y = lo[1] + j * dy
    z = lo[2] + k * dz
    even_layer = (k % 2) == 0
    x = x + np.where(even_layer, np.where(j % 2 == 1, 0.5 * dx, 0.0), np.where(j % 2 == 0, 0.5 * dx, 0.0))
    y = y + np.where(even_layer, 0.0, math.sqrt(3.0) / 6.0 * dx)
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], 1)
    inside = np.sum((pts - c) ** 2, 1) <= radius * radius
    pts = pts[inside]
    pts += c - pts.mean(0)
    r = np.empty((len(pts), 4))
    r[:, :3] = pts
    r[:, 3] = h * eta
    return r


def _body(n, radius, center, rho0, u0, eta, flag):
    r = hcp_sphere(n, radius, center, eta)
    cnt = len(r)
    volume = 4.0 / 3.0 * math.pi * radius ** 3
    m = np.full(cnt, volume * rho0 / cnt)
    rho_limit = float(np.min(m * W0 / r[:, 3] ** 3))
    return {
        "r": r, "v": np.zeros((cnt, 4)), "m": m, "rho": np.full(cnt, rho0), "u": np.full(cnt, u0),
        "flag": np.full(cnt, flag, dtype="u4"), "rho_min": max(rho_limit, 50.0), "volume": volume,
    }


def set_flaws(h, m, rho, material, rng, kernel_radius=2.0):
    """ScalarGradyKippModel::setFlaws, non-sampled branch: returns eps_min, m_zero, growth, n_flaws and sets
    material.young_modulus."""
    mu = material.shear_modulus
    A = material.bulk_modulus
    material.young_modulus = mu * 9.0 * A / (3.0 * A + mu)
    rho0 = material.density
    cg = 0.4 * math.sqrt((A + 4.0 / 3.0 * mu) / rho0)
    size = len(h)
    growth = cg / (kernel_radius * h)
    V = float(np.sum(m / rho))
    k_w, m_w = 4.0e35, 9.0
    denom = 1.0 / (k_w ** (1.0 / m_w) * V ** (1.0 / m_w))
    # flaws are assigned to random particles, the p-th flaw having activation strain denom * p^(1/m), until
    # every particle holds at least one flaw
    covered = np.zeros(size, dtype=bool)
    ncov = 0
    chunks = []
    while ncov < size:
        idx = (rng.random(size) * size).astype(np.int64)
        uniq, firstpos = np.unique(idx, return_index=True)
        fresh = ~covered[uniq]
        new, newpos = uniq[fresh], firstpos[fresh]
        if ncov + len(new) >= size:
            stop = int(np.sort(newpos)[size - ncov - 1])
            idx = idx[: stop + 1]
        covered[new] = True
        ncov = min(size, ncov + len(new))
        chunks.append(idx)
    seq = np.concatenate(chunks)
    count = np.bincount(seq, minlength=size)
    _, fpos = np.unique(seq, return_index=True)
    _, lpos = np.unique(seq[::-1], return_index=True)
    first = fpos + 1
    last = len(seq) - lpos
    eps_min = denom * first.astype("f8") ** (1.0 / m_w)
    eps_max = denom * last.astype("f8") ** (1.0 / m_w)
    with np.errstate(divide="ignore", invalid="ignore"):
        m_zero = np.where(count == 1, 1.0, np.log(count) / np.log(eps_max / eps_min))
    return eps_min, m_zero, growth, count.astype("u4")


def impact_state(n_target, r_target, n_imp, r_imp, speed=5.0e3, angle_deg=45.0, seed=1234, eta=1.3):
    """Solid impact of two basalt bodies (von Mises + Grady-Kipp). Returns (state, materials)."""
    rng = np.random.default_rng(seed)
    t = _body(n_target, r_target, (0.0, 0.0, 0.0), 2700.0, 0.0, eta, 0)
    h_t = float(t["r"][0, 3])
    phi = math.radians(angle_deg)
    dist = r_target + r_imp
    center = (dist * math.cos(phi) + 4.0 * h_t, dist * math.sin(phi), 0.0)
    im = _body(n_imp, r_imp, center, 2700.0, 0.0, eta, 1)
    im["v"][:, 0] = -speed
    mats = []
    parts = []
    for k, b in enumerate([t, im]):
        mat = abi.basalt()
        mat.density_range[:] = [b["rho_min"], abi.INFTY]
        eps_min, m_zero, growth, n_flaws = set_flaws(b["r"][:, 3], b["m"], b["rho"], mat, rng)
        b.update(eps_min=eps_min, m_zero=m_zero, growth=growth, n_flaws=n_flaws,
                 mat=np.full(len(b["m"]), k, dtype="u4"))
        mats.append(mat)
        parts.append(b)
    n = sum(len(b["m"]) for b in parts)
    st = {
        "r": np.concatenate([b["r"] for b in parts]).ravel(),
        "v": np.concatenate([b["v"] for b in parts]).ravel(),
        "dv": np.zeros(4 * n),
        "m": np.concatenate([b["m"] for b in parts]),
        "rho": np.concatenate([b["rho"] for b in parts]),
        "drho": np.zeros(n),
        "u": np.concatenate([b["u"] for b in parts]),
        "du": np.zeros(n),
        "p": np.zeros(n), "cs": np.zeros(n), "divv": np.zeros(n), "ncnt": np.zeros(n, "u4"),
        "flag": np.concatenate([b["flag"] for b in parts]),
        "mat": np.concatenate([b["mat"] for b in parts]),
        "S": np.zeros(5 * n), "dS": np.zeros(5 * n), "gradv": np.zeros(6 * n), "reduce": np.ones(n),
        "D": np.zeros(n), "dD": np.zeros(n),
        "eps_min": np.concatenate([b["eps_min"] for b in parts]),
        "m_zero": np.concatenate([b["m_zero"] for b in parts]),
        "growth": np.concatenate([b["growth"] for b in parts]),
        "n_flaws": np.concatenate([b["n_flaws"] for b in parts]),
    }
    return st, mats


def gas_impact(n_target, n_imp, gamma=5.0 / 3.0, mach=3.0, radius=1.0, imp_radius=None, eta=1.3,
               compression=0.05):
    """Ideal-gas target sphere (radius 1, rho 1, p 1, so u = 1 / ((gamma - 1) rho)) at the origin and an impactor
    of the same gas and density, touching it at 45 degrees and moving with -mach * c_s along x. Returns a state
    dict (r, v as 4 per particle, m, rho, u) and the number of target particles.

    Both bodies also contract uniformly about their centres, v += -kappa (r - centre) with
    kappa = compression * c_s / radius (the target's surface moves inwards at `compression` c_s). A body at rest
    or in rigid translation has v_ij . r_ij = 0 for every pair, exactly the switch of the artificial viscosity
    (core/sph/equations/av/Standard.h:75-77), where the loss has a kink; the contraction moves every initial
    pair off it. compression=0 gives the bodies at rest / in translation."""
    rho0, p0 = 1.0, 1.0
    u0 = p0 / ((gamma - 1.0) * rho0)
    cs = math.sqrt(gamma * p0 / rho0)
    if imp_radius is None:
        imp_radius = radius * (n_imp / n_target) ** (1.0 / 3.0)
    t = _body(n_target, radius, (0.0, 0.0, 0.0), rho0, u0, eta, 0)
    phi = math.radians(45.0)
    h_t = float(t["r"][0, 3])
    dist = radius + imp_radius
    center = (dist * math.cos(phi) + 0.5 * h_t, dist * math.sin(phi), 0.0)
    im = _body(n_imp, imp_radius, center, rho0, u0, eta, 1)
    im["v"][:, 0] = -mach * cs
    kappa = compression * cs / radius
    for b, c in ((t, (0.0, 0.0, 0.0)), (im, center)):
        b["v"][:, :3] -= kappa * (b["r"][:, :3] - np.asarray(c))
    parts = [t, im]
    st = {
        "r": np.concatenate([b["r"] for b in parts]).ravel(),
        "v": np.concatenate([b["v"] for b in parts]).ravel(),
        "m": np.concatenate([b["m"] for b in parts]),
        "rho": np.concatenate([b["rho"] for b in parts]),
        "u": np.concatenate([b["u"] for b in parts]),
    }
    return st, len(t["m"])


def plummer(n, seed=7, softening=1.0e-3, rmax=20.0):
    """Equal-mass Plummer sphere (scale radius 1, total mass 1): positions N x 4 (h = softening), masses."""
    rng = np.random.default_rng(seed)
    x = rng.random(n)
    rad = 1.0 / np.sqrt(np.power(x, -2.0 / 3.0) - 1.0)
    rad = np.minimum(rad, rmax)
    ct = 2.0 * rng.random(n) - 1.0
    ph = 2.0 * math.pi * rng.random(n)
    st = np.sqrt(1.0 - ct * ct)
    r = np.stack([rad * st * np.cos(ph), rad * st * np.sin(ph), rad * ct, np.full(n, softening)], 1)
    return r, np.full(n, 1.0 / n)


def rubble_cloud(n, radius, h=400.0, density=2500.0, inflow=1.0e-4, sigma=0.05, seed=5):
    """A cloud of n hard spheres for the N-body solver (the reaccumulation phase of the reference's
    impact presets, core/run/jobs/Presets.cpp:48): radii h (1 + U/2), density `density`, centres on a
    randomly jittered cubic lattice inside a sphere of `radius` (jitter small enough that no two spheres
    overlap), velocity -inflow r plus a normal dispersion sigma. Returns a state dict r, v, dv, m, w."""
    rng = np.random.default_rng(seed)
    spacing = (4.0 / 3.0 * math.pi * radius ** 3 / n) ** (1.0 / 3.0)
    hmax = 1.5 * h
    if spacing <= 2.0 * hmax:
        raise ValueError("the cloud is too dense for non-overlapping spheres")
    m = int(math.ceil(2.0 * radius / spacing)) + 2
    g = (np.arange(m) - (m - 1) / 2.0) * spacing
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    p = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    p = p[np.linalg.norm(p, axis=1) <= radius]
    while len(p) < n:
        spacing *= 0.99
        g = (np.arange(m + 2) - (m + 1) / 2.0) * spacing
        x, y, z = np.meshgrid(g, g, g, indexing="ij")
        p = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
        p = p[np.linalg.norm(p, axis=1) <= radius]
        m += 2
    p = p[rng.permutation(len(p))[:n]]
    hi = h * (1.0 + 0.5 * rng.random(n))
    jitter = 0.5 * (spacing - 2.0 * hmax) * 0.999
    p = p + rng.uniform(-jitter, jitter, size=(n, 3))
    r = np.zeros((n, 4))
    r[:, :3] = p
    r[:, 3] = hi
    v = np.zeros((n, 4))
    v[:, :3] = -inflow * p + sigma * rng.standard_normal((n, 3))
    mass = density * 4.0 / 3.0 * math.pi * hi ** 3
    return {"r": r.ravel(), "v": v.ravel(), "dv": np.zeros(4 * n), "m": mass, "w": np.zeros(4 * n)}
