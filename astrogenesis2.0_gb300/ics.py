"""Seeded synthetic initial conditions in G = 1 code units.

The reference ships no IC generator and names no public dataset for its hot
path, so the workloads are generated here from a counter-based RNG (Philox)
seeded per workload.  Shapes follow the workload definitions:

* ``plummer``      -- Plummer sphere, radius by inverse CDF, isotropic
                      directions, speed by rejection sampling from the
                      distribution function (Aarseth, Henon & Wielen 1974).
* ``disk_galaxy``  -- Hernquist dark halo with isotropic Jeans velocities
                      (Hernquist 1990, eq. 10), exponential stellar disk with a
                      sech^2 vertical profile, rotation from the enclosed mass
                      plus 10 % Gaussian dispersion, and a gas disk of the same
                      shape with uniform internal energy.
* ``merger``       -- two disk galaxies on a parabolic orbit.
* ``ensemble_sizes`` -- particle counts log-uniform in a range.

Types follow simulation/src/Physics/Particle.h:26: 1 star, 2 gas, 3 dark matter.
"""
from __future__ import annotations

import numpy as np


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(int(seed)))


def _iso(g: np.random.Generator, n: int) -> np.ndarray:
    ct = g.uniform(-1.0, 1.0, n)
    ph = g.uniform(0.0, 2 * np.pi, n)
    st = np.sqrt(1.0 - ct * ct)
    return np.stack([st * np.cos(ph), st * np.sin(ph), ct], axis=1)


def plummer(n: int, seed: int = 1, M: float = 1.0, a: float = 1.0, G: float = 1.0, xmax: float = 0.999):
    """Equal-mass Plummer sphere; returns dict(pos, vel, mass, type)."""
    g = rng(seed)
    X = g.uniform(1e-10, xmax, n)
    r = a / np.sqrt(X ** (-2.0 / 3.0) - 1.0)
    pos = _iso(g, n) * r[:, None]
    # speed fraction q of the local escape speed, density g(q) = q^2 (1-q^2)^(7/2)
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        x = g.uniform(0.0, 1.0, todo.size)
        y = g.uniform(0.0, 0.1, todo.size)
        ok = y < x * x * (1.0 - x * x) ** 3.5
        q[todo[ok]] = x[ok]
        todo = todo[~ok]
    vesc = np.sqrt(2.0 * G * M) * (r * r + a * a) ** -0.25
    vel = _iso(g, n) * (q * vesc)[:, None]
    pos -= pos.mean(axis=0)
    vel -= vel.mean(axis=0)
    return {"pos": pos, "vel": vel, "mass": np.full(n, M / n), "type": np.full(n, 1, np.uint8),
            "U": np.zeros(n)}


def _hernquist_sigma2(r, M, a, G=1.0):
    x = r / a
    t1 = 12.0 * r * (r + a) ** 3 / a ** 4 * np.log((r + a) / r)
    t2 = r / (r + a) * (25.0 + 52.0 * x + 42.0 * x * x + 12.0 * x ** 3)
    return np.maximum(G * M / (12.0 * a) * (t1 - t2), 0.0)


def _exp_disk(g, n, Rd, z0, rmax):
    R = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        s = g.gamma(2.0, Rd, todo.size)
        ok = s < rmax
        R[todo[ok]] = s[ok]
        todo = todo[~ok]
    ph = g.uniform(0.0, 2 * np.pi, n)
    z = z0 * np.arctanh(g.uniform(-0.999999, 0.999999, n))
    return R, ph, z


def disk_galaxy(n_dm: int = 786432, n_star: int = 196608, n_gas: int = 65536, seed: int = 2, M_halo: float = 10.0,
                a_halo: float = 5.0, M_star: float = 1.0, Rd: float = 1.0, z0: float = 0.1, u_gas: float = 0.01,
                G: float = 1.0, r_halo_max: float = 30.0):
    """Isolated disk galaxy; returns dict(pos, vel, mass, type, U, massInH)."""
    g = rng(seed)
    # halo: Hernquist M(<r) = M r^2/(r+a)^2, truncated at r_halo_max * a
    smax = r_halo_max / (1.0 + r_halo_max)
    s = np.sqrt(g.uniform(0.0, smax * smax, n_dm))
    r = a_halo * s / (1.0 - s)
    r = np.maximum(r, 1e-6)
    pos_h = _iso(g, n_dm) * r[:, None]
    sig = np.sqrt(_hernquist_sigma2(r, M_halo, a_halo, G))
    vel_h = g.standard_normal((n_dm, 3)) * sig[:, None]
    m_star = M_star / n_star
    M_gas = m_star * n_gas

    def disk(nn, M_part_total):
        R, ph, z = _exp_disk(g, nn, Rd, z0, 10.0 * Rd)
        p = np.stack([R * np.cos(ph), R * np.sin(ph), z], axis=1)
        Md = M_star + M_gas
        menc = M_halo * R * R / (R + a_halo) ** 2 + Md * (1.0 - (1.0 + R / Rd) * np.exp(-R / Rd))
        vc = np.sqrt(G * menc / np.maximum(R, 1e-6))
        v = np.stack([-vc * np.sin(ph), vc * np.cos(ph), np.zeros(nn)], axis=1)
        v += g.standard_normal((nn, 3)) * (0.1 * vc)[:, None]
        return p, v

    pos_s, vel_s = disk(n_star, M_star)
    pos_g, vel_g = disk(n_gas, M_gas)
    pos = np.concatenate([pos_h, pos_s, pos_g])
    vel = np.concatenate([vel_h, vel_s, vel_g])
    mass = np.concatenate([np.full(n_dm, M_halo / n_dm), np.full(n_star, m_star), np.full(n_gas, m_star)])
    typ = np.concatenate([np.full(n_dm, 3, np.uint8), np.full(n_star, 1, np.uint8), np.full(n_gas, 2, np.uint8)])
    U = np.where(typ == 2, u_gas, 0.0)
    com = (pos * mass[:, None]).sum(0) / mass.sum()
    vcom = (vel * mass[:, None]).sum(0) / mass.sum()
    return {"pos": pos - com, "vel": vel - vcom, "mass": mass, "type": typ, "U": U, "massInH": 64.0 * m_star}


def _rot_x(deg):
    t = np.radians(deg)
    c, s = np.cos(t), np.sin(t)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


def merger(n_per_galaxy: int = 2097152, seed: int = 3, r_peri: float = 5.0, separation: float = 40.0,
           incl=(30.0, 60.0), G: float = 1.0):
    """Two disk galaxies (3/4 dark matter, 3/16 stars, 1/16 gas) on a parabolic orbit."""
    n_dm = n_per_galaxy * 3 // 4
    n_gas = n_per_galaxy // 16
    n_star = n_per_galaxy - n_dm - n_gas
    gal = [disk_galaxy(n_dm, n_star, n_gas, seed=seed * 1000 + k) for k in range(2)]
    M1 = gal[0]["mass"].sum()
    M2 = gal[1]["mass"].sum()
    mu = G * (M1 + M2)
    v = np.sqrt(2.0 * mu / separation)
    vt = np.sqrt(2.0 * mu * r_peri) / separation
    vr = -np.sqrt(max(v * v - vt * vt, 0.0))
    rel_x = np.array([separation, 0.0, 0.0])
    rel_v = np.array([vr, vt, 0.0])
    parts = []
    for k, (gk, f) in enumerate(zip(gal, (-M2 / (M1 + M2), M1 / (M1 + M2)))):
        R = _rot_x(incl[k])
        parts.append({"pos": gk["pos"] @ R.T + f * rel_x, "vel": gk["vel"] @ R.T + f * rel_v, "mass": gk["mass"],
                      "type": gk["type"], "U": gk["U"]})
    out = {k: np.concatenate([p[k] for p in parts]) for k in ("pos", "vel", "mass", "type", "U")}
    out["massInH"] = gal[0]["massInH"]
    return out


def ensemble_sizes(count: int = 512, lo: int = 1024, hi: int = 65536, seed: int = 4) -> np.ndarray:
    g = rng(seed)
    return np.exp(g.uniform(np.log(lo), np.log(hi), count)).astype(np.int64)


def ensemble(count: int = 512, lo: int = 1024, hi: int = 65536, seed: int = 4) -> dict:
    """Independent Plummer spheres (M = 1, a = 1) with N_k log-uniform in
    [lo, hi], concatenated; instance k owns indices [first[k], first[k+1])."""
    sizes = ensemble_sizes(count, lo, hi, seed)
    parts = [plummer(int(nk), seed=seed * 100003 + k) for k, nk in enumerate(sizes)]
    out = {key: np.concatenate([q[key] for q in parts]) for key in ("pos", "vel", "mass", "type", "U")}
    out["first"] = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    return out


def serving_requests(count: int, seed: int = 7, lo: int = 4096, hi: int = 262144, gas_share: float = 0.3,
                     gas_fraction: float = 0.1, steps_lo: int = 50, steps_hi: int = 500) -> list:
    """Request mix of the serving workload: disk galaxies with N log-uniform in
    [lo, hi] (3/4 dark halo), a share of them with gas at `gas_fraction` of the
    particles (the rest of the disk in stars, otherwise all of it), and step
    counts uniform in [steps_lo, steps_hi].  Returns dicts with the particle
    arrays, massInH and steps."""
    g = rng(seed)
    sizes = np.exp(g.uniform(np.log(lo), np.log(hi), count)).astype(np.int64)
    with_gas = g.uniform(0.0, 1.0, count) < gas_share
    steps = g.integers(steps_lo, steps_hi + 1, count)
    out = []
    for k in range(count):
        n = int(sizes[k])
        n_dm = (3 * n) // 4
        n_gas = int(round(gas_fraction * n)) if with_gas[k] else 0
        d = disk_galaxy(n_dm, n - n_dm - n_gas, n_gas, seed=seed * 1009 + k)
        if not n_gas:
            d["massInH"] = 0.0
        d["steps"] = int(steps[k])
        out.append(d)
    return out


def poisson_arrivals(count: int, rate: float, seed: int = 8) -> np.ndarray:
    """Arrival times (s) of a Poisson stream of `count` requests at `rate`/s."""
    return np.cumsum(rng(seed).exponential(1.0 / rate, count))


def small_gas_cloud(n: int = 2000, seed: int = 5, gas_fraction: float = 0.5, u: float = 0.01):
    """Plummer sphere with a share of gas particles (SPH parity cases)."""
    d = plummer(n, seed=seed)
    g = rng(seed + 17)
    is_gas = g.uniform(0, 1, n) < gas_fraction
    d["type"] = np.where(is_gas, 2, 1).astype(np.uint8)
    d["U"] = np.where(is_gas, u, 0.0)
    d["massInH"] = 32.0 * d["mass"][0]
    return d
