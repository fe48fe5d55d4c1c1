"""The FP32 walk's node records against numpy's roundings of the exported FP64
moments, bit for bit: centre of mass as a two-float split in the instance's
scaled units, mass and gasMass scaled by ls^2, the opening threshold and the
gas velocity (zeros for a node without gas).  numpy's float32 casts round to nearest even, as the device's
conversions do.  The inputs add values on rounding ties, exact zeros and
magnitudes whose floats are subnormal or zero."""
import numpy as np
import pytest

import ics

pytestmark = pytest.mark.gpu

KPC, MSUN, G_SI = 3.08567758149137e19, 1.98847e30, 6.6743e-11


def _scale_exp(R):
    _, e = np.frexp(R)  # R = f 2^e, f in [0.5, 1)
    return int(-e)


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _check(d, theta=0.5, e0=0.02, G=1.0):
    import ag2

    n = len(d["mass"])
    c = ag2.Context(n, G=G, e0=e0, theta=theta, massInH=d.get("massInH", 0.0))
    c.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
    c.build_tree()
    t = c.topology()
    w = c.walk_records()
    k = _scale_exp(c.root_radius())
    c.close()
    C = w[:, 8:12].view(np.int32)
    live = C[:, 0] != 0  # an exported empty node is all zeros; a real one has first child >= 1 or -1
    assert live.sum() > 0.3 * len(live)
    com = t["com"][live]
    ok = ~np.isnan(com).any(axis=1)  # massless-first serial nodes carry a NaN centre
    s = np.ldexp(com[ok], k)
    hi = s.astype(np.float32)
    lo = (s - hi.astype(np.float64)).astype(np.float32)
    A, B, D = w[live][ok, 0:4], w[live][ok, 4:8], w[live][ok, 12:16]
    np.testing.assert_array_equal(_bits(A[:, :3]), _bits(hi))
    np.testing.assert_array_equal(_bits(B[:, :3]), _bits(lo))
    np.testing.assert_array_equal(_bits(A[:, 3]), _bits(np.ldexp(t["mass"][live][ok], 2 * k).astype(np.float32)))
    np.testing.assert_array_equal(_bits(D[:, 3]), _bits(np.ldexp(t["gas_mass"][live][ok], 2 * k).astype(np.float32)))
    leaf = t["is_leaf"][live][ok] != 0
    q = np.ldexp(t["radius"][live][ok], k).astype(np.float32) / np.float32(theta)
    mac = np.where(leaf, np.float32(-1.0), (q * q).astype(np.float32))
    np.testing.assert_array_equal(_bits(B[:, 3]), _bits(mac))
    part = t["particle"][live][ok]
    own = leaf & (part >= 0)
    gm = t["gas_mass"][live][ok]
    # the gas velocity: a leaf's own particle's, else the node's mVel; zeros without gas
    vel = np.where(own[:, None], d["vel"][np.maximum(part, 0)], t["mvel"][live][ok])
    vel = np.where((gm != 0)[:, None], vel, 0.0)
    np.testing.assert_array_equal(_bits(D[:, :3]), _bits(vel.astype(np.float32)))
    return int(ok.sum())


def _with_edges(d):
    """Particles whose coordinates, velocities and masses sit on float rounding
    ties (even and odd neighbours), are exact zeros, or are tiny, spaced so
    each gets a leaf of its own."""
    R = np.abs(d["pos"]).max()
    u = 2.0 ** -24
    vals = np.array([1 + u, 1 + 3 * u, -(1 + u), -(1 + 3 * u), 1 + u + 2.0 ** -40, 0.0, 1e-25, -3e-30, 0.75 + u / 2])
    m = len(vals)
    tiny = np.abs(vals) < 1e-20
    # powers of two keep the ties through the build's exact scalings
    p2 = 2.0 ** (np.floor(np.log2(R)) - 2)
    pos = np.stack([np.linspace(-0.5, 0.5, m) * R, np.where(tiny, vals, vals * p2), np.full(m, 0.125 * R)], axis=1)
    vel = np.stack([vals, -vals, vals * 8], axis=1)
    mass = np.where(tiny, 1.0, np.abs(vals)) * 2.0 ** np.round(np.log2(np.median(d["mass"])))
    out = {k: np.concatenate([d[k], v]) for k, v in
           (("pos", pos), ("vel", vel), ("mass", mass), ("type", np.full(m, 2, d["type"].dtype)),
            ("U", np.full(m, d["U"].mean())))}
    out["massInH"] = d["massInH"]
    return out


def test_walk_records_code_units():
    d = _with_edges(ics.disk_galaxy(n_dm=30000, n_star=10000, n_gas=8000, seed=12))
    assert _check(d) > 10000


def test_walk_records_si_units():
    d = ics.disk_galaxy(n_dm=20000, n_star=8000, n_gas=4000, seed=13)
    L, M = KPC, 1e10 * MSUN
    V = np.sqrt(G_SI * M / L)
    d = {"pos": d["pos"] * L, "vel": d["vel"] * V, "mass": d["mass"] * M, "U": d["U"] * V * V, "type": d["type"],
         "massInH": d["massInH"] * M}
    assert _check(_with_edges(d), e0=0.02 * L, G=G_SI) > 10000


def test_walk_records_far_from_origin():
    d = ics.small_gas_cloud(6000, seed=14)
    d["pos"] = d["pos"] + np.array([3.0e4, -1.5e4, 7.0e3])
    assert _check(_with_edges(d), e0=0.01) > 2000
