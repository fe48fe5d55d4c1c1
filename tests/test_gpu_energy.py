"""Energy diagnostic (ag2_energy): the potential of the walk's own pair force,
-(G m / e0) atan(e0 / r), over the FP64 walk's accepted nodes, and the drift of
the total energy under the step loop."""
import numpy as np
import pytest

import ics

pytestmark = pytest.mark.gpu


def _ctx(d, e0=0.01, theta=0.5, precision="fp32"):
    import ag2

    c = ag2.Context(len(d["mass"]), e0=e0, theta=theta, massInH=d.get("massInH", 0.0), precision=precision)
    c.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
    return c


def test_two_body_potential_is_exact():
    m1, m2, r, e0 = 0.3, 0.7, 1.25, 0.05
    d = {"pos": np.array([[0.1, -0.2, 0.05], [0.1 + r, -0.2, 0.05]]), "vel": np.array([[0.0, 0.1, 0.0], [0.0, -0.2, 0.3]]),
         "mass": np.array([m1, m2]), "type": np.array([1, 2], np.uint8), "U": np.array([0.0, 0.4])}
    c = _ctx(d, e0=e0)
    c.build_tree()
    e = c.energy()
    w = -(m1 * m2 / e0) * np.arctan(e0 / r)
    assert e["potential"] == pytest.approx(w, rel=1e-14)
    assert e["kinetic"] == pytest.approx(0.5 * m1 * 0.01 + 0.5 * m2 * (0.04 + 0.09), rel=1e-14)
    assert e["thermal"] == pytest.approx(m2 * 0.4, rel=1e-14)
    assert e["total"] == pytest.approx(e["kinetic"] + e["potential"] + e["thermal"], rel=1e-14)


def test_plummer_potential_energy_matches_analytic():
    # W = -3 pi G M^2 / (32 a) for a Plummer sphere; softening 0.01 and the
    # tree approximation move it by well under a percent at N = 16384
    d = ics.plummer(16384, seed=1)
    c = _ctx(d)
    c.build_tree()
    w = c.energy()["potential"]
    assert w == pytest.approx(-3 * np.pi / 32, rel=0.02)


def test_energy_drift_small_over_steps():
    d = ics.plummer(4096, seed=7)
    c = _ctx(d)
    c.build_tree()
    c.sph_density()
    c.forces()
    e0 = c.energy()["total"]
    for _ in range(200):
        c.step(1e-3)
    e1 = c.energy()["total"]
    assert abs(e1 - e0) / abs(e0) < 1e-3


def test_energy_rejects_general_softening_and_missing_tree():
    import ag2

    d = ics.plummer(64, seed=3)
    c = _ctx(d)
    with pytest.raises(ag2.AG2Error):
        c.energy()  # no tree yet
    c2 = _ctx(d, e0=1.0)
    c2.build_tree()
    with pytest.raises(ag2.AG2Error):
        c2.energy()
