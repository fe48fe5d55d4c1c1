"""Known-answer tests of the checker against formulas worked by hand from the
reference's source (no GPU)."""
import math

import numpy as np
import pytest

import ics
import oracle


@pytest.fixture(autouse=True)
def _port():
    if not oracle.available("port"):
        import build

        build.build_checkers()


def test_two_body_is_plummer_softened():
    # Node.cpp:285-305 with |e| < 1 truncating to 0 in int abs(): eps = e0
    pos = np.array([[0.3, -0.1, 0.2], [-0.25, 0.15, -0.05]])
    mass = np.array([0.6, 0.4])
    w = oracle.World(pos, mass, np.array([1, 1], np.uint8))
    w.build(1)
    w.forces(0.01, 0.5, 1)
    acc = w.get("acc")
    for i, j in ((0, 1), (1, 0)):
        d = pos[j] - pos[i]
        r = math.sqrt(d @ d)
        want = (mass[j] / (r * r + 0.01 ** 2)) * (d / r)
        np.testing.assert_allclose(acc[i], want, rtol=1e-15, atol=0)


def softening_kernel(u):
    if 0 <= u < 0.5:
        return 16 / 3 * u ** 2 - 48 / 5 * u ** 4 + 32 / 5 * u ** 5 - 14 / 5
    if 0.5 <= u < 1:
        return 1 / (15 * u) + 32 / 3 * u ** 2 - 16 * u ** 3 - 48 / 5 * u ** 4 - 32 / 15 * u ** 5 - 16 / 5
    if u >= 1:
        return -1 / u
    return 0.0


def law(r, e0):
    """Softening length of Node.cpp:287-305 with the int truncation of abs()."""
    K = softening_kernel(r / (2.8 * e0))
    e = -(2.8 * e0) / (K - r)
    ae = abs(math.trunc(e))
    return e if (ae > e0 * 1e-4 and ae < 1e30) else e0


@pytest.mark.parametrize("e0,r", [(0.01, 0.5), (0.01, 0.02), (1.0, 0.5), (1.0, 3.5), (2.0, 0.1)])
def test_pair_law_with_truncated_abs(e0, r):
    pos = np.array([[0.0, 0.0, 0.0], [r, 0.0, 0.0]])
    mass = np.array([1.0, 1.0])
    got = oracle.direct_sum(pos, mass, e0, np.array([0]))[0, 0]
    eps = law(r, e0)
    want = 1.0 / (r * r + eps * eps)
    assert got == pytest.approx(want, rel=1e-14)
    if e0 < 0.6:
        assert eps == e0  # the configs' softening reduces to Plummer softening


def test_node_count_is_one_plus_eight_per_split():
    d = ics.plummer(4096, seed=3)
    w = oracle.World(d["pos"], d["mass"], d["type"])
    w.build(1)
    t = w.topology()
    internal = int((t["is_leaf"] == 0).sum())
    assert w.node_count() == 1 + 8 * internal
    # every particle of the root box sits in exactly one leaf
    p = t["particle"][t["particle"] >= 0]
    assert len(np.unique(p)) == len(p)


def test_kick_drift_by_hand():
    d = ics.plummer(64, seed=4)
    w = oracle.World(d["pos"], d["mass"], d["type"], d["vel"])
    w.build(1)
    w.forces(0.01, 0.5, 1)
    a = w.get("acc")
    v0 = w.get("vel")
    x0 = w.get("pos")
    w.kick(1e-3)
    w.drift(1e-3)
    v1 = v0 + a * 1e-3 / 2
    np.testing.assert_array_equal(w.get("vel"), v1)
    np.testing.assert_array_equal(w.get("pos"), x0 + v1 * 1e-3)


def test_gas_density_by_hand():
    """Node.cpp:737-751 on four gas particles of mass 0.25 with massInH = 0.5.
    Particles 2 and 3 are alone in their root octants: the leaf (gas 0.25) is
    strictly closer to 0.5 than the root (gas 1.0), so each gets h = 2 * R/2 and
    rho = m W(0, h) = m / (pi h^3).  Particles 0 and 1 share every node down to
    depth 5 with gas 0.5 = massInH; the deepest such node's parent holds 0.5 too,
    so the strict test fails and they get no density (h stays 0)."""
    pos = np.array([[0.1, 0.1, 0.1], [0.12, 0.11, 0.1], [-0.3, 0.2, 0.1], [0.5, -0.4, -0.2]])
    w = oracle.World(pos, np.full(4, 0.25), np.full(4, 2, np.uint8), U=np.full(4, 0.01))
    w.build(1)
    w.gas_density(0.5)
    R = w.root_radius()
    h, rho, P = w.get("h"), w.get("rho"), w.get("P")
    assert R == pytest.approx(math.sqrt(0.5 ** 2 + 0.4 ** 2 + 0.2 ** 2), rel=1e-15)
    np.testing.assert_array_equal(h[:2], 0.0)
    np.testing.assert_array_equal(h[2:], R)
    np.testing.assert_allclose(rho[2:], 0.25 / (math.pi * R ** 3), rtol=1e-15)
    np.testing.assert_allclose(P[2:], (5 / 3 - 1) * 0.01 * rho[2:], rtol=1e-15)
