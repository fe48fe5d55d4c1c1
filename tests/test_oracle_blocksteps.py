"""The block-time-step restatement (oracle.block_steps, Simulation.cpp:188-341):
with min = max step it is the plain step loop; otherwise every particle moves on
its own power-of-two step and the global time only grows."""
import numpy as np
import pytest

import ics
import oracle

pytestmark = pytest.mark.skipif(not oracle.available("port"), reason="oracle not built")


def _world(d):
    return oracle.World(d["pos"], d["mass"], d["type"], d["vel"], d["U"], kind="port")


def test_equal_limits_is_the_plain_step_loop():
    d = ics.small_gas_cloud(600, seed=91)
    e0, theta, dt = 0.01, 0.5, 1.0 / 512
    a = _world(d)
    a.build(1)
    a.gas_density(d["massInH"])
    a.forces(e0, theta)
    log, ts, tn = oracle.block_steps(a, d["type"], 0.3, dt, dt, e0, theta, d["massInH"], 3)
    assert [k for _, k in log] == [600] * 3 and np.allclose([t for t, _ in log], dt * np.arange(1, 4), rtol=0, atol=0)
    b = _world(d)
    b.build(1)
    b.gas_density(d["massInH"])
    b.forces(e0, theta)
    g = d["type"] == 2
    for _ in range(3):
        b.kick(dt)
        b.drift(dt)
        b.build(1)
        b.gas_density(d["massInH"])
        b.forces(e0, theta)
        U, du = b.get("U"), b.get("dUdt")
        U[g] = U[g] + du[g] * dt
        du[g] = 0
        b.set("U", U)
        b.set("dUdt", du)
        b.kick(dt)
    for f in ("pos", "vel", "U"):
        np.testing.assert_array_equal(a.get(f), b.get(f), err_msg=f)


def test_steps_are_powers_of_two_and_time_grows():
    d = ics.plummer(800, seed=92)
    w = _world(d)
    w.build(1)
    w.forces(0.01, 0.5)
    log, ts, tn = oracle.block_steps(w, d["type"], 0.05, 2.0 ** -14, 2.0 ** -6, 0.01, 0.5, 0.0, 12)
    times = [t for t, _ in log]
    assert all(b > a for a, b in zip(times, times[1:]))
    m, e = np.frexp(ts)
    assert np.all(m == 0.5) and ts.min() >= 2.0 ** -14 and ts.max() <= 2.0 ** -6
    assert len(set(ts)) > 1  # the steps really differ
    # everyone is due together only where the step sizes line up
    assert all(0 < k <= 800 for _, k in log) and any(k < 800 for _, k in log)


def test_restatement_matches_the_reference_run():
    """Against the reference's own Simulation::run with block time steps
    (tests/golden/blocksteps/plummer2k.npz, made by make_blocksteps_golden.py):
    the same final global time, the same step and next integration time per
    particle (exact: powers of two), and the state to the FP64 tolerance of
    node moments summed in another order (run() builds at 100 * its host's
    cores per serial switch; the restatement builds with as many threads)."""
    import os

    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "blocksteps", "plummer2k.npz"))
    p = {k[2:]: float(z[k]) for k in z.files if k.startswith("p_")}
    w = oracle.World(z["in_pos"], z["in_mass"], z["in_type"], z["in_vel"], z["in_U"], kind="port")
    w.set("acc", z["acc0"])
    log, ts, tn = oracle.block_steps(w, z["in_type"], p["eta"], p["min_dt"], p["max_dt"], p["e0"], p["theta"], 0.0,
                                     0, threads=int(z["cores"]), end_time=p["end_time"])
    assert log[-1][0] == float(z["global_time"]) and len(log) >= 4
    assert any(k < len(ts) for _, k in log)  # not every particle is due at every iteration
    np.testing.assert_array_equal(ts, z["tstep"])
    np.testing.assert_array_equal(tn, z["tnext"])
    scale = np.max(np.abs(z["pos"]))
    np.testing.assert_allclose(w.get("pos"), z["pos"], rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(w.get("vel"), z["vel"], rtol=1e-9, atol=1e-12)
