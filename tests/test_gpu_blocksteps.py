"""Block time steps on the device (ag2_block_init / ag2_block_step) against the
oracle's restatement of Simulation.cpp:188-341: the same global times, the same
numbers of particles integrated, and the same state to the FP64 walk's
tolerance (the schedule itself is exact: power-of-two steps)."""
import numpy as np
import pytest

import ics
import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["plummer", "gas_cloud"])
def test_block_steps_match_oracle(case):
    import ag2

    d = ics.plummer(3000, seed=93) if case == "plummer" else ics.small_gas_cloud(2500, seed=94)
    mih = d.get("massInH", 0.0)
    e0, theta, eta, dmin, dmax, steps = 0.01, 0.5, 0.05, 2.0 ** -14, 2.0 ** -6, 10
    c = ag2.Context(len(d["mass"]), e0=e0, theta=theta, massInH=mih, precision="fp64")
    c.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
    c.build_tree()
    c.sph_density()
    c.forces()
    w = oracle.World(d["pos"], d["mass"], d["type"], d["vel"], d["U"], kind="port")
    w.build(1)
    if (d["type"] == 2).any():
        w.gas_density(mih)
    w.forces(e0, theta)
    c.block_init(eta, dmin, dmax, 0.0)
    np.testing.assert_array_equal(c.download("tstep"), oracle.block_dt(w.get("acc"), eta, e0, dmin, dmax))
    dev = [c.block_step() for _ in range(steps)]
    log, ts, tn = oracle.block_steps(w, d["type"], eta, dmin, dmax, e0, theta, mih, steps)
    assert [t for t, _ in dev] == [t for t, _ in log]
    assert [k for _, k in dev] == [k for _, k in log]
    np.testing.assert_array_equal(c.download("tstep"), ts)
    np.testing.assert_array_equal(c.download("tnext"), tn)
    scale = np.max(np.abs(w.get("pos")))
    np.testing.assert_allclose(c.download("pos"), w.get("pos"), rtol=0, atol=1e-11 * scale)
    np.testing.assert_allclose(c.download("vel"), w.get("vel"), rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(c.download("U"), w.get("U"), rtol=1e-9, atol=0)


def test_block_steps_with_equal_limits_match_plain_steps():
    import ag2

    d = ics.small_gas_cloud(2000, seed=95)
    dt = 1.0 / 512

    def ctx():
        c = ag2.Context(len(d["mass"]), e0=0.01, massInH=d["massInH"])
        c.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
        c.build_tree()
        c.sph_density()
        c.forces()
        return c

    a, b = ctx(), ctx()
    a.block_init(0.3, dt, dt, 0.0)
    for s in range(4):
        t, k = a.block_step()
        assert t == dt * (s + 1) and k == 2000
        b.step(dt)
    for f in ("pos", "vel", "acc", "U"):
        np.testing.assert_array_equal(a.download(f), b.download(f), err_msg=f)


def test_block_steps_match_reference_run():
    """Against the reference's own Simulation::run with block time steps
    (tests/golden/blocksteps/plummer2k.npz): ag2_block_init from the same
    initial accelerations, then ag2_block_step while the global time is below
    endTime, with the serial-switch threshold run() used (100 * the cores of
    the host that made the fixture).  The final global time and every
    particle's step and next integration time are bit-exact; positions and
    velocities agree to the FP64 walk's tolerance."""
    import os

    import ag2

    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "blocksteps", "plummer2k.npz"))
    p = {k[2:]: float(z[k]) for k in z.files if k.startswith("p_")}
    n = len(z["in_mass"])
    c = ag2.Context(n, e0=p["e0"], theta=p["theta"], split_threshold=100 * int(z["cores"]), precision="fp64")
    c.upload(z["in_pos"], z["in_mass"], z["in_type"], vel=z["in_vel"], U=z["in_U"])
    c.set_field("acc", z["acc0"])
    c.block_init(p["eta"], p["min_dt"], p["max_dt"], 0.0)
    t, iters, partial = 0.0, 0, False
    while t < p["end_time"]:
        t, k = c.block_step()
        iters += 1
        partial |= k < n
    assert t == float(z["global_time"]) and iters >= 4 and partial
    np.testing.assert_array_equal(c.download("tstep"), z["tstep"])
    np.testing.assert_array_equal(c.download("tnext"), z["tnext"])
    scale = np.max(np.abs(z["pos"]))
    np.testing.assert_allclose(c.download("pos"), z["pos"], rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(c.download("vel"), z["vel"], rtol=1e-9, atol=1e-12)
    c.close()
