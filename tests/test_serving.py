"""Continuous batching (astrogenesis2.0_gb300/serving.py): simulations that
arrive while others are resident are admitted at step boundaries within the
particle budget, and every result equals the same simulation run alone.

Tolerance: none.  Each simulation's tree, walk and update read only its own
particles, so the mix reproduces the lone run bit for bit."""
import numpy as np
import pytest

import ics

pytestmark = pytest.mark.gpu

E0, THETA, DT = 0.01, 0.5, 1e-3


def _requests():
    import serving

    specs = [(ics.plummer(1500, seed=61), 0.0, 4), (ics.small_gas_cloud(2200, seed=62), None, 6),
             (ics.plummer(700, seed=63), 0.0, 3), (ics.disk_galaxy(2000, 500, 300, seed=64), None, 5),
             (ics.plummer(1, seed=65), 0.0, 2)]
    out = []
    for k, (d, mih, steps) in enumerate(specs):
        out.append(serving.Request(rid=k, pos=d["pos"], vel=d["vel"], mass=d["mass"], type=d["type"], U=d["U"],
                                   steps=steps, massInH=d.get("massInH", 0.0) if mih is None else mih))
    return out


def _check_alone(results, reqs):
    import serving

    assert sorted(r.rid for r in results) == [q.rid for q in reqs]
    for r in results:
        q = reqs[r.rid]
        alone = serving.run_alone(q, e0=E0, theta=THETA, dt=DT)
        for f in ("pos", "vel", "acc", "U", "dUdt"):
            np.testing.assert_array_equal(r.state[f], alone[f], err_msg=f"request {r.rid} field {f}")


def test_staggered_arrivals_match_alone():
    import serving

    reqs = _requests()
    eng = serving.Engine(20000, e0=E0, theta=THETA, dt=DT)
    results = []
    arrivals = {0: [0, 1], 2: [2], 3: [3], 6: [4]}  # engine step -> requests submitted before it
    for s in range(40):
        for k in arrivals.get(s, []):
            eng.submit(reqs[k])
        results.extend(eng.step())
        if eng.idle() and s > max(arrivals):
            break
    eng.close()
    _check_alone(results, reqs)


def test_budget_admission_is_first_come_first_served():
    import serving

    reqs = _requests()
    cap = 3000  # the 2200-particle gas cloud cannot join the 1500-particle sphere
    eng = serving.Engine(cap, e0=E0, theta=THETA, dt=DT)
    for q in reqs:
        eng.submit(q)
    order, resident_max, step = [], 0, 0
    seen = set()
    while not eng.idle():
        done = eng.step()
        step += 1
        resident_max = max(resident_max, eng.n)
        for r in eng.resident:
            if r.req.rid not in seen:
                seen.add(r.req.rid)
                order.append(r.req.rid)
        for d in done:
            assert d.steps == reqs[d.rid].steps
        assert step < 200
    eng.close()
    assert resident_max <= cap
    assert order == sorted(order)  # admitted in arrival order
    with pytest.raises(ValueError):
        serving.Engine(100, e0=E0, theta=THETA, dt=DT).submit(reqs[0])


def test_serve_realtime_trace():
    import serving

    reqs = _requests()
    for k, q in enumerate(reqs):
        q.arrival = 0.01 * k
    eng = serving.Engine(20000, e0=E0, theta=THETA, dt=DT)
    results = serving.serve(eng, reqs, realtime=True)
    eng.close()
    assert all(r.completed >= r.admitted >= r.arrival for r in results)
    _check_alone(results, _requests())
