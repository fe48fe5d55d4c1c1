"""Steps replayed from a captured CUDA graph (ag2_step_graphs): the build's
level loop and moments levels run as conditional nodes on the device, and the
results are bit-identical to the same steps launched one by one."""
import numpy as np
import pytest

import ics

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "acc", "U", "h", "rho")


def _run(parts, steps, graphs, dt=1e-3, e0=0.01, mih=None, change_dt_at=None):
    import ag2

    n = sum(len(p["mass"]) for p in parts)
    c = ag2.Context(n, e0=e0, massInH=(mih[0] if mih and len(parts) == 1 else 0.0))
    cat = lambda k: np.concatenate([p[k] for p in parts])  # noqa: E731
    c.upload(cat("pos"), cat("mass"), cat("type"), vel=cat("vel"), U=cat("U"))
    if len(parts) > 1:
        c.set_instances(np.cumsum([0] + [len(p["mass"]) for p in parts]), mih)
    c.build_tree()
    c.sph_density()
    c.forces()
    if graphs:
        c.step_graphs(True)
    l0 = c.launches()
    for s in range(steps):
        c.step(dt if change_dt_at is None or s < change_dt_at else dt / 2)
    out = {f: c.download(f) for f in FIELDS}
    out["nodes"] = c.node_count()
    out["launches"] = c.launches() - l0
    out["inter"] = c.interactions()
    c.close()
    return out


@pytest.mark.parametrize("case", ["gas_cloud", "disk", "forest"])
def test_graph_steps_match_launched_steps(case):
    if case == "gas_cloud":
        d = ics.small_gas_cloud(6000, seed=81)
        parts, mih = [d], [d["massInH"]]
    elif case == "disk":
        d = ics.disk_galaxy(12000, 3000, 1500, seed=82)
        parts, mih = [d], [d["massInH"]]
    else:
        parts = [ics.plummer(3000, seed=83), ics.small_gas_cloud(2500, seed=84), ics.plummer(1, seed=85),
                 ics.disk_galaxy(4000, 1000, 500, seed=86)]
        mih = [0.0, parts[1]["massInH"], 0.0, parts[3]["massInH"]]
    a = _run(parts, 5, False, mih=mih)
    b = _run(parts, 5, True, mih=mih)
    for f in FIELDS:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)
    assert a["nodes"] == b["nodes"]
    assert a["inter"] == b["inter"]
    assert b["launches"] > 0


def test_graph_recaptured_when_dt_changes():
    d = ics.small_gas_cloud(3000, seed=87)
    a = _run([d], 4, False, mih=[d["massInH"]], change_dt_at=2)
    b = _run([d], 4, True, mih=[d["massInH"]], change_dt_at=2)
    for f in FIELDS:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)
