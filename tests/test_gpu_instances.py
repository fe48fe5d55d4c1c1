"""Several independent simulations in one context (ag2_set_instances): every
instance's results are bit-identical to the same simulation run alone, because
each instance has its own tree, root half-width, gasMass tables, massInH and
walk groups."""
import numpy as np
import pytest

import ics

pytestmark = pytest.mark.gpu


def _mix():
    parts = [ics.plummer(1000, seed=41), ics.small_gas_cloud(2500, seed=42), ics.plummer(40000, seed=43),
             ics.disk_galaxy(3000, 800, 300, seed=44), ics.plummer(33, seed=45)]
    mih = [0.0, parts[1]["massInH"], 0.0, parts[3]["massInH"], 0.0]
    return parts, mih


def _ctx(parts, mih, precision, e0=0.01):
    import ag2

    n = sum(len(p["mass"]) for p in parts)
    c = ag2.Context(n, e0=e0, precision=precision, massInH=mih[0] if len(parts) == 1 else 0.0)
    cat = lambda k: np.concatenate([p[k] for p in parts])  # noqa: E731
    c.upload(cat("pos"), cat("mass"), cat("type"), vel=cat("vel"), U=cat("U"))
    first = np.cumsum([0] + [len(p["mass"]) for p in parts])
    if len(parts) > 1:
        c.set_instances(first, mih)
    return c, first


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_instances_match_alone(precision):
    parts, mih = _mix()
    c, first = _ctx(parts, mih, precision)
    c.build_tree()
    c.visual_density(0.05)
    c.sph_density()
    c.forces()
    got = {k: c.download(k) for k in ("acc", "h", "rho", "dUdt", "vdens")}
    node = c.particle_node()
    radii = [c.instance_radius(k) for k in range(len(parts))]
    g_mix = c.interactions()
    g_sum = [0, 0]
    for k, p in enumerate(parts):
        a, _ = _ctx([p], [mih[k]], precision)
        a.build_tree()
        a.visual_density(0.05)
        a.sph_density()
        a.forces()
        assert a.root_radius() == radii[k]
        sl = slice(first[k], first[k + 1])
        for f in ("acc", "h", "rho", "dUdt", "vdens"):
            np.testing.assert_array_equal(got[f][sl], a.download(f), err_msg=f"{f} of instance {k}")
        alone_node = a.particle_node()
        assert np.array_equal(node[sl] >= 0, alone_node >= 0)
        gi, si = a.interactions()
        g_sum[0] += gi
        g_sum[1] += si
    assert list(g_mix) == g_sum


def test_instance_steps_and_direct_sum_match_alone():
    parts, mih = _mix()
    c, first = _ctx(parts, mih, "fp32")
    c.build_tree()
    c.sph_density()
    c.forces()
    for _ in range(3):
        c.step(1e-3)
    pos = c.download("pos")
    ids = np.array([first[0] + 3, first[2] + 17, first[3] + 5])
    ds = c.direct_sum(ids)
    for k, p in enumerate(parts):
        a, _ = _ctx([p], [mih[k]], "fp32")
        a.build_tree()
        a.sph_density()
        a.forces()
        for _ in range(3):
            a.step(1e-3)
        np.testing.assert_array_equal(pos[first[k]:first[k + 1]], a.download("pos"))
        for j, i in enumerate(ids):
            if first[k] <= i < first[k + 1]:
                np.testing.assert_array_equal(ds[j], a.direct_sum(np.array([i - first[k]]))[0])


def test_bad_instance_layouts():
    import ag2

    parts, mih = _mix()
    c, first = _ctx(parts, mih, "fp32")
    with pytest.raises(ag2.AG2Error):
        c.set_instances(np.array([0, 10, 5, first[-1]]))
    with pytest.raises(ag2.AG2Error):
        c.set_instances(np.array([1, first[-1]]))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_ragged_forest_with_empty_and_single_particle_simulations(precision):
    """A forest whose simulations include an empty one, single-particle ones
    and an all-gas one: the others are bit-identical to their lone runs, the
    single particles feel no force, and the empty simulation changes nothing."""
    import ag2

    gas = ics.small_gas_cloud(600, seed=47, gas_fraction=1.0)
    one = ics.plummer(1, seed=48)
    parts = [ics.plummer(500, seed=46), {k: v[:0] for k, v in one.items() if hasattr(v, "__len__")}, one, gas,
             ics.plummer(1, seed=49), ics.plummer(300, seed=50)]
    mih = [0.0, 0.0, 0.0, gas["massInH"], 0.0, 0.0]
    n = sum(len(p["mass"]) for p in parts)
    c = ag2.Context(n, e0=0.01, precision=precision)
    cat = lambda k: np.concatenate([p[k] for p in parts])  # noqa: E731
    c.upload(cat("pos"), cat("mass"), cat("type").astype(np.uint8), vel=cat("vel"), U=cat("U"))
    first = np.cumsum([0] + [len(p["mass"]) for p in parts])
    c.set_instances(first, mih)
    c.build_tree()
    c.sph_density()
    c.forces()
    for _ in range(2):
        c.step(1e-3)
    got = {k: c.download(k) for k in ("pos", "acc", "h", "rho")}
    for k, p in enumerate(parts):
        if len(p["mass"]) == 0:
            continue
        a = ag2.Context(len(p["mass"]), e0=0.01, precision=precision, massInH=mih[k])
        a.upload(p["pos"], p["mass"], p["type"].astype(np.uint8), vel=p["vel"], U=p["U"])
        a.build_tree()
        a.sph_density()
        a.forces()
        for _ in range(2):
            a.step(1e-3)
        sl = slice(first[k], first[k + 1])
        for f in got:
            np.testing.assert_array_equal(got[f][sl], a.download(f), err_msg=f"{f} of simulation {k}")
        if len(p["mass"]) == 1:
            assert not got["acc"][sl].any()
        a.close()
    c.close()
