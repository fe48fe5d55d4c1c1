"""Uploads keep the gasMass tables and the instance tables when nothing they
depend on changed (the end-to-end step loop uploads the same particles every
step).  These tests change exactly what the tables depend on between uploads
and check every result against a fresh context, bit for bit."""
import numpy as np
import pytest

import ics

pytestmark = pytest.mark.gpu


def _step_once(c, d):
    c.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
    if "first" in d:
        c.set_instances(d["first"], d.get("mih"))
    c.build_tree()
    c.sph_density()
    c.forces()
    return {k: c.download(k) for k in ("h", "rho", "acc", "dUdt")}


def _fresh(d, **kw):
    import ag2

    c = ag2.Context(len(d["mass"]), **kw)
    r = _step_once(c, d)
    c.close()
    return r


def _same(a, b):
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_gas_mass_change_rebuilds_table():
    import ag2

    d = ics.small_gas_cloud(3000, seed=9)
    kw = dict(e0=0.02, theta=0.5, massInH=d["massInH"])
    c = ag2.Context(3000, **kw)
    _same(_step_once(c, d), _fresh(d, **kw))
    d2 = dict(d)
    d2["mass"] = d["mass"] * np.where(d["type"] == 2, 1.5, 1.0)  # gas particles heavier
    _same(_step_once(c, d2), _fresh(d2, **kw))
    d3 = dict(d2)
    t = d2["type"].copy()
    t[np.flatnonzero(t == 2)[:100]] = 1  # fewer gas particles
    d3["type"] = t
    _same(_step_once(c, d3), _fresh(d3, **kw))
    _same(_step_once(c, d3), _fresh(d3, **kw))  # unchanged: the kept tables


def test_instance_layout_change_with_same_count():
    import ag2

    parts = [ics.small_gas_cloud(n, seed=20 + k) for k, n in enumerate((700, 1300, 1000))]
    d = {k: np.concatenate([p[k] for p in parts]) for k in ("pos", "vel", "mass", "type", "U")}
    d["first"] = np.array([0, 700, 2000, 3000])
    d["mih"] = np.array([p["massInH"] for p in parts])
    kw = dict(e0=0.02, theta=0.5)
    c = ag2.Context(3000, **kw)
    _same(_step_once(c, d), _fresh(d, **kw))
    d2 = dict(d)
    d2["first"] = np.array([0, 2000, 3000])  # same particles, two simulations now
    d2["mih"] = np.array([parts[0]["massInH"], parts[2]["massInH"]])
    _same(_step_once(c, d2), _fresh(d2, **kw))
    _same(_step_once(c, d), _fresh(d, **kw))


def test_reupload_keeps_slots_and_download_order():
    """A second upload of the same count takes the last build's slot order;
    downloads still return the caller's order, bit for bit."""
    import ag2

    d = ics.small_gas_cloud(5000, seed=31)
    c = ag2.Context(5000, e0=0.02, theta=0.5, massInH=d["massInH"])
    _step_once(c, d)
    rng = np.random.default_rng(2)
    pos2 = d["pos"] + rng.normal(0, 1e-3, d["pos"].shape)
    vel2 = rng.normal(0, 1, d["vel"].shape)
    c.upload(pos2, d["mass"], d["type"], vel=vel2, U=d["U"] * 2)
    np.testing.assert_array_equal(c.download("pos"), pos2)
    np.testing.assert_array_equal(c.download("vel"), vel2)
    np.testing.assert_array_equal(c.download("U"), d["U"] * 2)
    np.testing.assert_array_equal(c.download("mass"), d["mass"])


def test_download_fields_equals_download():
    import ag2

    d = ics.small_gas_cloud(4000, seed=32)
    c = ag2.Context(4000, e0=0.02, theta=0.5, massInH=d["massInH"])
    _step_once(c, d)
    c.step(1e-3)
    names = ["pos", "vel", "acc", "U", "h", "rho", "dUdt"]  # more fields than staging halves
    outs = {f: np.empty((4000, 3) if f in ("pos", "vel", "acc") else 4000) for f in names}
    c.download_fields(outs)
    for f in names:
        np.testing.assert_array_equal(outs[f], c.download(f), err_msg=f)
    with pytest.raises(ValueError):
        c.download_fields({"pos": np.empty(4000)})


def test_step_host_equals_separate_calls():
    """ag2_step_host gives the same state as upload + set_field + step +
    downloads, bit for bit, with the outputs written over the inputs."""
    import ag2

    d = ics.small_gas_cloud(6000, seed=33)
    kw = dict(e0=0.02, theta=0.5, massInH=d["massInH"])
    a, b = ag2.Context(6000, **kw), ag2.Context(6000, **kw)
    pos, vel, U = d["pos"].copy(), d["vel"].copy(), d["U"].copy()
    acc = np.zeros_like(pos)
    mass, typ = np.ascontiguousarray(d["mass"]), np.ascontiguousarray(d["type"], np.uint8)
    ref = {"pos": pos.copy(), "vel": vel.copy(), "acc": acc.copy(), "U": U.copy()}
    for _ in range(3):
        a.step_host(1e-3, pos, mass, typ, vel=vel, U=U, acc=acc, out={"pos": pos, "vel": vel, "acc": acc, "U": U})
        b.upload(ref["pos"], mass, typ, vel=ref["vel"], U=ref["U"])
        b.set_field("acc", ref["acc"])
        b.step(1e-3)
        ref = {f: b.download(f) for f in ("pos", "vel", "acc", "U")}
        for f, got in (("pos", pos), ("vel", vel), ("acc", acc), ("U", U)):
            np.testing.assert_array_equal(got, ref[f], err_msg=f)
    assert np.abs(acc).max() > 0


def test_step_host_with_instances():
    import ag2

    parts = [ics.small_gas_cloud(n, seed=40 + k) for k, n in enumerate((900, 2100, 1500))]
    d = {k: np.concatenate([p[k] for p in parts]) for k in ("pos", "vel", "mass", "type", "U")}
    first = np.array([0, 900, 3000, 4500])
    mih = np.array([p["massInH"] for p in parts])
    a, b = ag2.Context(4500, e0=0.02, theta=0.5), ag2.Context(4500, e0=0.02, theta=0.5)
    typ = np.ascontiguousarray(d["type"], np.uint8)
    pos, vel, U, acc = d["pos"].copy(), d["vel"].copy(), d["U"].copy(), np.zeros_like(d["pos"])
    ref = {"pos": pos.copy(), "vel": vel.copy(), "acc": acc.copy(), "U": U.copy()}
    for _ in range(2):
        a.step_host(1e-3, pos, d["mass"], typ, vel=vel, U=U, acc=acc,
                    out={"pos": pos, "vel": vel, "acc": acc, "U": U}, first=first, massInH=mih)
        b.upload(ref["pos"], d["mass"], typ, vel=ref["vel"], U=ref["U"])
        b.set_instances(first, mih)
        b.set_field("acc", ref["acc"])
        b.step(1e-3)
        ref = {f: b.download(f) for f in ("pos", "vel", "acc", "U")}
        for f, got in (("pos", pos), ("vel", vel), ("acc", acc), ("U", U)):
            np.testing.assert_array_equal(got, ref[f], err_msg=f)


def test_step_host_failure_after_readbacks_started():
    """A step_host that fails after its position and acceleration read-backs
    were queued (here a host-injected AG2_E_STACK right after the walk, the
    point where the walk's own stack check would report one) returns only once
    those copies have landed: the position buffer holds the drifted positions,
    and the next upload and step through the same staging area give the same
    bits as a fresh context."""
    import torch

    import ag2

    d = ics.small_gas_cloud(20000, seed=41)
    n = len(d["mass"])
    kw = dict(e0=0.02, theta=0.5, massInH=d["massInH"])
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()  # noqa: E731
    c = ag2.Context(n, **kw)
    c.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
    c.build_tree()
    c.sph_density()
    c.forces()
    acc0 = c.download("acc")
    hpos, hvel, hmass, hU, htype, hacc = (pin(d["pos"]), pin(d["vel"]), pin(d["mass"]), pin(d["U"]), pin(d["type"]),
                                          pin(acc0))
    out = {"pos": pin(np.zeros_like(d["pos"])), "acc": pin(np.zeros_like(acc0)), "vel": pin(np.zeros_like(d["vel"])),
           "U": pin(np.zeros_like(d["U"]))}
    c.inject_fault(1, ag2.E_STACK)
    with pytest.raises(ag2.AG2Error) as ei:
        c.step_host(1e-3, hpos, hmass, htype, vel=hvel, U=hU, acc=hacc, out=out)
    assert ei.value.code == ag2.E_STACK
    # the positions after the kick and drift, as a separate context computes them
    r = ag2.Context(n, **kw)
    r.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
    r.set_field("acc", acc0)
    r.kick_drift(1e-3)
    assert np.array_equal(out["pos"], r.download("pos"))
    r.close()
    # the same context, reused at once: a full step_host against a fresh context
    d2 = ics.small_gas_cloud(20000, seed=42)
    outs = {k: pin(np.zeros_like(v)) for k, v in out.items()}
    c.step_host(1e-3, pin(d2["pos"]), pin(d2["mass"]), pin(d2["type"]), vel=pin(d2["vel"]), U=pin(d2["U"]),
                acc=pin(acc0), out=outs)
    f = ag2.Context(n, **kw)
    ref = {k: pin(np.zeros_like(v)) for k, v in out.items()}
    f.step_host(1e-3, pin(d2["pos"]), pin(d2["mass"]), pin(d2["type"]), vel=pin(d2["vel"]), U=pin(d2["U"]),
                acc=pin(acc0), out=ref)
    for k in outs:
        assert np.array_equal(outs[k], ref[k]), k
    c.close()
    f.close()
