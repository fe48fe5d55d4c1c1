"""CUDA path (through the C-ABI) against the reference fixtures and the C
restatement.  Tolerances:

* topology (node count, per-node depth / leaf flag / leaf particle / childParticles
  count and membership hash / geometric centre / half-width), Particle::node,
  root half-width: bit-exact;
* gasMass of nodes: bit-exact when all gas particles share one mass (the
  reference's sequential sums are reproduced), else relative 1e-12;
* node mass / centre of mass / gas velocity: relative 1e-12 (sum order);
* h: bit-exact; rho, P, T, visualDensity: relative 1e-12;
* acc: FP64 walk relative 1e-12 per particle; FP32 walk median <= 1e-5 and
  99.9th percentile <= 1e-3 relative error (the accuracy contract);
* kick / drift / Ueuler applied to identical inputs: bit-exact.
"""
import glob
import os

import numpy as np
import pytest

import ics
import oracle

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
DT = 1e-3


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build

    build.build()
    if not oracle.available("port"):
        build.build_checkers()


def ctx_for(d, e0=0.01, theta=0.5, massInH=0.0, threads=1, precision="fp64"):
    import ag2

    c = ag2.Context(max(len(d["mass"]), 1), e0=e0, theta=theta, massInH=massInH, split_threshold=100 * threads,
                    precision=precision)
    c.upload(d["pos"], d["mass"], d["type"], vel=d.get("vel"), U=d.get("U"))
    return c


def rel_err(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def check_topology(t, ref, uniform_gas, exact_fp=False):
    for k in ("depth", "is_leaf", "particle", "cp_count", "cp_hash", "center", "radius"):
        assert np.array_equal(t[k], ref[k]), k
    if uniform_gas:
        assert np.array_equal(t["gas_mass"], ref["gas_mass"])
    # a leaf's centre of mass is the reference's one-insertion running mean,
    # (0*(m-m) + x*m)/m, or the position itself: bit-exact
    leaf = (t["is_leaf"] == 1) & (t["particle"] >= 0) & (ref["mass"] > 0)
    assert np.array_equal(t["com"][leaf], ref["com"][leaf])
    scale = np.max(np.abs(ref["center"])) + ref["radius"][0]
    for k in ("mass", "gas_mass", "mvel", "com"):
        s = scale if k == "com" else max(np.max(np.abs(ref[k])), 1e-300)
        np.testing.assert_allclose(t[k], ref[k], rtol=1e-12, atol=1e-13 * s, err_msg=k)


def fixture_dict(z):
    return {k[3:]: z[k] for k in z.files if k.startswith("in_")}, \
        {k[2:]: z[k].item() for k in z.files if k.startswith("p_")}


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def test_fixture(path, precision):
    z = np.load(path)
    d, p = fixture_dict(z)
    c = ctx_for(d, e0=p["e0"], theta=p["theta"], massInH=p["massInH"], threads=p["threads"], precision=precision)
    c.build_tree()
    nn, ni, _ = c.node_count()
    assert nn == int(z["nodes"]) and nn == 1 + 8 * ni
    assert c.root_radius() == float(z["R"])
    ref_topo = {k[5:]: z[k] for k in z.files if k.startswith("topo_")}
    gas_m = d["mass"][d["type"] == 2]
    check_topology(c.topology(), ref_topo, uniform_gas=gas_m.size == 0 or gas_m.min() == gas_m.max())
    np.testing.assert_array_equal(c.particle_node(), z["leaf_index"])
    c.visual_density(float(z["R"]) / 100.0)
    np.testing.assert_allclose(c.download("vdens"), z["vdens"], rtol=1e-12, atol=0)
    c.sph_density()
    np.testing.assert_array_equal(c.download("h"), z["h"])
    for k in ("rho", "P", "T"):
        np.testing.assert_allclose(c.download(k), z[k], rtol=1e-12, atol=0, err_msg=k)
    c.forces()
    acc = c.download("acc")
    e = rel_err(acc, z["acc"])
    if precision == "fp64":
        assert e.max() <= 1e-12 if p["threads"] == 1 else 1e-9, e.max()
    else:
        assert np.median(e) <= 1e-5 and np.quantile(e, 0.999) <= 1e-3, (np.median(e), e.max())
    du = c.download("dUdt")
    scale = max(np.max(np.abs(z["dUdt"])), 1e-300)
    tol = 1e-11 if precision == "fp64" else 1e-4
    assert np.max(np.abs(du - z["dUdt"])) <= tol * scale


@pytest.mark.parametrize("path", FIXTURES[:6], ids=[os.path.basename(f)[:-4] for f in FIXTURES[:6]])
def test_leapfrog_bit_exact(path):
    """Ueuler, kick, drift on the fixture's own acc/dUdt reproduce the reference."""
    z = np.load(path)
    d, p = fixture_dict(z)
    c = ctx_for(d, e0=p["e0"], theta=p["theta"], massInH=p["massInH"])
    c.set_field("acc", z["acc"])
    c.set_field("dUdt", z["dUdt"])
    c.ueuler(DT)
    c.kick(DT)
    c.drift(DT)
    np.testing.assert_array_equal(c.download("vel"), z["after_vel"])
    np.testing.assert_array_equal(c.download("pos"), z["after_pos"])
    U = z["after_U"].copy()
    g = d["type"] == 2
    np.testing.assert_array_equal(c.download("U")[g], U[g])


def port_world(d, threads=1, massInH=0.0, e0=0.01, theta=0.5):
    w = oracle.World(d["pos"], d["mass"], d["type"], d.get("vel"), d.get("U"), kind="port")
    w.build(threads)
    if (d["type"] == 2).any():
        w.gas_density(massInH)
    w.forces(e0, theta, os.cpu_count() or 1)
    return w


@pytest.mark.parametrize("name", ["plummer16k", "disk65k", "general4k", "plummer16k_t8", "disk65k_t16"])
def test_against_port_medium(name):
    """disk65k_t16: 16 threads put the parallel threshold at 1600, above what one
    warp builds in shared memory, so the level loop builds the serial levels too."""
    threads, e0, massInH = 1, 0.01, 0.0
    if name == "plummer16k":
        d = ics.plummer(16384, seed=1)
    elif name == "plummer16k_t8":
        d, threads = ics.plummer(16384, seed=1), 8
    elif name == "disk65k_t16":
        d, threads = ics.disk_galaxy(49152, 12288, 4096, seed=7), 16
        e0, massInH = 0.02, d["massInH"]
    elif name == "disk65k":
        d = ics.disk_galaxy(49152, 12288, 4096, seed=7)
        e0, massInH = 0.02, d["massInH"]
    else:
        d, e0 = ics.plummer(4096, seed=8), 1.0
    w = port_world(d, threads=threads, massInH=massInH, e0=e0)
    ref_t = w.topology()
    for precision in ("fp64", "fp32"):
        c = ctx_for(d, e0=e0, massInH=massInH, threads=threads, precision=precision)
        c.build_tree()
        assert c.node_count()[0] == w.node_count()
        t = c.topology()
        for k in ("depth", "is_leaf", "particle", "cp_count", "cp_hash"):
            assert np.array_equal(t[k], ref_t[k]), k
        np.testing.assert_array_equal(c.particle_node(), w.leaf_index())
        c.sph_density()
        if massInH:
            np.testing.assert_array_equal(c.download("h"), w.get("h"))
            np.testing.assert_allclose(c.download("rho"), w.get("rho"), rtol=1e-12, atol=0)
        c.forces()
        e = rel_err(c.download("acc"), w.get("acc"))
        if precision == "fp64":
            assert e.max() <= 1e-11, e.max()
        else:
            assert np.median(e) <= 1e-5 and np.quantile(e, 0.999) <= 1e-3, (np.median(e), np.quantile(e, 0.999))
        c.close()


def test_full_steps_match_port():
    """Three steps of the reference's step loop (Simulation.cpp:256-341) with
    the FP64 walk: kick+drift, build, density, forces, Ueuler, kick."""
    d = ics.disk_galaxy(6144, 1536, 512, seed=9)
    mih = d["massInH"]
    c = ctx_for(d, e0=0.02, massInH=mih)
    w = oracle.World(d["pos"], d["mass"], d["type"], d["vel"], d["U"], kind="port")
    # initial forces as Simulation::init does (Simulation.cpp:120-139)
    c.build_tree()
    c.sph_density()
    c.forces()
    w.build(1)
    w.gas_density(mih)
    w.forces(0.02, 0.5, os.cpu_count() or 1)
    for _ in range(3):
        c.step(DT)
        w.kick(DT)
        w.drift(DT)
        w.build(1)
        w.gas_density(mih)
        w.forces(0.02, 0.5, os.cpu_count() or 1)
        w.ueuler(DT)
        w.kick(DT)
    for k, tol in (("pos", 1e-12), ("vel", 1e-10), ("U", 1e-10)):
        a, b = c.download(k), w.get(k)
        scale = np.max(np.abs(b))
        assert np.max(np.abs(a - b)) <= tol * scale, k


def test_root_radius_after_reordering_builds():
    """The state is kept in tree order between builds; the root half-width must
    still be summed in the caller's particle order (Tree.cpp:99-103)."""
    for n in (3000, 70000):
        d = ics.plummer(n, seed=12)
        c = ctx_for(d)
        w = oracle.World(d["pos"], d["mass"], d["type"], d["vel"], kind="port")
        for _ in range(3):
            c.build_tree()
            c.forces()
            c.kick_drift(1e-3)
            w.build(1)
            w.forces(0.01, 0.5, os.cpu_count() or 1)
            w.kick(1e-3)
            w.drift(1e-3)
        c.set_field("pos", w.get("pos"))
        c.build_tree()
        w.build(1)
        if n <= 32768:
            assert c.root_radius() == w.root_radius()
        else:
            assert c.root_radius() == pytest.approx(w.root_radius(), rel=1e-15)


def test_large_properties():
    """1M Plummer sphere: node-count identity, one leaf per particle, FP32 walk
    against FP64 walk."""
    d = ics.plummer(1 << 20, seed=1)
    c = ctx_for(d, precision="fp64")
    c.build_tree()
    nn, ni, depth = c.node_count()
    assert nn == 1 + 8 * ni and depth < 40
    node = c.particle_node()
    inside = node >= 0
    assert inside.mean() > 0.999
    assert len(np.unique(node[inside])) == inside.sum()
    c.forces()
    a64 = c.download("acc")
    g64, _ = c.interactions()
    c.set(precision="fp32")
    c.forces()
    a32 = c.download("acc")
    g32, _ = c.interactions()
    e = rel_err(a32, a64)
    assert np.median(e) <= 1e-5 and np.quantile(e, 0.999) <= 1e-3
    assert abs(g32 - g64) <= 1e-4 * g64  # same accepted node set up to guard-band ties


def test_edge_cases():
    import ag2

    # empty, one and two particles
    for n in (0, 1, 2):
        d = ics.plummer(max(n, 1), seed=5)
        d = {k: (v[:n] if hasattr(v, "__len__") else v) for k, v in d.items()}
        c = ctx_for(d)
        c.build_tree()
        w = port_world(d) if n else None
        nn = c.node_count()[0]
        assert nn == (w.node_count() if n else 1)
        c.forces()
        if n:
            np.testing.assert_allclose(c.download("acc"), w.get("acc"), rtol=1e-12, atol=0)
    # coincident particles off the centre planes: the reference separates nothing
    # but drops them once the half-width falls below their ulp (depth ~58)
    pos = np.concatenate([[[0.1, 0.2, 0.3]] * 3, ics.plummer(40, seed=2)["pos"]])
    d = {"pos": pos, "mass": np.ones(len(pos)), "type": np.ones(len(pos), np.uint8)}
    w = port_world(d)
    c = ctx_for(d)
    c.build_tree()
    assert c.node_count()[0] == w.node_count()
    assert np.array_equal(c.topology()["cp_hash"], w.topology()["cp_hash"])
    np.testing.assert_array_equal(c.particle_node(), w.leaf_index())
    # coincident particles on every centre plane (the origin): the reference's
    # chain only ends when the half-width underflows (~1075 levels); here an error
    pos = np.concatenate([[[0.0, 0.0, 0.0]] * 3, ics.plummer(40, seed=2)["pos"]])
    d = {"pos": pos, "mass": np.ones(len(pos)), "type": np.ones(len(pos), np.uint8)}
    c = ctx_for(d)
    with pytest.raises(ag2.AG2Error) as ei:
        c.build_tree()
    assert ei.value.code == ag2.E_COINCIDENT
    # the same in the level loop: 150 coincident particles keep a parallel node
    # (threshold 100) splitting until the depth limit; the loop, one level ahead
    # of the host, reports the error from the control block it reads back
    pos = np.concatenate([[[0.0, 0.0, 0.0]] * 150, ics.plummer(400, seed=2)["pos"]])
    d = {"pos": pos, "mass": np.ones(len(pos)), "type": np.ones(len(pos), np.uint8)}
    c = ctx_for(d)
    with pytest.raises(ag2.AG2Error) as ei:
        c.build_tree()
    assert ei.value.code == ag2.E_COINCIDENT
    c.close()
    c = ctx_for(ics.plummer(550, seed=3))  # a context after the failed one builds normally
    c.build_tree()
    assert c.node_count()[0] > 1
    # non-finite position
    d = {"pos": np.array([[0.1, np.nan, 0.3], [0.0, 0.0, 0.0]]), "mass": np.ones(2), "type": np.ones(2, np.uint8)}
    c = ag2.Context(2)
    with pytest.raises(ag2.AG2Error) as ei:
        c.upload(d["pos"], d["mass"], d["type"])
    assert ei.value.code == ag2.E_NAN
    # capacity and call order
    c = ag2.Context(4)
    with pytest.raises(ag2.AG2Error) as ei:
        c.upload(np.zeros((5, 3)), np.ones(5), np.ones(5, np.uint8))
    assert ei.value.code == ag2.E_CAPACITY
    d = ics.plummer(8, seed=1)
    c = ctx_for(d)
    with pytest.raises(ag2.AG2Error) as ei:
        c.forces()
    assert ei.value.code == ag2.E_INVALID


def test_massless_and_out_of_box_particles():
    """Massless particles feel no force (Node.cpp:264-267); particles beyond the
    root box (|x| > mean + 10 sigma) are not inserted but still feel forces."""
    d = ics.plummer(3000, seed=6)
    d["mass"] = d["mass"].copy()
    d["mass"][:10] = 0.0
    d["pos"] = d["pos"].copy()
    d["pos"][10] = [500.0, 0.0, 0.0]
    w = port_world(d)
    c = ctx_for(d)
    c.build_tree()
    assert c.node_count()[0] == w.node_count()
    np.testing.assert_array_equal(c.particle_node(), w.leaf_index())
    c.forces()
    acc = c.download("acc")
    np.testing.assert_array_equal(acc[:10], 0.0)
    e = rel_err(acc[10:], w.get("acc")[10:])
    assert e.max() <= 1e-11
