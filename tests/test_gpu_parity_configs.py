"""CUDA path against the C restatement of the reference (pinned bit-exactly to
the reference's own outputs by tests/test_oracle_golden.py) at the sizes the
benchmark runs, not only at fixture sizes:

* the isolated disk galaxy of 1,048,576 particles (786,432 halo, 196,608
  stars, 65,536 gas; e0 = 0.02, massInH = 64 m_gas, theta = 0.5), every
  particle;
* the galaxy merger scaled to 262,144 particles at theta = 0.4, 0.5 and 0.7
  (Node.cpp:331-334: the opening test changes the walk, not the tree), every
  particle;
* the 4,194,304-particle merger itself at theta = 0.5: full topology, root
  half-width, h and rho, and the walk on 65,536 seeded particles;
* the 512-sphere ensemble: every 16th simulation against the restatement run
  on that simulation alone.

Tolerances (as tests/test_gpu_parity.py): node count, per-node depth / leaf
flag / leaf particle / childParticles count and membership hash / centre /
half-width, Particle::node, the root half-width and h bit-exact; rho and
visualDensity relative 1e-12; dU/dt within 1e-10 (FP64) and 1e-4 (FP32) of
its largest value; acc of the FP64 walk relative median <= 1e-12, 99.9th percentile <=
1e-11 and max <= 5e-11 per particle: node masses and centres of mass are
summed bottom-up, not as the reference's running mean (1e-12 relative), and a
particle whose net acceleration nearly cancels magnifies that relative to its
own |a| (the 1M disk's largest is 1.1e-11 at median 3e-13; a different
opening decision would differ by the monopole error, ~1e-3); FP32 walk median
<= 1e-5 and 99.9th percentile <= 1e-3 relative (the accuracy contract).  The
measured figures are printed (pytest -s).
"""
import os

import numpy as np
import pytest

import ics
import oracle

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build

    build.build()
    if not oracle.available("port"):
        build.build_checkers()


def rel_err(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def port_tree(d, massInH):
    w = oracle.World(d["pos"], d["mass"], d["type"], d.get("vel"), d.get("U"), kind="port")
    w.build(1)
    if massInH:
        w.gas_density(massInH)
    return w


def check_tree(c, w, massInH, label):
    """Returns the node count and both roots' (mass, centre of mass): GPU, restatement."""
    nn = c.node_count()[0]
    assert nn == w.node_count(), (label, nn, w.node_count())
    assert c.root_radius() == w.root_radius(), label
    t, ref = c.topology(), w.topology()
    for k in ("depth", "is_leaf", "particle", "cp_count", "cp_hash", "center", "radius"):
        assert np.array_equal(t[k], ref[k]), (label, k)
    np.testing.assert_array_equal(c.particle_node(), w.leaf_index())
    roots = ((t["mass"][0], t["com"][0].copy()), (ref["mass"][0], ref["com"][0].copy()))
    del t, ref
    if massInH:
        c.sph_density()
        np.testing.assert_array_equal(c.download("h"), w.get("h"))
        np.testing.assert_allclose(c.download("rho"), w.get("rho"), rtol=1e-12, atol=0)
    return nn, roots


def check_forces(c, ref_acc, idx, precision, label, fp64_bound=(1e-12, 1e-11, 5e-11)):
    c.forces()
    acc = c.download("acc")
    e = rel_err(acc[idx], ref_acc[idx])
    med, p999, mx = float(np.median(e)), float(np.quantile(e, 0.999)), float(e.max())
    print(f"\n{label} {precision}: {idx.size} particles, rel err median {med:.2e} p99.9 {p999:.2e} max {mx:.2e}")
    if precision == "fp64":
        assert med <= fp64_bound[0] and p999 <= fp64_bound[1] and mx <= fp64_bound[2], (label, med, p999, mx)
    else:
        assert med <= 1e-5 and p999 <= 1e-3, (label, med, p999)


def check_dudt(c, ref_du, gas, precision, label):
    """dU/dt of the gas (the SPH heating the walk adds): FP64 within 1e-10
    and FP32 within 1e-4 of the largest |dU/dt|."""
    du = c.download("dUdt")
    scale = max(np.max(np.abs(ref_du[gas])), 1e-300)
    err = np.max(np.abs(du[gas] - ref_du[gas])) / scale
    print(f"\n{label} {precision}: dU/dt max diff {err:.2e} of scale")
    assert err <= (1e-10 if precision == "fp64" else 1e-4), (label, err)


def ctx_for(d, e0, theta, massInH, precision):
    import ag2

    c = ag2.Context(len(d["mass"]), e0=e0, theta=theta, massInH=massInH, split_threshold=100, precision=precision)
    c.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
    return c


def test_disk1m_against_port():
    """The plain-method configuration: a 1,048,576-particle disk galaxy."""
    d = ics.disk_galaxy(seed=2)
    e0, theta, mih = 0.02, 0.5, d["massInH"]
    w = port_tree(d, mih)
    Rv = w.root_radius() / 1e5  # Simulation.cpp:126
    w.visual_density(Rv)
    w.forces(e0, theta, THREADS)
    ref_acc, ref_du, ref_vd = w.get("acc"), w.get("dUdt"), w.get("vdens")
    gas = d["type"] == 2
    idx = np.arange(len(d["mass"]))
    for precision in ("fp64", "fp32"):
        c = ctx_for(d, e0, theta, mih, precision)
        c.build_tree()
        nn, _ = check_tree(c, w, mih, "disk1m")
        c.visual_density(Rv)
        np.testing.assert_allclose(c.download("vdens"), ref_vd, rtol=1e-12, atol=0)
        check_forces(c, ref_acc, idx, precision, f"disk1m ({nn} nodes)")
        check_dudt(c, ref_du, gas, precision, "disk1m")
        c.close()


@pytest.mark.parametrize("theta", [0.4, 0.5, 0.7])
def test_merger262k_theta_sweep_against_port(theta):
    """The precision form's opening angles on the merger, scaled to 262,144."""
    d = ics.merger(131072, seed=3)
    e0, mih = 0.02, d["massInH"]
    w = port_tree(d, mih)
    w.forces(e0, theta, THREADS)
    ref_acc, ref_du = w.get("acc"), w.get("dUdt")
    idx = np.arange(len(d["mass"]))
    for precision in ("fp64", "fp32"):
        c = ctx_for(d, e0, theta, mih, precision)
        c.build_tree()
        check_tree(c, w, mih, f"merger262k theta {theta}")
        check_forces(c, ref_acc, idx, precision, f"merger262k theta {theta}")
        check_dudt(c, ref_du, d["type"] == 2, precision, f"merger262k theta {theta}")
        c.close()


def test_merger4m_against_port():
    """The benchmark's own 4,194,304-particle merger at theta = 0.5: the whole
    tree, h and rho bit for bit, and the walk on 65,536 seeded particles.

    The FP64 accelerations are held to median 1e-11, 99.9th percentile 1e-10
    and max 1e-9.  At this size the reference's own node sums carry rounding
    that grows with their lists: a parallel node adds its particles' masses and
    mass-weighted positions one after another in list order (Node.cpp:465-506),
    up to 4,194,304 terms here, where the GPU sums them as a tree.  The
    restatement's root mass is off by 3.7e-11 relative (the GPU's by ~1e-16),
    and a particle pulled mostly by the other galaxy feels that directly.  The
    test measures it: both roots' mass and centre of mass against the exactly
    rounded values (math.fsum of the masses and of the same rounded products
    x*m), and the GPU's are the closer."""
    import math

    d = ics.merger(2097152, seed=3)
    e0, theta, mih = 0.02, 0.5, d["massInH"]
    w = port_tree(d, mih)
    rng = np.random.default_rng(65536)
    idx = np.sort(rng.choice(len(d["mass"]), size=65536, replace=False)).astype(np.int32)
    w.forces_subset(e0, theta, idx, THREADS)
    ref_acc = w.get("acc")
    for precision in ("fp64", "fp32"):
        c = ctx_for(d, e0, theta, mih, precision)
        c.build_tree()
        if precision == "fp64":
            _, ((gm, gc), (rm, rc)) = check_tree(c, w, mih, "merger4m")
            m, x = d["mass"], d["pos"]
            M = math.fsum(m)
            exact = np.array([math.fsum(x[:, k] * m) / M for k in range(3)])
            egm, erm = abs(gm - M) / M, abs(rm - M) / M
            egc, erc = np.abs(gc - exact).max(), np.abs(rc - exact).max()
            print(f"\nmerger4m root against exactly rounded sums: mass rel err GPU {egm:.2e} restatement {erm:.2e}; "
                  f"centre of mass abs err GPU {egc:.2e} restatement {erc:.2e}")
            assert egm <= erm and egm <= 1e-14 and egc <= erc
        else:
            c.sph_density()
        check_forces(c, ref_acc, idx, precision, "merger4m", fp64_bound=(1e-11, 1e-10, 1e-9))
        c.close()


def test_ensemble_instances_against_port():
    """The 512-simulation ensemble in one context: every 16th simulation
    against the restatement run on that simulation alone."""
    import ag2

    d = ics.ensemble(512)
    first = d["first"]
    e0, theta = 0.01, 0.5
    c = ag2.Context(len(d["mass"]), e0=e0, theta=theta, split_threshold=100, precision="fp64")
    c.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
    c.set_instances(first)
    c.build_tree()
    c.forces()
    a64 = c.download("acc")
    c.set(precision="fp32")
    c.forces()
    a32 = c.download("acc")
    worst64, e32 = 0.0, []
    for k in range(0, len(first) - 1, 16):
        a, b = int(first[k]), int(first[k + 1])
        w = oracle.World(d["pos"][a:b], d["mass"][a:b], d["type"][a:b], d["vel"][a:b], d["U"][a:b], kind="port")
        w.build(1)
        w.forces(e0, theta, THREADS)
        r = rel_err(a64[a:b], w.get("acc"))
        worst64 = max(worst64, float(r.max()))
        assert r.max() <= 5e-11, (k, r.max())
        e32.append(rel_err(a32[a:b], w.get("acc")))
        assert c.instance_radius(k) == w.root_radius(), k
    e = np.concatenate(e32)
    print(f"\nensemble: 32 of 512 simulations ({e.size} particles), FP64 max {worst64:.2e}, "
          f"FP32 median {np.median(e):.2e} p99.9 {np.quantile(e, 0.999):.2e}")
    assert np.median(e) <= 1e-5 and np.quantile(e, 0.999) <= 1e-3
    c.close()
