"""Generate the golden fixtures under tests/golden/ by running the reference.

The reference's own Tree/Node/kernel/TimeIntegration sources are compiled into
oracle/_ref/libag2ref.so (``make -C oracle ref``, G = 1 shadow constants) and run
here on small seeded inputs.  Each fixture stores the inputs, the parameters and
the reference's outputs: the tree topology in depth-first preorder, the root
half-width, visualDensity, h/rho/P/T, acc, dUdt, and the state after one
kick/drift/Ueuler.  tests/test_oracle_golden.py pins the C restatement to these
files; the GPU tests compare the CUDA path with them.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "astrogenesis2.0_gb300"))

import ics  # noqa: E402
import oracle  # noqa: E402

DT = 1e-3


def _child(c, r, o):
    sgn = np.array([1.0 if o & 1 else -1.0, 1.0 if o & 2 else -1.0, 1.0 if o & 4 else -1.0])
    return c + r * (sgn * 0.5), r * 0.5, sgn


def _rounding_escape(c, r, o):
    """A point routed from node (c, r) into child o that lies outside the child's
    rounded bounds, or None.  Node.cpp:436-440 accumulates child centres as
    c + r*(+-0.5); the bounds test is inclusive (Node.cpp:606-608)."""
    cc, h, sgn = _child(c, r, o)
    lo, hi = cc - h, cc + h
    for ax in range(3):
        x = cc.copy()
        if sgn[ax] > 0 and lo[ax] > c[ax]:
            x[ax] = np.nextafter(c[ax], np.inf)
            if x[ax] < lo[ax]:
                return x
        elif sgn[ax] < 0 and hi[ax] < c[ax]:
            x[ax] = c[ax]
            if x[ax] > hi[ax]:
                return x
    return None


def boundary_case(seed: int = 21):
    """Particles that the reference drops because a child's rounded bounds do not
    cover its octant (Node.cpp:606-612, 706-711):
      * one below a node that takes the parallel path (>= 100 particles), where
        the dropped particle still counts in that node's mass (Node.cpp:477-499);
      * triplets below serial nodes, where the dropped particle is the first
        (and, elsewhere, not the first) to reach the parent, which decides
        whether its Particle::node keeps pointing at that parent."""
    g = ics.rng(seed)
    # root half-width with a rounding escape two or three levels down, in a cell
    # that lies inside the sphere of radius R (so the anchor at (R,0,0) stays the
    # farthest particle and sets the root half-width)
    hit = None
    for trial in range(5000):
        R = float(g.uniform(1.0, 2.0))
        for path in g.integers(0, 8, size=(64, 3)):
            c, r = np.zeros(3), R
            for lvl, o in enumerate(path):
                cc, h, _ = _child(c, r, int(o))
                x = _rounding_escape(c, r, int(o))
                if lvl >= 1 and x is not None and np.linalg.norm(cc) + np.sqrt(3.0) * h < 0.95 * R:
                    hit = (cc, h, x)
                    break
                c, r = cc, h
            if hit:
                break
        if hit:
            break
    if hit is None:
        raise RuntimeError("no rounding escape found")
    c2, r2, xpar = hit
    pos = [np.array([R, 0.0, 0.0])]
    # 150-particle cluster inside the level-2 cell: that cell and its parent take
    # the parallel path; xpar is routed into the cell and fails its bounds
    pos += list(c2 + g.uniform(-0.8 * r2, 0.8 * r2, (150, 3)))
    pos.append(xpar)
    pos += list(g.uniform(-0.45 * R, 0.45 * R, (40, 3)))
    # serial-path escapes deeper down, away from the cluster
    first = True
    added = 0
    for trial in range(20000):
        c, r = np.zeros(3), R
        for level in range(1, 14):
            o = int(g.integers(0, 8))
            x = _rounding_escape(c, r, o)
            cc, h, sgn = _child(c, r, o)
            far = np.all(np.abs(cc - c2) > 4 * r2) and np.linalg.norm(cc) + 2 * h < 0.9 * R and level >= 4
            if x is not None and far:
                partner, partner2 = cc + sgn * (h * 0.25), cc - sgn * (h * 0.3)
                # array order decides which particle lands first in the parent
                pos += [x, partner, partner2] if first else [partner, x, partner2]
                first = not first
                added += 1
                break
            c, r = cc, h
        if added >= 6:
            break
    pos = np.array(pos)
    n = len(pos)
    typ = np.where(g.uniform(0, 1, n) < 0.5, 2, 1).astype(np.uint8)
    return {"pos": pos, "vel": g.normal(0, 0.1, (n, 3)), "mass": np.full(n, 1.0 / n), "type": typ,
            "U": np.where(typ == 2, 0.01, 0.0), "massInH": 8.0 / n}


def cases():
    out = {}
    out["two_body"] = (dict(pos=np.array([[0.3, -0.1, 0.2], [-0.25, 0.15, -0.05]]), vel=np.zeros((2, 3)),
                            mass=np.array([0.6, 0.4]), type=np.array([1, 1], np.uint8), U=np.zeros(2)),
                       dict(e0=0.01, theta=0.5, threads=1, massInH=0.0))
    out["three"] = (ics.plummer(3, seed=9), dict(e0=0.01, theta=0.5, threads=1, massInH=0.0))
    out["plummer_99"] = (ics.plummer(99, seed=3), dict(e0=0.01, theta=0.5, threads=1, massInH=0.0))
    out["plummer_100"] = (ics.plummer(100, seed=3), dict(e0=0.01, theta=0.5, threads=1, massInH=0.0))
    out["plummer_1k"] = (ics.plummer(1024, seed=1), dict(e0=0.01, theta=0.5, threads=1, massInH=0.0))
    out["plummer_1k_t8"] = (ics.plummer(1024, seed=1), dict(e0=0.01, theta=0.5, threads=8, massInH=0.0))
    out["plummer_1k_theta07"] = (ics.plummer(1024, seed=2), dict(e0=0.01, theta=0.7, threads=1, massInH=0.0))
    gc = ics.small_gas_cloud(2000, seed=5)
    out["gas_cloud_2k"] = (gc, dict(e0=0.01, theta=0.5, threads=1, massInH=gc["massInH"]))
    dg = ics.disk_galaxy(3072, 768, 256, seed=7)
    out["disk_4k"] = (dg, dict(e0=0.02, theta=0.5, threads=1, massInH=dg["massInH"]))
    out["general_law"] = (ics.plummer(256, seed=8), dict(e0=1.0, theta=0.5, threads=1, massInH=0.0))
    bd = boundary_case()
    out["boundary_drops"] = (bd, dict(e0=0.01, theta=0.5, threads=1, massInH=bd["massInH"]))
    return out


def run(kind: str, d: dict, p: dict) -> dict:
    w = oracle.World(d["pos"], d["mass"], d["type"], d.get("vel"), d.get("U"), kind=kind)
    w.build(p["threads"])
    res = {"R": np.array(w.root_radius()), "nodes": np.array(w.node_count())}
    topo = w.topology()
    for k, v in topo.items():
        res["topo_" + k] = v
    res["leaf_index"] = w.leaf_index()
    w.visual_density(w.root_radius() / 100.0)
    res["vdens"] = w.get("vdens")
    w.gas_density(p["massInH"])
    for k in ("h", "rho", "P", "T"):
        res[k] = w.get(k)
    w.forces(p["e0"], p["theta"], 1)
    res["acc"] = w.get("acc")
    res["dUdt"] = w.get("dUdt")
    w.ueuler(DT)
    w.kick(DT)
    w.drift(DT)
    for k in ("pos", "vel", "U"):
        res["after_" + k] = w.get(k)
    w.close()
    return res


def main():
    if not oracle.available("reference"):
        raise SystemExit("oracle/_ref/libag2ref.so missing: make -C oracle ref")
    for name, (d, p) in cases().items():
        res = run("reference", d, p)
        blob = {"in_" + k: np.asarray(d[k]) for k in ("pos", "vel", "mass", "type", "U")}
        blob.update({"p_" + k: np.array(v) for k, v in p.items()})
        blob.update(res)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **blob)
        print(f"{name}: n={len(d['mass'])} nodes={int(res['nodes'])} -> {os.path.relpath(path, REPO)}")


if __name__ == "__main__":
    main()
