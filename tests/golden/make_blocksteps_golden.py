"""Writes tests/golden/blocksteps/plummer2k.npz from the reference itself.

Runs the reference's own step loop with block time steps, Simulation::run
(Simulation.cpp:166-364), through oracle/_ref/libag2ref.so (orc_ref_run) on a
seeded 2,048-particle Plummer sphere, gravity only (the reference's SPH
density races above one thread, and run() sets the thread count itself):

  * initial accelerations as Simulation::init computes them (orc_build with one
    thread, orc_forces);
  * run() with eta = 0.05, minTimeStep = 2^-14, maxTimeStep = 2^-6,
    endTime = 2^-5, e0 = 0.01, theta = 0.5, H0 = 0, no snapshots.

Stored: the inputs and parameters, the initial accelerations, the final
globalTime, positions, velocities and accelerations, every particle's time
step and next integration time, and the host's core count (run() builds its
trees at 100 * std::thread::hardware_concurrency() particles per serial
switch, Tree.cpp:59-60 and Node.cpp:420).

Run from the repository root, where oracle/_ref is built:
    python tests/golden/make_blocksteps_golden.py
"""
from __future__ import annotations

import ctypes
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "astrogenesis2.0_gb300"))

import ics  # noqa: E402
import oracle  # noqa: E402

PARAMS = dict(eta=0.05, min_dt=2.0 ** -14, max_dt=2.0 ** -6, end_time=2.0 ** -5, e0=0.01, theta=0.5, H0=0.0)


def main():
    assert oracle.available("reference"), "build oracle/_ref first (make -C oracle ref)"
    L = oracle.load("reference")
    D, P = ctypes.c_double, ctypes.c_void_p
    L.orc_ref_run.argtypes = [P, ctypes.c_char_p, D, D, D, D, D, D, D, D, P, P, P, P]
    d = ics.plummer(2048, seed=97)
    n = len(d["mass"])
    w = oracle.World(d["pos"], d["mass"], d["type"], d["vel"], d["U"], kind="reference")
    w.build(1)
    w.forces(PARAMS["e0"], PARAMS["theta"])
    acc0 = w.get("acc")
    gt = np.zeros(1)
    ts, tn = np.zeros(n), np.zeros(n)
    cores = ctypes.c_int()
    p = PARAMS
    with tempfile.TemporaryDirectory() as logdir:
        L.orc_ref_run(w.h, logdir.encode(), p["eta"], p["min_dt"], p["max_dt"], p["end_time"], p["e0"], p["theta"],
                      0.0, p["H0"], gt.ctypes.data, ts.ctypes.data, tn.ctypes.data, ctypes.byref(cores))
    out = {f"in_{k}": d[k] for k in ("pos", "vel", "mass", "type", "U")}
    out.update({f"p_{k}": np.array(v) for k, v in PARAMS.items()})
    out.update(acc0=acc0, global_time=gt[0], pos=w.get("pos"), vel=w.get("vel"), acc=w.get("acc"), tstep=ts,
               tnext=tn, cores=np.array(cores.value))
    np.savez_compressed(os.path.join(HERE, "blocksteps", "plummer2k.npz"), **out)
    print(f"global time {gt[0]!r}, cores {cores.value}, distinct steps {np.unique(ts)}")


if __name__ == "__main__":
    main()
