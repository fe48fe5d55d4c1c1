"""The walk's tuning knobs (ag2_autotune_walk, ag2_set_walk_variant,
params.group_size) on the GPU.

* Every candidate is timed and reported; the one kept is the fastest and is
  what later walks use.
* The compiled variants (register budget, first-pass stack depth down to 64
  entries, whose overflowing groups go to the retry pass, L1 prefetch of the
  children to open) give the same FP32
  accelerations bit for bit: the arithmetic is explicit (no contraction) and a
  retried group is walked again from the start.
* The FP64 walk's per-particle sums do not depend on the group size (each
  lane meets its nodes in the reference's depth-first order whatever the other
  lanes do), so group sizes 32 and 16 agree bit for bit; the FP32 walk with
  16-particle groups keeps the accuracy contract (median <= 1e-5, 99.9th
  percentile <= 1e-3 relative to the FP64 walk).
"""
import numpy as np
import pytest

import ics

pytestmark = pytest.mark.gpu


def _ctx(d, **kw):
    import ag2

    c = ag2.Context(len(d["mass"]), e0=0.02, theta=0.5, massInH=d["massInH"], **kw)
    c.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
    c.build_tree()
    c.sph_density()
    return c


def _rel(a, b):
    return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)


def test_autotune_reports_candidates_and_keeps_the_fastest():
    d = ics.disk_galaxy(49152, 12288, 4096, seed=7)
    c = _ctx(d, precision="fp32")
    c.forces()
    r = c.autotune_walk()
    cands = r["candidates"]
    assert len(cands) == 12 and {x["group_size"] for x in cands} == {32, 16}
    assert {x["variant"] for x in cands} == {0, 1, 2, 3, 4, 5}
    assert all(x["ms"] > 0 for x in cands)
    best = min(cands, key=lambda x: x["ms"])
    assert r["chosen"] == best
    assert c.params.group_size == best["group_size"]
    c.forces()
    a32 = c.download("acc")
    c.set(precision="fp64")
    c.forces()
    e = _rel(a32, c.download("acc"))
    assert np.median(e) <= 1e-5 and np.quantile(e, 0.999) <= 1e-3
    c.close()


def test_variants_give_identical_results():
    d = ics.merger(32768, seed=3)
    c = _ctx(d, precision="fp32")
    ref = None
    zero = np.zeros(len(d["mass"]))
    for v in range(6):
        c.set_walk_variant(v)
        c.set_field("dUdt", zero)  # forces adds the SPH heating to dUdt
        c.forces()
        a = c.download("acc")
        du = c.download("dUdt")
        if ref is None:
            ref = (a, du)
        else:
            assert np.array_equal(a, ref[0]) and np.array_equal(du, ref[1]), v
    c.close()


def test_group_size_16():
    d = ics.disk_galaxy(24576, 6144, 2048, seed=5)
    c32 = _ctx(d, precision="fp64")
    c32.forces()
    a64 = c32.download("acc")
    c16 = _ctx(d, precision="fp64")
    c16.set(group_size=16)
    c16.forces()
    assert np.array_equal(c16.download("acc"), a64)
    assert np.array_equal(c16.download("dUdt"), c32.download("dUdt"))
    c16.set(precision="fp32")
    c16.forces()
    e = _rel(c16.download("acc"), a64)
    assert np.median(e) <= 1e-5 and np.quantile(e, 0.999) <= 1e-3
    c16.close()
    c32.close()
