"""Snapshot writer and initial-condition loader on the device (ag2_io.cu)
against the restatement of DataManager::saveData / loadICs
(oracle/snapio.py): bit-exact file bytes and bit-exact loaded fields."""
import os

import numpy as np
import pytest

import snapio as S

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "mass", "T", "P", "vdens", "U")


def _ctx_with(p, build=True):
    import ag2

    n = len(p["mass"])
    c = ag2.Context(max(n, 1), e0=1e18, theta=0.5)
    c.upload(p["pos"], p["mass"], p["type"], vel=p["vel"], U=p["U"])
    for f in ("T", "P", "vdens"):
        c.set_field(f, p[f])
    c.set_tags(p["id"], p["gp"], p["sfr"])
    if build:
        c.build_tree()  # the state is now in tree order: the writer must undo it
    return c


def _state(c):
    """The context's particles in upload order, as oracle particles."""
    p = {k: c.download(k) for k in FIELDS}
    p["pos"] = p["pos"].reshape(-1, 3)
    p["vel"] = p["vel"].reshape(-1, 3)
    t = c.tags()
    p["id"], p["gp"], p["sfr"] = t["id"], t["gp"], t["sfr"]
    p["type"] = None
    return p


@pytest.mark.parametrize("fmt", ["ag", "agc", "age", "gadget"])
@pytest.mark.parametrize("n,count", [(5000, 5000), (5000, 4877), (3, 1), (64, 0)])
def test_snapshot_matches_oracle(fmt, n, count):
    p = S.random_particles(n, 17 + n)
    c = _ctx_with(p)
    q = _state(c)
    q["type"] = p["type"]
    # the build only permutes: upload-order values are the uploaded ones
    for k in ("pos", "mass", "T", "P", "vdens", "U", "id", "gp", "sfr"):
        assert np.array_equal(q[k], p[k]), k
    got = c.snapshot_bytes(fmt, count, 0.5, 100.0, 12.25)
    assert got == S.encode(S.NAMES[fmt], p, count, 0.5, 100.0, 12.25)


def test_snapshot_after_steps():
    """The writer reads the evolved, tree-ordered state."""
    import ics

    d = ics.plummer(20000, seed=4)
    import ag2

    c = ag2.Context(20000, e0=0.01, theta=0.5)
    c.upload(d["pos"], d["mass"], d["type"], vel=d["vel"], U=d["U"])
    rng = np.random.default_rng(1)
    gp = rng.integers(1, 4, 20000).astype(np.uint8)
    c.set_tags(None, gp, None)
    c.build_tree()
    c.sph_density()
    c.forces()
    for _ in range(3):
        c.step(1e-3)
    q = _state(c)
    q["type"] = d["type"].astype(np.uint8)
    for fmt in ("ag", "agc", "age", "gadget"):
        assert c.snapshot_bytes(fmt, None, 1e-3, 1.0, 3e-3) == S.encode(S.NAMES[fmt], q, 20000, 1e-3, 1.0, 3e-3)


def test_snapshot_write_async(tmp_path):
    p = S.random_particles(30000, 2)
    c = _ctx_with(p)
    paths = []
    for k, fmt in enumerate(["age", "gadget", "ag", "agc"]):
        path = tmp_path / f"{k}.{fmt}"
        c.snapshot_write(path, fmt, 30000 - k, 1.0, 2.0, 3.0 + k, wait=False)
        paths.append((path, fmt, 30000 - k, 3.0 + k))
        c.build_tree()  # device work continues while the file is written
    c.snapshot_wait()
    for path, fmt, count, t in paths:
        assert path.read_bytes() == S.encode(S.NAMES[fmt], p, count, 1.0, 2.0, t)
    c.snapshot_write(tmp_path / "sync.age", "age", 100)
    assert (tmp_path / "sync.age").read_bytes() == S.encode(S.FMT_AGE, p, 100)


def test_snapshot_write_reports_io_errors(tmp_path):
    import ag2

    c = _ctx_with(S.random_particles(10, 1))
    c.snapshot_write(tmp_path / "missing_dir" / "x.ag", "ag", wait=False)
    with pytest.raises(ag2.AG2Error) as e:
        c.snapshot_wait()
    assert e.value.code == -10
    with pytest.raises(ag2.AG2Error):
        c.snapshot_bytes("ag", 11)  # more than the particles


def _check_load(b, fmt, tmp_path, cap=None):
    import ag2

    f = tmp_path / ("ic." + fmt)
    f.write_bytes(b)
    o, times = S.decode(S.NAMES[fmt], b)
    n = len(o["mass"])
    assert ag2.ic_count(f, fmt) == n
    c = ag2.Context(cap or max(n, 1), e0=1e18)
    got_times = c.load_ics(f, fmt)
    assert got_times == tuple(times)
    q = _state(c)
    for k in ("pos", "vel", "mass", "T", "P", "vdens", "U", "id", "gp", "sfr"):
        assert np.array_equal(q[k], o[k]), k
    # the type array is checked through the snapshot writer, which reads it
    assert c.snapshot_bytes("ag") == S.encode(S.FMT_AG, o, n)
    return c, o


@pytest.mark.parametrize("fmt", ["ag", "agc", "age"])
@pytest.mark.parametrize("n", [1, 31, 33, 10000])
def test_load_records_matches_oracle(fmt, n, tmp_path):
    p = S.random_particles(n, 5 + n)
    _check_load(S.encode(S.NAMES[fmt], p, n, 0.5, 2.0, 1.5), fmt, tmp_path)


def _gadget(seed, individual, gas, short_mass=False, n_scale=1):
    rng = np.random.default_rng(seed)
    npart = [40 * n_scale if gas else 0, 300 * n_scale, 200 * n_scale, 50, 7, 3]
    n = sum(npart)
    massarr = [0.0] * 6 if individual else [0.01, 0.02, 0.003, 0.004, 0.005, 0.006]
    masses = rng.uniform(1e-4, 1e-2, n).astype(np.float32) if individual else None
    if short_mass:
        masses = masses[: n - 5]
    return S.gadget_ic(npart, rng.normal(0, 5, (n, 3)).astype(np.float32),
                       rng.normal(0, 150, (n, 3)).astype(np.float32), rng.permutation(n).astype(np.uint32), massarr,
                       masses, rng.uniform(1, 1e3, npart[0]).astype(np.float32) if gas else None, time=0.25)


@pytest.mark.parametrize("individual,gas,short", [(True, True, False), (False, True, False), (True, False, False),
                                                  (False, False, False), (True, True, True)])
def test_load_gadget_matches_oracle(individual, gas, short, tmp_path):
    _check_load(_gadget(8, individual, gas, short), "gadget", tmp_path)


@pytest.mark.parametrize("mass_block", [True, False])
def test_load_makegal_matches_oracle(mass_block, tmp_path):
    rng = np.random.default_rng(3)
    npart = [30, 120, 60, 20, 5, 4]
    n = sum(npart)
    mass = [0.0, 0.0, 0.001, 0.0, 0.002, 0.0] if mass_block else [0.01, 0.02, 0.003, 0.004, 0.005, 0.006]
    K = sum(npart[k] for k in range(6) if mass[k] == 0 and npart[k] > 0)
    b = S.makegal_ic(npart, rng.normal(0, 5, (n, 3)).astype(np.float32), rng.normal(0, 150, (n, 3)).astype(np.float32),
                     np.arange(n, dtype=np.uint32), mass,
                     rng.uniform(1e-4, 1e-2, K).astype(np.float32) if mass_block else None,
                     rng.uniform(1, 1e3, npart[0]).astype(np.float32), rng.uniform(0, 1, 30).astype(np.float32),
                     rng.uniform(0, 1, 30).astype(np.float32))
    _check_load(b, "makeGal", tmp_path)


def test_load_then_write_round_trip(tmp_path):
    """age and ag hold every field they write: load -> snapshot gives the
    file back, at a million particles."""
    p = S.random_particles(1 << 20, 77)
    for fmt in ("age", "ag"):
        b = S.encode(S.NAMES[fmt], p, 1 << 20, 0.5, 1.0, 0.75)
        f = tmp_path / ("big." + fmt)
        f.write_bytes(b)
        import ag2

        c = ag2.Context(1 << 20, e0=1e18)
        c.load_ics(f, fmt)
        c.build_tree()
        assert c.snapshot_bytes(fmt, None, 0.5, 1.0, 0.75) == b


def test_load_errors(tmp_path):
    import ag2

    p = S.random_particles(100, 1)
    b = S.encode(S.FMT_AGE, p, 100)
    f = tmp_path / "t.age"
    f.write_bytes(b[:-3])
    c = ag2.Context(1000, e0=1e18)
    with pytest.raises(ag2.AG2Error) as e:
        c.load_ics(f, "age")
    assert e.value.code == -9
    with pytest.raises(ag2.AG2Error) as e:
        c.load_ics(tmp_path / "nope", "age")
    assert e.value.code == -10
    f.write_bytes(b)
    small = ag2.Context(50, e0=1e18)
    with pytest.raises(ag2.AG2Error) as e:
        small.load_ics(f, "age")
    assert e.value.code == -8
