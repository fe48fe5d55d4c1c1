"""The snapshot / initial-condition restatement (oracle/snapio.py) pinned to
the reference's DataManager: golden hashes made by the reference
(tests/golden/ic_examples.json) and, where oracle/_ref is built, the
reference's saveData and loadICs run live on the same particles and files."""
import hashlib
import json
import os
import struct
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
import snapio as S  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "ic_examples.json")))
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
import oracle  # noqa: E402

_REF = oracle.reference_checkout()
EXAMPLES = os.path.join(_REF, "input_data", "Example") if _REF else ""
FIELDS = ("pos", "vel", "mass", "T", "P", "vdens", "U", "sfr", "type", "gp", "id")
need_ref = pytest.mark.skipif(S.ref_lib() is None, reason="oracle/_ref not built (no reference checkout)")


def zero_pad(fmt, b):
    b = bytearray(b)
    if fmt != "gadget":
        b[12:16] = bytes(4)  # AGFHeader padding the reference leaves uninitialised
    return bytes(b)


@pytest.mark.parametrize("fmt", ["ag", "agc", "age", "gadget"])
@pytest.mark.parametrize("count", [1000, 777])
def test_encode_matches_golden(fmt, count):
    p = S.random_particles(1000, 3)
    b = S.encode(S.NAMES[fmt], p, count, 1.5, 2.5, 3.5)
    g = GOLDEN["snapshots"][f"{fmt}_{count}"]
    assert len(b) == g["bytes"]
    assert hashlib.sha256(b).hexdigest() == g["sha256"]


@pytest.mark.skipif(not os.path.isdir(EXAMPLES), reason="reference example files not present")
@pytest.mark.parametrize("name", sorted(GOLDEN["examples"]))
def test_decode_examples_match_golden(name):
    g = GOLDEN["examples"][name]
    p, _ = S.decode(S.NAMES[g["format"]], open(os.path.join(EXAMPLES, name), "rb").read())
    assert len(p["mass"]) == g["n"]
    order = S.canonical_order(p) if g["format"] == "makeGal" else None
    assert S.field_digest(p, order) == g["sha256"]


@need_ref
@pytest.mark.parametrize("fmt", ["ag", "agc", "age", "gadget"])
@pytest.mark.parametrize("seed,n,count", [(1, 1, 1), (2, 37, 0), (5, 4096, 4096), (6, 3000, 1234)])
def test_encode_matches_reference(fmt, seed, n, count):
    p = S.random_particles(n, seed)
    assert zero_pad(fmt, S.ref_save(fmt, p, count, 0.25, 8.0, 1.0 / 3)) == S.encode(S.NAMES[fmt], p, count, 0.25, 8.0,
                                                                                  1.0 / 3)


@need_ref
def test_encode_gadget_only_gas_and_unlisted():
    """Gadget lists with no disk stars, and particles in no list (type 3 in
    the disk, type 1 in the halo): counted in npart[0], written nowhere."""
    p = S.random_particles(500, 9)
    p["type"][:] = np.where(np.arange(500) % 3 == 0, 2, np.where(np.arange(500) % 3 == 1, 3, 1))
    p["gp"][:] = np.where(np.arange(500) % 3 == 1, 1, 3)
    assert S.ref_save("gadget", p, 500) == S.encode(S.FMT_GADGET, p, 500)
    p["type"][:] = 3
    p["gp"][:] = 3
    assert S.ref_save("gadget", p, 500) == S.encode(S.FMT_GADGET, p, 500)  # no gas list: no U block


def same(a, b, fields=FIELDS):
    for k in fields:
        assert np.array_equal(a[k], b[k]), k


@need_ref
@pytest.mark.skipif(not os.path.isdir(EXAMPLES), reason="reference example files not present")
@pytest.mark.parametrize("name", sorted(GOLDEN["examples"]))
def test_decode_examples_match_reference(name):
    fmt = GOLDEN["examples"][name]["format"]
    path = os.path.join(EXAMPLES, name)
    r, _ = S.ref_load(path, fmt, 1 << 20)
    o, _ = S.decode(S.NAMES[fmt], open(path, "rb").read())
    if fmt == "makeGal":
        r = {k: v[S.canonical_order(r)] for k, v in r.items()}
        o = {k: v[S.canonical_order(o)] for k, v in o.items()}
    same(r, o)


@need_ref
@pytest.mark.parametrize("fmt", ["ag", "agc", "age"])
def test_decode_records_match_reference(fmt, tmp_path):
    p = S.random_particles(2000, 11)
    b = S.encode(S.NAMES[fmt], p, 2000, 1.0, 2.0, 3.0)
    f = tmp_path / "ic"
    f.write_bytes(b)
    r, ok = S.ref_load(str(f), fmt, 4096)
    o, times = S.decode(S.NAMES[fmt], b)
    assert ok and times == (1.0, 2.0, 3.0)
    # agc carries no id: the reference leaves Particle::id unset
    same(r, o, [k for k in FIELDS if not (fmt == "agc" and k == "id")])


def _gadget_case(seed, individual, gas, short_mass=False):
    rng = np.random.default_rng(seed)
    npart = [40 if gas else 0, 300, 200, 50, 7, 3]
    n = sum(npart)
    pos = rng.normal(0, 5, (n, 3)).astype(np.float32)
    vel = rng.normal(0, 150, (n, 3)).astype(np.float32)
    ids = rng.permutation(n).astype(np.uint32)
    massarr = [0.0] * 6 if individual else [0.01, 0.02, 0.003, 0.004, 0.005, 0.006]
    masses = rng.uniform(1e-4, 1e-2, n).astype(np.float32) if individual else None
    if short_mass:
        masses = masses[: n - 5]
    u = rng.uniform(1, 1e3, npart[0]).astype(np.float32) if gas else None
    return S.gadget_ic(npart, pos, vel, ids, massarr, masses, u, time=0.125)


@need_ref
@pytest.mark.parametrize("individual,gas,short", [(True, True, False), (False, True, False), (True, False, False),
                                                  (False, False, False), (True, True, True)])
def test_decode_gadget_matches_reference(individual, gas, short, tmp_path):
    b = _gadget_case(21, individual, gas, short)
    f = tmp_path / "ic"
    f.write_bytes(b)
    r, ok = S.ref_load(str(f), "gadget", 4096)
    o, times = S.decode(S.FMT_GADGET, b)
    assert ok and times[2] == 0.125
    same(r, o)


def _makegal_case(seed, mass_block, gas=True):
    rng = np.random.default_rng(seed)
    npart = [30 if gas else 0, 120, 60, 20, 5, 4]
    n = sum(npart)
    mass = [0.0, 0.0, 0.001, 0.0, 0.002, 0.0] if mass_block else [0.01, 0.02, 0.003, 0.004, 0.005, 0.006]
    K = sum(npart[k] for k in range(6) if mass[k] == 0 and npart[k] > 0)
    return S.makegal_ic(npart, rng.normal(0, 5, (n, 3)).astype(np.float32),
                        rng.normal(0, 150, (n, 3)).astype(np.float32), np.arange(n, dtype=np.uint32) + 100,
                        mass, rng.uniform(1e-4, 1e-2, K).astype(np.float32) if mass_block else None,
                        rng.uniform(1, 1e3, npart[0]).astype(np.float32),
                        rng.uniform(0, 1, npart[0]).astype(np.float32), rng.uniform(0, 1, npart[0]).astype(np.float32))


@need_ref
@pytest.mark.parametrize("mass_block", [True, False])
def test_decode_makegal_matches_reference(mass_block, tmp_path):
    """Without a MASS block the reader still consumes one, so U comes from 24
    bytes into the U block: the restatement reads the same bytes."""
    b = _makegal_case(5, mass_block)
    f = tmp_path / "ic"
    f.write_bytes(b)
    r, _ = S.ref_load(str(f), "makeGal", 4096)
    o, _ = S.decode(S.FMT_MAKEGAL, b)
    r = {k: v[S.canonical_order(r)] for k, v in r.items()}
    o = {k: v[S.canonical_order(o)] for k, v in o.items()}
    same(r, o)


def test_decode_rejects_what_the_reference_cannot_read():
    p = S.random_particles(10, 1)
    b = S.encode(S.FMT_AGE, p, 10)
    with pytest.raises(S.FormatError):
        S.decode(S.FMT_AGE, b[:-1])  # truncated record
    g = bytearray(_gadget_case(3, True, True))
    g[0:4] = struct.pack("<I", 255)
    with pytest.raises(S.FormatError):
        S.decode(S.FMT_GADGET, bytes(g))  # header block size
    with pytest.raises(S.FormatError):
        S.decode(S.FMT_GADGET, _gadget_case(3, True, True)[:-2])  # truncated U block


def test_round_trip_records():
    p = S.random_particles(333, 4)
    for fmt in (S.FMT_AG, S.FMT_AGE):
        q, _ = S.decode(fmt, S.encode(fmt, p, 333, 1, 2, 3))
        assert S.encode(fmt, q, 333, 1, 2, 3) == S.encode(fmt, p, 333, 1, 2, 3)


def test_ic_count_reads_headers(tmp_path):
    """ag2_ic_count is host code: it parses headers without a GPU."""
    ag2 = pytest.importorskip("ag2")
    try:
        ag2.load()
    except OSError:
        pytest.skip("libag2.so not built")
    f = tmp_path / "a.age"
    f.write_bytes(S.encode(S.FMT_AGE, S.random_particles(77, 2), 77))
    assert ag2.ic_count(f, "age") == 77
    f.write_bytes(_gadget_case(1, True, True))
    assert ag2.ic_count(f, "gadget") == 600
    f.write_bytes(_makegal_case(1, False))
    assert ag2.ic_count(f, "makeGal") == 239
    with pytest.raises(ag2.AG2Error):
        ag2.ic_count(tmp_path / "none", "age")
