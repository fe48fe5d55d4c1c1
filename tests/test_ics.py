import numpy as np

import ics


def test_plummer_deterministic_and_centred():
    a = ics.plummer(2048, seed=1)
    b = ics.plummer(2048, seed=1)
    np.testing.assert_array_equal(a["pos"], b["pos"])
    assert abs(a["mass"].sum() - 1.0) < 1e-12
    assert np.abs(a["pos"].mean(0)).max() < 1e-12
    r = np.linalg.norm(a["pos"], axis=1)
    # half-mass radius of a Plummer sphere: a / sqrt(2^(2/3) - 1) = 1.3048
    assert abs(np.median(r) - 1.3048) < 0.08


def test_disk_galaxy_shapes():
    d = ics.disk_galaxy(3000, 800, 200, seed=2)
    n = 4000
    assert d["pos"].shape == (n, 3) and d["type"].shape == (n,)
    assert (d["type"] == 2).sum() == 200 and (d["type"] == 3).sum() == 3000
    assert np.all(d["U"][d["type"] == 2] == 0.01)
    assert d["massInH"] == 64 * d["mass"][d["type"] == 2][0]


def test_merger_counts():
    m = ics.merger(n_per_galaxy=4096, seed=3)
    assert len(m["mass"]) == 8192
    assert (m["type"] == 2).sum() == 2 * 256


def test_ensemble_sizes_range():
    s = ics.ensemble_sizes(512, seed=4)
    assert s.min() >= 1024 and s.max() <= 65536 and len(s) == 512
