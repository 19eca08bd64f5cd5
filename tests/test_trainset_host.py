"""Training-set files (src/trainset.f90 records) on the host: write/read
round trip and the ts_normalize restatement."""
import numpy as np

from aenet_gb300.trainset import TrainSet, normalize, read_trainset, write_trainset


def _sample():
    rng = np.random.default_rng(3)
    ts = TrainSet(["Ti", "O"], [-1.5, -0.5])
    for k in range(3):
        n = 2 + k
        types = rng.integers(1, 3, n)
        sf = [rng.normal(size=4 if t == 1 else 6) for t in types]
        ts.add("s%d.xsf" % k, -3.0 * n + k, types, rng.normal(size=(n, 3)),
               rng.normal(size=(n, 3)), sf)
    ts.E_av, ts.E_min, ts.E_max = ts.energy_range()
    ts.setup_records = [[b"abc", b"\x01\x00\x00\x00"], [b"xyz", b"\x02\x00\x00\x00"]]
    return ts


def test_trainset_round_trip(tmp_path):
    ts = _sample()
    write_trainset(str(tmp_path / "a.train"), ts)
    r = read_trainset(str(tmp_path / "a.train"))
    assert r.type_names == ts.type_names and np.array_equal(r.E_atom, ts.E_atom)
    assert len(r.structures) == 3 and r.natoms_total == ts.natoms_total
    for a, b in zip(r.structures, ts.structures):
        assert a["file"] == b["file"] and a["energy"] == b["energy"]
        assert np.array_equal(a["types"], b["types"])
        assert np.array_equal(a["coords"], b["coords"]) and np.array_equal(a["forces"], b["forces"])
        assert all(np.array_equal(x, y) for x, y in zip(a["sfval"], b["sfval"]))
    assert (r.E_av, r.E_min, r.E_max) == (ts.E_av, ts.E_min, ts.E_max)
    assert r.setup_records == ts.setup_records


def test_normalize_matches_ts_normalize_formulas():
    ts = _sample()
    stats = {1: (np.full(4, 0.5), np.full(4, 2.0)), 2: (np.zeros(6), np.ones(6))}
    n = normalize(ts, stats)
    scale = 2.0 / (ts.E_max - ts.E_min)
    shift = 0.5 * (ts.E_max + ts.E_min)
    assert n.normalized and n.scale == scale and n.shift == shift
    for a, b in zip(n.structures, ts.structures):
        k = len(b["types"])
        assert np.isclose(a["energy"], scale * (b["energy"] - k * shift))
        assert np.allclose(a["forces"], scale * b["forces"])
        for t, x, y in zip(b["types"], a["sfval"], b["sfval"]):
            assert np.allclose(x, (y - stats[t][0][:len(y)]) * stats[t][1][:len(y)])
