"""The PyTorch export file of generate.x (pytorchoutput.f90:104-138):
record layout and Fortran (column-major) order, on the host."""
import struct

import numpy as np

from aenet_gb300.pytorch_export import read_forces_file, select_structures, write_forces_file


def test_selection_counts_like_pyo_select_force_structures():
    for n, frac in ((10, 0.5), (7, 0.3), (4, 1.0), (5, 0.0)):
        f = select_structures(n, frac, seed=1)
        assert f.sum() == int(np.rint(n * frac)) and set(f.tolist()) <= {0, 1}


def test_record_layout_and_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    dGi = rng.normal(size=(4, 3))
    dGj = rng.normal(size=(2, 4, 3))
    recs = [{"name": "a.xsf", "natoms": 1, "ntypes": 2, "selected": True,
             "atoms": [(2, np.array([1, 1]), dGi, dGj)]},
            {"name": "bb.xsf", "natoms": 3, "ntypes": 2, "selected": False, "atoms": []}]
    path = str(tmp_path / "x.forces")
    assert write_forces_file(path, recs) == 2
    raw = open(path, "rb").read()
    # header record: nStrucs
    assert struct.unpack_from("<iii", raw, 0) == (4, 2, 4)
    # sfderiv_i is written column-major: the first three doubles of that
    # record are dG_1/dx, dG_2/dx, dG_3/dx
    marker = struct.pack("<i", 4 * 3 * 8)
    off = raw.index(marker) + 4
    first = np.frombuffer(raw, "<f8", count=3, offset=off)
    np.testing.assert_array_equal(first, dGi[:3, 0])
    got, max_nnb = read_forces_file(path)
    assert max_nnb == 2
    assert [r["name"] for r in got] == ["a.xsf", "bb.xsf"]
    itype, nbl, gi, gj = got[0]["atoms"][0]
    assert itype == 2 and nbl.tolist() == [1, 1]
    np.testing.assert_array_equal(gi, dGi)
    np.testing.assert_array_equal(gj, dGj)
    assert got[1]["atoms"] == [] and not got[1]["selected"]
