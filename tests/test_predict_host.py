"""predict.x input parsing and XSF round trip (host only)."""
import numpy as np


def test_predict_input_parser(tmp_path):
    from aenet_gb300.predict import read_input
    p = tmp_path / "predict.in"
    p.write_text("TYPES\n2\nTi\nO\n\nNETWORKS\nTi Ti.nn\nO O.nn\n\nPRINT_ATOMIC_ENERGIES\n"
                 "RELAX\nmethod=bfgs F_conv=2.0d-3 E_conv=1.0d-5 steps=7\n\nFILES\n1\na.xsf\n")
    inp = read_input(str(p))
    assert inp["types"] == ["Ti", "O"]
    assert inp["forces"] and inp["print_atomic_energies"]
    assert inp["relax"]["F_conv"] == 2e-3 and inp["relax"]["steps"] == 7
    assert inp["files"][0].endswith("a.xsf")


def test_xsf_round_trip(tmp_path):
    from aenet_gb300.xsf import read_xsf, write_xsf
    pos = np.array([[0.0, 0.1, 0.2], [1.5, 1.6, 1.7]])
    cell = np.diag([5.0, 6.0, 7.0])
    write_xsf(str(tmp_path / "a.xsf"), ["Ti", "O"], pos, cell=cell, forces=pos * 2)
    s = read_xsf(str(tmp_path / "a.xsf"))
    assert s["pbc"] and s["symbols"] == ["Ti", "O"]
    assert np.allclose(s["positions"], pos) and np.allclose(s["cell"], cell)
    assert np.allclose(s["forces"], pos * 2)
    write_xsf(str(tmp_path / "b.xsf"), ["Cu", "Cu"], pos)
    s = read_xsf(str(tmp_path / "b.xsf"))
    assert not s["pbc"] and s["cell"] is None
