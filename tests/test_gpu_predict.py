"""The predict.x-style driver on the GPU: the reference's Cu-dimer input
(unittests/Cu-dimer-forces/predict.in: TYPES, NETWORKS, FORCES) over XSF
files, report lines compared with the reference outputs at their printed
precision (output-reference/dimer-x*.xsf.out)."""
import io
import re

import numpy as np
import pytest

from tests.golden import fixtures

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


def test_predict_driver_cu_dimer_report(cuda, tmp_path):
    from aenet_gb300 import predict
    from aenet_gb300.xsf import write_xsf
    k3 = fixtures.load("k3_cu_dimer.npz")
    pots = fixtures.potentials(k3)
    paths = fixtures.write_potential_files(pots, str(tmp_path))
    types = [str(t) for t in k3["types"]]
    picks = [0, 14, 40, 80]                     # 2.0, 3.4, 6.0 and 10.0 A
    files = []
    for q in picks:
        fn = tmp_path / ("dimer-%02d.xsf" % q)
        write_xsf(str(fn), ["Cu", "Cu"], k3["positions"][q], comment="dimer")
        files.append(str(fn))
    inp = tmp_path / "predict.in"
    with open(inp, "w") as fh:
        fh.write("TYPES\n%d\n%s\n\nNETWORKS\n" % (len(types), "\n".join(types)))
        for t in types:
            fh.write("%s  %s\n" % (t, paths[t]))
        fh.write("\nFORCES\n\n!RELAX\n!method=bfgs  F_conv=1.0d-2\n\nFILES\n%d\n%s\n"
                 % (len(files), "\n".join(files)))
    out = io.StringIO()
    assert predict.main([str(inp)], out=out) == 0
    text = out.getvalue()
    ecoh = [float(x) for x in re.findall(r"Cohesive energy\s+:\s+(\S+) eV", text)]
    etot = [float(x) for x in re.findall(r"Total energy\s+:\s+(\S+) eV", text)]
    rows = re.findall(r"^ Cu\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)\s+(\S+)\s*$", text, re.M)
    assert len(ecoh) == len(picks) and len(rows) == 2 * len(picks)
    for n, q in enumerate(picks):
        # F20.8 energies and F12.6 forces, as printed by predict.x
        assert abs(ecoh[n] - k3["E_coh"][q]) <= 1.01e-8
        assert abs(etot[n] - k3["E_total"][q]) <= 1.01e-8
        for a in range(2):
            F = np.array([float(x) for x in rows[2 * n + a][3:]])
            assert np.abs(F - k3["forces"][q][a]).max() <= 1.01e-6
    assert "The maximum force is acting on atom" in text


def test_predict_driver_relaxation_lowers_energy(cuda, oracle, tmp_path):
    """RELAX through the driver: a perturbed 256-atom Cu cell relaxes to a
    lower cohesive energy and a smaller RMS force, and the report shows the
    optimised coordinates."""
    from aenet_gb300 import predict, workloads
    from aenet_gb300.xsf import write_xsf
    from tests import helpers
    w = workloads.cu_fcc_256()
    paths = helpers.make_potentials(oracle, w, str(tmp_path), max_atoms=64)
    s = w.structures[0]
    write_xsf(str(tmp_path / "cu.xsf"), ["Cu"] * s.natoms, s.positions, cell=s.cell)
    inp = tmp_path / "predict.in"
    inp.write_text("TYPES\n1\nCu\n\nNETWORKS\nCu %s\n\nRELAX\nmethod=bfgs F_conv=1.0d-3 "
                   "E_conv=1.0d-9 steps=30\n\nFILES\n1\n%s\n" % (paths["Cu"], tmp_path / "cu.xsf"))
    out = io.StringIO()
    assert predict.main([str(inp)], out=out) == 0
    text = out.getvalue()
    assert "Geometry optimization:" in text and "(optimized)" in text
    rows = re.findall(r"^\s+(\d+)\s+(-?\d+\.\d+)\s+(\d+\.\d+)", text, re.M)
    dE = [float(r[1]) for r in rows]
    rms = [float(r[2]) for r in rows]
    assert len(rows) >= 2 and dE[-1] < 0.0 and rms[-1] < rms[0]
    final_rms = float(re.findall(r"RMS force\s+:\s+(\S+)", text)[-1])
    assert final_rms < rms[0]
