"""&inputPsiE on the host (SRC/mod_PsiE_01y2.f:19-88): the funE energies are
read only for iphoto > 0, from the file the namelist names."""
import os

import numpy as np

from madwave3_gb300.host import constants as C, setup


def test_input_psie(case_dirs, tmp_path):
    src = os.path.join(case_dirs["tiny_j0"], "input.dat")
    run = setup.load(src)
    assert run.efe_zot.size == 0                      # iphoto = 0: off
    run.inp.iphoto = 1
    d = tmp_path / "psie"
    d.mkdir()
    (d / "input.dat").write_text("&inputPsiE\n nofe=2, file_resonancesE='res.dat'\n/\n")
    (d / "res.dat").write_text("0.25\n0.75d0\n1.5\n")
    setup.input_psie(run, str(d / "input.dat"))
    assert np.allclose(run.efe_zot, np.array([0.25, 0.75]) * C.eV2cm * C.conve1, rtol=0, atol=0)
