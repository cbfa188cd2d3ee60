"""The reference's field files through the C ABI (host code, no GPU needed):
the field form of DEALII_SCFT/src/scft.cc:317-333 / scft_util.cc:14-41, the
MATLAB inputs, and the .res tables 1D_FEM.c:321-342 reads.  Fixture values come
from tests/golden (made from the reference's own files); when the reference
tree is present the original files are read as well."""
import json
import math
import os

import numpy as np
import pytest

from scft_gb300 import _lib, api

GOLD = os.path.join(os.path.dirname(__file__), "golden")
from oracle import oracle as orc

REF = orc.reference_dir()  # reference sources on this host (None when absent)


def load(name):
    return json.load(open(os.path.join(GOLD, name)))


def test_field_write_matches_the_reference_layout_and_reads_back(tmp_path):
    g = load("dealii_N33.json")
    p = str(tmp_path / "solution_yita_1D_N= 33.txt")
    api.write_field(p, g["x"], g["w"], g["file_error"], g["file_free_energy"])
    lines = open(p).read().splitlines()
    assert lines[:2] == g["header"]
    assert len(lines) == 2 + 33 and lines[2].startswith("0,0.000000000000000,")
    f = api.read_field(p)
    np.testing.assert_array_equal(f["x"], g["x"])
    np.testing.assert_array_equal(f["w"], g["w"])
    assert f["err"] == g["file_error"] and f["free_energy"] == g["file_free_energy"]


def test_matlab_form_without_energy_line(tmp_path):
    g = load("matlab_N33.json")
    p = tmp_path / "solution_yita_1D_N= 33.txt"
    with open(p, "w") as fh:
        fh.write("N= 33 \n")
        for i, (x, w) in enumerate(zip(g["x"], g["w"])):
            fh.write(f"{i},{x:.15f},{w:.15f}\n")
    f = api.read_field(str(p))
    assert len(f["x"]) == 33 and math.isnan(f["err"]) and math.isnan(f["free_energy"])
    np.testing.assert_allclose(f["w"], g["w"], rtol=0, atol=5e-16 * 100)
    assert f["w"][0] == g["w"][0]  # node 0 is kept (read_yita_middle_1D would skip its line)


def test_missing_node_and_missing_file_are_errors(tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("N= 3, ERROR= 1e-3 \nmean_field_free_energy, 0.5 \n0,0.0,0.0\n2,1.0,0.0\n")
    with pytest.raises(_lib.ScftError) as e:
        api.read_field(str(p))
    assert e.value.code == _lib.SCFT_EINVAL
    with pytest.raises(_lib.ScftError) as e:
        api.read_field(str(tmp_path / "absent.txt"))
    assert e.value.code == _lib.SCFT_EIO


def test_res_table_in_the_reference_layout(tmp_path):
    g = load("res_m32.json")
    p = tmp_path / "Exp_m32_n2048_IE.res"
    rows = [f" {a:.6e}  {b:.14e}   {0.0:.14e}  {0.0:.14e}  {0.0:.14e}" for a, b in zip(g["x_over_l"], g["phi"])]
    p.write_text("\n\nm = 32   n = 2048\n\n"
                 f"N=1000  l={g['l']:.14e}  cp=0.00000000000000e+00  mphi={g['mphi']:.14e}  t={g['t']:.14e}\n"
                 "Z=1.002289e+00  f=2.01673546641703e-03  |f|max=7.628679e-11\n\n"
                 "     x/l               phi                   eta                    phie                  phij\n"
                 "------------- --------------------- ---------------------- --------------------- "
                 "---------------------\n" + "\n".join(rows) + "\n")
    r = api.read_res(str(p), max_rows=64)
    assert r["m"] == 32 and r["nsteps"] == 2048 and len(r["phi"]) == 33
    assert r["l"] == pytest.approx(g["l"], rel=1e-14) and r["t"] == pytest.approx(g["t"], rel=1e-14)
    assert r["mphi"] == pytest.approx(g["mphi"], rel=1e-14)
    assert r["Z"] == 1.002289 and r["f"] == 2.01673546641703e-03 and r["fmax"] == 7.628679e-11
    np.testing.assert_allclose(r["x_over_l"], g["x_over_l"], rtol=1e-6)
    np.testing.assert_allclose(r["phi"], g["phi"], rtol=1e-13)
    with pytest.raises(_lib.ScftError):
        api.read_res(str(p), max_rows=8)


@pytest.mark.skipif(REF is None, reason="reference tree absent")
def test_reference_files_themselves():
    g = load("dealii_N33.json")
    f = api.read_field(os.path.join(REF, "DEALII_SCFT/inputFiles/N=33_for_read.txt"))
    np.testing.assert_array_equal(f["w"], g["w"])
    assert f["err"] == g["file_error"] and f["free_energy"] == g["file_free_energy"]
    m = api.read_field(os.path.join(REF, "Matlab_files/inputFiles/solution_yita_1D_N= 33.txt"))
    assert len(m["w"]) == 33 and math.isnan(m["free_energy"])
    r = api.read_res(os.path.join(REF, "Exp_m32_n2048_IE.res"))
    rg = load("res_m32.json")
    assert r["m"] == 32 and r["nsteps"] == 2048 and r["l"] == rg["l"]
    np.testing.assert_array_equal(r["phi"], rg["phi"])
    assert r["Z"] == 1.002289 and r["fmax"] == 7.628679e-11
