"""Measurement output records: the reference's edit descriptors, field by
field, and the values they carry."""
import numpy as np

from hofstadter_hubbard_tsc_gb300 import output as O
from hofstadter_hubbard_tsc_gb300.measure import structure_factor


def test_edit_descriptors():
    assert O.fortran_i(32, 6) == "    32"
    assert O.fortran_i(-3, 8) == "      -3"
    assert O.fortran_i(1234567, 6) == "******"
    assert O.fortran_f(0.5, 14, 8) == "    0.50000000"
    assert O.fortran_f(-1.25, 21, 14) == "    -1.25000000000000"
    assert O.fortran_f(-1e-12, 14, 8) == "   -0.00000000"
    assert O.fortran_f(123456.0, 14, 8) == "**************"
    assert O.list_directed("Nx=", 32, "Ny=", 4) == " Nx=          32 Ny=           4"


def test_site_profile_record(tmp_path):
    prof = np.array([0.9, 0.8, 0.75, 0.85])
    p = tmp_path / "num_elec.dat"
    O.write_site_profile(p, prof, 2, 2, 2, 64, 128)
    O.write_site_profile(p, prof, 2, 2, 2, 64, 128)   # appended
    lines = p.read_text().split("\n")
    assert lines[0].split() == ["Nx=", "2", "Ny=", "2", "N_up=", "2", "N_down=", "2", "M1=", "64", "M2=", "128"]
    assert lines[1] == "     1     1    0.90000000    0.90000000"
    assert lines[4] == "     2     2    0.85000000    3.30000000"
    assert lines[5] == " " and lines[6] == lines[0]
    assert all(len(x) == 40 for x in lines[1:5])


def test_correlation_records(tmp_path):
    C = np.zeros((4, 4), dtype=complex)
    C[0, 2] = 0.125 - 0.5j
    C[3, 1] = -0.25
    p = tmp_path / "elec_cor.dat"
    O.write_correlations(p, C, 2, 0.0, 256)
    lines = p.read_text().rstrip("\n").split("\n")
    assert lines[0].split()[:4] == ["Nx=", "2", "Ny=", "2"] and lines[0].split()[-2:] == ["kept_max=", "256"]
    assert lines[1:] == ["       1       3       1     0.12500000000000    -0.50000000000000",
                         "       4       2      -1    -0.25000000000000     0.00000000000000"]
    p2 = tmp_path / "density_cor.dat"
    O.write_correlations(p2, C.real, 2, 0.0, 256, density=np.array([1.0, 0.5, 0.75, 1.25]))
    assert p2.read_text().split("\n")[1].split() == ["1", "3", "1", "0.12500000000000", "1.00000000000000",
                                                   "0.75000000000000"]


def test_structure_factor_record(tmp_path):
    rng = np.random.default_rng(3)
    C = rng.standard_normal((8, 8))
    kx, ky, S = structure_factor(C, 2, 4, 0)
    p = tmp_path / "strfac_spin.dat"
    O.write_structure_factor(p, kx, ky, S, 2, 4, 3, 3, 64, 64)
    lines = p.read_text().split("\n")
    rows = lines[1:1 + len(kx) * len(ky)]
    assert all(len(r) == 50 for r in rows)
    vals = np.array([[float(t) for t in r.split()] for r in rows])
    np.testing.assert_allclose(vals[:, 0], np.tile(kx, len(ky)), atol=1e-12)
    np.testing.assert_allclose(vals[:, 1], np.repeat(ky, len(kx)), atol=1e-12)
    np.testing.assert_allclose(vals[:, 2], S.T.ravel(), atol=1e-12)
    assert lines[1 + len(kx) * len(ky)] == " "
