"""WAMIT-format result files (bem_write_wamit) against the values they print.

The writer follows Generate_Output_File_WAMIT / Update_Output_File_WAMIT
(Hydrodynamic_Solver_IO.cpp:430-646): column order, units (forces / g, C / (rho g),
M / rho, frequency column = 2 pi Omega), the conjugated .2sc phase and the
number format (6 significant digits, blank-padded fields).  Host only."""
import os

import numpy as np
import pytest

import bemuse_gb300 as bg


def _orc_case(orc):
    mesh, aux = orc.cylinder(5.0, 8.0, 12, 3, 4)
    om = np.array([0.0, 0.4, 1.1])
    betas = np.deg2rad([0.0, 60.0])
    M, C, vc = orc.mass_hydrostatics(mesh, aux, mass=0.0, cog=(0.0, 0.0, -1.0))
    out = orc.solve(mesh, om, betas, M=M, C=C)
    return om, betas, out, M, C, vc


def _rows(path):
    with open(path) as f:
        return [ln.split() for ln in f if ln.strip()]


def test_wamit_files(orc, tmp_path):
    om, betas, out, M, C, vc = _orc_case(orc)
    prefix = str(tmp_path / "case")
    bg.write_wamit(prefix, om, out, betas, M, C, vc[0], vc[1:], (0.0, 0.0, -1.0), rho=1025.0, gravity=9.81)
    for ext in (".1", ".2", ".2fk", ".2sc", ".4", ".hst", ".mmx"):
        assert os.path.exists(prefix + ext)
    rel = lambda a, b: abs(a - b) <= 1e-5 * max(1.0, abs(b))
    # .1: Omega = 0 -> (0, i, j, A); otherwise (2 pi Omega, i, j, A, B)
    r1 = _rows(prefix + ".1")
    assert len(r1) == 36 * len(om)
    for k, w in enumerate(om):
        for i in range(6):
            for j in range(6):
                row = r1[36 * k + 6 * i + j]
                assert int(row[1]) == i + 1 and int(row[2]) == j + 1
                assert rel(float(row[0]), 2 * np.pi * w)
                assert rel(float(row[3]), out["A"][k, i, j])
                if w != 0.0:
                    assert rel(float(row[4]), out["B"][k, i, j])
                else:
                    assert len(row) == 4
    # .2 / .2fk / .2sc / .4: (freq, beta deg, dof, |X|/s, arg, Re/s, Im/s), no rows at Omega = 0
    for ext, key, scale, conj in ((".2", "F", 9.81, False), (".2fk", "FK", 9.81, False),
                                  (".2sc", "SC", 9.81, True), (".4", "RAO", 1.0, False)):
        rows = _rows(prefix + ext)
        live = [k for k, w in enumerate(om) if w != 0.0]
        assert len(rows) == len(live) * len(betas) * 6
        n = 0
        for k in live:
            for b in range(len(betas)):
                for i in range(6):
                    row = [float(x) for x in rows[n]]
                    n += 1
                    z = out[key][k, i, b]
                    z = np.conj(z) if conj else z
                    assert rel(row[0], 2 * np.pi * om[k]) and rel(row[1], np.rad2deg(betas[b])) and row[2] == i + 1
                    assert rel(row[3], abs(z) / scale)
                    assert abs(row[5] - z.real / scale) <= 1e-5 * max(abs(z) / scale, 1e-30)
                    assert abs(row[6] - z.imag / scale) <= 1e-5 * max(abs(z) / scale, 1e-30)
    # .hst: C / (rho g); .mmx: M / rho after the header
    hst = _rows(prefix + ".hst")
    assert len(hst) == 36
    for i in range(6):
        for j in range(6):
            assert rel(float(hst[6 * i + j][2]), C[i, j] / 1025.0 / 9.81)
    mmx = _rows(prefix + ".mmx")
    assert mmx[0][0] == "Gravity:" and float(mmx[0][1]) == 9.81
    assert rel(float(mmx[1][1]), vc[0])
    body = mmx[-36:]
    for i in range(6):
        for j in range(6):
            assert rel(float(body[6 * i + j][2]), M[i, j] / 1025.0)


def test_number_format(tmp_path):
    """Fields: 6 significant digits, a leading blank for values >= 0, padded to 15."""
    z = np.zeros((1, 6, 6))
    z[0, 0, 0] = 1234.56789
    z[0, 0, 1] = -0.000123456
    prefix = str(tmp_path / "fmt")
    bg.write_wamit(prefix, [0.0], {"A": z, "B": z}, [], np.eye(6), np.eye(6), 1.0, (0, 0, 0), (0, 0, 0))
    with open(prefix + ".1") as f:
        first = f.readline()
        second = f.readline()
    assert first.startswith(" 0" + " " * 13 + "1     1      1234.57")
    assert "-0.000123456" in second
