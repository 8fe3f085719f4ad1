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


def test_kochin_and_wave_files(orc, tmp_path):
    """_KochinRad.bem (freq, dof, theta deg, |H|, arg, Re, Im), _KochinDiff.bem
    (freq, beta deg, theta deg, ...), .6r (freq, point, |eta|, arg per dof) and
    _WaveElPos.bem (Hydrodynamic_Solver_IO.cpp:488-500, 589-645)."""
    mesh, _ = orc.cylinder(5.0, 8.0, 12, 3, 4)
    om = np.array([0.0, 0.7])
    betas = np.deg2rad([0.0, 30.0])
    wp = np.array([[15.0, 0.0, 0.0], [0.0, 15.0, 0.0], [-10.0, -10.0, 0.0]])
    nk = 8
    out = dict(kochin_rad=np.zeros((2, nk, 6), complex), kochin_diff=np.zeros((2, nk, 2), complex),
               fs_rad=np.zeros((2, 3, 6), complex))
    for k, w in enumerate(om):
        r = orc.solve(mesh, [w], betas, want_phi=True)
        fr, _, kr, kd = orc.exterior(mesh, w, betas, r["phiJ"], r["phiS"], wp, nk)
        out["kochin_rad"][k], out["kochin_diff"][k], out["fs_rad"][k] = kr, kd, fr
    prefix = str(tmp_path / "ext")
    bg.write_wamit(prefix, om, out, betas, np.eye(6), np.eye(6), 1.0, (0, 0, 0), (0, 0, 0), wave_points=wp)
    rel = lambda a, b: abs(a - b) <= 1e-5 * max(1.0, abs(b))
    kr = _rows(prefix + "_KochinRad.bem")
    assert len(kr) == nk * 6  # the Omega = 0 frequency writes no rows
    for i in range(nk):
        for d in range(6):
            row = [float(x) for x in kr[6 * i + d]]
            z = out["kochin_rad"][1, i, d]
            assert rel(row[0], 2 * np.pi * 0.7) and row[1] == d + 1 and rel(row[2], (0.5 + i) * 360.0 / nk)
            assert rel(row[3], abs(z)) and abs(row[5] - z.real) <= 1e-5 * abs(z)
    kd = _rows(prefix + "_KochinDiff.bem")
    assert len(kd) == 2 * nk
    row = [float(x) for x in kd[nk + 3]]  # heading 1, angle 3
    z = out["kochin_diff"][1, 3, 1]
    assert rel(row[1], 30.0) and rel(row[2], 3.5 * 360.0 / nk) and rel(row[3], abs(z))
    r6 = _rows(prefix + ".6r")
    assert len(r6) == 3 and int(r6[2][1]) == 2 and len(r6[0]) == 14
    z = out["fs_rad"][1, 2, 2]
    assert rel(float(r6[2][6]), abs(z)) and abs(float(r6[2][7]) - np.angle(z)) < 1e-5
    pos = _rows(prefix + "_WaveElPos.bem")
    assert [int(p[0]) for p in pos] == [0, 1, 2] and float(pos[2][1]) == -10.0
    assert os.path.exists(prefix + ".6")


def test_bem_summary_file(orc, tmp_path):
    """.bem summary (Hydrodynamic_Solver_IO.cpp:107-426): header, M and C tables, and per
    frequency Omega, period 1/(2 pi Omega), wavenumber, the A/B table and the FK and
    excitation tables (|F|/g, phase)."""
    om, betas, out, M, C, vc = _orc_case(orc)
    mesh, _ = orc.cylinder(5.0, 8.0, 12, 3, 4)
    prefix = str(tmp_path / "sum")
    bg.write_bem(prefix, om, out, betas, M, C, vc[0], vc[1:], (0.0, 0.0, -1.0), mesh=bg.Mesh(mesh.nodes, mesh.elems),
                 mass=M[0, 0], file_info="generated")
    text = open(prefix + ".bem").read()
    lines = text.split("\n")
    assert lines[1].startswith("------------------------ BEMUse Output")
    assert "Gravity:                 9.81 m s^{-2}." in text and "Incoming wave angles: (deg)" in text
    assert "Input Mesh has:          %d panels." % mesh.n in text
    area = float([ln for ln in lines if ln.startswith("Surface area:")][0].split()[2])
    assert abs(area - np.sum(bg.panel_areas(bg.Mesh(mesh.nodes, mesh.elems)))) < 1e-3 * area
    blocks = text.split("----------\nFrequency:")[1:]
    assert len(blocks) == len(om)
    rel = lambda a, b: abs(a - b) <= 1e-5 * max(1e-12, abs(b))
    for k, blk in enumerate(blocks):
        bl = blk.split("\n")
        assert rel(float(bl[0].split()[0]), om[k])
        assert rel(float(bl[2].split()[1]), om[k] ** 2 / 9.81) or om[k] == 0
        heave = [ln for ln in bl if ln.startswith("Heave ")][0].split()
        assert rel(float(heave[5]), out["A"][k, 2, 2]) and (rel(float(heave[6]), out["B"][k, 2, 2])
                                                             or abs(out["B"][k, 2, 2]) < 1e-9)
        ex = blk.split("Excitation Forces:")[1].split("\n")
        hv = [ln for ln in ex if ln.startswith("Heave: ")][0].split()
        assert rel(float(hv[1]), abs(out["F"][k, 2, 0]) / 9.81) or abs(out["F"][k, 2, 0]) < 1e-9


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


def test_read_gdf(tmp_path):
    """GDF import (GDF_Geo.cpp:12-103): three-field lines are vertices, four make a
    panel, a repeated third vertex makes a triangle, header lines are skipped."""
    p = tmp_path / "box.gdf"
    p.write_text("WAMIT-style header line with words\n"
                 "1.0 9.80665\n"
                 "0 0\n"
                 "2\n"
                 " 0.0  0.0 -1.0\n"
                 " 1.0  0.0 -1.0\n"
                 " 1.0  1.0 -1.0\n"
                 " 0.0  1.0 -1.0\n"
                 "0.0 0.0 0.0\r\n"
                 "0.0 0.0 -1.0\r\n"
                 "1.0 0.0 -1.0\r\n"
                 "1.0 0.0 -1.0\r\n"
                 "9 9 9 \n")          # trailing blank: four fields, not a vertex
    m = bg.read_mesh(p)
    assert m.n == 2
    assert m.nodes.shape == (7, 3)
    assert list(m.elems[0]) == [0, 1, 2, 3]
    assert list(m.elems[1]) == [4, 5, 6, -1]
    assert np.allclose(m.nodes[2], [1.0, 1.0, -1.0])
    bad = tmp_path / "bad.gdf"
    bad.write_text("a b c\n")
    with pytest.raises(bg.BEMError):
        bg.GDF_Geometry(bad)


def test_read_mar(tmp_path):
    """NEMOH .mar (MAR_Geo.cpp:12-96): nodes until a four-field line with id 0, then
    1-based panels; third == fourth (as text) is a triangle."""
    p = tmp_path / "hull.mar"
    p.write_text("2 0\n"
                 "1 0.0 0.0 -1.0\n"
                 "2 1.0 0.0 -1.0\n"
                 "3 1.0 1.0 -1.0\n"
                 "4 0.0 1.0 -1.0\n"
                 "0 0.00 0.00 0.00\n"
                 "1 2 3 4\n"
                 "1 3 4 4\n"
                 "0 0 0 0\n")
    m = bg.MAR_Geometry(p)
    assert m.nodes.shape == (4, 3)
    assert m.elems.tolist() == [[0, 1, 2, 3], [0, 2, 3, -1]]
    q = tmp_path / "broken.mar"
    q.write_text("1 0 0 0\n0 0 0 0\n1 2 3 4\n")
    with pytest.raises(bg.BEMError, match="does not exist"):
        bg.read_mesh(q)


def test_read_stl(tmp_path):
    """ASCII STL (STL_Geo.cpp:12-94): positions x 100, corners stored C3 C2 C1."""
    p = tmp_path / "tri.stl"
    p.write_text("solid t\n"
                 "  facet normal 0 0 1\n"
                 "    outer loop\n"
                 "      vertex 0 0 -0.01\n"
                 "      vertex 0.01 0 -0.01\n"
                 "      vertex 0 0.01 -0.01\n"
                 "    endloop\n"
                 "  endfacet\n"
                 "endsolid t\n")
    m = bg.read_mesh(p)
    assert m.nodes.shape == (3, 3)
    assert np.allclose(m.nodes, [[0, 0, -1], [1, 0, -1], [0, 1, -1]])
    assert m.elems.tolist() == [[2, 1, 0, -1]]


def test_read_pnl(tmp_path):
    """HAMS .pnl (PNL_Geo.cpp:17-129): sections by marker lines, 1-based panels with
    their vertex count."""
    p = tmp_path / "hull.pnl"
    p.write_text("    --------------Hull Mesh File---------------\n\n"
                 "    # Number of Panels, Nodes, X-Symmetry and Y-Symmetry\n"
                 "         2         5         0         0\n\n"
                 "    #Start Definition of Node Coordinates     ! node_number   x   y   z\n"
                 "    1   0.0  0.0  -1.0\n"
                 "    2   1.0  0.0  -1.0\n"
                 "    3   1.0  1.0  -1.0\n"
                 "    4   0.0  1.0  -1.0\n"
                 "    5   2.0  0.0  -1.0\n"
                 "    #End Definition of Node Coordinates\n\n"
                 "    #Start Definition of Node Relations   ! panel_number  number_of_vertices   Vertex1_ID\n"
                 "    1   4   1   2   3   4\n"
                 "    2   3   2   5   3\n"
                 "    #End Definition of Node Relations\n")
    m = bg.PNL_Geometry(p)
    assert m.nodes.shape == (5, 3)
    assert m.elems.tolist() == [[0, 1, 2, 3], [1, 4, 2, -1]]
