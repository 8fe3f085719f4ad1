"""CPU tests of the FP64 oracle: pinned against the reference's own compiled
Kernels.cpp (golden fixtures, and live when oracle/_ref exists) and against
known answers of the panel method (no GPU)."""
import os

import numpy as np
import pytest

import cases
from conftest import normwise

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_havelock_matches_reference_golden(orc):
    g = np.load(os.path.join(GOLD, "havelock_ref.npz"))
    got = orc.havelock(g["x"], g["y"], g["v"])
    rel = np.abs(got - g["G"]) / np.maximum(np.abs(g["G"]), 1e-300)
    # the oracle restates Kernels.cpp operation by operation: agreement to a few ulp
    assert np.max(rel) < 1e-13


def test_havelock_matches_reference_live(orc):
    from oracle.oracle import RefKernels
    if not RefKernels.available():
        pytest.skip("reference kernels not built here")
    ref = RefKernels()
    rng = np.random.default_rng(11)
    x, y = rng.uniform(-150, 150, (2, 5000))
    v = -10 ** rng.uniform(-4, 2, 5000)
    assert np.array_equal(orc.havelock(x, y, v), ref.havelock(x, y, v))


def test_havelock_guard_and_dgz(orc):
    g = np.load(os.path.join(GOLD, "havelock_ref.npz"))
    tail = orc.havelock(g["x"][-10:], g["y"][-10:], g["v"][-10:])
    assert np.all(tail[:2, 1] == 0) and np.all(tail[:2, 2] == 0)   # h <= 1e-6 -> dG/dx = dG/dy = 0
    assert np.array_equal(tail[:, 3], tail[:, 0])                   # dG/dz = G (Kernels.cpp:411)


def test_struve_against_scipy():
    g = np.load(os.path.join(GOLD, "havelock_ref.npz"))
    sp = pytest.importorskip("scipy.special")
    h, s = g["h"], g["special"]
    assert np.max(np.abs(s[:, 2] - sp.j0(h))) < 1e-12
    assert np.max(np.abs(s[:, 3] - sp.j1(h))) < 1e-12
    # the reference's Struve fits are ~1e-8-accurate approximations
    assert np.max(np.abs(s[:, 0] - sp.struve(0, h))) < 2e-7


def test_analytic_panel_far_field_matches_point_kernels(orc):
    """Inf_SourceKernel (Panel.cpp:86-156) tends to the Gauss quadrature of the
    reference's Source_Kernel / Dipole_Kernel (Kernels.cpp:11-27) far away."""
    pk = np.load(os.path.join(GOLD, "point_kernels_ref.npz"))
    S, D, A = pk["S"], pk["D"], pk["A"]
    r = np.linalg.norm(D - S, axis=1)
    assert np.allclose(pk["src"], -1.0 / (4 * np.pi * r), rtol=1e-14)
    assert np.allclose(pk["dip"], np.sum(A * (D - S), 1) / r ** 3 / (4 * np.pi), rtol=1e-12, atol=1e-18)
    m, _ = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    P = orc.panels(m)
    for i in (0, 20, 60, 140):
        p = P[i]
        d = np.array([0.3, 0.5, -0.8]) / np.linalg.norm([0.3, 0.5, -0.8])
        pt = p[13:16] + 500.0 * d
        Sv, Dv = orc.source_kernel(p, pt[None, :])
        qp, qw, qn = p[27:39].reshape(4, 3), p[39:43], p[43:55].reshape(4, 3)
        nq = int(p[26])
        rq = np.linalg.norm(pt[None, :] - qp[:nq], axis=1)
        src = np.sum(qw[:nq] * (-1.0 / (4 * np.pi * rq)))
        dip = np.sum(qw[:nq] * np.sum(qn[:nq] * (pt[None, :] - qp[:nq]), 1) / rq ** 3 / (4 * np.pi))
        assert abs(Sv[0] - src) < 1e-9 * abs(src)
        assert abs(Dv[0] - dip) < 1e-7 * abs(dip)


def test_dipole_self_influence_and_closed_surface(orc):
    """d_ii -> 1/2 (solid angle of the panel seen from 1e-5 above it) and the
    body + mirror image form a closed polyhedron: sum_S (d + dr) = 1 exactly."""
    m, _ = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    s, sr, d, dr, rn = orc.rankine(m)
    assert np.max(np.abs(np.diag(d) - 0.5)) < 1e-3
    assert np.max(np.abs((d + dr).sum(1) - 1.0)) < 1e-12
    b, _ = orc.barge(30.0, 12.0, 8.0, 8, 4, 3)
    s, sr, d, dr, rn = orc.rankine(b)
    assert np.max(np.abs((d + dr).sum(1) - 1.0)) < 1e-12


def test_mesh_counts_and_geometry(orc):
    m, aux = orc.cylinder(10.0, 20.0, 48, 8, 16, NRFS=8)
    assert m.n == 1152 and np.sum(m.elems[:, 3] < 0) == 48
    P = orc.panels(m)
    # inscribed 48-gon: side area and volume
    side = 48 * 2 * 10 * np.sin(np.pi / 48) * 20
    bottom = 48 * 0.5 * 100 * np.sin(2 * np.pi / 48)
    assert abs(P[:, 25].sum() - side - bottom) < 1e-8 * side
    M, C, vc = orc.mass_hydrostatics(m, aux)
    assert abs(vc[0] - bottom * 20) < 1e-8 * vc[0]
    assert abs(vc[3] - (-10.0)) < 1e-8                         # centre of buoyancy at half draft
    assert abs(C[2, 2] - 1025 * 9.81 * bottom) < 1e-6 * C[2, 2]  # rho g A_wp
    # mirrored panels: z reflected, normal z reversed
    Pm = orc.panels(m, mirror=True)
    assert np.allclose(Pm[:, 15], -P[:, 15]) and np.allclose(Pm[:, 24], -P[:, 24])
    b, _ = orc.barge(30.0, 12.0, 8.0, 8, 4, 3)
    assert b.n == 2 * 4 * 3 + 2 * 8 * 3 + 8 * 4


def test_oracle_regression_fixture(orc):
    g = np.load(os.path.join(GOLD, "cyl144_oracle.npz"))
    m, aux = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    r = orc.solve(m, g["omegas"], g["betas"], M=g["M"], C=g["C"])
    for k in ("A", "B", "F", "FK", "SC", "RAO"):
        assert normwise(r[k], g[k]) < 1e-12, k


def test_added_mass_symmetry_and_cylinder_symmetry(orc):
    g = np.load(os.path.join(GOLD, "cyl144_oracle.npz"))
    for f in range(len(g["omegas"])):
        A, B = g["A"][f], g["B"][f]
        s = np.max(np.abs(A))
        # reciprocity holds to discretisation accuracy for constant panels
        assert np.max(np.abs(A - A.T)) < 2e-2 * s
        assert abs(A[0, 0] - A[1, 1]) < 1e-6 * s and abs(B[0, 0] - B[1, 1]) < 1e-6 * np.max(np.abs(B))
        assert abs(A[0, 4] + A[1, 3]) < 1e-6 * s


def test_low_frequency_limit(orc):
    """Omega -> 0 approaches the Omega = 0 branch (Solve, Hydrodynamic_Solver.cpp:415-419)."""
    m, _ = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    r = orc.solve(m, [0.0, 1e-3], [0.0])
    assert normwise(r["A"][1], r["A"][0]) < 1e-3
    assert np.all(r["F"][0] == 0) and np.all(r["FK"][0] == 0)


def test_wave_integral_vs_subpanel_midpoint(orc):
    """2x2 Gauss wave-panel integration vs a dense sub-panel midpoint rule on the
    same flat panel (the reference's brute-force aid, Panel.cpp:828-868)."""
    m, _ = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    Pm = orc.panels(m, mirror=True)
    i = 20  # a mirrored bottom-disc quad (z = +20, flat)
    p = Pm[i]
    K = 0.05
    x = np.array([[3.0, 4.0, -5.0]])
    # Gauss (oracle) through the wave matrices of a 1-panel 'mesh' is not exposed;
    # integrate with the oracle's HavelockGF directly.
    def integrand(pts):
        R = (x - pts) * K
        g = orc.havelock(R[:, 0], R[:, 1], R[:, 2])
        return g[:, 0] * K / (4 * np.pi)
    qp, qw = p[27:39].reshape(4, 3), p[39:43]
    gauss = np.sum(qw * integrand(qp))
    v = p[1:13].reshape(4, 3)
    n = 60
    u = (np.arange(n) + 0.5) / n
    U, W = np.meshgrid(u, u, indexing="ij")
    U, W = U.ravel(), W.ravel()
    pts = ((1 - U) * (1 - W))[:, None] * v[0] + ((1 - U) * W)[:, None] * v[1] + (U * W)[:, None] * v[2] + \
          (U * (1 - W))[:, None] * v[3]
    # bilinear map Jacobian
    dU = (-(1 - W))[:, None] * v[0] - W[:, None] * v[1] + W[:, None] * v[2] + (1 - W)[:, None] * v[3]
    dW = (-(1 - U))[:, None] * v[0] + (1 - U)[:, None] * v[1] + U[:, None] * v[2] - U[:, None] * v[3]
    jac = np.linalg.norm(np.cross(dU, dW), axis=1)
    brute = np.sum(jac * integrand(pts)) / n ** 2
    assert abs(gauss - brute) < 1e-4 * abs(brute)
