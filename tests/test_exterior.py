"""Exterior outputs: free-surface elevation (Hydrodynamic_Solver.cpp:205-266,
498-505) and Kochin functions (:492-494, 598-642; defined E, see the oracle).

CPU tests pin the oracle by physics: the heave Kochin function of an
axisymmetric body is independent of the angle, the radiation damping equals
K/(4 pi) times the angular integral of |H|^2 (energy conservation, Newman),
and mirror-image wave points see mirror-equal heave elevations.  GPU tests
compare the library with the oracle on the same mesh and frequency."""
import numpy as np
import pytest

from conftest import normwise


def _cyl(orc, na=16, nr=3, nv=5):
    m, _ = orc.cylinder(5.0, 8.0, na, nr, nv)
    return m


def test_kochin_heave_axisymmetric(orc):
    m = _cyl(orc)
    r = orc.solve(m, [0.9], [0.0], want_phi=True)
    _, _, kr, _ = orc.exterior(m, 0.9, [0.0], r["phiJ"], r["phiS"], np.zeros((0, 3)), 36)
    h = np.abs(kr[:, 2])
    assert (h.max() - h.min()) / h.max() < 1e-12


@pytest.mark.parametrize("om", [0.6, 1.3])
def test_kochin_energy_relation(orc, om):
    """B_jj = K / (4 pi) * int |H_j(theta)|^2 dtheta (surge and heave), to the
    discretisation error of a 24 x 9 panel cylinder."""
    m = _cyl(orc, 24, 3, 6)
    r = orc.solve(m, [om], [0.0], want_phi=True)
    nk = 72
    _, _, kr, _ = orc.exterior(m, om, [0.0], r["phiJ"], r["phiS"], np.zeros((0, 3)), nk)
    K = om * om / 9.81
    for j in (0, 2):
        energy = K / (4 * np.pi) * np.sum(np.abs(kr[:, j]) ** 2) * 2 * np.pi / nk
        assert abs(r["B"][0][j, j] - energy) / r["B"][0][j, j] < 0.03, j


def test_fs_elevation_mirror_points(orc):
    m = _cyl(orc)
    wp = np.array([[12.0, 7.0, 0.0], [12.0, -7.0, 0.0], [-12.0, 7.0, 0.0]])
    r = orc.solve(m, [0.8], [0.0], want_phi=True)
    fr, fd, _, _ = orc.exterior(m, 0.8, [0.0], r["phiJ"], r["phiS"], wp, 0)
    assert abs(fr[0, 2] - fr[1, 2]) < 1e-10 * abs(fr[0, 2])
    assert abs(fr[0, 2] - fr[2, 2]) < 1e-10 * abs(fr[0, 2])
    assert abs(fd[0, 0] - fd[1, 0]) < 1e-10 * abs(fd[0, 0])  # heading 0 is symmetric in y
    zero, _, _, _ = orc.exterior(m, 0.0, [0.0], r["phiJ"], r["phiS"], wp, 0)
    assert np.all(zero == 0)  # -i Omega / g factor


@pytest.fixture(scope="module")
def bg():
    import bemuse_gb300
    bemuse_gb300.build.build()
    return bemuse_gb300


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_exterior_matches_oracle(bg, orc, precision):
    mesh = bg.Half_Cylinder(5.0, 8.0, 16, 3, 5, 0, False)
    m = _cyl(orc)  # the same mesh from the oracle's generator
    om = np.array([0.4, 1.1])
    betas = [0.0, 0.7]
    wp = np.array([[x, y, 0.0] for x in np.linspace(-30, 30, 7) for y in np.linspace(-30, 30, 5)])
    wp[:, :2] *= 1.001
    s = bg.Hydrodynamic_Radiation_Solver(precision=precision)
    s.Set_Parameters([bg.Parameter("WaveAngle", b) for b in betas] + [bg.Parameter("NKochin", 24)])
    s.Setup(mesh)
    s.set_wave_points(wp)
    out = s.solve_omegas(om, want_fs=True, want_kochin=True)
    tol = 1e-9 if precision == 0 else 1e-7
    for f, w in enumerate(om):
        r = orc.solve(m, [w], betas, want_phi=True)
        fr, fd, kr, kd = orc.exterior(m, w, betas, r["phiJ"], r["phiS"], wp, 24)
        assert normwise(out["fs_rad"][f], fr) < tol
        assert normwise(out["fs_diff"][f], fd) < tol
        assert normwise(out["kochin_rad"][f], kr) < tol
        assert normwise(out["kochin_diff"][f], kd) < tol

