"""Irregular-frequency removal (IFR; Hydrodynamic_Solver.cpp:17, 45-55, 406): the
interior free-surface panels join the system after the hull panels.

CPU tests pin the oracle by the physics IFR exists for: a truncated cylinder of
radius 5 has its first irregular frequency near K a = 2.405 (omega ~ 2.17 rad/s);
without IFR the heave damping there turns negative and the heave excitation
spikes, with IFR both stay smooth.  The GPU tests compare the library's IFR
solves (plain FP64 and mixed) with the oracle's."""
import numpy as np
import pytest

from conftest import normwise

OM = np.array([0.0, 0.9, 2.2])


def test_ifr_removes_the_irregular_frequency(orc):
    m, aux = orc.cylinder(5.0, 8.0, 16, 3, 5, NRFS=3)
    om = np.linspace(1.9, 2.5, 7)
    plain = orc.solve(m, om, [0.0])
    ifr = orc.solve(m, om, [0.0], ifr_aux=aux)
    b_plain, b_ifr = plain["B"][:, 2, 2], ifr["B"][:, 2, 2]
    assert b_plain.min() < -0.1              # the spike: negative radiation damping
    assert np.all(b_ifr > 0)                 # removed
    assert np.all(np.diff(b_ifr) < 0)        # and monotone over the band
    f_ifr = np.abs(ifr["F"][:, 2, 0])
    assert np.all(np.diff(f_ifr) < 0)
    # away from the irregular frequency the two formulations agree closely
    low = orc.solve(m, [0.6], [0.0])
    low_ifr = orc.solve(m, [0.6], [0.0], ifr_aux=aux)
    assert abs(low["A"][0, 2, 2] - low_ifr["A"][0, 2, 2]) < 2e-3 * abs(low["A"][0, 2, 2])


def test_ifr_zero_frequency_is_solved_at_1e_3(orc):
    m, aux = orc.cylinder(5.0, 8.0, 12, 3, 4, NRFS=2)
    a = orc.solve(m, [0.0], [0.0], ifr_aux=aux)
    b = orc.solve(m, [1.0e-3], [0.0], ifr_aux=aux)
    for k in ("A", "B", "F", "FK"):
        assert np.array_equal(a[k], b[k]), k


@pytest.fixture(scope="module")
def bg():
    import bemuse_gb300
    bemuse_gb300.build.build()
    return bemuse_gb300


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_ifr_matches_oracle(bg, orc, precision):
    mesh = bg.Half_Cylinder(5.0, 8.0, 16, 3, 5, 3, False)
    m, aux = orc.cylinder(5.0, 8.0, 16, 3, 5, NRFS=3)
    betas = [0.0, 0.6]
    s = bg.Hydrodynamic_Radiation_Solver(precision=precision)
    s.Set_Parameters([bg.Parameter("IFR", True)] + [bg.Parameter("WaveAngle", b) for b in betas])
    s.Setup(mesh)
    assert s.N == m.n  # hull panels
    got = s.solve_omegas(OM, want_phi=True)
    ref = orc.solve(m, OM, betas, M=s.M_ij, C=s.C_ij, want_phi=True, ifr_aux=aux)
    # plain FP64: rounding-level agreement; mixed: the 1e-6 bound on A and B that the
    # mixed path is specified to (B at Omega = 1e-3 is ~1e-7 of A, so its relative error
    # reflects the refinement tolerance on the whole right-hand side)
    tol = 1e-8 if precision == 0 else 1e-6
    for k in ("A", "B", "F", "FK", "SC", "RAO"):
        e = max(normwise(got[k][f], ref[k][f]) for f in range(len(OM)))
        assert e < tol, (k, e)
    assert normwise(got["phiJ"], ref["phiJ"]) < tol
    # the spike is gone on the GPU too
    assert got["B"][2, 2, 2] > 0
