"""Edge cases of the hydrodynamic solve against the FP64 oracle:
  * the largest right-hand-side count (10 headings, R = 16) and a count between the
    assembly kernel's accumulator sizes (5 headings, R = 11), plain and mixed;
  * a tiny body (a 1 x 1 x 1 barge: 5 panels, padded to one 128-row block; cosine
    spacing, since the linear-spacing barge's interior free-surface panels are
    degenerate at this size and are rejected);
  * a ragged panel count (144, not a multiple of 128) at Omega = 0 (no wave term,
    incident potential defined as 0) next to wave frequencies in one call;
  * an empty frequency list, and more headings than the interface holds.
Tolerances as in test_gpu_parity: plain 1e-8, mixed 1e-6 normwise."""
import numpy as np
import pytest

import cases
from conftest import normwise

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg():
    import bemuse_gb300
    bemuse_gb300.build.build()
    return bemuse_gb300


def _solver(bg, mesh, betas, precision):
    s = bg.Hydrodynamic_Radiation_Solver(precision=precision)
    s.Set_Parameters([bg.Parameter("WaveAngle", b) for b in betas])
    s.Set_Mass_Properties(mass=0.0, cog=(0, 0, 0), gyration=np.eye(3))
    s.Setup(mesh)
    return s


def _worst(got, ref, keys):
    return {k: max(normwise(got[k][f], ref[k][f]) for f in range(got[k].shape[0])) for k in keys}


@pytest.mark.parametrize("nb", [5, 10])
@pytest.mark.parametrize("precision,tol", [("PLAIN_FP64", 1e-8), ("MIXED", 1e-6)])
def test_many_headings(bg, orc, nb, precision, tol):
    betas = np.linspace(0.0, np.pi, nb, endpoint=False)
    m, _ = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    s = _solver(bg, cases.lib_cylinder(cases.CYL_SMALL), betas, getattr(bg, precision))
    om = np.array([0.4, 1.3])
    got = s.solve_omegas(om)
    ref = orc.solve(m, om, betas, M=s.M_ij, C=s.C_ij)
    assert got["F"].shape == (2, 6, nb)
    w = _worst(got, ref, ("A", "B", "F", "FK", "SC"))
    print(nb, precision, w)
    for k, e in w.items():
        assert e < tol, (k, e)


@pytest.mark.parametrize("precision,tol", [("PLAIN_FP64", 1e-8), ("MIXED", 1e-6)])
def test_tiny_body(bg, orc, precision, tol):
    om_o, _ = orc.barge(6.0, 4.0, 3.0, 1, 1, 1, cosine=True)
    mesh = bg.Barge(6.0, 4.0, 3.0, 1, 1, 1, True)
    assert mesh.n == om_o.n == 5
    s = _solver(bg, mesh, [0.0, 0.7], getattr(bg, precision))
    om = np.array([0.5, 1.5])
    got = s.solve_omegas(om)
    ref = orc.solve(om_o, om, [0.0, 0.7], M=s.M_ij, C=s.C_ij)
    w = _worst(got, ref, ("A", "B", "F"))
    print(precision, w)
    for k, e in w.items():
        assert e < tol, (k, e)


def test_zero_frequency_beside_wave_frequencies(bg, orc):
    m, _ = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    for precision, tol in (("PLAIN_FP64", 1e-8), ("MIXED", 1e-6)):
        s = _solver(bg, cases.lib_cylinder(cases.CYL_SMALL), [0.0], getattr(bg, precision))
        assert s.N == 144
        om = np.array([0.0, 0.8, 0.0])
        got = s.solve_omegas(om)
        ref = orc.solve(m, om, [0.0], M=s.M_ij, C=s.C_ij)
        # no wave term and no incident potential at Omega = 0: A from the Rankine part only
        for f in (0, 2):
            assert np.all(got["FK"][f] == 0) and np.all(got["SC"][f] == 0) and np.all(got["F"][f] == 0)
            assert normwise(got["A"][f], ref["A"][f]) < tol
            assert np.abs(got["B"][f]).max() <= 1e-12 * np.abs(got["A"][f]).max()
        assert normwise(got["A"][0], got["A"][2]) < 1e-11
        w = _worst(got, ref, ("A", "B", "F"))
        for k, e in w.items():
            assert e < tol, (precision, k, e)


def test_empty_frequency_list_and_too_many_headings(bg):
    s = _solver(bg, cases.lib_cylinder(cases.CYL_SMALL), [0.0], bg.MIXED)
    got = s.solve_omegas(np.array([]))
    assert got["A"].shape == (0, 6, 6)
    with pytest.raises(bg.BEMError):
        s2 = bg.Hydrodynamic_Radiation_Solver()
        s2.Set_Parameters([bg.Parameter("WaveAngle", b) for b in np.linspace(0, 1, 11)])
        s2.Setup(cases.lib_cylinder(cases.CYL_SMALL))
