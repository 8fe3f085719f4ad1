"""Parity on the plain-method workload at its full size: a floating truncated
vertical cylinder (radius 10 m, draft 20 m, 48 azimuthal x (8 bottom rings + 16
vertical) panels with linear spacing = 1,152 panels: 48 triangles + 1,104
quads), infinite depth, 20 frequencies uniform on 0.1-2.0 rad/s, heading 0,
6 radiation + 1 diffraction right-hand sides, unit radii of gyration with the
centre of gravity at the waterline centre.

Both GPU paths are compared with the FP64 oracle on every frequency, with the
oracle's own mass and stiffness matrices (not the library's):
  plain FP64 GPU path   1e-8 normwise on A, B, F, FK, SC, RAO
  mixed path            1e-6 normwise on A, B, F, FK, SC; residual <= 1e-12"""
import numpy as np
import pytest

from conftest import normwise

pytestmark = pytest.mark.gpu

OMEGAS = np.linspace(0.1, 2.0, 20)
BETAS = [0.0]


@pytest.fixture(scope="module")
def bg():
    import bemuse_gb300
    bemuse_gb300.build.build()
    return bemuse_gb300


@pytest.fixture(scope="module")
def ref(orc):
    m, _ = orc.cylinder(10.0, 20.0, 48, 8, 16, cosine=False)
    assert m.n == 1152 and int((m.elems[:, 3] < 0).sum()) == 48
    M, C, _ = orc.mass_hydrostatics(m, None, rho=1025.0, g=9.81, mass=0.0, cog=(0, 0, 0), gyr=np.eye(3))
    return orc.solve(m, OMEGAS, BETAS, M=M, C=C), M, C


def _solve(bg, precision):
    mesh = bg.Half_Cylinder(10.0, 20.0, 48, 8, 16, 0, False)
    s = bg.Hydrodynamic_Radiation_Solver(precision=precision)
    s.Set_Parameters([bg.Parameter("WaveAngle", b) for b in BETAS])
    s.Set_Mass_Properties(mass=0.0, cog=(0.0, 0.0, 0.0), gyration=np.eye(3))
    s.Setup(mesh)
    assert s.N == 1152
    return s, s.solve_omegas(OMEGAS)


def _worst(got, want, keys):
    return {k: max(normwise(got[k][f], want[k][f]) for f in range(len(OMEGAS))) for k in keys}


def test_plain_fp64_matches_oracle_on_all_20_frequencies(bg, ref):
    want, M, C = ref
    s, got = _solve(bg, bg.PLAIN_FP64)
    assert np.allclose(s.M_ij, M, rtol=1e-12, atol=0) and np.allclose(s.C_ij, C, rtol=1e-12, atol=1e-9)
    worst = _worst(got, want, ("A", "B", "F", "FK", "SC", "RAO"))
    print("plain vs oracle", worst)
    for k, e in worst.items():
        assert e < 1e-8, (k, e)


def test_mixed_matches_oracle_on_all_20_frequencies(bg, ref):
    want, _, _ = ref
    _, got = _solve(bg, bg.MIXED)
    print("refine sweeps", got["iters"], "max residual", got["residual"].max())
    assert np.all(got["residual"] <= 1e-12)
    worst = _worst(got, want, ("A", "B", "F", "FK", "SC"))
    print("mixed vs oracle", worst)
    for k, e in worst.items():
        assert e < 1e-6, (k, e)
