"""Mass and hydrostatic stiffness matrices of the library (bem_get_body_matrices,
computed by host_mesh.cpp::mass_and_stiffness during bem_setup) against the
oracle's restatement of Calculate_Mass_Matrix and
Calculate_Hydrostatic_Stiffness_Matrix (Hydrodynamic_Solver.cpp:300-397),
including the reference's quirks (Q5): the waterplane integrals come from the
interior free-surface (aux) panels only, C mixes the Density parameter with the
1025 constant, and the symmetry lines overwrite the upper off-diagonal entries.
These matrices feed the RAO, so they are pinned here rather than passed from
the library into the oracle."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bg():
    import bemuse_gb300
    bemuse_gb300.build.build()
    return bemuse_gb300


def _lib(bg, mesh, rho, g, mass, cog, gyr):
    s = bg.Hydrodynamic_Radiation_Solver(precision=bg.PLAIN_FP64)
    s.Set_Parameters([bg.Parameter("WaveAngle", 0.0), bg.Parameter("Density", rho), bg.Parameter("Gravity", g)])
    s.Set_Mass_Properties(mass=mass, cog=cog, gyration=gyr)
    s.Setup(mesh)
    return s


def _close(a, b, tol=1e-12):
    d = np.max(np.abs(b))
    return np.max(np.abs(a - b)) <= tol * (d if d > 0 else 1.0)


PROPS = [
    # (density, gravity, mass (0: volume x 1025), centre of gravity, radii of gyration)
    (1025.0, 9.81, 0.0, (0.0, 0.0, 0.0), np.zeros((3, 3))),
    (1000.0, 9.80665, 0.0, (0.0, 0.0, -5.0), np.eye(3)),
    (1025.0, 9.81, 3.2e6, (0.5, -0.25, -3.0), np.diag([6.0, 7.0, 4.0]) + 0.5),
]


@pytest.mark.parametrize("props", PROPS)
def test_cylinder_with_waterplane_panels(bg, orc, props):
    rho, g, mass, cog, gyr = props
    om, oa = cases.oracle_cylinder(orc, cases.CYL_MED)
    s = _lib(bg, cases.lib_cylinder(cases.CYL_MED), rho, g, mass, cog, gyr)
    M, C, vc = orc.mass_hydrostatics(om, oa, rho=rho, g=g, mass=mass, cog=cog, gyr=gyr)
    print("M", M.diagonal(), "C", C.diagonal())
    assert _close(s.M_ij, M) and _close(s.C_ij, C)
    assert abs(s.Volume - vc[0]) <= 1e-12 * vc[0]
    assert np.allclose(s.Centre_Buoyancy, vc[1:], rtol=0, atol=1e-12 * max(1.0, np.abs(vc[1:]).max()))
    assert C[2, 2] != 0.0  # the aux panels give a waterplane area


@pytest.mark.parametrize("props", PROPS[1:])
def test_barge_with_waterplane_panels(bg, orc, props):
    rho, g, mass, cog, gyr = props
    c = cases.BARGE_SMALL
    om, oa = orc.barge(c["L"], c["W"], c["D"], c["NX"], c["NY"], c["NZ"], cosine=c["cosine"])
    s = _lib(bg, bg.Barge(c["L"], c["W"], c["D"], c["NX"], c["NY"], c["NZ"], c["cosine"]), rho, g, mass, cog, gyr)
    M, C, vc = orc.mass_hydrostatics(om, oa, rho=rho, g=g, mass=mass, cog=cog, gyr=gyr)
    assert _close(s.M_ij, M) and _close(s.C_ij, C)
    assert abs(s.Volume - vc[0]) <= 1e-12 * vc[0]


def test_without_waterplane_panels_c33_is_zero(bg, orc):
    # no aux (interior free-surface) panels: the reference's waterplane sums are empty
    c = dict(cases.CYL_SMALL, NRFS=0)
    om, oa = cases.oracle_cylinder(orc, c)
    s = _lib(bg, cases.lib_cylinder(c), 1025.0, 9.81, 0.0, (0.0, 0.0, 0.0), np.eye(3))
    M, C, vc = orc.mass_hydrostatics(om, None, rho=1025.0, g=9.81, mass=0.0, cog=(0, 0, 0), gyr=np.eye(3))
    assert _close(s.M_ij, M) and _close(s.C_ij, C)
    assert C[2, 2] == 0.0 and s.C_ij[2, 2] == 0.0
