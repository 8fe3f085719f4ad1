"""Steady lifting flow past a wing with a trailing wake: the full-size steady
workload, a rectangular NACA 0012 wing (chord 1, span 8, 120 panels around the
section x 60 strips = 7,200 panels) at 5 deg, with a flat wake of 60 strips 20
chords long carrying the Kutta jumps, surface pressure from the surface gradient
of the potential, and the lift coefficient from the integrated pressure.

The reference's Aerodynamic_Solver (Aerodynamic_Solver.cpp:12-180) has no wake,
no Kutta condition and no pressure; this workload defines them (the oracle's
orc_aero_wake and oracle/aero_post.py) and the library matches the oracle:
  X (plain FP64 and mixed)   1e-10 normwise
  cp per panel               1e-9 absolute
  CL, CD, CF                 1e-10 absolute
and the physics: CL close to the lifting-line value 2 pi a / (1 + 2 / AR), odd
in the angle of attack, and near zero without the wake."""
import numpy as np
import pytest

from conftest import normwise

CHORD, SPAN, NC, NS, LENGTH = 1.0, 8.0, 120, 60, 20.0


def _U(alpha_deg):
    a = np.radians(alpha_deg)
    return np.array([np.cos(a), 0.0, np.sin(a)])


def test_wing_wake_geometry_matches_the_restatement():
    """bem_mesh_wing_wake (host only) against oracle/aero_post.wing_wake."""
    import os
    import bemuse_gb300 as bg
    from bemuse_gb300 import build
    from oracle import aero_post
    if not os.path.exists(build.LIB):
        pytest.skip("library not built")
    q, up, lo = bg.NACA_Wing_Wake(CHORD, SPAN, NC, NS, LENGTH)
    q2, up2, lo2 = aero_post.wing_wake(CHORD, SPAN, NC, NS, LENGTH)
    assert np.array_equal(q, q2) and np.array_equal(up, up2) and np.array_equal(lo, lo2)
    # the Kutta pair of every strip sits at the trailing edge, one on each side
    w = bg.NACA_Wing(CHORD, SPAN, 0.12, NC, NS)
    for e in (up[0], lo[0], up[-1], lo[-1]):
        xs = w.nodes[w.elems[e][w.elems[e] >= 0], 0]
        assert xs.max() == pytest.approx(CHORD)
    with pytest.raises(bg.BEMError):
        bg.NACA_Wing_Wake(CHORD, SPAN, 7, NS, LENGTH)


def test_oracle_lift_is_close_to_lifting_line():
    """The oracle's wake solve on a coarse wing (40 x 16 panels): CL(5 deg) within
    6 % of the lifting-line estimate, CL(-5 deg) = -CL(5 deg), no wake -> CL ~ 0."""
    import bemuse_gb300 as bg
    from oracle.oracle import Oracle, Mesh as OMesh
    from oracle import aero_post
    import os
    from bemuse_gb300 import build
    if not os.path.exists(build.LIB):
        pytest.skip("library not built")
    orc = Oracle()
    nc, ns = 40, 16
    w = bg.NACA_Wing(CHORD, SPAN, 0.12, nc, ns)
    om = OMesh(w.nodes, w.elems)
    q, up, lo = aero_post.wing_wake(CHORD, SPAN, nc, ns, LENGTH)
    P = orc.panels(om)
    cl = {}
    for a in (5.0, -5.0):
        X, _ = orc.aero_wake(om, q, up, lo, _U(a))
        cl[a] = aero_post.surface(P, w.elems, X, _U(a), CHORD * SPAN)[2]
    X0, _ = orc.aero(om, _U(5.0))
    cl0 = aero_post.surface(P, w.elems, X0, _U(5.0), CHORD * SPAN)[2]
    ll = 2 * np.pi * np.radians(5.0) / (1 + 2 / (SPAN / CHORD))
    assert abs(cl[5.0] / ll - 1) < 0.06
    assert cl[-5.0] == pytest.approx(-cl[5.0], rel=1e-9)
    assert abs(cl0) < 0.1 * cl[5.0]


@pytest.fixture(scope="module")
def wing(orc):
    import bemuse_gb300 as bg
    from oracle.oracle import Mesh as OMesh
    from oracle import aero_post
    bg.build.build()
    w = bg.NACA_Wing(CHORD, SPAN, 0.12, NC, NS)
    assert w.n == 7200
    q, up, lo = bg.NACA_Wing_Wake(CHORD, SPAN, NC, NS, LENGTH)
    om = OMesh(w.nodes, w.elems)
    X, BC = orc.aero_wake(om, q, up, lo, _U(5.0))
    cp, CF, CL, CD = aero_post.surface(orc.panels(om), w.elems, X, _U(5.0), CHORD * SPAN)
    return bg, w, (q, up, lo), dict(X=X, BC=BC, cp=cp, CF=CF, CL=CL, CD=CD)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["PLAIN_FP64", "MIXED"])
def test_wake_solve_and_pressure_match_oracle_at_7200_panels(wing, precision):
    bg, w, wake, ref = wing
    a = bg.Aerodynamic_Solver(precision=getattr(bg, precision))
    a.Set_Wake(*wake)
    a.Setup(w)
    a.Set_External_BC([_U(5.0)])
    X = a.Solve_Steady()
    assert np.max(np.abs(a.BC - ref["BC"])) < 1e-14
    e = normwise(X, ref["X"])
    cp, co = a.Surface(_U(5.0), CHORD * SPAN)
    print(precision, "X", e, "cp", np.max(np.abs(cp - ref["cp"])), "CL", co["CL"], ref["CL"])
    assert e < 1e-10
    assert np.max(np.abs(cp - ref["cp"])) < 1e-9
    assert abs(co["CL"] - ref["CL"]) < 1e-10 and abs(co["CD"] - ref["CD"]) < 1e-10
    assert np.max(np.abs(co["CF"] - ref["CF"])) < 1e-10
    # the library's pressure of the oracle's potential is the oracle's pressure
    cp2, co2 = a.Surface(_U(5.0), CHORD * SPAN, X=ref["X"])
    assert np.max(np.abs(cp2 - ref["cp"])) < 1e-12 and abs(co2["CL"] - ref["CL"]) < 1e-12


@pytest.mark.gpu
def test_lift_physics_on_the_gpu(wing):
    """CL(5 deg) within 6 % of lifting line, odd in alpha; removing the wake
    (n_wake = 0) takes the lift away."""
    bg, w, wake, ref = wing
    a = bg.Aerodynamic_Solver(precision=bg.MIXED)
    a.Set_Wake(*wake)
    a.Setup(w)
    a.Set_External_BC([_U(5.0)])
    a.Solve_Steady()
    cl_p = a.Surface(_U(5.0), CHORD * SPAN)[1]["CL"]
    a.Set_External_BC([_U(-5.0)])
    a.Solve_Steady()
    cl_m = a.Surface(_U(-5.0), CHORD * SPAN)[1]["CL"]
    ll = 2 * np.pi * np.radians(5.0) / (1 + 2 / (SPAN / CHORD))
    assert abs(cl_p / ll - 1) < 0.06
    assert cl_m == pytest.approx(-cl_p, rel=1e-8)
    a.Set_Wake(np.zeros((0, 4, 3)), [], [])
    a.Setup(w)
    a.Set_External_BC([_U(5.0)])
    a.Solve_Steady()
    assert abs(a.Surface(_U(5.0), CHORD * SPAN)[1]["CL"]) < 0.1 * cl_p


@pytest.mark.gpu
def test_wake_rejects_kutta_index_outside_the_mesh(wing):
    bg, w, wake, _ = wing
    q, up, lo = wake
    a = bg.Aerodynamic_Solver()
    bad = up.copy()
    bad[3] = w.n
    a.Set_Wake(q, bad, lo)
    with pytest.raises(bg.BEMError):
        a.Setup(w)
