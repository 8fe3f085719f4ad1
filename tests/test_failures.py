"""Failure detection, in the forms that fault, trap or hang no GPU: bad inputs
caught on the host, a refinement that runs out of its solve budget, and a
device-side wait that runs into its deadline because the flag it waits for is
never published (the kernel gives up, sets FLAG_TIMEOUT and finishes; the host
reports BEM_ERR_CUDA).  After each failure the same context must still solve
correctly.  The reference has no error codes (it prints and returns,
BEMUser_Console.cpp:30-33); these are the C ABI's."""
import numpy as np
import pytest

import cases
from conftest import normwise

pytestmark = pytest.mark.gpu

BEM_ERR_ARG, BEM_ERR_CUDA, BEM_ERR_STATE, BEM_ERR_NUMERIC = 1, 2, 3, 4


@pytest.fixture(scope="module")
def bg():
    import bemuse_gb300
    bemuse_gb300.build.build()
    return bemuse_gb300


def _solver(bg, precision):
    s = bg.Hydrodynamic_Radiation_Solver(precision=precision)
    s.Set_Parameters([bg.Parameter("WaveAngle", 0.0)])
    s.Set_Mass_Properties(gyration=np.eye(3))
    return s


def _status(excinfo):
    return excinfo.value.status


def test_degenerate_panel_is_rejected(bg):
    m = cases.lib_cylinder(cases.CYL_SMALL)
    nodes = m.nodes.copy()
    e = m.elems[len(m.elems) // 2]
    # collapse one quad onto a line: its area is zero
    nodes[e[1]] = nodes[e[0]]
    nodes[e[2]] = nodes[e[3]]
    bad = bg.Mesh(nodes, m.elems)
    s = _solver(bg, bg.PLAIN_FP64)
    with pytest.raises(bg.BEMError) as ex:
        s.Setup(bad)
    assert _status(ex) == BEM_ERR_ARG and "degenerate" in str(ex.value)
    nodes2 = m.nodes.copy()
    nodes2[3, 2] = np.nan
    with pytest.raises(bg.BEMError) as ex:
        s.Setup(bg.Mesh(nodes2, m.elems))
    assert _status(ex) == BEM_ERR_ARG


def test_solve_before_setup_is_out_of_order(bg):
    s = _solver(bg, bg.MIXED)
    with pytest.raises(bg.BEMError) as ex:
        s.solve_omegas([0.5])
    assert _status(ex) == BEM_ERR_STATE


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_non_finite_frequency_is_rejected(bg, orc, bad):
    s = _solver(bg, bg.MIXED)
    s.Setup(cases.lib_cylinder(cases.CYL_SMALL))
    with pytest.raises(bg.BEMError) as ex:
        s.solve_omegas([0.5, bad])
    assert _status(ex) == BEM_ERR_ARG
    # the context still solves
    m, _ = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    ref = orc.solve(m, [0.5], [0.0], M=s.M_ij, C=s.C_ij)
    got = s.solve_omegas([0.5])
    assert normwise(got["A"][0], ref["A"][0]) < 1e-6


@pytest.mark.parametrize("graph", [0, 1])
@pytest.mark.parametrize("omegas", [[0.8], [0.8, 1.0, 1.3, 1.7]])
def test_refinement_out_of_solves_is_numeric_failure(bg, orc, omegas, graph):
    # with several frequencies the failure comes while the next frequency's LU and the
    # one after's assembly are in flight on their own streams; graph = 1: the convergence
    # test runs on the device (refine_graph) and reports the same failure
    s = _solver(bg, bg.MIXED)
    s.Setup(cases.lib_cylinder(cases.CYL_SMALL))
    s.set_tuning("refine_graph", graph)
    s.set_tuning("refine_max_solves", 0)
    with pytest.raises(bg.BEMError) as ex:
        s.solve_omegas(omegas)
    assert _status(ex) == BEM_ERR_NUMERIC and "did not reach the tolerance" in str(ex.value)
    s.set_tuning("refine_max_solves", 60)
    m, _ = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    ref = orc.solve(m, omegas, [0.0], M=s.M_ij, C=s.C_ij)
    got = s.solve_omegas(omegas)
    assert np.all(got["residual"] <= 1e-12)
    for f in range(len(omegas)):
        assert normwise(got["A"][f], ref["A"][f]) < 1e-6
    with pytest.raises(bg.BEMError):
        s.set_tuning("refine_max_solves", -1)


@pytest.mark.parametrize("gmres,graph", [(0, 0), (1, 0), (0, 1)])
def test_expired_device_wait_is_reported_and_context_survives(bg, orc, gmres, graph):
    # Every wait of the triangular-solve chain asks for a flag value nothing publishes;
    # each gives up 1 ms after its CTA starts, sets FLAG_TIMEOUT and the chain finishes
    # (all accesses stay in bounds, the results are garbage).  The host must report
    # BEM_ERR_CUDA, not a refinement failure, and the context must solve correctly after.
    # 288 panels: two 256-row super-blocks, so the chain has waits across them
    s = _solver(bg, bg.MIXED)
    s.Setup(cases.lib_cylinder(cases.CYL_MED))
    assert s.N == 288
    s.set_tuning("refine_gmres", gmres)
    s.set_tuning("refine_graph", graph)
    s.set_tuning("test_wait_ms", 1.0)
    s.set_tuning("test_wait_skew", 1)
    with pytest.raises(bg.BEMError) as ex:
        s.solve_omegas([0.8, 1.1, 1.5])
    assert _status(ex) == BEM_ERR_CUDA and "expired" in str(ex.value)
    s.set_tuning("test_wait_skew", 0)
    s.set_tuning("test_wait_ms", 2000.0)
    m, _ = cases.oracle_cylinder(orc, cases.CYL_MED)
    ref = orc.solve(m, [0.8, 1.2], [0.0], M=s.M_ij, C=s.C_ij)
    got = s.solve_omegas([0.8, 1.2])
    assert np.all(got["residual"] <= 1e-12)
    for f in range(2):
        assert normwise(got["A"][f], ref["A"][f]) < 1e-6
        assert normwise(got["B"][f], ref["B"][f]) < 1e-6


def test_bad_tuning_values_are_rejected(bg):
    s = _solver(bg, bg.MIXED)
    for key, val in (("test_wait_skew", 2), ("test_wait_ms", 0.0), ("refine_graph", 2), ("no_such_key", 1)):
        with pytest.raises(bg.BEMError) as ex:
            s.set_tuning(key, val)
        assert _status(ex) == BEM_ERR_ARG
