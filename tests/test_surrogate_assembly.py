"""The surrogate form of the mixed assembly (k_wave_surrogate): far-field pairs inside
the network's domain take the tensor-core network's G and dG/dh; near pairs,
out-of-domain pairs and the judged sample take the FP32 closed form.  Checked here:
  * with an empty domain every pair takes the closed form, and the solve keeps the
    mixed path's accuracy against the oracle (1e-6);
  * with every far pair judged, the network is evaluated but never used: the same
    accuracy, and the judge records its error;
  * strict mode with a network that misses the tolerance solves every frequency again
    with the closed form (results within 1e-6 of the oracle);
  * accept mode keeps the network's values: the refinement still converges on its own
    operator, and the error against the oracle is reported, not hidden."""
import numpy as np
import pytest

import cases
from conftest import normwise

pytestmark = pytest.mark.gpu

OMEGAS = np.array([0.3, 0.6, 1.0])


@pytest.fixture(scope="module")
def bg():
    import bemuse_gb300
    bemuse_gb300.build.build()
    return bemuse_gb300


@pytest.fixture(scope="module")
def array_case(bg, orc):
    """Four small cylinders 50 m apart: most pairs are far field."""
    from oracle.oracle import Mesh as OMesh
    c = cases.ARRAY_SMALL
    om, _ = orc.cylinder(c["R"], c["draft"], c["NA"], c["NR"], c["NV"], cosine=False)
    omesh = OMesh.concat([om] * 4, cases.ARRAY_ORIGINS)
    lm = bg.Half_Cylinder(c["R"], c["draft"], c["NA"], c["NR"], c["NV"], 0, False)
    lmesh = bg.unify([lm] * 4, cases.ARRAY_ORIGINS)
    ref = orc.solve(omesh, OMEGAS, cases.BETAS)
    return lmesh, ref


@pytest.fixture(scope="module")
def trained(bg):
    """A network trained briefly on the domain (a few seconds of the library's own
    training kernels): good enough to be used, far from the 1e-6 the solve needs."""
    x, y, t = bg.HavelockSurrogate.domain_set(1 << 17, seed=0)
    s = bg.HavelockSurrogate(seed=0)
    s.set_domain_normalization(t)
    for e in range(40):
        s.train(x, t, epochs=1, batch=4096, lr=2e-3 * (0.93 ** e), seed=e)
    return s


def _solver(bg, mesh):
    s = bg.Hydrodynamic_Radiation_Solver(precision=bg.MIXED)
    s.Set_Parameters([bg.Parameter("WaveAngle", b) for b in cases.BETAS])
    s.Setup(mesh)
    return s


def _err(got, ref):
    return {k: max(normwise(got[k][f], ref[k][f]) for f in range(len(OMEGAS))) for k in ("A", "B", "F")}


def test_empty_domain_is_the_closed_form(bg, array_case, trained):
    mesh, ref = array_case
    s = _solver(bg, mesh)
    s.set_surrogate(trained, mode="accept", judge_fraction=0.0, domain=[1e9, 1e9, 0.0, 3.0])
    got = s.solve_omegas(OMEGAS)
    st = s.surrogate_stats()
    print(st, _err(got, ref))
    assert st["gauss_points_network"] == 0 and st["judged_pairs"] == 0
    assert st["frequencies_with_surrogate"] == len(OMEGAS)
    n = mesh.n
    nq = int(np.sum(np.where(mesh.elems[:, 3] < 0, 3, 4)))
    assert st["gauss_points_closed_form"] == len(OMEGAS) * n * nq
    assert np.all(got["residual"] <= 1e-12)
    for k, e in _err(got, ref).items():
        assert e < 1e-6, (k, e)


def test_fully_judged_uses_the_closed_form_and_records_the_error(bg, array_case, trained):
    mesh, ref = array_case
    s = _solver(bg, mesh)
    s.set_surrogate(trained, mode="accept", judge_fraction=1.0)
    got = s.solve_omegas(OMEGAS)
    st = s.surrogate_stats()
    print(st, _err(got, ref))
    assert st["gauss_points_network"] == 0
    assert st["judged_pairs"] > 0 and 0.0 < st["judged_error_max"] < 10.0
    for k, e in _err(got, ref).items():
        assert e < 1e-6, (k, e)


def test_strict_mode_falls_back_and_keeps_accuracy(bg, array_case, trained):
    mesh, ref = array_case
    s = _solver(bg, mesh)
    s.set_surrogate(trained, mode="strict", judge_tol=1e-6, judge_fraction=0.05)
    got = s.solve_omegas(OMEGAS)
    st = s.surrogate_stats()
    print(st, _err(got, ref))
    assert st["gauss_points_network"] > 0
    assert st["frequencies_resolved"] == len(OMEGAS)  # a BF16 network misses 1e-6 everywhere
    assert np.all(got["residual"] <= 1e-12)
    for k, e in _err(got, ref).items():
        assert e < 1e-6, (k, e)


def test_accept_mode_converges_and_reports_its_error(bg, array_case, trained):
    mesh, ref = array_case
    s = _solver(bg, mesh)
    s.set_surrogate(trained, mode="accept", judge_fraction=0.01)
    got = s.solve_omegas(OMEGAS)
    st = s.surrogate_stats()
    err = _err(got, ref)
    print(st, err)
    frac = st["gauss_points_network"] / (st["gauss_points_network"] + st["gauss_points_closed_form"])
    print("share of Gauss points by the network: %.3f" % frac)
    assert frac > 0.3
    assert np.all(got["residual"] <= 1e-12)
    # the network's values enter the operator: the results move, but stay the same solution
    assert 1e-6 < max(err.values()) < 0.2


def test_bad_surrogate_settings_are_rejected(bg, array_case, trained):
    s = _solver(bg, array_case[0])
    for kw in (dict(mode="strict", judge_fraction=0.0), dict(mode="accept", judge_fraction=2.0),
               dict(mode="accept", domain=[0.0, 1.0, -1.0, 3.0])):
        with pytest.raises(bg.BEMError):
            s.set_surrogate(trained, **kw)
