"""GPU parity: every stage of the CUDA path against the FP64 CPU oracle.

Tolerances (normwise = max|gpu - oracle| / max|oracle|):
  HavelockGF FP64        1e-9  relative per point (CUDA j0/y0 vs libstdc++)
  HavelockGF FP32        2e-4  relative to max(|G|, 1) per point
  Rankine influence      1e-11 absolute (values are O(1))
  wave influence FP64    1e-9  normwise
  plain FP64 solve       1e-8  normwise per frequency on A, B, F, FK, SC, RAO
  mixed solve            1e-6  normwise per frequency on A, B, F
"""
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


def _grid(n=4000, seed=0):
    rng = np.random.default_rng(seed)
    kr = 10 ** rng.uniform(-3, np.log10(200), n)
    th = rng.uniform(0, 2 * np.pi, n)
    v = -10 ** rng.uniform(-3, 2, n)
    return kr * np.cos(th), kr * np.sin(th), v


def test_havelock_fp64_matches_oracle(bg, orc):
    x, y, v = _grid()
    g = bg.havelock_gf(x, y, v, bg.PLAIN_FP64)
    o = orc.havelock(x, y, v)
    rel = np.abs(g - o) / np.maximum(np.abs(o), 1e-300)
    assert np.max(rel) < 1e-9, np.max(rel)


def test_havelock_fp32_accuracy(bg, orc):
    x, y, v = _grid(seed=1)
    g = bg.havelock_gf(x, y, v, bg.MIXED)
    o = orc.havelock(x, y, v)
    err = np.abs(g - o) / np.maximum(np.abs(o), 1.0)
    print("fp32 HavelockGF max err", err.max(axis=0))
    assert np.max(err) < 2e-4


def test_havelock_branches_and_small_h(bg, orc):
    # both Struve branches (h <= 3, h > 3) and the h <= 1e-6 guard
    h = np.array([1e-8, 1e-7, 5e-7, 0.5, 2.999, 3.0, 3.001, 10.0, 150.0])
    v = np.full_like(h, -0.7)
    g = bg.havelock_gf(h, 0 * h, v, bg.PLAIN_FP64)
    o = orc.havelock(h, 0 * h, v)
    assert np.allclose(g, o, rtol=1e-9, atol=1e-12)
    assert np.all(g[:3, 1] == 0) and np.all(g[:3, 2] == 0)


def _solver(bg, mesh, betas=cases.BETAS, precision=0, gyr=cases.GYR_UNIT):
    s = bg.Hydrodynamic_Radiation_Solver(precision=precision)
    s.Set_Parameters([bg.Parameter("WaveAngle", b) for b in betas])
    s.Set_Mass_Properties(mass=0.0, cog=(0, 0, 0), gyration=gyr)
    s.Setup(mesh)
    return s


def test_rankine_matches_oracle(bg, orc):
    m, _ = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    s = _solver(bg, cases.lib_cylinder(cases.CYL_SMALL))
    got = s.rankine()
    ref = orc.rankine(m)[:4]
    for a, b in zip(got, ref):
        assert np.max(np.abs(a - b)) < 1e-11


@pytest.mark.parametrize("K", [0.01, 0.2, 1.0])
def test_wave_matrices_match_oracle(bg, orc, K):
    m, _ = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    s = _solver(bg, cases.lib_cylinder(cases.CYL_SMALL))
    ws, wd = s.wave_matrices(K, bg.PLAIN_FP64)
    ows, owd = orc.wave(m, K)
    assert normwise(ws, ows) < 1e-9
    assert normwise(wd, owd) < 1e-9
    ws32, wd32 = s.wave_matrices(K, bg.MIXED)
    e32 = max(normwise(ws32, ows), normwise(wd32, owd))
    print("fp32 wave matrices normwise err", e32)
    assert e32 < 1e-4


def _oracle_solve(orc, mesh, aux, omegas, betas, s):
    return orc.solve(mesh, omegas, betas, M=s.M_ij, C=s.C_ij)


def _compare(got, ref, tol, keys=("A", "B", "F", "FK", "SC")):
    worst = {}
    for k in keys:
        e = max(normwise(got[k][f], ref[k][f]) for f in range(got[k].shape[0]))
        worst[k] = e
    print(worst)
    for k, e in worst.items():
        assert e < tol, (k, e)


def test_plain_fp64_solve_matches_oracle_cylinder(bg, orc):
    m, aux = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    s = _solver(bg, cases.lib_cylinder(cases.CYL_SMALL))
    got = s.solve_omegas(cases.OMEGAS)
    ref = _oracle_solve(orc, m, aux, cases.OMEGAS, cases.BETAS, s)
    _compare(got, ref, 1e-8, keys=("A", "B", "F", "FK", "SC", "RAO"))


def test_mixed_solve_matches_oracle_cylinder(bg, orc):
    m, aux = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    s = _solver(bg, cases.lib_cylinder(cases.CYL_SMALL), precision=bg.MIXED)
    got = s.solve_omegas(cases.OMEGAS)
    ref = _oracle_solve(orc, m, aux, cases.OMEGAS, cases.BETAS, s)
    print("refine sweeps", got["iters"], "residual", got["residual"])
    assert np.all(got["residual"] <= 1e-12)
    _compare(got, ref, 1e-6)


def test_refinement_variants_agree_near_irregular_frequency(bg, orc):
    # The 144-panel cylinder (R = 10, draft 20) has its first irregular frequency near
    # K R = 2.405 coth(2.405 draft / R), Omega ~ 1.54: the system is nearly singular there
    # and classic refinement contracts slowly.  Classic (0), flexible GMRES (1) and the
    # default switch from classic to GMRES (2) must meet the same residual test, agree
    # with the oracle, and GMRES must not need more preconditioner solves than classic.
    m, aux = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    om = np.linspace(1.45, 1.65, 9)
    s = _solver(bg, cases.lib_cylinder(cases.CYL_SMALL), precision=bg.MIXED)
    ref = _oracle_solve(orc, m, aux, om, cases.BETAS, s)
    got = {}
    for mode in (0, 1, 2):
        s.set_tuning("refine_gmres", mode)
        got[mode] = s.solve_omegas(om)
        print("refine_gmres", mode, "iterations", got[mode]["iters"], "residual", got[mode]["residual"].max())
        assert np.all(got[mode]["residual"] <= 1e-12)
        _compare(got[mode], ref, 1e-6)
    assert np.all(got[1]["iters"] <= got[0]["iters"] + 1)
    assert np.all(got[2]["iters"] <= got[0]["iters"] + 1)


def test_device_side_refinement_matches_host_loop(bg, orc):
    """The classic refinement with its convergence test on the device (refine_graph = 1: a
    conditional while node of a CUDA graph repeats the sweeps, k_refine_step decides) makes
    the decisions of the host loop: the same sweeps, the switch to GMRES near the irregular
    frequency of the 144-panel cylinder (Omega ~ 1.54), the coarse first residual, the
    same results; with one LU in flight and with two beside the refinement."""
    m, aux = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    om = np.array([0.5, 1.0, 1.50, 1.54, 1.58, 2.2])
    got = {}
    for lo in (0, 2):
        for g in (0, 1):
            s = _solver(bg, cases.lib_cylinder(cases.CYL_SMALL), precision=bg.MIXED)
            s.set_tuning("lu_overlap", lo)
            s.set_tuning("refine_graph", g)
            got[lo, g] = s.solve_omegas(om)
            print("lu_overlap", lo, "refine_graph", g, "sweeps", got[lo, g]["iters"])
            assert np.all(got[lo, g]["residual"] <= 1e-12)
    ref = _oracle_solve(orc, m, aux, om, cases.BETAS, s)
    _compare(got[2, 1], ref, 1e-6)
    for lo in (0, 2):
        assert np.array_equal(got[lo, 0]["iters"], got[lo, 1]["iters"]), lo
        for k in ("A", "B", "F"):
            assert max(normwise(got[lo, 1][k][f], got[lo, 0][k][f]) for f in range(om.size)) < 1e-11, (lo, k)


def test_coarse_first_residual_keeps_the_sweeps(bg, orc):
    # The first sweep's residual from the FP32 high words of Re D (refine_coarse_first = 1,
    # the default, used after a solve that contracted by less than 3e-4 per sweep) against
    # every residual in double-float: the same residual test and the same results to the
    # mixed-path tolerance.  Neighbouring frequencies contract alike, so the coarse
    # residual adds at most one sweep where the contraction changes.
    m, aux = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    om = np.array([0.7, 0.8, 1.0, 1.2, 2.0])
    s = _solver(bg, cases.lib_cylinder(cases.CYL_SMALL), precision=bg.MIXED)
    ref = _oracle_solve(orc, m, aux, om, cases.BETAS, s)
    got = {}
    for coarse in (0, 1):
        s.set_tuning("refine_coarse_first", coarse)
        got[coarse] = s.solve_omegas(om)
        print("refine_coarse_first", coarse, "iterations", got[coarse]["iters"], "residual",
              got[coarse]["residual"].max())
        assert np.all(got[coarse]["residual"] <= 1e-12)
        _compare(got[coarse], ref, 1e-6)
    assert np.all(got[1]["iters"] <= got[0]["iters"] + 1)
    assert got[1]["iters"].sum() <= got[0]["iters"].sum() + 1
    with pytest.raises(bg.BEMError):
        s.set_tuning("refine_coarse_first", 2)


def test_lu_schedule_variants_agree(bg):
    # 1200 panels: the TF32 LU has 10 block steps, so the paired schedule runs four full
    # pairs and a final single step.  Every schedule / inverse variant must meet the
    # refinement test and agree with the plain FP64 GPU solve (itself pinned to the
    # oracle above) to the mixed-path tolerance.
    mesh = bg.Half_Cylinder(10.0, 20.0, 40, 6, 24, 0, False)
    om = np.array([0.6, 1.4])
    ref = _solver(bg, mesh).solve_omegas(om)
    s = _solver(bg, mesh, precision=bg.MIXED)
    variants = [
        # (two steps per pass, CTAs per inverse, blocked inverse, split panel)
        (1, 4, 1, 1), (0, 4, 1, 1), (1, 2, 0, 1), (1, 8, 1, 1), (1, 1, 0, 1), (1, 4, 1, 0), (0, 2, 1, 0),
        (1, 4, 2, 1), (1, 2, 2, 1), (1, 8, 2, 1), (0, 4, 2, 0),
    ]
    for pair, cl, blk, split in variants:
        s.set_tuning("lu_pair_update", pair)
        s.set_tuning("lu_cluster_inverse", cl)
        s.set_tuning("lu_block_inverse", blk)
        s.set_tuning("lu_split_panel", split)
        got = s.solve_omegas(om)
        print((pair, cl, blk, split), "iterations", got["iters"], "residual", got["residual"].max())
        assert np.all(got["residual"] <= 1e-12)
        _compare(got, ref, 1e-6, keys=("A", "B", "F"))


def test_lu_beside_refinement_matches_serial_schedule(bg):
    """The split pipelines (the LU of frequency f + 1 beside the refinement of f, f + 2
    assembled meanwhile, three frequency slots; or four or five slots with the LUs of
    f + 1 .. f + 3 on as many streams), cycled by seven frequencies, give the results of the schedule
    that factors and refines one frequency after the other."""
    mesh = cases.lib_cylinder(cases.CYL_MED)
    om = np.array([0.3, 0.7, 1.1, 1.5, 1.9, 2.3, 0.5])
    out = {}
    for lo in (0, 1, 2, 3):
        s = _solver(bg, mesh, precision=bg.MIXED)
        s.set_tuning("lu_overlap", lo)
        out[lo] = s.solve_omegas(om)
        assert np.all(out[lo]["residual"] <= 1e-12)
    for lo in (1, 2, 3):
        for k in ("A", "B", "F"):
            assert max(normwise(out[lo][k][f], out[0][k][f]) for f in range(om.size)) < 1e-11, (lo, k)
        assert np.array_equal(out[0]["iters"], out[lo]["iters"])


def test_programmatic_launches_keep_the_results(bg):
    """The LU with its block inverses and first W21 tiles launched as programmatic
    dependents (lu_pdl = 1) gives the results of ordinary launches."""
    mesh = cases.lib_cylinder(cases.CYL_MED)
    om = np.array([0.4, 1.2, 2.0])
    out = {}
    for pdl in (0, 1):
        s = _solver(bg, mesh, precision=bg.MIXED)
        s.set_tuning("lu_pdl", pdl)
        out[pdl] = s.solve_omegas(om)
        assert np.all(out[pdl]["residual"] <= 1e-12)
    for k in ("A", "B", "F"):
        assert max(normwise(out[1][k][f], out[0][k][f]) for f in range(om.size)) < 1e-11, k


def test_autotune_picks_a_setting(bg):
    # the autotuner times seven schedule settings on the sample frequencies, marks the one
    # it keeps, and the solver then solves with it to the mixed-path tolerance
    mesh = bg.Half_Cylinder(10.0, 20.0, 40, 6, 24, 0, False)
    om = np.array([0.6, 1.4])
    ref = _solver(bg, mesh).solve_omegas(om)
    s = _solver(bg, mesh, precision=bg.MIXED)
    ms, report = s.autotune([0.4, 0.9, 1.6, 2.4])
    print("\n".join(report))
    assert ms > 0.0
    assert len(report) == 7
    assert sum(line.startswith("*") for line in report) == 1
    got = s.solve_omegas(om)
    assert np.all(got["residual"] <= 1e-12)
    _compare(got, ref, 1e-6, keys=("A", "B", "F"))
    with pytest.raises(bg.BEMError):
        s.autotune([0.5])


def test_plain_fp64_solve_matches_oracle_array(bg, orc):
    c = cases.ARRAY_SMALL
    om, _ = orc.cylinder(c["R"], c["draft"], c["NA"], c["NR"], c["NV"], cosine=False)
    from oracle.oracle import Mesh as OMesh
    omesh = OMesh.concat([om] * 4, cases.ARRAY_ORIGINS)
    lm = bg.Half_Cylinder(c["R"], c["draft"], c["NA"], c["NR"], c["NV"], 0, False)
    lmesh = bg.unify([lm] * 4, cases.ARRAY_ORIGINS)
    s = _solver(bg, lmesh)
    got = s.solve_omegas(cases.OMEGAS[:3])
    ref = orc.solve(omesh, cases.OMEGAS[:3], cases.BETAS, M=s.M_ij, C=s.C_ij)
    _compare(got, ref, 1e-8)


def test_plain_fp64_solve_matches_oracle_barge(bg, orc):
    c = cases.BARGE_SMALL
    om, oa = orc.barge(c["L"], c["W"], c["D"], c["NX"], c["NY"], c["NZ"], cosine=c["cosine"])
    s = _solver(bg, bg.Barge(c["L"], c["W"], c["D"], c["NX"], c["NY"], c["NZ"], c["cosine"]), betas=[0.0])
    got = s.solve_omegas(cases.OMEGAS[1:4])
    ref = orc.solve(om, cases.OMEGAS[1:4], [0.0], M=s.M_ij, C=s.C_ij)
    _compare(got, ref, 1e-8)


def test_set_real_uses_frequency_over_two_pi(bg, orc):
    m, aux = cases.oracle_cylinder(orc, cases.CYL_SMALL)
    s = _solver(bg, cases.lib_cylinder(cases.CYL_SMALL))
    s.Set_Real(2 * np.pi * 0.8)
    s.Solve()
    ref = orc.solve(m, [0.8], cases.BETAS, M=s.M_ij, C=s.C_ij, want_phi=True)
    assert normwise(s.A_ij, ref["A"][0]) < 1e-8
    assert normwise(s.RadSolArray[-1], ref["phiJ"]) < 1e-8
    assert normwise(s.DiffSolArray[-1], ref["phiS"]) < 1e-8


def test_dense_solve_plain_and_mixed(bg):
    rng = np.random.default_rng(3)
    # padded sizes 128, 384, 768, 1152: one 128-block, then odd and even block counts (the
    # triangular solves pair the 128-blocks; an odd count leaves the last one single)
    for n in (100, 300, 700, 1100):
        A = 0.5 * np.eye(n) + 0.3 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
        A += np.diag(np.sign(rng.standard_normal(n)) * 0.0)
        B = rng.standard_normal((n, 5)) + 1j * rng.standard_normal((n, 5))
        ref = np.linalg.solve(A, B)
        x, _, _ = bg.dense_solve(A, B, bg.PLAIN_FP64)
        assert normwise(x, ref) < 1e-11
        x, it, res = bg.dense_solve(A, B, bg.MIXED)
        assert res <= 1e-12 and normwise(x, ref) < 1e-10


def test_aero_steady_solve_matches_oracle(bg, orc):
    """Aerodynamic_Solver constant-panel steady solve (Aerodynamic_Solver.cpp:42-58,
    150-180) on a 240-panel NACA 0012 wing at 5 deg: X = H^-1 (G (U . n))."""
    from oracle.oracle import Mesh as OMesh
    w = bg.NACA_Wing(1.0, 8.0, 0.12, 24, 10)
    U = [np.cos(np.radians(5.0)), 0.0, np.sin(np.radians(5.0))]
    Xo, BCo = orc.aero(OMesh(w.nodes, w.elems), U)
    for prec, tol in ((bg.PLAIN_FP64, 1e-10), (bg.MIXED, 1e-10)):
        a = bg.Aerodynamic_Solver(precision=prec)
        a.Setup(w)
        a.Set_External_BC([U])
        X = a.Solve_Steady()
        assert np.max(np.abs(a.BC - BCo)) < 1e-14
        assert normwise(X, Xo) < tol, (prec, normwise(X, Xo))


@pytest.mark.gpu
def test_batch_solve_matches_single_bodies(bg):
    """bem_batch_solve (concurrent per-body pipelines) gives each body the results
    of its own single-context solve."""
    meshes = [bg.Half_Cylinder(5.0, 8.0, 12, 3, 4, 0, False), bg.Barge(20.0, 8.0, 4.0, 8, 4, 3, True),
              bg.Half_Cylinder(3.0, 6.0, 16, 2, 5, 0, False)]
    om = np.array([0.3, 0.9])
    outs, sec = bg.batch_solve(meshes, om, [0.0, 0.5], bg.MIXED, n_workers=3)
    for m, o in zip(meshes, outs):
        s = bg.Hydrodynamic_Radiation_Solver(precision=bg.MIXED)
        s.Set_Parameters([bg.Parameter("WaveAngle", 0.0), bg.Parameter("WaveAngle", 0.5)])
        s.Setup(m)
        ref = s.solve_omegas(om)
        for k in ("A", "B", "F"):
            assert normwise(o[k], ref[k]) < 1e-12, k


@pytest.mark.gpu
def test_gdf_import_solves_like_generated_mesh(bg, tmp_path):
    """A body written to .gdf and read back (GDF_Geo.cpp: unshared nodes per panel)
    solves to the generated body's coefficients."""
    m = bg.Half_Cylinder(5.0, 8.0, 16, 3, 5, 0, False)
    lines = ["round trip of a cylinder mesh", "1.0 9.81", "0 0", str(m.n)]
    for e in m.elems:
        ids = [int(i) for i in e if i >= 0]
        ids += [ids[2]] * (4 - len(ids))
        lines += ["%.17g %.17g %.17g" % tuple(m.nodes[i]) for i in ids]
    p = tmp_path / "cyl.gdf"
    p.write_text("\n".join(lines) + "\n")
    g = bg.read_mesh(p)
    assert g.n == m.n
    om = np.array([0.2, 0.7])
    out = []
    for mesh in (m, g):
        s = bg.Hydrodynamic_Radiation_Solver(precision=bg.PLAIN_FP64)
        s.Set_Parameters([bg.Parameter("WaveAngle", 0.0)])
        s.Setup(mesh)
        out.append(s.solve_omegas(om))
    for k in ("A", "B", "F"):
        assert normwise(out[1][k], out[0][k]) < 1e-12, k


@pytest.mark.gpu
def test_batch_solve_many_concurrent_contexts(bg):
    """Eight contexts at once on one GPU (the bench's batched form in small): every body
    gets its single-context result.  Catches work lost to SM admission or cross-context
    waits when the GPU is full of other contexts' kernels."""
    meshes = [bg.Half_Cylinder(4.0 + 0.5 * i, 10.0 + i, 32, 4, 12 + i, 0, False) for i in range(8)]
    om = np.array([0.3, 0.7, 1.1, 1.5, 1.9, 2.3])
    outs, sec = bg.batch_solve(meshes, om, [0.0], bg.MIXED, n_workers=8)
    for m, o in zip(meshes, outs):
        s = bg.Hydrodynamic_Radiation_Solver(precision=bg.MIXED)
        s.Set_Parameters([bg.Parameter("WaveAngle", 0.0)])
        s.Setup(m)
        ref = s.solve_omegas(om)
        for k in ("A", "B", "F"):
            assert normwise(o[k], ref[k]) < 1e-9, k


def test_cusolver_reference_lu_runs(bg):
    """bem_cusolver_zgetrf_ms (measurement only: cuSOLVER's partial-pivot complex LU,
    opened at run time) returns a positive device time, growing with the order."""
    t1 = bg.cusolver_zgetrf_ms(512)
    t2 = bg.cusolver_zgetrf_ms(2048)
    print("cusolver zgetrf ms", t1, t2)
    assert 0.0 < t1 < t2
