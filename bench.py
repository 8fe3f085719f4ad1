"""Benchmark: frequency-solves/s of the panel-method hot path on GB300.

Workload (default): the four-column array -- four truncated cylinders, radius
6 m, draft 20 m, 64 azimuthal x (8 bottom + 24 side) panels each (2048 panels,
8192 in total), centred at (+-25, +-25, 0) m; infinite depth; 100 frequencies
uniform on 0.05-3.0 rad/s; headings 0/45/90 deg (6 radiation + 3 diffraction
right-hand sides).  Synthetic by construction (generated mesh, no dataset).

One step = one frequency-solve in the mixed-precision mode: wave assembly
(FP32 real parts, FP64-accurate imaginary parts), TF32 tensor-core LU, FP64
iterative refinement to 1e-12 relative residual, hull integrals.  The library runs
the timed frequencies as a pipeline (the assembly of f + 3, the LUs of f + 1 and
f + 2 and the refinement of f on their own streams); the autotuner picks the SM
split and the number of LUs in flight before the warm-up, outside the timed region.

  value         = freq-solves/s from device time (CUDA events on the library stream)
  e2e           = freq-solves/s of wall time around bem_solve (host in, host out)
  roofline      = the wave-assembly kernel on its FP32 bound (345 FP operations per
                  Green-function evaluation against a measured FMA rate), with the HBM view;
                  roofline.alone: the same kernel on the whole GPU (one frequency alone)
  lu_roofline   = the tensor-core LU against a measured cuBLAS TF32 rate
  cpu_baseline  = one unscaled frequency-solve of the same array by the oracle port on the
                  host cores (setup excluded); the same solve pins accuracy_vs_oracle
  plain_fp64    = the plain FP64 GPU path on --plain-steps of the timed frequencies, with
                  cuSOLVER zgetrf at the same order beside its LU (plain_lu_vs_cusolver)
  surrogate     = the learned form measured on the same frequencies (accept and strict)
  steady        = the steady lifting-wing workload: NACA 0012 wing of 7,200 panels at 5 deg
                  with a 60-strip trailing wake (Kutta condition), surface pressure and CL;
                  GPU wall time of setup (Rankine matrices + wake fold) and solve, and the
                  oracle's solve of the same case on the host cores beside it
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "freq-solves/s at 8k panels: mixed+surrogate vs FP64 GPU, A/B err <=1e-6"
OMEGAS = np.linspace(0.05, 3.0, 100)
BETAS = np.deg2rad([0.0, 45.0, 90.0])
ORIGINS = [[25.0, 25.0, 0.0], [-25.0, 25.0, 0.0], [-25.0, -25.0, 0.0], [25.0, -25.0, 0.0]]


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--plain-steps", type=int, default=2)
    p.add_argument("--na", type=int, default=64, help="azimuthal panels per cylinder (64 -> 8192 panels)")
    p.add_argument("--batched", type=int, default=1, help="1: also run the 64-body batched form")
    p.add_argument("--cpu-baseline", type=int, default=1,
                   help="1: time one unscaled oracle frequency-solve on the host cores (also the accuracy pin)")
    p.add_argument("--autotune", type=int, default=1,
                   help="1: time a small grid of schedule settings on 8 sample frequencies before the "
                        "warm-up (outside the timed region) and keep the fastest")
    p.add_argument("--surrogate-seconds", type=float, default=45.0,
                   help="training budget of the Green-function surrogate legs (0 skips them)")
    p.add_argument("--steady", type=int, default=1, help="1: also run the steady lifting-wing leg")
    return p.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="gloo")
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def shard(omegas, rank, world):
    """This rank's frequencies: a round-robin share of the sweep (frequencies are
    independent units; no data-path collective)."""
    return list(np.asarray(omegas)[rank::world])


def pick_timed(my, steps, warmup):
    """The timed frequencies sample this rank's share evenly over the sweep (the
    plane-wave angle count, and so the work, grows with frequency); warm-up
    frequencies are drawn from the same share."""
    n_my = len(my)
    timed = [my[(i * n_my) // max(1, steps) + (n_my // max(1, steps)) // 2] if steps <= n_my
             else my[i % n_my] for i in range(steps)]
    warm = [my[(7 * i + 3) % n_my] for i in range(warmup)]
    return timed, warm


def timed_sweep(solve, my, steps, dist, world):
    """Times `steps` frequency-solves of this rank's share between barriers.
    solve(omegas) -> (device_ms, result) runs them and reports their device span.
    The whole-job rate divides the frequency-solves of all ranks by the slowest
    rank's time (max over ranks of device time and of wall time)."""
    timed, _ = pick_timed(my, steps, 0)
    barrier(dist)
    t0 = time.perf_counter()
    dev_ms, res = solve(timed)
    wall = time.perf_counter() - t0
    barrier(dist)
    dev_ms_max = allmax(dist, dev_ms)
    wall_max = allmax(dist, wall)
    total = steps * world
    return {"timed": timed, "result": res, "dev_ms": dev_ms, "dev_ms_max": dev_ms_max, "wall_max": wall_max,
            "value": total / (dev_ms_max / 1000.0), "e2e": total / wall_max}


def build_mesh(bg, na):
    cyl = bg.Half_Cylinder(6.0, 20.0, na, 8, 24, 0, False)
    return bg.unify([cyl] * 4, ORIGINS)


def oracle_frequency_solve(na, omega):
    """One full frequency-solve of the four-column array by the FP64 oracle (the CPU
    restatement of the reference's path) on all host cores, unscaled: wave assembly of
    every row and compose (OpenMP over source columns, as the reference), complex LU
    with partial pivoting at n = N, the 9 right-hand sides, solves and post.  The
    frequency-independent Rankine setup is timed apart and not counted, as on the GPU.
    Returns the oracle's results at omega and the cpu_baseline record."""
    from oracle.oracle import Oracle, Mesh as OMesh
    orc = Oracle()
    cyl, _ = orc.cylinder(6.0, 20.0, na, 8, 24, cosine=False)
    mesh = OMesh.concat([cyl] * 4, ORIGINS)
    res, clk = orc.solve_timed(mesh, [omega], BETAS)
    wave, lu, rest = float(clk["wave"][0]), float(clk["lu"][0]), float(clk["rest"][0])
    per = wave + lu + rest
    info = {"value": 1.0 / per, "unit": "freq-solves/s", "cores": orc.num_threads(), "kind": "port",
            "sample": "one unscaled frequency-solve of the %d-panel array at Omega = %.4f rad/s by the oracle port "
                      "(wave assembly + compose %.1f s, partial-pivot complex LU at n = %d %.1f s, right-hand sides, "
                      "solves and post %.1f s); the Rankine setup (%.1f s, frequency-independent) not counted"
                      % (mesh.n, omega, wave, mesh.n, lu, rest, clk["setup"]),
            "seconds_per_solve": per, "stage_s": {"wave": wave, "lu": lu, "rest": rest, "setup": clk["setup"]},
            "omega": float(omega)}
    return res, info


def run_reference(args, world, rank, dist):
    """The reference arm: the reference's CPU path (its oracle port, kind "port") on the
    host cores, on this arm's workload.  Each warm-up step is a small frequency-solve
    (it starts the OpenMP pool and pages the library in); the timed part is one unscaled
    frequency-solve of the full array at the highest timed frequency.  Further steps
    would repeat the same work: the line reports that one measured solve per step."""
    if rank != 0:
        return
    from oracle.oracle import Oracle, Mesh as OMesh
    orc = Oracle()
    small, _ = orc.cylinder(6.0, 20.0, 16, 2, 6, cosine=False)
    for _ in range(args.warmup):
        orc.solve(small, [1.0], BETAS)
    timed, _ = pick_timed(shard(OMEGAS, 0, 1), args.steps, 0)
    _, info = oracle_frequency_solve(args.na, timed[-1])
    v = info["value"]
    info["sample"] += "; 1 of %d steps measured, the rest taken equal" % args.steps
    line = {"metric": METRIC, "impl": "reference", "value": v, "unit": "freq-solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "timed_steps": 1, "warmup": args.warmup, "ms_per_step": 1000.0 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "four-cylinder array, %d panels, 100 freqs 0.05-3.0 rad/s, 3 headings"
                                   % (4 * args.na * 32)},
            "cpu_baseline": {k: info[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "stage_s": info["stage_s"],
            "e2e": {"value": v, "unit": "freq-solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def tf32_peak_tflops(device, n=8192):
    """cuBLAS TF32 GEMM throughput (torch.matmul on FP32 with TF32 allowed, n^3, best
    of 5 with CUDA events): the roofline denominator of the tensor-core LU."""
    import torch
    dev = torch.device("cuda", device)
    torch.backends.cuda.matmul.allow_tf32 = True
    a = torch.randn(n, n, device=dev)
    b = torch.randn(n, n, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize(dev)
    best = float("inf")
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize(dev)
        best = min(best, e0.elapsed_time(e1))
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def batched_bodies(bg, n_bodies=64, seed=0):
    """Seeded set of independent bodies: truncated cylinders (radius U[3,15], draft
    U[5,30]) or boxes (length, beam U[5,40], draft U[5,30]) at even odds, target
    panel count U{400..6000} met as closely as the panel grid allows (numpy PCG64)."""
    rng = np.random.default_rng(seed)
    bodies = []
    for _ in range(n_bodies):
        target = int(rng.integers(400, 6001))
        if rng.random() < 0.5:
            R, draft = rng.uniform(3, 15), rng.uniform(5, 30)
            side = np.sqrt((2 * np.pi * R * draft + np.pi * R * R) / target)
            NA = max(8, int(round(2 * np.pi * R / side)))
            NR = max(2, int(round(R / side)))
            NV = max(2, int(round(target / NA)) - NR)
            bodies.append(("cylinder", (R, draft, NA, NR, NV), bg.Half_Cylinder(R, draft, NA, NR, NV, 0, False)))
        else:
            L, B, D = rng.uniform(5, 40), rng.uniform(5, 40), rng.uniform(5, 30)
            side = np.sqrt((L * B + 2 * (L + B) * D) / target)
            NX, NY, NZ = (max(2, int(round(v / side))) for v in (L, B, D))
            bodies.append(("box", (L, B, D, NX, NY, NZ), bg.Barge(L, B, D, NX, NY, NZ, True)))
    return bodies


def batched_report(bg, n_workers=8):
    """Batched form: 64 seeded bodies, 30 frequencies log-spaced on 0.1-2.5 rad/s,
    heading 0, mixed precision, n_workers concurrent body pipelines (bem_batch_solve)."""
    bodies = batched_bodies(bg)
    meshes = [b[2] for b in bodies]
    om = np.logspace(np.log10(0.1), np.log10(2.5), 30)
    outs, sec = bg.batch_solve(meshes[:4], om[:2], [0.0], bg.MIXED, n_workers=4)  # warm-up
    outs, sec = bg.batch_solve(meshes, om, [0.0], bg.MIXED, n_workers=n_workers)
    panels = [m.n for m in meshes]
    iters = np.concatenate([o["iters"] for o in outs])
    return {"workload": "64 seeded bodies (cylinders/boxes), 30 freqs log-spaced 0.1-2.5 rad/s, heading 0",
            "seed": 0, "panels_min": int(min(panels)), "panels_max": int(max(panels)),
            "panels_total": int(sum(panels)), "workers": n_workers, "wall_s": sec,
            "freq_solves_per_s": len(meshes) * om.size / sec, "refine_sweeps_max": int(iters.max()),
            "note": "wall time of one bem_batch_solve call (setup of each body included)"}


def steady_report(bg, with_oracle, reps=3):
    """Steady lifting flow: NACA 0012 wing (chord 1, span 8, 120 x 60 = 7,200 panels) at
    alpha = 5 deg, flat wake of 60 strips 20 chords long carrying the Kutta jumps; setup
    (Rankine G and H on the GPU, wake dipoles folded into H), solve in both precisions,
    surface pressure and CL on the host.  Wall times (the calls are synchronous), median of
    reps after one warm-up."""
    c, span, nc, ns = 1.0, 8.0, 120, 60
    w = bg.NACA_Wing(c, span, 0.12, nc, ns)
    wake = bg.NACA_Wing_Wake(c, span, nc, ns, 20.0)
    a = np.radians(5.0)
    U = np.array([np.cos(a), 0.0, np.sin(a)])
    out = {"workload": "NACA 0012 wing 7200 panels, 60 wake strips x 20 chords, alpha 5 deg", "panels": w.n}
    sol = {}
    for name, prec in (("mixed", bg.MIXED), ("plain_fp64", bg.PLAIN_FP64)):
        sv = bg.Aerodynamic_Solver(precision=prec)
        sv.Set_Wake(*wake)
        ts, tv, tp = [], [], []
        for r in range(reps + 1):
            t0 = time.perf_counter()
            sv.Setup(w)
            t1 = time.perf_counter()
            sv.Set_External_BC([U])
            X = sv.Solve_Steady()
            t2 = time.perf_counter()
            cp, co = sv.Surface(U, c * span)
            t3 = time.perf_counter()
            if r:
                ts.append(t1 - t0); tv.append(t2 - t1); tp.append(t3 - t2)
        sol[name] = X
        out[name] = {"setup_ms": 1e3 * float(np.median(ts)), "solve_ms": 1e3 * float(np.median(tv)),
                     "surface_ms": 1e3 * float(np.median(tp)), "CL": co["CL"], "CD": co["CD"],
                     "cp_min": float(cp.min())}
    out["lifting_line_CL"] = 2 * np.pi * a / (1 + 2 / (span / c))
    if with_oracle:
        from oracle.oracle import Oracle, Mesh as OMesh
        from oracle import aero_post
        orc = Oracle()
        om = OMesh(w.nodes, w.elems)
        t0 = time.perf_counter()
        Xo, _ = orc.aero_wake(om, *wake, U)
        t1 = time.perf_counter()
        cpo, CF, CL, CD = aero_post.surface(orc.panels(om), w.elems, Xo, U, c * span)
        out["oracle"] = {"solve_s": t1 - t0, "threads": orc.num_threads(), "CL": CL, "CD": CD,
                         "note": "setup and solve of the oracle port (FP64, OpenMP) on the host cores"}
        out["accuracy_vs_oracle"] = {k: normwise(sol[k], Xo) for k in sol}
        out["accuracy_vs_oracle"]["CL_abs_err_mixed"] = abs(out["mixed"]["CL"] - CL)
    return out


def surrogate_report(bg, solver, timed, budget_s, results, oref, hi):
    """The learned form of the metric, measured: the surrogate network (2 -> 128 x 4 -> 6,
    SiLU, BF16 weights, FP32 accumulation) trained by the library's own kernels on 2^22
    samples of the plain FP64 integrator in its domain for a bounded time, then fused into
    the mixed assembly (tensor-core forward) and run on the same timed frequencies in the
    two modes of bem_set_surrogate: "accept" keeps the network's far-field values, "strict"
    solves a frequency again with the closed form when the judged error (1 % of the far
    pairs, checked against the closed form) exceeds 1e-6.  Rates are device time of the
    whole call, as for the headline."""
    t0 = time.perf_counter()
    HS = bg.HavelockSurrogate
    x, y, t = HS.domain_set(1 << 22, seed=0)
    xv, yv, tv = HS.domain_set(1 << 16, seed=1)
    sur = HS(seed=0)
    sur.set_domain_normalization(t)
    t1 = time.perf_counter()
    epochs, losses = 0, []
    while time.perf_counter() - t1 < budget_s and epochs < 200:
        frac = (time.perf_counter() - t1) / budget_s
        lr = 2e-3 * 0.5 * (1.0 + np.cos(np.pi * min(frac, 1.0))) + 1e-5
        losses += list(sur.train(x, t, epochs=1, batch=4096, lr=lr, seed=epochs))
        epochs += 1
    train_s = time.perf_counter() - t1
    pred = sur.predict(xv)
    env = HS.envelope(10.0 ** xv[:, 0], xv[:, 1])
    rel_env = np.abs(pred - yv) / env
    rep = {"network": "2-128x4-6 SiLU, BF16 weights and activations, FP32 accumulation (tcgen05 kind::f16, TMEM)",
           "domain": {"KR": list(HS.KR_RANGE), "KZ": list(HS.KZ_RANGE), "near_field_panel_diameters": 3.0},
           "train_samples": int(x.shape[0]), "epochs": epochs, "train_s": train_s,
           "data_s": t1 - t0, "final_loss": float(losses[-1]) if losses else None,
           "validation": {"median_err_over_envelope": [float(v) for v in np.median(rel_env, axis=0)],
                          "max_err_over_envelope": [float(v) for v in rel_env.max(axis=0)],
                          "max_err_over_max_target": [float(v) for v in
                                                      np.max(np.abs(pred - yv), axis=0) / np.max(np.abs(yv), axis=0)]},
           "evals_per_s_tensor_core_network": sur.throughput_tc(1 << 22),
           "evals_per_s_fp32_closed_form": bg.havelock_throughput(1 << 22, bg.MIXED)}
    rep["network_slowdown"] = rep["evals_per_s_fp32_closed_form"] / rep["evals_per_s_tensor_core_network"]
    legs = {}
    for mode in ("accept", "strict"):
        solver.set_surrogate(sur, mode=mode, judge_tol=1e-6, judge_fraction=0.01)
        solver.solve_omegas(timed[:2])  # warm-up
        solver.surrogate_stats(reset=True)
        solver.kernel_times(reset=True)
        w0 = time.perf_counter()
        r = solver.solve_omegas(timed)
        wall = time.perf_counter() - w0
        kt = solver.kernel_times(reset=True)
        st = solver.surrogate_stats(reset=True)
        n = len(timed)
        keys = ("A", "B", "F")
        legs[mode] = {"value": n / (kt[3] / 1000.0), "unit": "freq-solves/s", "ms_per_step": kt[3] / n,
                      "e2e": n / wall,
                      "accuracy_vs_oracle": {k: normwise(r[k][hi], oref[k][0]) for k in keys} if oref else None,
                      "accuracy_vs_closed_form_mixed": {
                          k: max(normwise(r[k][i], results[i][k][0]) for i in range(n)) for k in keys},
                      "network_share_of_gauss_points": st["gauss_points_network"] / max(
                          1, st["gauss_points_network"] + st["gauss_points_closed_form"]),
                      "judged_pairs": st["judged_pairs"], "judged_error_max": st["judged_error_max"],
                      "frequencies_resolved_with_closed_form": st["frequencies_resolved"],
                      "refine_sweeps_max": int(np.max(r["iters"]))}
    solver.set_surrogate(None, mode=None)
    rep["mixed_plus_surrogate"] = legs
    rep["omega_of_oracle_check"] = float(timed[hi])
    rep["used_in_headline"] = False
    rep["headline_note"] = ("measured, not composed; the headline is the closed-form mixed path, which meets "
                            "the accuracy target and is faster: the network is slower than the closed form it "
                            "replaces, and its BF16 error, once in the operator, moves A/B far beyond 1e-6 "
                            "(accept), so strict mode falls back to the closed form")
    return rep


def normwise(a, b):
    d = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (d if d > 0 else 1.0))


def main():
    args = parse()
    world, rank, local, dist = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
        return
    import bemuse_gb300 as bg
    bg.build.build()
    mesh = build_mesh(bg, args.na)
    N = mesh.n
    s = bg.Hydrodynamic_Radiation_Solver(device=local, precision=bg.MIXED)
    s.Set_Parameters([bg.Parameter("WaveAngle", b) for b in BETAS])
    t0 = time.perf_counter()
    s.Setup(mesh)
    setup_s = time.perf_counter() - t0
    my = shard(OMEGAS, rank, world)
    n_my = len(my)
    timed, warm = pick_timed(my, args.steps, args.warmup)
    tune = None
    if args.autotune and n_my >= 2:
        t0 = time.perf_counter()
        sample = [my[(i * n_my) // 8 + n_my // 16] for i in range(8)] if n_my >= 8 else list(my)
        tune_ms, tune_rep = s.autotune(sample)
        tune = {"ms_per_freq": tune_ms, "sample_omegas": len(sample), "settings": tune_rep,
                "wall_s": time.perf_counter() - t0}
    if args.warmup > 0:
        s.solve_omegas(warm)
    s.stage_times(reset=True)
    s.kernel_times(reset=True)
    launches0 = bg.launch_count()
    kt_box = {}

    def solve(oms):
        # the timed steps: one call with this rank's K frequencies (the library pipelines the
        # assembly of frequency f+1 with the factorization and refinement of frequency f)
        r = s.solve_omegas(oms)
        kt_box["kt"] = s.kernel_times(reset=True)
        return float(kt_box["kt"][3]), r  # device span: first assembly start -> last result copy

    with Clocks(local) as clk:
        tr = timed_sweep(solve, my, args.steps, dist, world)
    launches = bg.launch_count() - launches0
    st = s.stage_times(reset=True)
    kt_timed = kt_box["kt"]
    res, dev_ms_max, value, e2e = tr["result"], tr["dev_ms_max"], tr["value"], tr["e2e"]
    KEYS = ("A", "B", "F", "FK", "SC")
    results = [{k: res[k][i:i + 1] for k in KEYS} for i in range(len(timed))]
    iters = [int(x) for x in res["iters"]]
    # LU and assembly alone (one frequency, nothing overlapping: the tensor-core roofline,
    # and k_wave_mixed on the whole GPU beside the pipelined figure)
    s.stage_times(reset=True)
    s.kernel_times(reset=True)
    s.solve_omegas([timed[-1]])
    lu_alone_ms = float(s.stage_times(reset=True)[2])
    kt_alone = s.kernel_times(reset=True)
    # plain FP64 GPU path at frequencies spread over the timed ones (highest and lowest
    # first); the mixed results are compared with it
    pick = []
    if args.plain_steps > 0 and args.steps > 0:
        cand = [args.steps - 1, 0] + [(i * args.steps) // max(1, args.plain_steps) for i in range(args.plain_steps)]
        for c in cand:
            if c not in pick and len(pick) < min(args.plain_steps, args.steps):
                pick.append(c)
    plain_om = [timed[i] for i in pick]
    sp = bg.Hydrodynamic_Radiation_Solver(device=local, precision=bg.PLAIN_FP64)
    sp.Set_Parameters([bg.Parameter("WaveAngle", b) for b in BETAS])
    if plain_om:
        sp.Setup(mesh)
    sp.stage_times(reset=True)
    err_plain = {k: 0.0 for k in KEYS}
    plain_res = {}
    t0 = time.perf_counter()
    for i, om in enumerate(plain_om):
        rp = sp.solve_omegas([om])
        plain_res[pick[i]] = rp
        for k in KEYS:
            err_plain[k] = max(err_plain[k], normwise(results[pick[i]][k][0], rp[k][0]))
    plain_wall = time.perf_counter() - t0
    stp = sp.stage_times(reset=True)
    plain_ms = float(np.sum(stp[:5])) / max(1, len(plain_om))
    plain_value = 1000.0 / plain_ms if plain_om else float("nan")
    names = ["incident+static rhs", "wave assembly", "lu factor", "solve+refine", "post"]
    per = st[:5] / args.steps
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    Np = (N + 127) // 128 * 128
    kt = kt_timed
    wk_ms = kt[0] / max(1.0, kt[1])
    ntri = 4 * args.na
    evals = float(N) * (4.0 * (N - ntri) + 3.0 * ntri)  # Green-function evaluations per launch
    fp32_peak = bg.fp32_peak(local)
    # roofline of the dominant kernel, k_wave_mixed (CUDA events on its stream around each
    # launch): FP32-pipe bound at 345 FP operations per Green-function evaluation (a hand
    # count of HavelockGF and the wave-kernel scaling, special functions excluded),
    # against the measured FP32 FMA rate; the HBM view uses 16 N^2 bytes per launch (one
    # complex FP64 operator's worth of output).
    roof = {"kernel": "k_wave_mixed (wave-influence assembly)", "bound": "fp32",
            "achieved": 345.0 * evals / (wk_ms / 1000.0) / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
            "peak_source": "measured: FP32 FMA loop timed with CUDA events (bem_fp32_peak); not in MEASURED_PEAKS.json",
            "ops_per_eval": 345, "evals_per_launch": evals, "avg_launch_ms": wk_ms, "launches": int(kt[1]),
            "green_evals_per_s": evals / (wk_ms / 1000.0),
            "traffic": 32.0 * N * N * (480.9e6 / (32.0 * 4096 * 4096)),
            "traffic_source": "ncu dram__bytes_read+write of one 4096-panel launch (270.7 MB + 210.2 MB), scaled by "
                              "N^2 (the pair count)",
            "hbm": {"bytes_per_launch": 16.0 * N * N, "achieved_gbs": 16.0 * N * N / (wk_ms / 1000.0) / 1e9,
                    "peak_gbs": hbm_peak, "peak_source": "measured, MEASURED_PEAKS.json"}}
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["hbm"]["frac"] = roof["hbm"]["achieved_gbs"] / hbm_peak
    if kt_alone[1] > 0:
        a_ms = float(kt_alone[0] / kt_alone[1])
        a_tf = 345.0 * evals / (a_ms / 1000.0) / 1e12
        roof["alone"] = {"avg_launch_ms": a_ms, "achieved": a_tf, "frac": a_tf / roof["peak"],
                         "note": "one frequency solved alone after the timed steps: the assembly on the whole "
                                 "GPU; the timed launches keep off the SMs reserved for the LUs and refinement"}
    if rank != 0:
        return
    honesty = {}
    try:
        honesty["tf32_peak_tflops"] = tf32_peak_tflops(local)
        honesty["cusolver_zgetrf_ms"] = bg.cusolver_zgetrf_ms(Np, local)
    except Exception as exc:  # torch or cuSOLVER unavailable: report why
        honesty["unavailable"] = str(exc)[:200]
    F_lu = 8.0 / 3.0 * float(Np) ** 3
    lu = {"flops": F_lu, "ms_alone": lu_alone_ms, "ms_pipelined": float(per[2]),
          "tflops_alone": F_lu / (lu_alone_ms * 1e-3) / 1e12, "tflops_pipelined": F_lu / (per[2] * 1e-3) / 1e12,
          "plain_fp64_lu_ms": float(stp[2]) / max(1, len(plain_om))}
    if "tf32_peak_tflops" in honesty:
        lu["peak_tf32_tflops"] = honesty["tf32_peak_tflops"]
        lu["peak_source"] = "measured: cuBLAS TF32 GEMM 8192^3 (torch.matmul, CUDA events)"
        lu["frac_alone"] = lu["tflops_alone"] / lu["peak_tf32_tflops"]
        lu["frac_pipelined"] = lu["tflops_pipelined"] / lu["peak_tf32_tflops"]
    if "cusolver_zgetrf_ms" in honesty:
        honesty["plain_fp64_lu_ms"] = lu["plain_fp64_lu_ms"]
        honesty["note"] = ("cuSOLVER zgetrf (FP64 complex, partial pivoting) at n = %d beside this library's plain "
                           "FP64 LU (no row exchanges) at the same order" % N)
    # the measured CPU baseline: one unscaled frequency-solve by the oracle port at the highest
    # timed frequency, which also pins the GPU results at benchmark size
    hi = len(timed) - 1
    oref, cpu, acc = None, None, None
    if args.cpu_baseline:
        oref, cpu = oracle_frequency_solve(args.na, timed[hi])
        cpu.pop("seconds_per_solve", None)
        acc = {"omega": float(timed[hi]), "metric": "max|x-ref|/max|ref| per 6x6 (or 6 x NB) block, FP64 oracle",
               "mixed": {k: normwise(results[hi][k][0], oref[k][0]) for k in KEYS}}
        if hi in plain_res:
            acc["plain_fp64"] = {k: normwise(plain_res[hi][k][0], oref[k][0]) for k in KEYS}
        # F = conj(FK + SC): where F is small beside FK (the two nearly cancel) its relative
        # error grows; the same errors against the size of the incident-wave force
        fk = float(np.max(np.abs(oref["FK"][0])))
        if fk > 0:
            acc["vs_max_FK"] = {
                "metric": "max|x-ref| / max|FK_ref| in the 6 x NB block",
                "F": float(np.max(np.abs(results[hi]["F"][0] - oref["F"][0]))) / fk,
                "SC": float(np.max(np.abs(results[hi]["SC"][0] - oref["SC"][0]))) / fk,
                "max_F_over_max_FK": float(np.max(np.abs(oref["F"][0]))) / fk,
                "max_SC_over_max_FK": float(np.max(np.abs(oref["SC"][0]))) / fk}
    batched = batched_report(bg) if args.batched else None
    sur = None
    if args.surrogate_seconds > 0:
        sur = surrogate_report(bg, s, timed, args.surrogate_seconds, results, oref, hi)
    steady = steady_report(bg, args.cpu_baseline) if args.steady else None
    h2d = 8 + 6 * N * 8
    d2h = (36 + 12 * len(BETAS)) * 16 + int(np.mean(iters)) * (2 * 9 * 8) + 4
    line = {"metric": METRIC, "value": value, "unit": "freq-solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+tf32+f64", "data": "synthetic",
            "config": {"workload": "four-cylinder array, %d panels, 100 freqs 0.05-3.0 rad/s, 3 headings, mixed "
                                   "precision (FP32 assembly, TF32 LU, FP64 refinement to 1e-12)" % N,
                       "panels": N, "rhs": 9, "l2": "inputs larger than L2 (Rankine matrices 3 x %.0f MB)"
                       % (8.0 * N * Np / 1e6), "parallelism": "frequencies sharded over ranks"},
            "e2e": {"value": e2e, "unit": "freq-solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches),
            "roofline": roof,
            "lu_roofline": lu,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "accuracy_vs_oracle": acc,
            "plain_fp64": {"value": plain_value, "unit": "freq-solves/s", "steps": len(plain_om),
                           "ms_per_step": plain_ms, "wall_s": plain_wall,
                           "stage_ms": [float(x) / max(1, len(plain_om)) for x in stp[:5]]},
            "speedup_vs_plain_fp64": value / plain_value,
            "accuracy_vs_plain_fp64": dict(err_plain, metric="max|x-ref|/max|ref| per 6x6 (or 6 x NB) block"),
            "plain_lu_vs_cusolver": honesty,
            "refine_sweeps": iters,
            "surrogate": sur,
            "batched": batched,
            "steady": steady,
            "stage_ms": dict(zip(names, [float(x) for x in per])),
            "stage_ms_note": "per frequency; assembly of f+1 overlaps factor+solve of f, so stages sum to more than ms_per_step",
            "setup_s": setup_s,
            "autotune": tune}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
