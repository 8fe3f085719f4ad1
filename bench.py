"""Benchmark: frequency-solves/s of the panel-method hot path on GB300.

Workload (default): the four-column array -- four truncated cylinders, radius
6 m, draft 20 m, 64 azimuthal x (8 bottom + 24 side) panels each (2048 panels,
8192 in total), centred at (+-25, +-25, 0) m; infinite depth; 100 frequencies
uniform on 0.05-3.0 rad/s; headings 0/45/90 deg (6 radiation + 3 diffraction
right-hand sides).  Synthetic by construction (generated mesh, no dataset).

One step = one frequency-solve in the mixed-precision mode: wave assembly
(FP32 real parts, FP64-accurate imaginary parts), TF32 tensor-core LU, FP64
iterative refinement to 1e-12 relative residual, hull integrals.  The plain
FP64 GPU path is timed on `--plain-steps` of the same frequencies and the
mixed results are compared with it (A, B normwise).

  value  = freq-solves/s from device time (CUDA events on the library stream)
  e2e    = freq-solves/s of wall time around bem_solve (host in, host out)
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
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--plain-steps", type=int, default=2)
    p.add_argument("--na", type=int, default=64, help="azimuthal panels per cylinder (64 -> 8192 panels)")
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU baseline sample")
    p.add_argument("--batched", type=int, default=1, help="1: also run the 64-body batched form")
    p.add_argument("--autotune", type=int, default=1,
                   help="1: time a small grid of schedule settings on 8 sample frequencies before the "
                        "warm-up (outside the timed region) and keep the fastest")
    p.add_argument("--surrogate-seconds", type=float, default=20.0,
                   help="training budget of the Green-function surrogate report (0 skips it)")
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


def build_mesh(bg, na):
    cyl = bg.Half_Cylinder(6.0, 20.0, na, 8, 24, 0, False)
    return bg.unify([cyl] * 4, ORIGINS)


def cpu_baseline(na, budget_s):
    """The FP64 oracle (CPU restatement of the reference path) on the host cores,
    on a bounded sample of one frequency-solve: wave assembly of a block of
    rows and a dense complex LU + solve of a smaller order, each scaled to the
    full workload by its operation count (rows x N x Q, and n^3)."""
    from oracle.oracle import Oracle, Mesh as OMesh
    orc = Oracle()
    cyl, _ = orc.cylinder(6.0, 20.0, na, 8, 24, cosine=False)
    mesh = OMesh.concat([cyl] * 4, ORIGINS)
    N = mesh.n
    K = OMEGAS[50] ** 2 / 9.81
    rows = 16
    t0 = time.perf_counter()
    orc.wave_rows(mesh, K, 0, rows)
    t_rows = time.perf_counter() - t0
    while t_rows < 0.25 * budget_s and rows < N // 4:
        rows *= 2
        t0 = time.perf_counter()
        orc.wave_rows(mesh, K, 0, rows)
        t_rows = time.perf_counter() - t0
    t_asm = t_rows * N / rows
    n = 512
    rng = np.random.default_rng(0)
    t_lu = 0.0
    while True:
        A = 0.5 * np.eye(n) + (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * (0.2 / np.sqrt(n))
        B = rng.standard_normal((n, 9)) + 0j
        t0 = time.perf_counter()
        orc.lu_solve(A, B)
        t_lu = time.perf_counter() - t0
        if t_lu > 0.25 * budget_s or n >= 4096:
            break
        n *= 2
    t_lu_full = t_lu * (N / n) ** 3
    per_solve = t_asm + t_lu_full
    return {"value": 1.0 / per_solve, "unit": "freq-solves/s", "cores": orc.num_threads(), "kind": "port",
            "sample": "oracle wave assembly of %d of %d rows (scaled x%.0f) + oracle complex LU/solve at n=%d "
                      "(scaled x%.0f by n^3); %.2f s + %.2f s per freq-solve" % (rows, N, N / rows, n, (N / n) ** 3,
                                                                                 t_asm, t_lu_full),
            "seconds_per_solve": per_solve}


def run_reference(args, world, rank, dist):
    if rank != 0:
        return
    steps = []
    for _ in range(args.warmup):
        pass
    info = None
    for _ in range(max(1, args.steps)):
        info = cpu_baseline(args.na, args.cpu_seconds / max(1, args.steps))
        steps.append(info["seconds_per_solve"])
    v = 1.0 / float(np.mean(steps))
    line = {"metric": METRIC, "impl": "reference", "value": v, "unit": "freq-solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "four-cylinder array, %d panels, 100 freqs 0.05-3.0 rad/s, 3 headings"
                                   % (4 * args.na * 32)},
            "cpu_baseline": {"value": v, "unit": "freq-solves/s", "cores": info["cores"], "kind": "port",
                             "sample": info["sample"]},
            "e2e": {"value": v, "unit": "freq-solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


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


def surrogate_report(bg, budget_s, ms_per_solve, wave_kernel_ms, evals_per_solve):
    """The MLP stand-in for HavelockGF (2 -> 128 x 4 -> 6, SiLU, BF16 weights / FP32
    accumulation): trained on 2^22 samples of the plain FP64 integrator for a bounded
    time, then measured against the FP32 closed form it would replace.  The
    mixed+surrogate rate is composed from measured parts: the mixed frequency-solve
    with its wave-kernel time replaced by the same number of surrogate evaluations."""
    t0 = time.perf_counter()
    x, y = bg.HavelockSurrogate.training_set(1 << 22, seed=0)
    xv, yv = bg.HavelockSurrogate.training_set(1 << 14, seed=1)
    s = bg.HavelockSurrogate(seed=0)
    s.set_normalization(x.mean(0), x.std(0), y.mean(0), y.std(0) + 1e-12)
    lr, epochs, losses = 1e-3, 0, []
    while time.perf_counter() - t0 < budget_s and epochs < 40:
        losses += list(s.train(x, y, epochs=1, batch=8192, lr=lr, seed=epochs))
        epochs += 1
        if epochs % 8 == 0:
            lr *= 0.5
    pred = s.eval(xv)
    err = np.max(np.abs(pred - yv), axis=0) / np.max(np.abs(yv), axis=0)
    far = xv[:, 0] > 0.0  # KR > 1
    err_far = np.max(np.abs(pred[far] - yv[far]), axis=0) / np.max(np.abs(yv[far]), axis=0)
    mlp_rate = s.throughput(1 << 20)
    closed_rate = bg.havelock_throughput(1 << 22, bg.MIXED)
    mlp_wave_ms = evals_per_solve / mlp_rate * 1000.0
    ms_sur = ms_per_solve - wave_kernel_ms + mlp_wave_ms
    return {"network": "2-128x4-6 SiLU, BF16 weights, FP32 accumulate", "train_samples": int(x.shape[0]),
            "epochs": epochs, "train_s": time.perf_counter() - t0, "final_loss": float(losses[-1]) if losses else None,
            "max_err_over_max_target": [float(v) for v in err],
            "max_err_over_max_target_KR_gt_1": [float(v) for v in err_far],
            "evals_per_s_surrogate": mlp_rate, "evals_per_s_fp32_closed_form": closed_rate,
            "surrogate_slowdown": closed_rate / mlp_rate,
            "mixed_plus_surrogate_freq_solves_per_s": 1000.0 / ms_sur,
            "mixed_plus_surrogate_note": "composed: measured mixed frequency-solve minus its measured wave-kernel "
                                         "time plus %.3g surrogate evaluations at the measured surrogate rate; the "
                                         "headline value uses the closed form" % evals_per_solve,
            "used_in_headline": False}


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
    my = OMEGAS[rank::world]
    # timed steps sample this rank's frequencies evenly over the whole sweep (the
    # plane-wave angle count, and so the work, grows with frequency)
    n_my = len(my)
    timed = [my[(i * n_my) // max(1, args.steps) + (n_my // max(1, args.steps)) // 2] if args.steps <= n_my
             else my[i % n_my] for i in range(args.steps)]
    warm = [my[(7 * i + 3) % n_my] for i in range(args.warmup)]
    seq = warm + timed
    tune = None
    if args.autotune and n_my >= 2:
        t0 = time.perf_counter()
        sample = [my[(i * n_my) // 8 + n_my // 16] for i in range(8)] if n_my >= 8 else list(my)
        tune_ms, tune_rep = s.autotune(sample)
        tune = {"ms_per_freq": tune_ms, "sample_omegas": len(sample), "settings": tune_rep,
                "wall_s": time.perf_counter() - t0}
    if args.warmup > 0:
        s.solve_omegas(seq[:args.warmup])
    s.stage_times(reset=True)
    s.kernel_times(reset=True)
    launches0 = bg.launch_count()
    barrier(dist)
    # the timed steps: one call with this rank's K frequencies (the library pipelines the
    # assembly of frequency f+1 with the factorization and refinement of frequency f)
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        res = s.solve_omegas(timed)
        wall = time.perf_counter() - t0
    barrier(dist)
    launches = bg.launch_count() - launches0
    st = s.stage_times(reset=True)
    kt_timed = s.kernel_times(reset=True)
    dev_ms = float(kt_timed[3])  # device span of the call (events: first assembly start -> last result copy)
    dev_ms_max = allmax(dist, dev_ms)
    wall_max = allmax(dist, wall)
    total = args.steps * world
    value = total / (dev_ms_max / 1000.0)
    e2e = total / wall_max
    results = [{k: res[k][i:i + 1] for k in ("A", "B", "F")} for i in range(len(timed))]
    iters = [int(x) for x in res["iters"]]
    # plain FP64 GPU path on the first frequencies of this rank, and accuracy of mixed vs plain
    # plain FP64 reference at frequencies spread over the timed ones (lowest and highest first)
    pick = []
    if args.plain_steps > 0 and args.steps > 0:
        cand = [0, args.steps - 1] + [(i * args.steps) // max(1, args.plain_steps) for i in range(args.plain_steps)]
        for c in cand:
            if c not in pick and len(pick) < min(args.plain_steps, args.steps):
                pick.append(c)
    plain_om = [timed[i] for i in pick]
    sp = bg.Hydrodynamic_Radiation_Solver(device=local, precision=bg.PLAIN_FP64)
    sp.Set_Parameters([bg.Parameter("WaveAngle", b) for b in BETAS])
    if plain_om:
        sp.Setup(mesh)
    sp.stage_times(reset=True)
    errA, errB, errF = 0.0, 0.0, 0.0
    t0 = time.perf_counter()
    for i, om in enumerate(plain_om):
        rp = sp.solve_omegas([om])
        rm = results[pick[i]]
        errA = max(errA, normwise(rm["A"][0], rp["A"][0]))
        errB = max(errB, normwise(rm["B"][0], rp["B"][0]))
        errF = max(errF, normwise(rm["F"][0], rp["F"][0]))
    plain_wall = time.perf_counter() - t0
    stp = sp.stage_times(reset=True)
    plain_ms = float(np.sum(stp[:5])) / max(1, len(plain_om))
    plain_value = 1000.0 / plain_ms if plain_om else float("nan")
    # roofline of the dominant kernel, k_wave_mixed (largest single-kernel share of the
    # launch list): CUDA events on the solve stream around each of its launches.
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
    # algorithmic bytes per launch: per panel pair it reads RD, RSR as float pairs (16 B)
    # and writes Re D as a float pair plus the FP32 copy (Re, Im) for the LU (16 B)
    wk_bytes = 32.0 * N * N
    ntri = 4 * args.na
    evals = float(N) * (4.0 * (N - ntri) + 3.0 * ntri)
    roof = {"kernel": "k_wave_mixed (wave-influence assembly)", "bound": "hbm",
            "achieved": wk_bytes / (wk_ms / 1000.0) / 1e9, "peak": hbm_peak, "unit": "GB/s",
            "traffic": 32.0 * N * N * (499.0e6 / (32.0 * 4096 * 4096)),
            "traffic_source": "ncu dram__bytes_read+write of the 4096-panel launch (271 MB + 228 MB for 537 MB "
                              "algorithmic; part of the writes still in L2 at exit), scaled by N^2", "avg_launch_ms": wk_ms, "launches": int(kt[1]),
            "green_evals_per_s": evals / (wk_ms / 1000.0),
            "note": "bound in practice by the FP32/SFU pipes (special functions per Gauss point), not HBM",
            "peak_source": "measured, MEASURED_PEAKS.json"}
    roof["frac"] = roof["achieved"] / roof["peak"]
    if rank != 0:
        return
    cpu = cpu_baseline(args.na, args.cpu_seconds)
    cpu.pop("seconds_per_solve", None)
    batched = batched_report(bg) if args.batched else None
    sur = None
    if args.surrogate_seconds > 0:
        sur = surrogate_report(bg, args.surrogate_seconds, dev_ms_max / args.steps, wk_ms, evals)
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
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "plain_fp64": {"value": plain_value, "unit": "freq-solves/s", "steps": len(plain_om),
                           "ms_per_step": plain_ms, "wall_s": plain_wall,
                           "stage_ms": [float(x) / max(1, len(plain_om)) for x in stp[:5]]},
            "speedup_vs_plain_fp64": value / plain_value,
            "accuracy_vs_plain_fp64": {"A": errA, "B": errB, "F": errF, "metric": "max|x-ref|/max|ref| per 6x6"},
            "refine_sweeps": iters,
            "surrogate": sur,
            "batched": batched,
            "stage_ms": dict(zip(names, [float(x) for x in per])),
            "stage_ms_note": "per frequency; assembly of f+1 overlaps factor+solve of f, so stages sum to more than ms_per_step",
            "setup_s": setup_s,
            "autotune": tune}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
