"""Generate the golden fixtures in tests/golden/ (run where the reference tree
exists; the fixtures travel with the repository, the reference does not).

havelock_ref.npz   HavelockGF (src/Kernels.cpp:342-412) and the Struve/Bessel
                   helpers (:31-116) evaluated by the reference's own Kernels.cpp,
                   compiled unmodified into oracle/_ref (oracle/Makefile `ref`),
                   on seeded points covering log10(KR) in [-3, log10 200],
                   KZ in [-100, 0] and both Struve branches (h <= 3, h > 3).
point_kernels_ref.npz  Source_Kernel / Dipole_Kernel (:11-27) at seeded points.
cyl144_oracle.npz  FP64 oracle results for a 144-panel cylinder (R=10, T=20,
                   16 x (3+6) panels, linear spacing) at 5 frequencies and 3
                   headings: a regression fixture for the oracle itself.

Usage: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle.oracle import Oracle, RefKernels, build  # noqa: E402


def havelock_points(n=3000, seed=20261203):
    rng = np.random.default_rng(seed)
    kr = 10 ** rng.uniform(-3, np.log10(200), n)
    th = rng.uniform(0, 2 * np.pi, n)
    kz = rng.uniform(-100, 0, n)
    kz[: n // 4] = -10 ** rng.uniform(-4, 0, n // 4)   # near-surface band
    # both Struve branches and the h <= 1e-6 guard
    extra_h = np.array([1e-8, 5e-7, 0.1, 1.0, 2.999999, 3.0, 3.000001, 8.0, 25.0, 199.0])
    x = np.concatenate([kr * np.cos(th), extra_h])
    y = np.concatenate([kr * np.sin(th), np.zeros_like(extra_h)])
    v = np.concatenate([kz, np.full_like(extra_h, -0.3)])
    return x, y, v


def main():
    build()
    if not RefKernels.available():
        raise SystemExit("oracle/_ref/libref_kernels.so is missing (needs the reference tree)")
    ref = RefKernels()
    x, y, v = havelock_points()
    g = ref.havelock(x, y, v)
    hx = np.concatenate([np.linspace(1e-4, 3.0, 100), np.linspace(3.0, 200.0, 100)])
    sp = ref.special(hx)
    np.savez_compressed(os.path.join(HERE, "havelock_ref.npz"), x=x, y=y, v=v, G=g, h=hx, special=sp)
    rng = np.random.default_rng(7)
    S = rng.uniform(-5, 5, (200, 3))
    D = rng.uniform(-5, 5, (200, 3))
    A = rng.standard_normal((200, 3))
    src, dip = ref.point_kernels(S, D, A)
    np.savez_compressed(os.path.join(HERE, "point_kernels_ref.npz"), S=S, D=D, A=A, src=src, dip=dip)
    orc = Oracle()
    m, aux = orc.cylinder(10.0, 20.0, 16, 3, 6, NRFS=3, cosine=False)
    M, C, vc = orc.mass_hydrostatics(m, aux, gyr=np.eye(3).ravel())
    om = np.array([0.1, 0.55, 1.0, 1.6, 2.0])
    be = np.array([0.0, np.pi / 4, np.pi / 2])
    r = orc.solve(m, om, be, M=M, C=C)
    np.savez_compressed(os.path.join(HERE, "cyl144_oracle.npz"), omegas=om, betas=be, M=M, C=C, vol_cob=vc, **r)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
