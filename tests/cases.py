"""Seeded mesh cases shared by the CPU and GPU tests (built with both the
oracle's and the library's generators)."""
import numpy as np

CYL_SMALL = dict(R=10.0, draft=20.0, NA=16, NR=3, NV=6, NRFS=3, cosine=False)      # 144 panels
CYL_MED = dict(R=10.0, draft=20.0, NA=24, NR=4, NV=8, NRFS=4, cosine=False)        # 288 panels
ARRAY_ORIGINS = [[25.0, 25.0, 0.0], [-25.0, 25.0, 0.0], [-25.0, -25.0, 0.0], [25.0, -25.0, 0.0]]
ARRAY_SMALL = dict(R=6.0, draft=20.0, NA=12, NR=2, NV=5, NRFS=0, cosine=False)     # 4 x 84 panels
BARGE_SMALL = dict(L=30.0, W=12.0, D=8.0, NX=8, NY=4, NZ=3, cosine=True)           # 104 panels
OMEGAS = np.array([0.1, 0.55, 1.0, 1.6, 2.0])
BETAS = np.array([0.0, np.pi / 4, np.pi / 2])
GYR_UNIT = np.eye(3)


def oracle_cylinder(orc, c):
    return orc.cylinder(c["R"], c["draft"], c["NA"], c["NR"], c["NV"], NRFS=c["NRFS"], cosine=c["cosine"])


def lib_cylinder(c):
    import bemuse_gb300 as bg
    return bg.Half_Cylinder(c["R"], c["draft"], c["NA"], c["NR"], c["NV"], c["NRFS"], c["cosine"])
