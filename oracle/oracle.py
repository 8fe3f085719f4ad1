"""ctypes front end of the FP64 CPU oracle (oracle/bem_oracle.cpp).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker; the product package never imports
it.  The optional ``ref`` handle loads oracle/_ref/libref_kernels.so, the
reference's own src/Kernels.cpp compiled unmodified (built only where the
reference tree is present).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(HERE, "_build", "liboracle.so")
_REF = os.path.join(HERE, "_ref", "libref_kernels.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_i = ctypes.c_int
_d = ctypes.c_double


def build(ref=None):
    """Compile liboracle.so (and the reference kernels when the tree exists)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref_root = ref or os.environ.get("BEM_REFERENCE_ROOT")
    args = ["REF=" + ref_root] if ref_root else []
    subprocess.run(["make", "-s", "-C", HERE, "ref-if-present"] + args, check=True)


def _p(a, typ=_dp):
    if a is None:
        return None
    return a.ctypes.data_as(typ)


class Mesh:
    """A panel mesh in the oracle's layout: body-local nodes (nn x 3), element
    connectivity (ne x 4, column 3 = -1 for triangles) and components, each a
    contiguous element range with a translation-only frame origin."""

    def __init__(self, nodes, elems, comp_first=None, comp_origin=None):
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        self.elems = np.ascontiguousarray(elems, dtype=np.int32)
        ne = self.elems.shape[0]
        if comp_first is None:
            comp_first = [0, ne]
            comp_origin = [[0.0, 0.0, 0.0]]
        self.comp_first = np.ascontiguousarray(comp_first, dtype=np.int32)
        self.comp_origin = np.ascontiguousarray(comp_origin, dtype=np.float64).reshape(-1, 3)

    @property
    def n(self):
        return self.elems.shape[0]

    def args(self):
        return (self.nodes.shape[0], _p(self.nodes), self.elems.shape[0], _p(self.elems, _ip),
                self.comp_first.shape[0] - 1, _p(self.comp_first, _ip), _p(self.comp_origin))

    @staticmethod
    def concat(meshes, origins):
        """Unify several body-local meshes into one system (Triple_Spar.cpp:120-166)."""
        nodes, elems, first, org = [], [], [0], []
        off = 0
        for m, o in zip(meshes, origins):
            nodes.append(m.nodes)
            e = m.elems.copy()
            e[e >= 0] += off
            elems.append(e)
            off += m.nodes.shape[0]
            first.append(first[-1] + m.n)
            org.append(o)
        return Mesh(np.concatenate(nodes), np.concatenate(elems), first, org)


class Oracle:
    def __init__(self, path=_LIB):
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        self.L = L
        L.orc_cylinder_sizes.argtypes = [_i, _i, _i, _i, _ip, _ip, _ip, _ip]
        L.orc_cylinder.argtypes = [_d, _d, _i, _i, _i, _i, _i, _dp, _ip, _dp, _ip]
        L.orc_barge_sizes.argtypes = [_i, _i, _i, _ip, _ip, _ip, _ip]
        L.orc_barge.argtypes = [_d, _d, _d, _i, _i, _i, _i, _dp, _ip, _dp, _ip]
        mesh_args = [_i, _dp, _i, _ip, _i, _ip, _dp]
        L.orc_panels.argtypes = mesh_args + [_i, _dp]
        L.orc_collocation.argtypes = mesh_args + [_dp]
        L.orc_havelock.argtypes = [_i, _dp, _dp, _dp, _dp]
        L.orc_source_kernel.argtypes = [_dp, _i, _dp, _dp, _dp]
        L.orc_rankine.argtypes = mesh_args + [_dp, _dp, _dp, _dp, _dp]
        L.orc_wave.argtypes = mesh_args + [_d, _dp, _dp]
        L.orc_wave_rows.argtypes = mesh_args + [_d, _i, _i, _dp, _dp]
        L.orc_lu_solve.argtypes = [_i, _dp, _i, _dp]
        L.orc_aero_wake.argtypes = mesh_args + [_i, _dp, _i, _ip, _ip, _ip, _i, _dp, _dp, _dp]
        L.orc_aero.argtypes = mesh_args + [_i, _dp, _dp, _dp]
        L.orc_mass_hydrostatics.argtypes = mesh_args + mesh_args + [_d, _d, _d, _dp, _dp, _dp, _dp, _dp]
        L.orc_solve.argtypes = mesh_args + [_i, _dp, _i, _dp, _d, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                            _dp, _dp]
        L.orc_solve_timed.argtypes = mesh_args + [_i, _dp, _i, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_solve_ifr.argtypes = mesh_args + mesh_args + [_i, _dp, _i, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                                            _dp, _dp, _dp]
        L.orc_exterior.argtypes = mesh_args + [_d, _i, _dp, _dp, _dp, _i, _dp, _i, _dp, _dp, _dp, _dp]
        L.orc_num_threads.restype = _i
        L.orc_set_threads.argtypes = [_i]

    # ---- meshes -----------------------------------------------------------
    def cylinder(self, R, draft, NA, NR, NV, NRFS=0, cosine=False):
        """Half_Cylinder mesh (+ optional interior waterplane 'aux' mesh)."""
        nn, ne, nna, nea = (ctypes.c_int() for _ in range(4))
        self.L.orc_cylinder_sizes(NA, NR, NV, NRFS, nn, ne, nna, nea)
        nodes = np.zeros((nn.value, 3))
        elems = np.zeros((ne.value, 4), np.int32)
        an = np.zeros((max(nna.value, 1), 3))
        ae = np.zeros((max(nea.value, 1), 4), np.int32)
        self.L.orc_cylinder(R, draft, NA, NR, NV, NRFS, int(cosine), _p(nodes), _p(elems, _ip), _p(an),
                            _p(ae, _ip))
        aux = Mesh(an[:nna.value], ae[:nea.value]) if NRFS > 0 else None
        return Mesh(nodes, elems), aux

    def barge(self, L, W, D, NX, NY, NZ, cosine=True):
        nn, ne, nna, nea = (ctypes.c_int() for _ in range(4))
        self.L.orc_barge_sizes(NX, NY, NZ, nn, ne, nna, nea)
        nodes = np.zeros((nn.value, 3))
        elems = np.zeros((ne.value, 4), np.int32)
        an = np.zeros((nna.value, 3))
        ae = np.zeros((nea.value, 4), np.int32)
        self.L.orc_barge(L, W, D, NX, NY, NZ, int(cosine), _p(nodes), _p(elems, _ip), _p(an), _p(ae, _ip))
        return Mesh(nodes, elems), Mesh(an, ae)

    # ---- geometry and kernels --------------------------------------------
    def panels(self, mesh, mirror=False):
        out = np.zeros((mesh.n, 56))
        self.L.orc_panels(*mesh.args(), int(mirror), _p(out))
        return out

    def collocation(self, mesh):
        out = np.zeros((mesh.n, 3))
        self.L.orc_collocation(*mesh.args(), _p(out))
        return out

    def havelock(self, x, y, v):
        x, y, v = (np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (x, y, v))
        out = np.zeros((x.size, 8))
        self.L.orc_havelock(x.size, _p(x), _p(y), _p(v), _p(out))
        g = out[:, 0::2] + 1j * out[:, 1::2]
        return g  # columns: G, dGx, dGy, dGz

    def source_kernel(self, packed_panel, P):
        pp = np.ascontiguousarray(packed_panel, dtype=np.float64)
        P = np.ascontiguousarray(P, dtype=np.float64).reshape(-1, 3)
        S = np.zeros(P.shape[0])
        D = np.zeros(P.shape[0])
        self.L.orc_source_kernel(_p(pp), P.shape[0], _p(P), _p(S), _p(D))
        return S, D

    def rankine(self, mesh):
        N = mesh.n
        s, sr, d, dr = (np.zeros((N, N)) for _ in range(4))
        rn = np.zeros(N)
        self.L.orc_rankine(*mesh.args(), _p(s), _p(sr), _p(d), _p(dr), _p(rn))
        return s, sr, d, dr, rn

    def wave(self, mesh, K):
        N = mesh.n
        ws = np.zeros((N, N), np.complex128)
        wd = np.zeros((N, N), np.complex128)
        self.L.orc_wave(*mesh.args(), K, _p(ws.view(np.float64)), _p(wd.view(np.float64)))
        return ws, wd

    def wave_rows(self, mesh, K, r0, r1):
        N = mesh.n
        ws = np.zeros((r1 - r0, N), np.complex128)
        wd = np.zeros((r1 - r0, N), np.complex128)
        self.L.orc_wave_rows(*mesh.args(), K, r0, r1, _p(ws.view(np.float64)), _p(wd.view(np.float64)))
        return ws, wd

    def lu_solve(self, A, B):
        A = np.array(A, dtype=np.complex128, order="C")
        B = np.array(B, dtype=np.complex128, order="C")
        if B.ndim == 1:
            B = B[:, None]
        self.L.orc_lu_solve(A.shape[0], _p(A.view(np.float64)), B.shape[1], _p(B.view(np.float64)))
        return B

    def mass_hydrostatics(self, mesh, aux=None, rho=1025.0, g=9.81, mass=0.0, cog=(0, 0, 0), gyr=None):
        if aux is None:
            aux = Mesh(np.zeros((0, 3)), np.zeros((0, 4), np.int32))
        cog = np.ascontiguousarray(cog, dtype=np.float64)
        gyr = np.ascontiguousarray(np.zeros(9) if gyr is None else gyr, dtype=np.float64).ravel()
        M = np.zeros((6, 6))
        C = np.zeros((6, 6))
        vc = np.zeros(4)
        self.L.orc_mass_hydrostatics(*mesh.args(), *aux.args(), rho, g, mass, _p(cog), _p(gyr), _p(M), _p(C),
                                     _p(vc))
        return M, C, vc

    def solve(self, mesh, omegas, betas, M=None, C=None, want_phi=False, ifr_aux=None):
        """Full FP64 frequency loop; omegas are the internal angular frequencies.
        ifr_aux: the interior free-surface mesh, solved with IFR (hull + lid panels)."""
        omegas = np.ascontiguousarray(omegas, dtype=np.float64).ravel()
        betas = np.ascontiguousarray(betas, dtype=np.float64).ravel()
        nf, nb, N = omegas.size, betas.size, mesh.n
        M = np.ascontiguousarray(np.zeros((6, 6)) if M is None else M, dtype=np.float64)
        C = np.ascontiguousarray(np.zeros((6, 6)) if C is None else C, dtype=np.float64)
        A = np.zeros((nf, 6, 6))
        B = np.zeros((nf, 6, 6))
        FK, SC, F, RAO = (np.zeros((nf, 6, nb), np.complex128) for _ in range(4))
        pj = np.zeros((N, 6), np.complex128) if want_phi else None
        ps = np.zeros((N, nb), np.complex128) if want_phi else None
        tail = (_p(M), _p(C), _p(A), _p(B), _p(FK.view(np.float64)), _p(SC.view(np.float64)),
                _p(F.view(np.float64)), _p(RAO.view(np.float64)), _p(pj.view(np.float64)) if want_phi else None,
                _p(ps.view(np.float64)) if want_phi else None)
        if ifr_aux is None:
            self.L.orc_solve(*mesh.args(), nf, _p(omegas), nb, _p(betas), 9.81, *tail)
        else:
            self.L.orc_solve_ifr(*mesh.args(), *ifr_aux.args(), nf, _p(omegas), nb, _p(betas), *tail)
        out = dict(A=A, B=B, FK=FK, SC=SC, F=F, RAO=RAO)
        if want_phi:
            out["phiJ"] = pj
            out["phiS"] = ps
        return out

    def solve_timed(self, mesh, omegas, betas, M=None, C=None):
        """solve() with wall-clock seconds per stage: 'setup' (the frequency-independent
        Rankine matrices) and per frequency 'wave' (assembly + compose), 'lu' and 'rest'
        (right-hand sides, solves, post)."""
        omegas = np.ascontiguousarray(omegas, dtype=np.float64).ravel()
        betas = np.ascontiguousarray(betas, dtype=np.float64).ravel()
        nf, nb = omegas.size, betas.size
        M = np.ascontiguousarray(np.zeros((6, 6)) if M is None else M, dtype=np.float64)
        C = np.ascontiguousarray(np.zeros((6, 6)) if C is None else C, dtype=np.float64)
        A = np.zeros((nf, 6, 6))
        B = np.zeros((nf, 6, 6))
        FK, SC, F, RAO = (np.zeros((nf, 6, nb), np.complex128) for _ in range(4))
        clk = np.zeros(1 + 3 * nf)
        self.L.orc_solve_timed(*mesh.args(), nf, _p(omegas), nb, _p(betas), _p(M), _p(C), _p(A), _p(B),
                               _p(FK.view(np.float64)), _p(SC.view(np.float64)), _p(F.view(np.float64)),
                               _p(RAO.view(np.float64)), _p(clk))
        t = clk[1:].reshape(nf, 3)
        return dict(A=A, B=B, FK=FK, SC=SC, F=F, RAO=RAO), {"setup": float(clk[0]), "wave": t[:, 0], "lu": t[:, 1],
                                                            "rest": t[:, 2]}

    def exterior(self, mesh, omega, betas, phiJ, phiS, wave_points, n_kochin):
        """Free-surface elevation at wave_points (n x 3) and Kochin functions at
        n_kochin angles for one frequency from the potentials phiJ (N x 6) and
        phiS (N x nb): (fs_rad, fs_diff, kochin_rad, kochin_diff)."""
        betas = np.ascontiguousarray(betas, dtype=np.float64).ravel()
        nb, N = betas.size, mesh.n
        pj = np.ascontiguousarray(phiJ, dtype=np.complex128).reshape(N, 6)
        ps = np.ascontiguousarray(phiS, dtype=np.complex128).reshape(N, nb)
        wp = np.ascontiguousarray(wave_points, dtype=np.float64).reshape(-1, 3)
        nw = wp.shape[0]
        fr = np.zeros((nw, 6), np.complex128)
        fd = np.zeros((nw, nb), np.complex128)
        kr = np.zeros((n_kochin, 6), np.complex128)
        kd = np.zeros((n_kochin, nb), np.complex128)
        self.L.orc_exterior(*mesh.args(), float(omega), nb, _p(betas), _p(pj.view(np.float64)),
                            _p(ps.view(np.float64)), nw, _p(wp), int(n_kochin), _p(fr.view(np.float64)),
                            _p(fd.view(np.float64)), _p(kr.view(np.float64)), _p(kd.view(np.float64)))
        return fr, fd, kr, kd

    def aero(self, mesh, vel):
        """Aerodynamic_Solver steady constant-panel solve: returns (X, BC)."""
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
        X = np.zeros(mesh.n)
        BC = np.zeros(mesh.n)
        self.L.orc_aero(*mesh.args(), vel.shape[0], _p(vel), _p(X), _p(BC))
        return X, BC

    def aero_wake(self, mesh, wake_quads, te_up, te_lo, vel):
        """The steady constant-panel solve with a trailing wake (orc_aero_wake): wake strip w
        is the quad wake_quads[w] (4 x 3 vertices), its strength the Kutta jump
        X[te_up[w]] - X[te_lo[w]].  Returns (X, BC)."""
        q = np.ascontiguousarray(wake_quads, dtype=np.float64).reshape(-1, 4, 3)
        nw = q.shape[0]
        wn = np.ascontiguousarray(q.reshape(-1, 3))
        we = np.ascontiguousarray(np.arange(4 * nw, dtype=np.int32).reshape(nw, 4))
        up = np.ascontiguousarray(te_up, dtype=np.int32)
        lo = np.ascontiguousarray(te_lo, dtype=np.int32)
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
        X = np.zeros(mesh.n)
        BC = np.zeros(mesh.n)
        self.L.orc_aero_wake(*mesh.args(), wn.shape[0], _p(wn), nw, _p(we, _ip), _p(up, _ip), _p(lo, _ip),
                             vel.shape[0], _p(vel), _p(X), _p(BC))
        return X, BC

    def set_threads(self, n):
        self.L.orc_set_threads(int(n))

    def num_threads(self):
        return self.L.orc_num_threads()


class RefKernels:
    """The reference's own Kernels.cpp (compiled unmodified); None if unbuilt."""

    def __init__(self, path=_REF):
        L = ctypes.CDLL(path)
        self.L = L
        L.ref_havelock.argtypes = [_i, _dp, _dp, _dp, _dp]
        L.ref_special.argtypes = [_i, _dp, _dp]
        L.ref_point_kernels.argtypes = [_i, _dp, _dp, _dp, _dp, _dp]

    @staticmethod
    def available(path=_REF):
        return os.path.exists(path)

    def havelock(self, x, y, v):
        x, y, v = (np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (x, y, v))
        out = np.zeros((x.size, 8))
        self.L.ref_havelock(x.size, _p(x), _p(y), _p(v), _p(out))
        return out[:, 0::2] + 1j * out[:, 1::2]

    def special(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        out = np.zeros((x.size, 6))
        self.L.ref_special(x.size, _p(x), _p(out))
        return out

    def point_kernels(self, S, D, A):
        S, D, A = (np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 3) for a in (S, D, A))
        src = np.zeros(S.shape[0])
        dip = np.zeros(S.shape[0])
        self.L.ref_point_kernels(S.shape[0], _p(S), _p(D), _p(A), _p(src), _p(dip))
        return src, dip
