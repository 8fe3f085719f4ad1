"""bemuse_gb300 -- GB300-native frequency-domain panel-method solver.

Python mirror of the reference's hydrodynamic solver interface (ZeppSav/BEMUse,
src/Solver/Hydrodynamic_Solver.h:35-160 behind src/Solver/Solver_Base.h:39-153)
over the C ABI in include/bemgpu.h.  All computation happens in
bemuse_gb300/_lib/libbemgpu.so (hand-written sm_103a kernels); this module only
marshals arguments.  There is no CPU fallback: importing works without the
library, but every call that needs it raises if it is missing.
"""
import ctypes
import os

import numpy as np

from . import build as _build

__all__ = [
    "BEMError", "lib", "Parameter", "Mesh", "Half_Cylinder", "Barge", "unify",
    "Hydrodynamic_Radiation_Solver", "Aerodynamic_Solver", "NACA_Wing", "NACA_Wing_Wake", "havelock_gf", "dense_solve",
    "PLAIN_FP64", "MIXED", "read_mesh", "GDF_Geometry", "MAR_Geometry", "STL_Geometry", "PNL_Geometry",
    "write_wamit",
]

PLAIN_FP64 = 0
MIXED = 1

_STATUS = {0: "BEM_OK", 1: "BEM_ERR_ARG", 2: "BEM_ERR_CUDA", 3: "BEM_ERR_STATE", 4: "BEM_ERR_NUMERIC",
           5: "BEM_ERR_NOMEM", 6: "BEM_ERR_UNSUPPORTED"}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_fp = ctypes.POINTER(ctypes.c_float)


class BEMError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (_STATUS.get(status, str(status)), msg))
        self.status = status


class _Mesh(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int), ("nodes", _dp), ("n_elems", ctypes.c_int), ("elems", _ip),
                ("n_comp", ctypes.c_int), ("comp_first", _ip), ("comp_origin", _dp)]


class _Props(ctypes.Structure):
    _fields_ = [("mass", ctypes.c_double), ("cog", ctypes.c_double * 3), ("gyration", ctypes.c_double * 9),
                ("mass_matrix", _dp), ("stiffness", _dp), ("aux", ctypes.POINTER(_Mesh))]


class _WamitInfo(ctypes.Structure):
    _fields_ = [("n_beta", ctypes.c_int), ("betas", _dp), ("rho", ctypes.c_double), ("gravity", ctypes.c_double),
                ("M", ctypes.c_double * 36), ("C", ctypes.c_double * 36), ("volume", ctypes.c_double),
                ("cob", ctypes.c_double * 3), ("cog", ctypes.c_double * 3), ("n_kochin", ctypes.c_int),
                ("n_wave", ctypes.c_int), ("wave_points", _dp)]


class _SummaryInfo(ctypes.Structure):
    _fields_ = [("w", ctypes.POINTER(_WamitInfo)), ("n_nodes", ctypes.c_int), ("n_elems", ctypes.c_int),
                ("n_aux_elems", ctypes.c_int), ("surface_area", ctypes.c_double), ("mass", ctypes.c_double),
                ("file_info", ctypes.c_char_p)]


class _Result(ctypes.Structure):
    _fields_ = [("A", _dp), ("B", _dp), ("FK", _dp), ("SC", _dp), ("F", _dp), ("RAO", _dp),
                ("refine_iters", _ip), ("residual", _dp), ("phi_rad", _dp), ("phi_scat", _dp),
                ("fs_rad", _dp), ("fs_diff", _dp), ("kochin_rad", _dp), ("kochin_diff", _dp)]


_LIB = None


def lib():
    """Load libbemgpu.so (raises if it has not been built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        raise BEMError(6, "native library %s is missing; run bemuse_gb300.build.build()" % path)
    L = ctypes.CDLL(path)
    c_int, c_double, vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
    sig = {
        "bem_version": ([], ctypes.c_char_p),
        "bem_last_error": ([vp], ctypes.c_char_p),
        "bem_mesh_cylinder_sizes": ([c_int] * 4 + [_ip] * 4, c_int),
        "bem_mesh_cylinder": ([c_double, c_double, c_int, c_int, c_int, c_int, c_int, _dp, _ip, _dp, _ip], c_int),
        "bem_mesh_barge_sizes": ([c_int] * 3 + [_ip] * 4, c_int),
        "bem_mesh_barge": ([c_double] * 3 + [c_int] * 4 + [_dp, _ip, _dp, _ip], c_int),
        "bem_create": ([ctypes.POINTER(vp), c_int], c_int),
        "bem_destroy": ([vp], None),
        "bem_set_params": ([vp, c_double, c_double, c_int, _dp], c_int),
        "bem_setup": ([vp, ctypes.POINTER(_Mesh), ctypes.POINTER(_Props)], c_int),
        "bem_solve": ([vp, c_int, _dp, c_int, c_double, ctypes.POINTER(_Result)], c_int),
        "bem_get_sizes": ([vp, _ip, _ip], c_int),
        "bem_get_body_matrices": ([vp, _dp, _dp, _dp], c_int),
        "bem_get_rankine": ([vp, _dp, _dp, _dp, _dp], c_int),
        "bem_wave_matrices": ([vp, c_double, c_int, _dp, _dp], c_int),
        "bem_havelock": ([c_int, c_int, _dp, _dp, _dp, c_int, _dp], c_int),
        "bem_dense_solve": ([vp, c_int, _dp, c_int, _dp, c_int, c_double, _ip, _dp], c_int),
        "bem_stage_times": ([vp, _dp, c_int], c_int),
        "bem_kernel_times": ([vp, _dp, c_int], c_int),
        "bem_lu_timeline": ([vp, c_int, c_int, _dp, _ip], c_int),
        "bem_set_tuning": ([vp, ctypes.c_char_p, c_double], c_int),
        "bem_autotune": ([vp, c_int, _dp, _dp, ctypes.c_char_p, c_int], c_int),
        "bem_mlp_num_params": ([], c_int),
        "bem_mlp_create": ([ctypes.POINTER(vp), c_int, ctypes.c_ulonglong], c_int),
        "bem_mlp_destroy": ([vp], None),
        "bem_mlp_last_error": ([vp], ctypes.c_char_p),
        "bem_mlp_set_normalization": ([vp, _dp, _dp, _dp, _dp], c_int),
        "bem_mlp_get_params": ([vp, _dp], c_int),
        "bem_mlp_set_params": ([vp, _dp], c_int),
        "bem_mlp_eval": ([vp, c_int, _dp, _dp], c_int),
        "bem_mlp_grad": ([vp, c_int, _dp, _dp, _dp, _dp], c_int),
        "bem_mlp_train": ([vp, c_int, _dp, _dp, c_int, c_int, ctypes.c_double, ctypes.c_ulonglong, _dp], c_int),
        "bem_mlp_throughput": ([vp, c_int, _dp], c_int),
        "bem_mlp_eval_tc": ([vp, c_int, _dp, _dp], c_int),
        "bem_mlp_throughput_tc": ([vp, c_int, _dp], c_int),
        "bem_havelock_throughput": ([c_int, c_int, c_int, _dp], c_int),
        "bem_batch_solve": ([c_int, c_int, ctypes.POINTER(_Mesh), ctypes.POINTER(_Props), c_double, c_double, c_int,
                             _dp, c_int, _dp, c_int, c_double, c_int, ctypes.POINTER(_Result), _dp], c_int),
        "bem_read_mesh": ([ctypes.c_char_p, c_int, _ip, _dp, _ip, _ip], c_int),
        "bem_set_wave_points": ([vp, c_int, _dp], c_int),
        "bem_set_kochin": ([vp, c_int], c_int),
        "bem_set_ifr": ([vp, c_int], c_int),
        "bem_read_mesh_error": ([], ctypes.c_char_p),
        "bem_write_bem": ([ctypes.c_char_p, ctypes.POINTER(_SummaryInfo), c_int, _dp, ctypes.POINTER(_Result)],
                          c_int),
        "bem_write_wamit": ([ctypes.c_char_p, ctypes.POINTER(_WamitInfo), c_int, _dp, ctypes.POINTER(_Result)], c_int),
        "bem_launch_count": ([], ctypes.c_ulonglong),
        "bem_mesh_wing_sizes": ([c_int, c_int, _ip, _ip], c_int),
        "bem_mesh_wing": ([c_double, c_double, c_double, c_int, c_int, c_int, _dp, _ip], c_int),
        "bem_aero_setup": ([vp, ctypes.POINTER(_Mesh)], c_int),
        "bem_aero_solve": ([vp, c_int, _dp, c_int, c_double, _dp, _dp], c_int),
        "bem_aero_set_wake": ([vp, c_int, _dp, _ip, _ip], c_int),
        "bem_aero_surface": ([vp, _dp, _dp, c_double, _dp, _dp], c_int),
        "bem_mesh_wing_wake": ([c_double, c_double, c_int, c_int, c_double, _dp, _ip, _ip], c_int),
        "bem_fp32_peak": ([c_int, _dp], c_int),
        "bem_cusolver_zgetrf_ms": ([c_int, c_int, _dp], c_int),
        "bem_set_surrogate": ([vp, vp, c_int, c_double, c_double, _dp], c_int),
        "bem_surrogate_stats": ([vp, _dp, c_int], c_int),
        "bem_tc_probe": ([c_int, c_int, c_int, _fp, _fp, _fp, _fp, _fp, _fp, _fp], c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _LIB = L
    return L


def _p(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


def _check(st, ctx=None):
    if st != 0:
        msg = lib().bem_last_error(ctx)
        raise BEMError(st, msg.decode() if msg else "")


class Parameter(tuple):
    """(name, value) pair as in Boundary_Base.h:47-55."""

    def __new__(cls, name, value):
        return super().__new__(cls, (name, value))


class Mesh:
    """Panel mesh: component-local nodes (n x 3), elements (m x 4, -1 = triangle),
    components (element ranges + translation origins) and an optional interior
    waterplane ('aux') mesh for hydrostatics."""

    def __init__(self, nodes, elems, comp_first=None, comp_origin=None, aux=None):
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64).reshape(-1, 3)
        self.elems = np.ascontiguousarray(elems, dtype=np.int32).reshape(-1, 4)
        if comp_first is None:
            comp_first, comp_origin = [0, self.elems.shape[0]], [[0.0, 0.0, 0.0]]
        self.comp_first = np.ascontiguousarray(comp_first, dtype=np.int32)
        self.comp_origin = np.ascontiguousarray(comp_origin, dtype=np.float64).reshape(-1, 3)
        self.aux = aux

    @property
    def n(self):
        return self.elems.shape[0]

    def _struct(self):
        return _Mesh(self.nodes.shape[0], _p(self.nodes), self.elems.shape[0], _p(self.elems, _ip),
                     self.comp_first.shape[0] - 1, _p(self.comp_first, _ip), _p(self.comp_origin))


def _cylinder_arrays(R, draft, NA, NR, NV, NRFS, cosine):
    L = lib()
    nn, ne, nna, nea = (ctypes.c_int() for _ in range(4))
    _check(L.bem_mesh_cylinder_sizes(NA, NR, NV, NRFS, nn, ne, nna, nea))
    nodes = np.zeros((nn.value, 3))
    elems = np.zeros((ne.value, 4), np.int32)
    an = np.zeros((max(nna.value, 1), 3))
    ae = np.zeros((max(nea.value, 1), 4), np.int32)
    _check(L.bem_mesh_cylinder(R, draft, NA, NR, NV, NRFS, int(cosine), _p(nodes), _p(elems, _ip), _p(an),
                               _p(ae, _ip)))
    aux = Mesh(an[:nna.value], ae[:nea.value]) if NRFS > 0 else None
    return nodes, elems, aux


def Half_Cylinder(Radius, Draft, NPanels_Azimuthal, NPanels_Radial, NPanels_Vertical,
                  NPanels_FreeSurface_Int_Radial=0, Cosine_Disc=True):
    """Half_Cylinder (Volume_of_Revolution.cpp:167-199); parameter names as the
    reference's Set_Parameters keys."""
    nodes, elems, aux = _cylinder_arrays(Radius, Draft, NPanels_Azimuthal, NPanels_Radial, NPanels_Vertical,
                                         NPanels_FreeSurface_Int_Radial, Cosine_Disc)
    return Mesh(nodes, elems, aux=aux)


def Barge(Tank_Length, Tank_Width, Tank_Depth, NPanels_Tank_Length, NPanels_Tank_Width, NPanels_Tank_Depth,
          Cosine_Disc=True):
    """Barge (Barge.cpp:12-204)."""
    L = lib()
    nn, ne, nna, nea = (ctypes.c_int() for _ in range(4))
    _check(L.bem_mesh_barge_sizes(NPanels_Tank_Length, NPanels_Tank_Width, NPanels_Tank_Depth, nn, ne, nna, nea))
    nodes = np.zeros((nn.value, 3))
    elems = np.zeros((ne.value, 4), np.int32)
    an = np.zeros((nna.value, 3))
    ae = np.zeros((nea.value, 4), np.int32)
    _check(L.bem_mesh_barge(Tank_Length, Tank_Width, Tank_Depth, NPanels_Tank_Length, NPanels_Tank_Width,
                            NPanels_Tank_Depth, int(Cosine_Disc), _p(nodes), _p(elems, _ip), _p(an), _p(ae, _ip)))
    return Mesh(nodes, elems, aux=Mesh(an, ae))


def NACA_Wing(chord=1.0, span=8.0, thickness=0.12, n_chord=120, n_span=60, cosine=True):
    """Rectangular wing of a symmetric NACA 00xx section (n_chord panels around
    the section, n_span strips; normals into the wing)."""
    L = lib()
    nn, ne = ctypes.c_int(), ctypes.c_int()
    _check(L.bem_mesh_wing_sizes(n_chord, n_span, nn, ne))
    nodes = np.zeros((nn.value, 3))
    elems = np.zeros((ne.value, 4), np.int32)
    _check(L.bem_mesh_wing(chord, span, thickness, n_chord, n_span, int(cosine), _p(nodes), _p(elems, _ip)))
    return Mesh(nodes, elems)


def NACA_Wing_Wake(chord=1.0, span=8.0, n_chord=120, n_span=60, length=20.0):
    """Flat trailing wake of NACA_Wing's wing: one strip per panel column from the
    trailing edge (x = chord, z = 0) to length chords downstream (normal -z).
    Returns (quads n_span x 4 x 3, te_upper, te_lower): the Kutta pair of strip j is
    the upper trailing-edge panel j n_chord + n_chord - 1 and the lower one j n_chord."""
    quads = np.zeros((n_span, 4, 3))
    up = np.zeros(n_span, np.int32)
    lo = np.zeros(n_span, np.int32)
    _check(lib().bem_mesh_wing_wake(chord, span, n_chord, n_span, length, _p(quads), _p(up, _ip), _p(lo, _ip)))
    return quads, up, lo


def unify(meshes, origins):
    """Several component meshes in translated frames as one system
    (Triple_Spar::Unify_Geometries, Triple_Spar.cpp:120-166)."""
    nodes, elems, first, org, an, ae, afirst = [], [], [0], [], [], [], [0]
    off = aoff = 0
    for m, o in zip(meshes, origins):
        nodes.append(m.nodes)
        e = m.elems.copy()
        e[e >= 0] += off
        elems.append(e)
        off += m.nodes.shape[0]
        first.append(first[-1] + m.n)
        org.append(o)
        if m.aux is not None:
            an.append(m.aux.nodes)
            a = m.aux.elems.copy()
            a[a >= 0] += aoff
            ae.append(a)
            aoff += m.aux.nodes.shape[0]
            afirst.append(afirst[-1] + m.aux.n)
    aux = None
    if an and len(an) == len(meshes):
        aux = Mesh(np.concatenate(an), np.concatenate(ae), afirst, org)
    return Mesh(np.concatenate(nodes), np.concatenate(elems), first, org, aux=aux)


MESH_FORMATS = {"auto": 0, "gdf": 1, "mar": 2, "stl": 3, "pnl": 4}


def read_mesh(path, fmt="auto"):
    """A mesh file as a Mesh, read by the rules of the reference's importers:
    GDF (GDF_Geo.cpp:12-103), MAR (MAR_Geo.cpp:12-96), ASCII STL (STL_Geo.cpp:12-94,
    positions x 100) and PNL (PNL_Geo.cpp:17-129); ``fmt="auto"`` picks by extension."""
    code = MESH_FORMATS[fmt.lower()]
    nn, ne = ctypes.c_int(), ctypes.c_int()
    rc = lib().bem_read_mesh(str(path).encode(), code, ctypes.byref(nn), None, ctypes.byref(ne), None)
    if rc != 0:
        raise BEMError(rc, lib().bem_read_mesh_error().decode())
    nodes = np.zeros((max(nn.value, 1), 3))
    elems = np.zeros((max(ne.value, 1), 4), np.int32)
    rc = lib().bem_read_mesh(str(path).encode(), code, ctypes.byref(nn), _p(nodes), ctypes.byref(ne), _p(elems, _ip))
    if rc != 0:
        raise BEMError(rc, lib().bem_read_mesh_error().decode())
    return Mesh(nodes[:nn.value], elems[:ne.value])


def GDF_Geometry(path):
    """The reference's GDF_Geometry importer (GDF_Geo.cpp)."""
    return read_mesh(path, "gdf")


def MAR_Geometry(path):
    """The reference's MAR_Geometry importer (MAR_Geo.cpp), NEMOH meshes."""
    return read_mesh(path, "mar")


def STL_Geometry(path):
    """The reference's STL_Geometry importer (STL_Geo.cpp), ASCII STL scaled by 100."""
    return read_mesh(path, "stl")


def PNL_Geometry(path):
    """The reference's PNL_Geometry importer (PNL_Geo.cpp), HAMS meshes."""
    return read_mesh(path, "pnl")


def write_wamit(prefix, omegas, out, betas, M, C, volume, cob, cog, rho=1025.0, gravity=9.81, wave_points=None):
    """WAMIT-format result files (.1 .2 .2fk .2sc .4 .6 .hst .mmx, _KochinRad.bem,
    _KochinDiff.bem, and with wave points .6r and _WaveElPos.bem) as the reference's
    Generate/Update_Output_File_WAMIT write them (Hydrodynamic_Solver_IO.cpp:430-646).
    omegas are the internal angular frequencies; out holds A, B (nf x 6 x 6),
    FK, SC, F, RAO (nf x 6 x nb complex) and optionally kochin_rad / kochin_diff and
    fs_rad from solve_omegas."""
    om = np.ascontiguousarray(omegas, dtype=np.float64).ravel()
    betas = np.ascontiguousarray(betas, dtype=np.float64).ravel()
    info = _WamitInfo()
    info.n_beta = betas.size
    info.betas = _p(betas)
    info.rho, info.gravity, info.volume = float(rho), float(gravity), float(volume)
    info.M[:] = list(np.asarray(M, dtype=np.float64).ravel())
    info.C[:] = list(np.asarray(C, dtype=np.float64).ravel())
    info.cob[:] = list(np.asarray(cob, dtype=np.float64).ravel())
    info.cog[:] = list(np.asarray(cog, dtype=np.float64).ravel())
    keys = ("A", "B", "FK", "SC", "F", "RAO", "kochin_rad", "kochin_diff", "fs_rad")
    keep = {k: np.ascontiguousarray(out[k]) for k in keys if k in out}
    res = _Result()
    res.A = _p(keep["A"]) if "A" in keep else None
    res.B = _p(keep["B"]) if "B" in keep else None
    for k in keys[2:]:
        setattr(res, k, _p(keep[k].view(np.float64)) if k in keep else None)
    if "kochin_rad" in keep:
        info.n_kochin = keep["kochin_rad"].shape[1]
    elif "kochin_diff" in keep:
        info.n_kochin = keep["kochin_diff"].shape[1]
    wp = None
    if wave_points is not None and "fs_rad" in keep:
        wp = np.ascontiguousarray(wave_points, dtype=np.float64).reshape(-1, 3)
        info.n_wave = wp.shape[0]
        info.wave_points = _p(wp)
    elif "fs_rad" in keep:
        res.fs_rad = None
    rc = lib().bem_write_wamit(str(prefix).encode(), ctypes.byref(info), om.size, _p(om), ctypes.byref(res))
    if rc != 0:
        raise BEMError(rc, "bem_write_wamit could not write %s.*" % prefix)


def panel_areas(mesh):
    """Flat-panel areas (Geo_Elements.cpp: quads 1/2 |d1 x d2|, triangles 1/2 |e1 x e2|)."""
    nodes = mesh.nodes
    e = mesh.elems
    p0, p1, p2 = nodes[e[:, 0]], nodes[e[:, 1]], nodes[e[:, 2]]
    p3 = nodes[np.where(e[:, 3] >= 0, e[:, 3], e[:, 0])]
    quad = 0.5 * np.linalg.norm(np.cross(p2 - p0, p3 - p1), axis=1)
    tri = 0.5 * np.linalg.norm(np.cross(p1 - p0, p2 - p0), axis=1)
    return np.where(e[:, 3] >= 0, quad, tri)


def write_bem(prefix, omegas, out, betas, M, C, volume, cob, cog, mesh=None, mass=0.0, n_aux=0, file_info=""):
    """The .bem summary file of Generate/Update_Output_File_BEMUse
    (Hydrodynamic_Solver_IO.cpp:107-426)."""
    om = np.ascontiguousarray(omegas, dtype=np.float64).ravel()
    betas = np.ascontiguousarray(betas, dtype=np.float64).ravel()
    w = _WamitInfo()
    w.n_beta = betas.size
    w.betas = _p(betas)
    w.rho, w.gravity, w.volume = 1025.0, 9.81, float(volume)
    w.M[:] = list(np.asarray(M, dtype=np.float64).ravel())
    w.C[:] = list(np.asarray(C, dtype=np.float64).ravel())
    w.cob[:] = list(np.asarray(cob, dtype=np.float64).ravel())
    w.cog[:] = list(np.asarray(cog, dtype=np.float64).ravel())
    info = _SummaryInfo()
    info.w = ctypes.pointer(w)
    if mesh is not None:
        info.n_nodes, info.n_elems = mesh.nodes.shape[0], mesh.elems.shape[0]
        info.surface_area = float(np.sum(panel_areas(mesh)))
    info.n_aux_elems = int(n_aux)
    info.mass = float(mass)
    info.file_info = file_info.encode()
    keep = {k: np.ascontiguousarray(out[k]) for k in ("A", "B", "FK", "F") if k in out}
    res = _Result()
    res.A = _p(keep["A"]) if "A" in keep else None
    res.B = _p(keep["B"]) if "B" in keep else None
    res.FK = _p(keep["FK"].view(np.float64)) if "FK" in keep else None
    res.F = _p(keep["F"].view(np.float64)) if "F" in keep else None
    rc = lib().bem_write_bem(str(prefix).encode(), ctypes.byref(info), om.size, _p(om), ctypes.byref(res))
    if rc != 0:
        raise BEMError(rc, "bem_write_bem could not write %s.bem" % prefix)


def barge_free_surface_points(LFS, WFS, NXFS, NYFS):
    """The Barge free-surface grid (Barge.cpp:125-140): (NXFS+1) x (NYFS+1) nodes over
    LFS x WFS, x-major, pushed out by the factor 1.001, at z = 0."""
    pts = []
    for i in range(NXFS + 1):
        for j in range(NYFS + 1):
            x = -0.5 * LFS + LFS * i / NXFS
            y = -0.5 * WFS + WFS * j / NYFS
            pts.append((1.001 * x, 1.001 * y, 0.0))
    return np.array(pts)


class Hydrodynamic_Radiation_Solver:
    """Drop-in for BEMUse::Hydrodynamic_Radiation_Solver (Hydrodynamic_Solver.h:35-160).

    Set_Parameters([...Parameter...]) -> Setup(mesh) -> Set_Real(Frequency) -> Solve().
    As in the reference, Solve() uses Omega = Frequency / (2 pi)
    (Hydrodynamic_Solver.cpp:405).  Results: A_ij, B_ij, FK_i, SC_i, F_i, RAO_i
    (Hydrodynamic_Solver.h:55-62) and RadSolArray / DiffSolArray
    (Solver_Base.h:148-151).  solve_omegas() runs a whole frequency list in one
    call.  precision: PLAIN_FP64 (the reference's arithmetic) or MIXED.
    """

    def __init__(self, device=0, precision=PLAIN_FP64, refine_tol=1e-12):
        L = lib()
        h = ctypes.c_void_p()
        _check(L.bem_create(ctypes.byref(h), int(device)))
        self._h = h
        self.precision = precision
        self.refine_tol = refine_tol
        self.Rho = 1025.0
        self.Grav = 9.81
        self.BetaArray = []
        self.Frequency = 0.0
        self.N, self.NBeta = 0, 0  # set by Setup
        self.mass = 0.0
        self.cog = np.zeros(3)
        self.gyration = np.zeros((3, 3))
        self.Mass_Mat = None
        self.Stiffness_Mat = None
        self.RadSolArray, self.DiffSolArray = [], []
        self.N = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().bem_destroy(h)
            self._h = None

    def close(self):
        self.__del__()

    # Set_Parameters (Hydrodynamic_Solver.cpp:11-27)
    def Set_Parameters(self, params):
        for name, val in params:
            if name == "WaveAngle":
                self.BetaArray.append(float(val))
            elif name == "Density":
                self.Rho = float(val)
            elif name == "Gravity":
                self.Grav = float(val)
            elif name == "IFR":
                self.IFR = bool(val)
                _check(lib().bem_set_ifr(self._h, int(self.IFR)), self._h)
            elif name == "NKochin":
                self.NKochin = int(val)
                _check(lib().bem_set_kochin(self._h, self.NKochin), self._h)
        b = np.asarray(self.BetaArray, dtype=np.float64)
        _check(lib().bem_set_params(self._h, self.Rho, self.Grav, b.size, _p(b) if b.size else None), self._h)

    def Set_Mass_Properties(self, mass=0.0, cog=(0, 0, 0), gyration=None, Mass_Mat=None, Stiffness_Mat=None):
        self.mass = float(mass)
        self.cog = np.asarray(cog, dtype=np.float64)
        self.gyration = np.zeros((3, 3)) if gyration is None else np.asarray(gyration, dtype=np.float64)
        self.Mass_Mat = None if Mass_Mat is None else np.ascontiguousarray(Mass_Mat, dtype=np.float64)
        self.Stiffness_Mat = None if Stiffness_Mat is None else np.ascontiguousarray(Stiffness_Mat, dtype=np.float64)

    def Setup(self, mesh):
        self.mesh = mesh
        ms = mesh._struct()
        props = _Props()
        props.mass = self.mass
        props.cog[:] = list(self.cog)
        props.gyration[:] = list(self.gyration.ravel())
        props.mass_matrix = _p(self.Mass_Mat)
        props.stiffness = _p(self.Stiffness_Mat)
        aux_s = mesh.aux._struct() if mesh.aux is not None else None
        props.aux = ctypes.pointer(aux_s) if aux_s is not None else None
        _check(lib().bem_setup(self._h, ctypes.byref(ms), ctypes.byref(props)), self._h)
        n, nb = ctypes.c_int(), ctypes.c_int()
        _check(lib().bem_get_sizes(self._h, n, nb), self._h)
        self.N, self.NBeta = n.value, nb.value
        M = np.zeros((6, 6))
        C = np.zeros((6, 6))
        vc = np.zeros(4)
        _check(lib().bem_get_body_matrices(self._h, _p(M), _p(C), _p(vc)), self._h)
        self.M_ij, self.C_ij = M, C
        self.Volume, self.Centre_Buoyancy = vc[0], vc[1:]

    def write_wamit(self, prefix, omegas, out):
        """Result files of solve_omegas(omegas) in the reference's WAMIT formats."""
        write_wamit(prefix, omegas, out, self.BetaArray, self.M_ij, self.C_ij,
                    self.Volume, self.Centre_Buoyancy, self.cog, rho=self.Rho, gravity=self.Grav,
                    wave_points=getattr(self, "wave_points", None))

    def write_bem(self, prefix, omegas, out, file_info=""):
        """The .bem summary file of solve_omegas(omegas) (Hydrodynamic_Solver_IO.cpp:107-426)."""
        aux = getattr(self.mesh, "aux", None)
        write_bem(prefix, omegas, out, self.BetaArray, self.M_ij, self.C_ij, self.Volume, self.Centre_Buoyancy,
                  self.cog, mesh=self.mesh, mass=self.M_ij[0][0], n_aux=0 if aux is None else aux.n,
                  file_info=file_info)

    def Set_Real(self, D):
        self.Frequency = float(D)

    def Solve(self):
        r = self.solve_omegas([self.Frequency * (0.5 / np.pi)], want_phi=True)
        self.A_ij, self.B_ij = r["A"][0], r["B"][0]
        self.FK_i, self.SC_i, self.F_i, self.RAO_i = r["FK"][0], r["SC"][0], r["F"][0], r["RAO"][0]
        self.RadSolArray.append(r["phiJ"])
        self.DiffSolArray.append(r["phiS"])
        return r

    def set_wave_points(self, xyz):
        """Exterior free-surface points (n x 3) for the elevation outputs (the
        reference's Wave_Nodes, Hydrodynamic_Solver.cpp:208-213)."""
        self.wave_points = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        n = self.wave_points.shape[0]
        _check(lib().bem_set_wave_points(self._h, n, _p(self.wave_points) if n else None), self._h)

    def solve_omegas(self, omegas, want_phi=False, precision=None, want_fs=False, want_kochin=False):
        """Solve at the internal angular frequencies `omegas`.  want_fs adds fs_rad
        [f][nw][6] and fs_diff [f][nw][nb] (ExtRadMat / ExtDiffMat at the wave points);
        want_kochin adds kochin_rad [f][nk][6] and kochin_diff [f][nk][nb]."""
        om = np.ascontiguousarray(omegas, dtype=np.float64).ravel()
        nf, nb, N = om.size, self.NBeta, self.N
        out = dict(A=np.zeros((nf, 6, 6)), B=np.zeros((nf, 6, 6)), FK=np.zeros((nf, 6, nb), np.complex128),
                   SC=np.zeros((nf, 6, nb), np.complex128), F=np.zeros((nf, 6, nb), np.complex128),
                   RAO=np.zeros((nf, 6, nb), np.complex128), iters=np.zeros(nf, np.int32),
                   residual=np.zeros(nf))
        res = _Result()
        res.A, res.B = _p(out["A"]), _p(out["B"])
        for k in ("FK", "SC", "F", "RAO"):
            setattr(res, k, _p(out[k].view(np.float64)))
        res.refine_iters = _p(out["iters"], _ip)
        res.residual = _p(out["residual"])
        if want_phi:
            out["phiJ"] = np.zeros((N, 6), np.complex128)
            out["phiS"] = np.zeros((N, nb), np.complex128)
            res.phi_rad = _p(out["phiJ"].view(np.float64))
            res.phi_scat = _p(out["phiS"].view(np.float64)) if nb else None
        if want_fs:
            nw = getattr(self, "wave_points", np.zeros((0, 3))).shape[0]
            out["fs_rad"] = np.zeros((nf, nw, 6), np.complex128)
            out["fs_diff"] = np.zeros((nf, nw, nb), np.complex128)
            res.fs_rad = _p(out["fs_rad"].view(np.float64))
            res.fs_diff = _p(out["fs_diff"].view(np.float64)) if nb else None
        if want_kochin:
            nk = getattr(self, "NKochin", 36)
            out["kochin_rad"] = np.zeros((nf, nk, 6), np.complex128)
            out["kochin_diff"] = np.zeros((nf, nk, nb), np.complex128)
            res.kochin_rad = _p(out["kochin_rad"].view(np.float64))
            res.kochin_diff = _p(out["kochin_diff"].view(np.float64)) if nb else None
        prec = self.precision if precision is None else precision
        _check(lib().bem_solve(self._h, nf, _p(om), int(prec), float(self.refine_tol), ctypes.byref(res)), self._h)
        return out

    # Influence matrices
    def rankine(self):
        N = self.N
        s, sr, d, dr = (np.zeros((N, N)) for _ in range(4))
        _check(lib().bem_get_rankine(self._h, _p(s), _p(sr), _p(d), _p(dr)), self._h)
        return s, sr, d, dr

    def wave_matrices(self, K, precision=PLAIN_FP64):
        N = self.N
        ws = np.zeros((N, N), np.complex128)
        wd = np.zeros((N, N), np.complex128)
        _check(lib().bem_wave_matrices(self._h, float(K), int(precision), _p(ws.view(np.float64)),
                                       _p(wd.view(np.float64))), self._h)
        return ws, wd

    def stage_times(self, reset=False):
        t = np.zeros(6)
        _check(lib().bem_stage_times(self._h, _p(t), int(reset)), self._h)
        return t

    def set_surrogate(self, surrogate, mode="strict", judge_tol=1e-6, judge_fraction=0.01, domain=None):
        """Far-field wave terms from a trained HavelockSurrogate (bem_set_surrogate): mode
        "strict" solves again, with the closed form, every frequency whose judged error
        exceeds judge_tol; "accept" keeps the network's values; None turns it off."""
        m = {None: 0, "off": 0, "strict": 1, "accept": 2}[mode]
        dom = None if domain is None else np.ascontiguousarray(domain, dtype=np.float64)
        self._surrogate = surrogate if m else None  # keeps the network alive while it is used
        _check(lib().bem_set_surrogate(self._h, surrogate._h if m else None, m, float(judge_tol),
                                       float(judge_fraction), _p(dom) if dom is not None else None), self._h)

    def surrogate_stats(self, reset=True):
        """Totals of the surrogate form since the last reset (bem_surrogate_stats)."""
        v = np.zeros(7)
        _check(lib().bem_surrogate_stats(self._h, _p(v), int(reset)), self._h)
        return {"gauss_points_network": int(v[0]), "gauss_points_closed_form": int(v[1]), "judged_pairs": int(v[2]),
                "judged_error_max": float(v[3]), "frequencies_resolved": int(v[4]),
                "frequencies_with_surrogate": int(v[5])}

    def set_tuning(self, key, value):
        _check(lib().bem_set_tuning(self._h, key.encode(), float(value)), self._h)

    def autotune(self, omegas):
        """Times the mixed pipelined solve on the sample frequencies for a small grid of
        schedule settings (bem_autotune) and keeps the fastest on this solver.  Returns
        (ms per frequency of the chosen setting, one report line per setting)."""
        om = np.ascontiguousarray(omegas, dtype=np.float64)
        ms = ctypes.c_double()
        buf = ctypes.create_string_buffer(4096)
        _check(lib().bem_autotune(self._h, int(om.size), om.ctypes.data_as(_dp), ctypes.byref(ms), buf, 4096),
               self._h)
        self.stage_times(reset=True)
        return ms.value, buf.value.decode().splitlines()

    def lu_timeline(self, enable=-1):
        """Per block step of the last mixed LU: ms of [cross start, cross done, inverse done,
        W21 done, panel ready, rest done] (enable=1 starts recording)."""
        n = ctypes.c_int()
        _check(lib().bem_lu_timeline(self._h, int(enable), 0, None, ctypes.byref(n)), self._h)
        out = np.zeros((max(n.value, 1), 6))
        _check(lib().bem_lu_timeline(self._h, -1, n.value, _p(out), ctypes.byref(n)), self._h)
        return out[:n.value]

    def kernel_times(self, reset=False):
        """[wave-assembly kernel ms (summed), launches, panel pairs per launch, 0]."""
        t = np.zeros(4)
        _check(lib().bem_kernel_times(self._h, _p(t), int(reset)), self._h)
        return t


class Aerodynamic_Solver:
    """Drop-in for BEMUse::Aerodynamic_Solver with constant panels
    (Aerodynamic_Solver.cpp:12-180): Setup(mesh) -> Set_External_BC(vels) ->
    Solve_Steady(); the perturbation potential is X (one value per panel)."""

    def __init__(self, device=0, precision=PLAIN_FP64, refine_tol=1e-12):
        L = lib()
        h = ctypes.c_void_p()
        _check(L.bem_create(ctypes.byref(h), int(device)))
        self._h = h
        self.precision = precision
        self.refine_tol = refine_tol
        self.vels = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().bem_destroy(h)
            self._h = None

    def Set_Parameters(self, params):
        for name, _ in params:
            if name == "BilinearPanels":
                raise BEMError(6, "bilinear panels are not implemented (constant panels only)")

    def Setup(self, mesh):
        self.mesh = mesh
        ms = mesh._struct()
        _check(lib().bem_aero_setup(self._h, ctypes.byref(ms)), self._h)
        self.N = mesh.n

    def Set_Wake(self, quads, te_upper, te_lower):
        """Flat constant-doublet wake strips carrying the Kutta jumps
        X[te_upper] - X[te_lower] (no reference counterpart: the reference's steady
        solve has no wake); takes effect at the next Setup."""
        q = np.ascontiguousarray(quads, dtype=np.float64).reshape(-1, 4, 3)
        up = np.ascontiguousarray(te_upper, dtype=np.int32).ravel()
        lo = np.ascontiguousarray(te_lower, dtype=np.int32).ravel()
        if not (q.shape[0] == up.size == lo.size):
            raise BEMError(1, "wake: one Kutta pair per strip")
        _check(lib().bem_aero_set_wake(self._h, q.shape[0], _p(q), _p(up, _ip), _p(lo, _ip)), self._h)

    def Set_External_BC(self, vels):
        self.vels = np.ascontiguousarray(vels, dtype=np.float64).reshape(-1, 3)

    def Surface(self, U, s_ref, X=None):
        """Surface pressure of the solution for the uniform onset flow U: cp per panel
        (1 - |U_t + grad X|^2 / |U|^2, least-squares surface gradient) and the force
        coefficients {CF (3), CL, CD} with CF = sum cp n A / s_ref."""
        X = np.ascontiguousarray(self.X if X is None else X, dtype=np.float64)
        U = np.ascontiguousarray(U, dtype=np.float64).ravel()
        cp = np.zeros(self.N)
        co = np.zeros(5)
        _check(lib().bem_aero_surface(self._h, _p(X), _p(U), float(s_ref), _p(cp), _p(co)), self._h)
        return cp, {"CF": co[:3].copy(), "CL": float(co[3]), "CD": float(co[4])}

    def Solve_Steady(self):
        X = np.zeros(self.N)
        BC = np.zeros(self.N)
        _check(lib().bem_aero_solve(self._h, self.vels.shape[0], _p(self.vels), int(self.precision),
                                    float(self.refine_tol), _p(X), _p(BC)), self._h)
        self.X, self.BC = X, BC
        return X


def havelock_gf(x, y, v, precision=PLAIN_FP64, device=0):
    """HavelockGF (Kernels.cpp:342-412) on the GPU; returns n x 4 complex: G, dGx, dGy, dGz."""
    x, y, v = (np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (x, y, v))
    out = np.zeros((x.size, 8))
    _check(lib().bem_havelock(int(device), x.size, _p(x), _p(y), _p(v), int(precision), _p(out)))
    return out[:, 0::2] + 1j * out[:, 1::2]


class HavelockSurrogate:
    """MLP stand-in for HavelockGF (Kernels.cpp:342-412): inputs (log10 KR, KZ),
    outputs Re/Im of G, dG/dR, dG/dZ; BF16 weights, FP32 accumulation, trained on
    the GPU by the library's own forward/backward kernels (k_mlp.cu)."""

    def __init__(self, device=0, seed=0):
        h = ctypes.c_void_p()
        rc = lib().bem_mlp_create(ctypes.byref(h), int(device), int(seed))
        if rc != 0:
            raise BEMError(rc, lib().bem_last_error(None).decode())
        self._h = h
        self.n_params = int(lib().bem_mlp_num_params())

    def __del__(self):
        if getattr(self, "_h", None):
            lib().bem_mlp_destroy(self._h)
            self._h = None

    def _chk(self, rc):
        if rc != 0:
            raise BEMError(rc, lib().bem_mlp_last_error(self._h).decode())

    def set_normalization(self, in_shift, in_scale, out_shift, out_scale):
        a = [np.ascontiguousarray(v, dtype=np.float64).ravel() for v in (in_shift, in_scale, out_shift, out_scale)]
        self._chk(lib().bem_mlp_set_normalization(self._h, *[_p(v) for v in a]))

    def params(self):
        w = np.zeros(self.n_params)
        self._chk(lib().bem_mlp_get_params(self._h, _p(w)))
        return w

    def set_params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float64)
        self._chk(lib().bem_mlp_set_params(self._h, _p(w)))

    def eval(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 2)
        y = np.zeros((x.shape[0], 6))
        self._chk(lib().bem_mlp_eval(self._h, x.shape[0], _p(x), _p(y)))
        return y

    def eval_tc(self, x):
        """Forward pass on the tensor cores (BF16 activations; bem_mlp_eval_tc)."""
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 2)
        y = np.zeros((x.shape[0], 6))
        self._chk(lib().bem_mlp_eval_tc(self._h, x.shape[0], _p(x), _p(y)))
        return y

    def throughput_tc(self, n=1 << 20):
        r = np.zeros(1)
        self._chk(lib().bem_mlp_throughput_tc(self._h, int(n), _p(r)))
        return float(r[0])

    def grad(self, x, y):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 2)
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(-1, 6)
        g = np.zeros(self.n_params)
        loss = np.zeros(1)
        self._chk(lib().bem_mlp_grad(self._h, x.shape[0], _p(x), _p(y), _p(g), _p(loss)))
        return float(loss[0]), g

    def train(self, x, y, epochs, batch=4096, lr=1e-3, seed=0):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 2)
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(-1, 6)
        losses = np.zeros(max(1, int(epochs)))
        self._chk(lib().bem_mlp_train(self._h, x.shape[0], _p(x), _p(y), int(epochs), int(batch), float(lr),
                                      int(seed), _p(losses)))
        return losses[:int(epochs)]

    def throughput(self, n=1 << 20):
        r = np.zeros(1)
        self._chk(lib().bem_mlp_throughput(self._h, int(n), _p(r)))
        return float(r[0])

    # The domain where the surrogate stands in for HavelockGF: far-field pairs with
    # K R and K Z inside these ranges (the rest is out of domain and keeps the closed form).
    KR_RANGE = (1.0e-3, 20.0)
    KZ_RANGE = (-40.0, 0.0)

    @staticmethod
    def envelope(kr, kz):
        """Per-sample scales of the six outputs (Re/Im of G, dG/dR, dG/dZ) that make the
        targets O(1) over the domain: 2/(d + 0.05) + w for G and dG/dZ (= G in the
        reference form), 2 KR/(d^2 (1 + d)) + w for dG/dR and w = 2 pi e^KZ / sqrt(1 + KR)
        (the wave part's envelope) for the imaginary parts; d = sqrt(KR^2 + KZ^2).  The
        fused assembly kernel computes the same expressions in FP32."""
        kr = np.asarray(kr, dtype=np.float64)
        kz = np.asarray(kz, dtype=np.float64)
        d = np.sqrt(kr * kr + kz * kz)
        w = 2.0 * np.pi * np.exp(kz) / np.sqrt(1.0 + kr)
        eg = 2.0 / (d + 0.05) + w
        er = 2.0 * kr / (d * d * (1.0 + d) + 1e-12) + w
        return np.stack([eg, w, er, w, eg, w], axis=-1)

    @staticmethod
    def domain_set(n, seed=0, device=0):
        """Samples of the surrogate's domain and their targets from the plain FP64
        integrator: inputs (log10 KR, KZ) with KR log-uniform on KR_RANGE and KZ on
        KZ_RANGE (half uniform, half concentrated near the free surface, where the wave
        part is largest); returns inputs x (n x 2), the six outputs y (n x 6) and the
        scaled targets t = y / envelope."""
        rng = np.random.default_rng(seed)
        lo, hi = np.log10(HavelockSurrogate.KR_RANGE[0]), np.log10(HavelockSurrogate.KR_RANGE[1])
        lkr = rng.uniform(lo, hi, n)
        u = rng.uniform(0.0, 1.0, n)
        half = rng.uniform(0.0, 1.0, n) < 0.5
        kz = HavelockSurrogate.KZ_RANGE[0] * np.where(half, u, u ** 3)
        g = havelock_gf(10.0 ** lkr, np.zeros(n), kz, PLAIN_FP64, device)
        y = np.stack([g[:, 0].real, g[:, 0].imag, g[:, 1].real, g[:, 1].imag, g[:, 3].real, g[:, 3].imag], axis=1)
        return np.stack([lkr, kz], axis=1), y, y / HavelockSurrogate.envelope(10.0 ** lkr, kz)

    def set_domain_normalization(self, t):
        """Fixed input normalisation of the domain (log10 KR and KZ mapped to [-1, 1]) and
        per-output standardisation of the scaled targets t."""
        lo, hi = np.log10(self.KR_RANGE[0]), np.log10(self.KR_RANGE[1])
        z0, z1 = self.KZ_RANGE
        self.set_normalization([(lo + hi) / 2, (z0 + z1) / 2], [(hi - lo) / 2, (z1 - z0) / 2], t.mean(0),
                               t.std(0) + 1e-12)

    def predict(self, x, tensor_cores=True):
        """The six outputs at raw inputs x = (log10 KR, KZ): the network's scaled output
        times the envelope."""
        x = np.asarray(x, dtype=np.float64).reshape(-1, 2)
        t = self.eval_tc(x) if tensor_cores else self.eval(x)
        return t * self.envelope(10.0 ** x[:, 0], x[:, 1])

    @staticmethod
    def training_set(n, seed=0, device=0, kr=(1e-3, 200.0), kz=(-100.0, 0.0)):
        """Inputs (log10 KR, KZ) with KR log-uniform and KZ uniform, and targets from the
        plain FP64 integrator: Re/Im of G, dG/dR (= dG/dx at y = 0), dG/dZ."""
        rng = np.random.default_rng(seed)
        lkr = rng.uniform(np.log10(kr[0]), np.log10(kr[1]), n)
        z = rng.uniform(kz[0], kz[1], n)
        g = havelock_gf(10.0 ** lkr, np.zeros(n), z, PLAIN_FP64, device)
        y = np.stack([g[:, 0].real, g[:, 0].imag, g[:, 1].real, g[:, 1].imag, g[:, 3].real, g[:, 3].imag], axis=1)
        return np.stack([lkr, z], axis=1), y


def batch_solve(meshes, omegas, betas=(0.0,), precision=MIXED, n_workers=8, refine_tol=1e-12, density=1025.0,
                gravity=9.81, device=0):
    """Independent bodies at the same frequencies (bem_batch_solve): returns a list of
    per-body dicts (A, B, FK, SC, F, RAO, iters) and the wall time in seconds."""
    om = np.ascontiguousarray(omegas, dtype=np.float64).ravel()
    b = np.ascontiguousarray(betas, dtype=np.float64).ravel()
    nf, nb, n = om.size, b.size, len(meshes)
    structs = (_Mesh * n)()
    keep = []
    for i, m in enumerate(meshes):
        ms = m._struct()
        keep.append(ms)
        structs[i] = ms
    outs, res = [], (_Result * n)()
    for i in range(n):
        o = dict(A=np.zeros((nf, 6, 6)), B=np.zeros((nf, 6, 6)), FK=np.zeros((nf, 6, nb), np.complex128),
                 SC=np.zeros((nf, 6, nb), np.complex128), F=np.zeros((nf, 6, nb), np.complex128),
                 RAO=np.zeros((nf, 6, nb), np.complex128), iters=np.zeros(nf, np.int32), residual=np.zeros(nf))
        outs.append(o)
        r = res[i]
        r.A, r.B = _p(o["A"]), _p(o["B"])
        for k in ("FK", "SC", "F", "RAO"):
            setattr(r, k, _p(o[k].view(np.float64)))
        r.refine_iters = _p(o["iters"], _ip)
        r.residual = _p(o["residual"])
    sec = np.zeros(1)
    _check(lib().bem_batch_solve(int(device), n, structs, None, float(density), float(gravity), nb,
                                 _p(b) if nb else None, nf, _p(om), int(precision), float(refine_tol),
                                 int(n_workers), res, _p(sec)))
    return outs, float(sec[0])


def havelock_throughput(n=1 << 22, precision=MIXED, device=0):
    """Closed-form HavelockGF evaluations per second of device time."""
    r = np.zeros(1)
    _check(lib().bem_havelock_throughput(int(device), int(n), int(precision), _p(r)))
    return float(r[0])


def launch_count():
    """Kernel launches issued by libbemgpu.so in this process."""
    return int(lib().bem_launch_count())


def fp32_peak(device=0):
    """Measured FP32 FMA throughput of the device in TFLOP/s (bem_fp32_peak)."""
    t = ctypes.c_double()
    _check(lib().bem_fp32_peak(int(device), ctypes.byref(t)))
    return t.value


def cusolver_zgetrf_ms(n, device=0):
    """Device time in ms of cuSOLVER's complex LU with partial pivoting at order n
    (bem_cusolver_zgetrf_ms): the library figure beside the plain FP64 path's LU."""
    t = ctypes.c_double()
    _check(lib().bem_cusolver_zgetrf_ms(int(device), int(n), ctypes.byref(t)))
    return t.value


def _planar32(z):
    z = np.asarray(z)
    return np.ascontiguousarray(np.stack([z.real, z.imag]).astype(np.float32))


def tc_probe(mode, C, Wa=None, Ua=None, Wb=None, Ub=None, T=None, device=0):
    """One launch of the tensor-core product kernel in tile mode `mode` (bem_tc_probe)
    on complex operands (C n x n; Wa, Ua, Wb, Ub n x 128; T 128 x 128 or
    (n / 256) x 128 x 128), stored as FP32 planes.  Returns the updated C and, for
    mode 3, the second destination W (n x 128)."""
    n = C.shape[0]
    c = _planar32(C)
    ops = [None if x is None else _planar32(x) for x in (Wa, Ua, Wb, Ub, T)]
    w = np.zeros((2, n, 128), np.float32)
    fp = lambda a: None if a is None else a.ctypes.data_as(_fp)
    st = lib().bem_tc_probe(int(device), int(mode), int(n), fp(c), *[fp(x) for x in ops], fp(w))
    if st != 0:
        raise BEMError(st, lib().bem_last_error(None).decode())
    return c[0] + 1j * c[1].astype(np.float64), w[0] + 1j * w[1].astype(np.float64)


def dense_solve(A, B, precision=PLAIN_FP64, refine_tol=1e-12, device=0):
    """Solve A X = B (complex) with the GPU LU; returns (X, refine_iters, residual)."""
    A = np.ascontiguousarray(A, dtype=np.complex128)
    B = np.array(B, dtype=np.complex128, order="C")
    squeeze = B.ndim == 1
    if squeeze:
        B = B[:, None].copy()
    L = lib()
    h = ctypes.c_void_p()
    _check(L.bem_create(ctypes.byref(h), int(device)))
    try:
        it, res = ctypes.c_int(), ctypes.c_double()
        _check(L.bem_dense_solve(h, A.shape[0], _p(A.view(np.float64)), B.shape[1], _p(B.view(np.float64)),
                                 int(precision), float(refine_tol), it, res), h)
    finally:
        L.bem_destroy(h)
    return (B[:, 0] if squeeze else B), it.value, res.value
