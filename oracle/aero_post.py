"""Post-processing of the steady constant-panel solve with a trailing wake, restated in
numpy (test infrastructure only; the library computes the same quantities in
bem_aero_surface).  Not in the reference, whose Aerodynamic_Solver stops at the surface
potential (Aerodynamic_Solver.cpp:169-180); defined here:

  * wake of the rectangular wing: strip j is the flat quad from the trailing edge
    (x = chord, z = 0) to `length` chords downstream over panel column j, normal
    pointing down; its Kutta pair is (upper trailing-edge panel j nc + nc - 1, lower j nc);
  * surface velocity: V = U - (U . n) n + grad_s X, with grad_s X the least-squares
    gradient of the panel potentials X in each panel's tangent plane over its edge
    neighbours that face the same side (n_i . n_j > 0, so the two sides of the sharp
    trailing edge do not mix);
  * Cp = 1 - |V|^2 / |U|^2;  force coefficient CF = sum_i Cp_i n_i A_i / S_ref (n into
    the body), CL = CF . e_L with e_L the unit vector normal to U in the x-z plane
    (+z for U along +x), CD = CF . U / |U|."""
import numpy as np


def wing_wake(chord, span, nc, ns, length=20.0):
    quads = np.zeros((ns, 4, 3))
    for j in range(ns):
        y0, y1 = -0.5 * span + span * j / ns, -0.5 * span + span * (j + 1) / ns
        x0, x1 = chord, chord * (1.0 + length)
        quads[j] = [[x0, y0, 0.0], [x1, y0, 0.0], [x1, y1, 0.0], [x0, y1, 0.0]]
    te_up = np.array([j * nc + nc - 1 for j in range(ns)], np.int32)
    te_lo = np.array([j * nc for j in range(ns)], np.int32)
    return quads, te_up, te_lo


def edge_neighbours(elems, normals):
    edges = {}
    for e, el in enumerate(elems):
        ids = [int(i) for i in el if i >= 0]
        for k in range(len(ids)):
            key = tuple(sorted((ids[k], ids[(k + 1) % len(ids)])))
            edges.setdefault(key, []).append(e)
    nbr = [[] for _ in range(len(elems))]
    for pans in edges.values():
        for a in pans:
            for b in pans:
                if a != b and np.dot(normals[a], normals[b]) > 0.0:
                    nbr[a].append(b)
    return nbr


def surface(panels, elems, X, U, s_ref):
    """panels: oracle panel records (Oracle.panels); returns (cp, CF, CL, CD)."""
    c, ex, ey, n, area = panels[:, 13:16], panels[:, 16:19], panels[:, 19:22], panels[:, 22:25], panels[:, 25]
    U = np.asarray(U, dtype=np.float64)
    nbr = edge_neighbours(elems, n)
    N = len(X)
    cp = np.zeros(N)
    for i in range(N):
        A = np.zeros((2, 2))
        b = np.zeros(2)
        for j in nbr[i]:
            d = c[j] - c[i]
            t = np.array([d @ ex[i], d @ ey[i]])
            A += np.outer(t, t)
            b += (X[j] - X[i]) * t
        g = np.linalg.solve(A, b) if abs(np.linalg.det(A)) > 1e-300 else np.zeros(2)
        V = U - (U @ n[i]) * n[i] + g[0] * ex[i] + g[1] * ey[i]
        cp[i] = 1.0 - (V @ V) / (U @ U)
    CF = (cp[:, None] * n * area[:, None]).sum(axis=0) / s_ref
    eL = np.array([-U[2], 0.0, U[0]]) / np.hypot(U[0], U[2])
    return cp, CF, float(CF @ eL), float(CF @ U / np.linalg.norm(U))
