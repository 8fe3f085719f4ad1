// host_mesh.cpp -- mesh generators and panel geometry (host, FP64).
//
// Mesh generators restate the reference's Boundary classes:
//   Half_Cylinder / Volume_of_Revolution  src/Boundary/Volume_of_Revolution.cpp:12-199
//   Barge                                 src/Boundary/Barge.cpp:12-204
// Panel geometry restates src/Geometry/Geo_Elements.cpp:45-214 (centroid,
// normal, area, 2x2 Gauss-Legendre / 3-point Dunavant nodes), the panel frame
// of CoordSys.h:87-94 (rows = q*UnitX, q*UnitY, q*UnitZ with
// q = Quaternion::FromTwoVectors(UnitZ, n)) and the mirror images of
// Boundary_Base.cpp:51-85.
#include "host_geom.h"
#include <algorithm>
#include <cmath>

namespace bem {

namespace {
const double kPi = 3.14159265358979323846;

struct V { double x, y, z; };
inline V mk(double a, double b, double c) { return V{a, b, c}; }
inline V operator+(V a, V b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V operator-(V a, V b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V operator*(V a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
inline V crossv(V a, V b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline double len(V a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline V unit(V a) { double n = len(a); return n > 0 ? mk(a.x / n, a.y / n, a.z / n) : a; }

// Rotation taking +z onto n (Eigen's setFromTwoVectors algorithm: axis = z x n,
// w = sqrt(2(1+c))/2; for n = -z, a half turn about x), returned as the three
// rotated unit axes.
void frame_from_normal(V n, V& ex, V& ey, V& ez) {
    V v1 = unit(n);
    double c = v1.z;
    double w;
    V qv;
    if (c < -1.0 + 1e-12) {
        c = std::max(c, -1.0);
        double w2 = (1.0 + c) * 0.5;
        w = std::sqrt(w2);
        qv = mk(std::sqrt(1.0 - w2), 0, 0);
    } else {
        V axis = crossv(mk(0, 0, 1), v1);
        double s = std::sqrt((1.0 + c) * 2.0);
        qv = axis * (1.0 / s);
        w = s * 0.5;
    }
    auto rot = [&](V v) {
        V uv = crossv(qv, v);
        uv = uv + uv;
        return v + uv * w + crossv(qv, uv);
    };
    ex = rot(mk(1, 0, 0));
    ey = rot(mk(0, 1, 0));
    ez = rot(mk(0, 0, 1));
}

inline double pi_cos_fac(int i, int itot) { return 0.5 * (1.0 - std::cos(i * kPi / (itot - 1))); }

void make_panel(int nv, const V* pl, V origin, PanelGeom& p) {
    p.nv = nv;
    V n;
    V pc;
    if (nv == 3) {
        pc = (pl[0] + pl[1] + pl[2]) * (1.0 / 3.0);
        V X1 = pl[0] - (pl[1] + pl[2]) * 0.5;
        V X2 = pl[2] - pl[1];
        V X3 = crossv(X1, X2);
        p.area = 0.5 * len(X3);
        n = unit(X3);
    } else {
        pc = (pl[0] + pl[1] + pl[2] + pl[3]) * 0.25;
        V X1 = (pl[3] + pl[2]) * 0.5 - (pl[0] + pl[1]) * 0.5;
        V X2 = (pl[2] + pl[1]) * 0.5 - (pl[3] + pl[0]) * 0.5;
        n = unit(crossv(X1, X2));
        p.area = 0.5 * len(crossv(pl[2] - pl[0], pl[3] - pl[1]));
    }
    V ex, ey, ez;
    frame_from_normal(n, ex, ey, ez);
    V c = pc + origin;
    p.c[0] = c.x; p.c[1] = c.y; p.c[2] = c.z;
    p.e[0] = ex.x; p.e[1] = ex.y; p.e[2] = ex.z;
    p.e[3] = ey.x; p.e[4] = ey.y; p.e[5] = ey.z;
    p.e[6] = ez.x; p.e[7] = ez.y; p.e[8] = ez.z;
    for (int k = 0; k < 4; ++k) {
        V g = pl[k < nv ? k : nv - 1] + origin;
        p.v[3 * k] = g.x; p.v[3 * k + 1] = g.y; p.v[3 * k + 2] = g.z;
    }
    // Quadrature nodes on the panel (bilinear / linear map of the vertices).
    for (int k = 0; k < 4; ++k) { p.qw[k] = 0; p.qp[3 * k] = p.qp[3 * k + 1] = p.qp[3 * k + 2] = 0; }
    if (nv == 3) {
        const double a = 0.666666666666667, b = 0.166666666666667, wt = 0.333333333333333;
        const double xi_[3] = {a, b, b}, eta_[3] = {b, b, a};
        p.nq = 3;
        V Rxi = pl[2] - pl[0], Reta = pl[1] - pl[0];
        V Rn = crossv(Rxi, Reta);
        double jac = len(Rn);
        V qe1, qe2, qn;
        frame_from_normal(unit(Rn), qe1, qe2, qn);
        for (int i = 0; i < 3; ++i) {
            V P = pl[0] * (1. - xi_[i] - eta_[i]) + pl[1] * eta_[i] + pl[2] * xi_[i] + origin;
            p.qp[3 * i] = P.x; p.qp[3 * i + 1] = P.y; p.qp[3 * i + 2] = P.z;
            p.qw[i] = jac * (wt * 0.5);
            p.qn[3 * i] = qn.x; p.qn[3 * i + 1] = qn.y; p.qn[3 * i + 2] = qn.z;
        }
    } else {
        const double g = 1.0 / std::sqrt(3.0);
        const double pt[2] = {-g, g};
        p.nq = 4;
        int k = 0;
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j) {
                double px = pt[i], py = pt[j];
                V P = pl[0] * (0.25 * (1 - px) * (1 - py)) + pl[1] * (0.25 * (1 - px) * (1 + py)) +
                      pl[2] * (0.25 * (1 + px) * (1 + py)) + pl[3] * (0.25 * (1 + px) * (1 - py));
                V Rxi = pl[0] * (-0.25 * (1 - py)) + pl[1] * (-0.25 * (1 + py)) + pl[2] * (0.25 * (1 + py)) +
                        pl[3] * (0.25 * (1 - py));
                V Reta = pl[0] * (-0.25 * (1 - px)) + pl[1] * (0.25 * (1 - px)) + pl[2] * (0.25 * (1 + px)) +
                         pl[3] * (-0.25 * (1 + px));
                V Rn = crossv(Rxi, Reta);
                double jac = len(Rn);
                V qe1, qe2, qn;
                frame_from_normal(unit(Rn), qe1, qe2, qn);
                P = P + origin;
                p.qp[3 * k] = P.x; p.qp[3 * k + 1] = P.y; p.qp[3 * k + 2] = P.z;
                p.qw[k] = jac;
                p.qn[3 * k] = qn.x; p.qn[3 * k + 1] = qn.y; p.qn[3 * k + 2] = qn.z;
                ++k;
            }
    }
}
}  // namespace

bool build_geometry(const MeshView& m, std::vector<PanelGeom>& body, std::vector<PanelGeom>& mirror,
                    std::string& err) {
    if (m.n_elems <= 0 || m.n_nodes <= 0 || !m.nodes || !m.elems) { err = "empty mesh"; return false; }
    body.resize(m.n_elems);
    mirror.resize(m.n_elems);
    int ncomp = m.n_comp > 0 ? m.n_comp : 1;
    for (int c = 0; c < ncomp; ++c) {
        int e0 = m.n_comp > 0 ? m.comp_first[c] : 0;
        int e1 = m.n_comp > 0 ? m.comp_first[c + 1] : m.n_elems;
        if (e0 < 0 || e1 > m.n_elems || e0 > e1) { err = "bad component element range"; return false; }
        V org = m.n_comp > 0 ? mk(m.comp_origin[3 * c], m.comp_origin[3 * c + 1], m.comp_origin[3 * c + 2])
                             : mk(0, 0, 0);
        for (int e = e0; e < e1; ++e) {
            const int* el = m.elems + 4 * (size_t)e;
            int nv = el[3] < 0 ? 3 : 4;
            V pl[4], pm[4];
            for (int k = 0; k < nv; ++k) {
                int id = el[k];
                if (id < 0 || id >= m.n_nodes) { err = "element references a missing node"; return false; }
                pl[k] = mk(m.nodes[3 * (size_t)id], m.nodes[3 * (size_t)id + 1], m.nodes[3 * (size_t)id + 2]);
            }
            for (int k = 0; k < nv; ++k) {
                V g = pl[nv - 1 - k] + org;  // reversed winding, z -> -z
                g.z *= -1.0;
                pm[k] = g;
            }
            make_panel(nv, pl, org, body[e]);
            make_panel(nv, pm, mk(0, 0, 0), mirror[e]);
            if (!(body[e].area > 0)) { err = "degenerate panel (zero area)"; return false; }
        }
    }
    return true;
}

// Vertices in the panel frame, edge slopes and lengths (Panel.cpp:86-146).
void rankine_record(const PanelGeom& p, double* rec) {
    for (int i = 0; i < RK_STRIDE; ++i) rec[i] = 0;
    rec[0] = p.nv;
    for (int i = 0; i < 3; ++i) rec[1 + i] = p.c[i];
    for (int i = 0; i < 9; ++i) rec[4 + i] = p.e[i];
    double lx[4], ly[4];
    for (int k = 0; k < p.nv; ++k) {
        double dx = p.v[3 * k] - p.c[0], dy = p.v[3 * k + 1] - p.c[1], dz = p.v[3 * k + 2] - p.c[2];
        lx[k] = p.e[0] * dx + p.e[1] * dy + p.e[2] * dz;
        ly[k] = p.e[3] * dx + p.e[4] * dy + p.e[5] * dz;
        rec[13 + k] = lx[k];
        rec[17 + k] = ly[k];
    }
    for (int k = 0; k < p.nv; ++k) {
        int k1 = (k + 1) % p.nv;
        rec[21 + k] = (ly[k1] - ly[k]) / (lx[k1] - lx[k]);
        rec[25 + k] = std::sqrt((lx[k1] - lx[k]) * (lx[k1] - lx[k]) + (ly[k1] - ly[k]) * (ly[k1] - ly[k]));
    }
}

void collocation_points(const std::vector<PanelGeom>& body, std::vector<double>& xr) {
    const size_t N = body.size();
    xr.assign(3 * N, 0.0);
    for (size_t i = 0; i < N; ++i)
        for (int d = 0; d < 3; ++d) xr[d * N + i] = body[i].c[d] + 1.e-5 * body[i].e[6 + d];
}

// ---- generators -------------------------------------------------------------
void cylinder_sizes(int NA, int NR, int NV, int NRFS, int* nn, int* ne, int* nna, int* nea) {
    int NZ = NR + NV;
    *nn = 1 + NZ * NA;
    *ne = NA * NZ;
    *nna = NRFS > 0 ? 1 + NRFS * NA : 0;
    *nea = NRFS > 0 ? NA * NRFS : 0;
}

void cylinder_mesh(double R, double draft, int NA, int NR, int NV, int NRFS, bool cosine, double* nodes, int* elems,
                   double* aux_nodes, int* aux_elems) {
    const double Z = -draft;
    std::vector<double> pr, pz;  // perimeter (r, z), bottom centre first
    for (int i = 0; i < NR; ++i) {
        pr.push_back(cosine ? R * pi_cos_fac(i, NR + 1) : R * i / NR);
        pz.push_back(Z);
    }
    for (int i = 0; i <= NV; ++i) {
        pr.push_back(R);
        pz.push_back(cosine ? Z * (1.0 - pi_cos_fac(i, NV + 1)) : Z * (1.0 - 1.0 * i / NV));
    }
    const int NZ = (int)pr.size() - 1;
    size_t k = 0;
    for (int i = 0; i <= NZ; ++i) {
        int nar = i == 0 ? 1 : NA;
        for (int j = 0; j < nar; ++j, ++k) {
            double u = j * (2.0 * kPi) / nar;
            nodes[3 * k] = pr[i] * std::cos(u);
            nodes[3 * k + 1] = pr[i] * std::sin(u);
            nodes[3 * k + 2] = pz[i];
        }
    }
    auto id = [&](int a, int z) {
        if (z == 0) return 0;
        int aa = a >= NA ? a - NA : (a < 0 ? a + NA : a);
        return 1 + (z - 1) * NA + aa;
    };
    size_t e = 0;
    for (int i = 0; i < NA; ++i, ++e) {
        elems[4 * e] = id(0, 0); elems[4 * e + 1] = id(i + 1, 1); elems[4 * e + 2] = id(i, 1); elems[4 * e + 3] = -1;
    }
    for (int z = 1; z < NZ; ++z)
        for (int i = 0; i < NA; ++i, ++e) {
            elems[4 * e] = id(i, z); elems[4 * e + 1] = id(i + 1, z);
            elems[4 * e + 2] = id(i + 1, z + 1); elems[4 * e + 3] = id(i, z + 1);
        }
    if (NRFS > 0 && aux_nodes && aux_elems) {
        k = 0;
        for (int i = 0; i <= NRFS; ++i) {
            double r = cosine ? R * pi_cos_fac(i, NRFS + 1) : R * i / NRFS;
            int nar = i == 0 ? 1 : NA;
            for (int j = 0; j < nar; ++j, ++k) {
                double u = j * (2.0 * kPi) / nar;
                aux_nodes[3 * k] = r * std::cos(u); aux_nodes[3 * k + 1] = r * std::sin(u); aux_nodes[3 * k + 2] = 0.0;
            }
        }
        e = 0;
        for (int i = 0; i < NA; ++i, ++e) {
            aux_elems[4 * e] = id(0, 0); aux_elems[4 * e + 1] = id(i, 1); aux_elems[4 * e + 2] = id(i + 1, 1);
            aux_elems[4 * e + 3] = -1;
        }
        for (int z = 1; z < NRFS; ++z)
            for (int i = 0; i < NA; ++i, ++e) {
                aux_elems[4 * e] = id(i, z + 1); aux_elems[4 * e + 1] = id(i + 1, z + 1);
                aux_elems[4 * e + 2] = id(i + 1, z); aux_elems[4 * e + 3] = id(i, z);
            }
    }
}

void barge_sizes(int NX, int NY, int NZ, int* nn, int* ne, int* nna, int* nea) {
    *nn = 2 * (NY + 1) * (NZ + 1) + 2 * (NX + 1) * (NZ + 1) + (NX + 1) * (NY + 1);
    *ne = 2 * NY * NZ + 2 * NX * NZ + NX * NY;
    *nna = (NX + 1) * (NY + 1);
    *nea = NX * NY;
}

void barge_mesh(double L, double W, double D, int NX, int NY, int NZ, bool cosine, double* nodes, int* elems,
                double* aux_nodes, int* aux_elems) {
    auto f = [&](int i, int n) { return cosine ? pi_cos_fac(i, n + 1) : 1.0 * i / n; };
    const int sx = (NY + 1) * (NZ + 1), sy = (NX + 1) * (NZ + 1);
    const int x1 = 0, x2 = sx, y1 = 2 * sx, y2 = 2 * sx + sy, zf = 2 * sx + 2 * sy;
    auto put = [&](int idx, double x, double y, double z) {
        nodes[3 * idx] = x; nodes[3 * idx + 1] = y; nodes[3 * idx + 2] = z;
    };
    for (int j = 0; j <= NY; ++j)
        for (int k = 0; k <= NZ; ++k) {
            double y = cosine ? -0.5 * W + W * f(j, NY) : -0.5 * W + W * j / NY;
            double z = cosine ? -D + D * f(k, NZ) : -D + D * k / NZ;
            put(x1 + j * (NZ + 1) + k, -0.5 * L, y, z);
            put(x2 + j * (NZ + 1) + k, 0.5 * L, y, z);
        }
    for (int i = 0; i <= NX; ++i)
        for (int k = 0; k <= NZ; ++k) {
            double x = cosine ? -0.5 * L + L * f(i, NX) : -0.5 * L + L * i / NX;
            double z = cosine ? -D + D * f(k, NZ) : -D + D * k / NZ;
            put(y1 + i * (NZ + 1) + k, x, -0.5 * W, z);
            put(y2 + i * (NZ + 1) + k, x, 0.5 * W, z);
        }
    for (int i = 0; i <= NX; ++i)
        for (int j = 0; j <= NY; ++j) {
            double x = cosine ? -0.5 * L + L * f(i, NX) : -0.5 * L + L * i / NX;
            double y = cosine ? -0.5 * W + W * f(j, NY) : -0.5 * W + W * j / NY;
            put(zf + i * (NY + 1) + j, x, y, -D);
        }
    size_t e = 0;
    auto quad = [&](int a, int b, int c, int d) {
        elems[4 * e] = a; elems[4 * e + 1] = b; elems[4 * e + 2] = c; elems[4 * e + 3] = d; ++e;
    };
    for (int j = 0; j < NY; ++j)
        for (int k = 0; k < NZ; ++k) {
            int a = j * (NZ + 1) + k, b = (j + 1) * (NZ + 1) + k;
            quad(x1 + a, x1 + a + 1, x1 + b + 1, x1 + b);
            quad(x2 + a, x2 + b, x2 + b + 1, x2 + a + 1);
        }
    for (int i = 0; i < NX; ++i)
        for (int k = 0; k < NZ; ++k) {
            int a = i * (NZ + 1) + k, b = (i + 1) * (NZ + 1) + k;
            quad(y1 + a, y1 + b, y1 + b + 1, y1 + a + 1);
            quad(y2 + a, y2 + a + 1, y2 + b + 1, y2 + b);
        }
    for (int i = 0; i < NX; ++i)
        for (int j = 0; j < NY; ++j) {
            int a = i * (NY + 1) + j, b = (i + 1) * (NY + 1) + j;
            quad(zf + a, zf + a + 1, zf + b + 1, zf + b);
        }
    if (aux_nodes && aux_elems) {
        size_t k = 0;
        for (int i = 0; i <= NX; ++i)
            for (int j = 0; j <= NY; ++j, ++k) {
                double x = cosine ? -0.5 * L + L * f(i, NX) : -0.5 * L + L * i / NX;
                // Barge.cpp:115 uses i (not j) for y in the linear branch; kept.
                double y = cosine ? -0.5 * W + W * f(j, NY) : -0.5 * W + W * i / NY;
                aux_nodes[3 * k] = x; aux_nodes[3 * k + 1] = y; aux_nodes[3 * k + 2] = 0.0;
            }
        e = 0;
        for (int i = 0; i < NX; ++i)
            for (int j = 0; j < NY; ++j, ++e) {
                aux_elems[4 * e] = i * (NY + 1) + j; aux_elems[4 * e + 1] = (i + 1) * (NY + 1) + j;
                aux_elems[4 * e + 2] = (i + 1) * (NY + 1) + j + 1; aux_elems[4 * e + 3] = i * (NY + 1) + j + 1;
            }
    }
}

// Rectangular wing of a symmetric NACA 00xx section (chord c, span b, thickness
// ratio t): half-cosine chordwise spacing on both surfaces, uniform spanwise
// strips, open tips.  Section nodes run from the trailing edge along the lower
// surface to the leading edge and back along the upper surface; the trailing
// edge is closed (thickness coefficient -0.1036, Airfoil_Profiles.h:93).
// x chordwise (0 = leading edge), y spanwise (centred), z thickness; panel
// normals point into the wing, as the reference's body panels do.
void wing_sizes(int nc, int ns, int* nn, int* ne) {
    *nn = nc * (ns + 1);
    *ne = nc * ns;
}

void wing_mesh(double chord, double span, double t, int nc, int ns, bool cosine, double* nodes, int* elems) {
    const int half = nc / 2;
    std::vector<double> xs(nc), zs(nc);
    for (int k = 0; k < nc; ++k) {
        // k = 0: trailing edge; k = half: leading edge
        int i = k <= half ? half - k : k - half;                 // chordwise station 0..half
        double f = cosine ? 0.5 * (1.0 - std::cos(kPi * i / half)) : 1.0 * i / half;
        double x = f;
        double yt = 5.0 * t * (0.2969 * std::sqrt(x) - 0.1260 * x - 0.3516 * x * x + 0.2843 * x * x * x -
                               0.1036 * x * x * x * x);
        xs[k] = chord * x;
        zs[k] = chord * (k <= half ? -yt : yt);
    }
    for (int j = 0; j <= ns; ++j) {
        double y = -0.5 * span + span * j / ns;
        for (int k = 0; k < nc; ++k) {
            size_t id = (size_t)j * nc + k;
            nodes[3 * id] = xs[k];
            nodes[3 * id + 1] = y;
            nodes[3 * id + 2] = zs[k];
        }
    }
    size_t e = 0;
    for (int j = 0; j < ns; ++j)
        for (int k = 0; k < nc; ++k, ++e) {
            int k1 = (k + 1) % nc;
            elems[4 * e] = j * nc + k;
            elems[4 * e + 1] = j * nc + k1;
            elems[4 * e + 2] = (j + 1) * nc + k1;
            elems[4 * e + 3] = (j + 1) * nc + k;
        }
}

// Flat trailing wake of the rectangular wing of wing_mesh: one constant-doublet strip per
// spanwise panel column, from the trailing edge (x = chord, z = 0) to length chords
// downstream, vertices ordered so the strip's normal points down (-z).  The Kutta
// pairing of strip j: upper trailing-edge panel j nc + nc - 1, lower j nc.
void wing_wake(double chord, double span, int nc, int ns, double length, double* quads, int* te_up, int* te_lo) {
    for (int j = 0; j < ns; ++j) {
        const double y0 = -0.5 * span + span * j / ns, y1 = -0.5 * span + span * (j + 1) / ns;
        const double x0 = chord, x1 = chord * (1.0 + length);
        const double v[4][3] = {{x0, y0, 0.0}, {x1, y0, 0.0}, {x1, y1, 0.0}, {x0, y1, 0.0}};
        for (int k = 0; k < 4; ++k)
            for (int d = 0; d < 3; ++d) quads[12 * (size_t)j + 3 * k + d] = v[k][d];
        te_up[j] = j * nc + nc - 1;
        te_lo[j] = j * nc;
    }
}

// Calculate_Volume / Calculate_COB (Boundary_Base.cpp:177-224, with
// Calculate_GridParams :125-150 for the zero clean-up), Calculate_Mass_Matrix
// and Calculate_Hydrostatic_Stiffness_Matrix (Hydrodynamic_Solver.cpp:300-397).
void mass_and_stiffness(const std::vector<PanelGeom>& body, const std::vector<PanelGeom>* aux, double rho, double g,
                        double mass, const double* cog, const double* gyr, double* M, double* C, double* vc) {
    double Vx = 0, Vy = 0, Vz = 0;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (const PanelGeom& p : body) {
        const double* n = p.e + 6;
        Vx += -p.c[0] * n[0] * p.area;
        Vy += -p.c[1] * n[1] * p.area;
        Vz += -p.c[2] * n[2] * p.area;
        for (int k = 0; k < p.nv; ++k)
            for (int d = 0; d < 3; ++d) {
                lo[d] = std::min(lo[d], p.v[3 * k + d]);
                hi[d] = std::max(hi[d], p.v[3 * k + d]);
            }
    }
    double V = (Vx + Vy + Vz) / 3.0;
    double maxdim = 0;
    for (int d = 0; d < 3; ++d) maxdim = std::max(maxdim, hi[d] - lo[d]);
    double cb[3] = {0, 0, 0};
    for (const PanelGeom& p : body) {
        const double* n = p.e + 6;
        for (int d = 0; d < 3; ++d) cb[d] -= n[d] * p.c[d] * p.c[d] * p.area;
    }
    for (int d = 0; d < 3; ++d) {
        cb[d] *= 0.5 / V;
        if (std::fabs(cb[d]) < maxdim * 1e-6) cb[d] = 0;
    }
    vc[0] = V; vc[1] = cb[0]; vc[2] = cb[1]; vc[3] = cb[2];
    const double Mass = mass == 0 ? V * 1025.0 : mass;
    for (int i = 0; i < 36; ++i) { M[i] = 0; C[i] = 0; }
    M[0 * 6 + 0] = M[1 * 6 + 1] = M[2 * 6 + 2] = Mass;
    M[0 * 6 + 4] = Mass * cog[2];
    M[1 * 6 + 3] = -Mass * cog[2];
    M[0 * 6 + 5] = -Mass * cog[1];
    M[2 * 6 + 3] = Mass * cog[1];
    M[1 * 6 + 5] = Mass * cog[0];
    M[2 * 6 + 4] = -Mass * cog[0];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            M[(3 + i) * 6 + j] = -M[i * 6 + 3 + j];
            M[(3 + i) * 6 + 3 + j] = Mass * gyr[3 * i + j] * std::fabs(gyr[3 * i + j]);
        }
    double AFS = 0, Mx = 0, My = 0, Mxx = 0, Mxy = 0, Myy = 0;
    if (aux)
        for (const PanelGeom& p : *aux) {
            AFS += p.area;
            My += p.area * p.c[1];
            Mx += p.area * p.c[0];
            Mxy += p.area * p.c[0] * p.c[1];
            Mxx += p.area * p.c[0] * p.c[0];
            Myy += p.area * p.c[1] * p.c[1];
        }
    const double rw = 1025.0;  // the reference mixes Rho and the Rho_wat constant (:372-391)
    C[2 * 6 + 2] = rho * g * AFS;
    C[2 * 6 + 3] = rho * g * My;
    C[2 * 6 + 4] = -rho * g * Mx;
    C[3 * 6 + 3] = rho * g * Myy + rw * g * V * cb[2] - Mass * g * cog[2];
    C[3 * 6 + 4] = -rho * g * Mxy;
    C[3 * 6 + 5] = -rho * g * V * cb[0] + Mass * g * cog[0];
    C[4 * 6 + 4] = rho * g * Mxx + rw * g * V * cb[2] - Mass * g * cog[2];
    C[4 * 6 + 5] = -rho * g * V * cb[1] + Mass * g * cog[1];
    // :394-396 copy the (zero) lower entries over the upper ones; kept.
    C[2 * 6 + 3] = C[3 * 6 + 2];
    C[2 * 6 + 4] = C[4 * 6 + 2];
    C[3 * 6 + 4] = C[4 * 6 + 3];
}

}  // namespace bem
