// bem_oracle.cpp -- FP64 CPU restatement of the reference's frequency-domain
// panel-method path (ZeppSav/BEMUse).  TEST INFRASTRUCTURE ONLY: this file is
// the oracle that the GPU library is checked against.  It is never linked into,
// loaded by, or called from the product path (bemuse_gb300/).  Tests, smoke()
// and bench.py's CPU-baseline leg are its only callers.
//
// Every function cites the reference file:line it restates.  The arithmetic is
// kept in the reference's order where that order affects rounding, so that the
// oracle and the reference agree to a few ulp.  Eigen is not available, so:
//   * Eigen::Quaternion::FromTwoVectors and q*v are restated from Eigen's
//     published algorithm (axis = a x b, w = sqrt(2(1+c))/2);
//   * Eigen::PartialPivLU<MatrixXcd> is replaced by a partial-pivot LU with the
//     same pivot rule (largest |a_ik| in the column, first on ties).
// Special functions: std::cyl_bessel_j / std::cyl_neumann (C++17) are the same
// libstdc++ implementation as the std::tr1 calls at Kernels.cpp:31-34.

#include <cmath>
#include <complex>
#include <cstring>
#include <vector>
#include <algorithm>
#include <cstdint>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> cplx;

namespace {

// BEMUse_Math_Types.h:99-117
const double EUL = 0.5772156649;
const double PI_ = M_PI;
const double TwoPI = 2.0 * M_PI;
const double FourPIinv = 0.25 / M_PI;
const double TwoPIinv = 0.5 / M_PI;
const double Rho_wat = 1025;
const double Gravity = 9.81;

struct V3 { double x, y, z; };
static inline V3 v3(double a, double b, double c) { V3 r = {a, b, c}; return r; }
static inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 scl(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline double norm(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
// Eigen MatrixBase::normalized(): v / sqrt(squaredNorm()) when nonzero.
static inline V3 normalized(V3 a) { double n = norm(a); return n > 0 ? v3(a.x / n, a.y / n, a.z / n) : a; }

// Unit quaternion (w, x, y, z).
struct Quat { double w; V3 v; };

// Eigen QuaternionBase::setFromTwoVectors(a, b) with a = UnitZ (CoordSys.h:35,
// Geo_Elements.cpp:66,144).  Generic branch: axis = v0 x v1, s = sqrt(2(1+c)).
// Antiparallel branch (c < -1 + 1e-12): Eigen takes the null vector of [v0;v1]
// from a JacobiSVD; for v0 = +z, v1 = -z that is the x axis, i.e. a rotation
// by pi about x.  (All panel integrals are invariant to this in-plane choice.)
static Quat quat_from_z(V3 n) {
    V3 v0 = v3(0, 0, 1);
    V3 v1 = normalized(n);
    double c = dot(v1, v0);
    Quat q;
    if (c < -1.0 + 1e-12) {
        c = std::max(c, -1.0);
        double w2 = (1.0 + c) * 0.5;
        q.w = std::sqrt(w2);
        q.v = scl(v3(1, 0, 0), std::sqrt(1.0 - w2));
        return q;
    }
    V3 axis = cross(v0, v1);
    double s = std::sqrt((1.0 + c) * 2.0);
    double invs = 1.0 / s;
    q.v = scl(axis, invs);
    q.w = s * 0.5;
    return q;
}

// Eigen's q * v (_transformVector): uv = 2 (q.vec x v); v + w uv + q.vec x uv.
static V3 qrot(const Quat& q, V3 v) {
    V3 uv = cross(q.v, v);
    uv = add(uv, uv);
    return add(add(v, scl(uv, q.w)), cross(q.v, uv));
}

// One flat panel with its frame and quadrature nodes (Geo_Elements.cpp).
struct Panel {
    int nv;
    V3 vtx[4];      // global vertex positions
    V3 c;           // centroid (global)
    V3 ex, ey, ez;  // OrientMat rows (CoordSys.h:87-94)
    double area;
    int nq;
    V3 qp[4];
    double qw[4];
    V3 qn[4];
};

// Tri_Element::Set_Centroid (Geo_Elements.cpp:45-67) and Set_Quad_Nodes (:69-119),
// Dunavant rule 2 (3 points, Quadrule.cpp dunavant_subrule_02) with w *= 0.5.
static void tri_panel(const V3 pl[3], V3 origin, Panel& p) {
    p.nv = 3;
    V3 PC = scl(add(add(pl[0], pl[1]), pl[2]), 1.0 / 3.0);
    V3 X1 = sub(pl[0], scl(add(pl[1], pl[2]), 0.5));
    V3 X2 = sub(pl[2], pl[1]);
    V3 X3 = cross(X1, X2);
    p.area = 0.5 * norm(X3);
    X3 = normalized(X3);
    Quat q = quat_from_z(X3);
    p.c = add(PC, origin);
    p.ex = qrot(q, v3(1, 0, 0));
    p.ey = qrot(q, v3(0, 1, 0));
    p.ez = qrot(q, v3(0, 0, 1));
    for (int i = 0; i < 3; ++i) p.vtx[i] = add(pl[i], origin);
    p.vtx[3] = p.vtx[2];
    // Dunavant rule 2: barycentric suborder (0.666666666666667, 0.166666666666667,
    // 0.166666666666667), weight 0.333333333333333; points (a,b),(b,b),(b,a).
    const double a = 0.666666666666667, b = 0.166666666666667, w = 0.333333333333333;
    const double PX[3] = {a, b, b}, PY[3] = {b, b, a};
    p.nq = 3;
    for (int i = 0; i < 3; ++i) {
        double xi = PX[i], eta = PY[i];
        V3 P = v3(0, 0, 0);
        P = add(P, scl(pl[0], 1. - xi - eta));
        P = add(P, scl(pl[1], eta));
        P = add(P, scl(pl[2], xi));
        V3 R_xi = v3(0, 0, 0), R_eta = v3(0, 0, 0);
        R_xi = add(R_xi, scl(pl[0], -1));
        R_xi = add(R_xi, scl(pl[2], 1));
        R_eta = add(R_eta, scl(pl[0], -1));
        R_eta = add(R_eta, scl(pl[1], 1));
        V3 R_n = cross(R_xi, R_eta);
        double Jac = norm(R_n);
        R_n = normalized(R_n);
        Quat qq = quat_from_z(R_n);
        p.qp[i] = add(P, origin);
        p.qw[i] = Jac * (w * 0.5);
        p.qn[i] = qrot(qq, v3(0, 0, 1));
    }
    p.qp[3] = v3(0, 0, 0); p.qw[3] = 0; p.qn[3] = v3(0, 0, 0);
}

// Quad_Element::Set_Centroid (Geo_Elements.cpp:123-145) and Set_Quad_Nodes
// (:147-214): 2x2 Gauss-Legendre (cdgqf kind 1: nodes -+1/sqrt(3), weights 1).
static void quad_panel(const V3 pl[4], V3 origin, Panel& p) {
    p.nv = 4;
    V3 PC = scl(add(add(add(pl[0], pl[1]), pl[2]), pl[3]), 0.25);
    V3 X1 = sub(scl(add(pl[3], pl[2]), 0.5), scl(add(pl[0], pl[1]), 0.5));
    V3 X2 = sub(scl(add(pl[2], pl[1]), 0.5), scl(add(pl[3], pl[0]), 0.5));
    V3 X3 = normalized(cross(X1, X2));
    V3 C1 = sub(pl[2], pl[0]);
    V3 C2 = sub(pl[3], pl[1]);
    p.area = 0.5 * norm(cross(C1, C2));
    Quat q = quat_from_z(X3);
    p.c = add(PC, origin);
    p.ex = qrot(q, v3(1, 0, 0));
    p.ey = qrot(q, v3(0, 1, 0));
    p.ez = qrot(q, v3(0, 0, 1));
    for (int i = 0; i < 4; ++i) p.vtx[i] = add(pl[i], origin);
    const double g = 1.0 / std::sqrt(3.0);
    const double PX[2] = {-g, g}, WX[2] = {1.0, 1.0};
    p.nq = 4;
    int k = 0;
    for (int i = 0; i < 2; ++i) {
        for (int j = 0; j < 2; ++j) {
            double px = PX[i], py = PX[j];
            V3 P = v3(0, 0, 0);
            P = add(P, scl(pl[0], 0.25 * (1 - px) * (1 - py)));
            P = add(P, scl(pl[1], 0.25 * (1 - px) * (1 + py)));
            P = add(P, scl(pl[2], 0.25 * (1 + px) * (1 + py)));
            P = add(P, scl(pl[3], 0.25 * (1 + px) * (1 - py)));
            V3 R_xi = v3(0, 0, 0);
            R_xi = add(R_xi, scl(pl[0], -0.25 * (1 - py)));
            R_xi = add(R_xi, scl(pl[1], -0.25 * (1 + py)));
            R_xi = add(R_xi, scl(pl[2], 0.25 * (1 + py)));
            R_xi = add(R_xi, scl(pl[3], 0.25 * (1 - py)));
            V3 R_eta = v3(0, 0, 0);
            R_eta = add(R_eta, scl(pl[0], -0.25 * (1 - px)));
            R_eta = add(R_eta, scl(pl[1], 0.25 * (1 - px)));
            R_eta = add(R_eta, scl(pl[2], 0.25 * (1 + px)));
            R_eta = add(R_eta, scl(pl[3], -0.25 * (1 + px)));
            V3 R_n = cross(R_xi, R_eta);
            double Jac = norm(R_n);
            R_n = normalized(R_n);
            Quat qq = quat_from_z(R_n);
            p.qp[k] = add(P, origin);
            p.qw[k] = Jac * WX[i] * WX[j];
            p.qn[k] = qrot(qq, v3(0, 0, 1));
            ++k;
        }
    }
}

// A panel mesh: body-local nodes, connectivity (elems[4*i+3] < 0 for tris), and
// component frames (Triple_Spar.cpp:60-67: translation-only CoordSys per leg).
struct Mesh {
    int nn; const double* nodes;
    int ne; const int* elems;
    int ncomp; const int* comp_first; const double* comp_origin;
};

static V3 node_local(const Mesh& m, int i) {
    return v3(m.nodes[3 * i], m.nodes[3 * i + 1], m.nodes[3 * i + 2]);
}
static V3 comp_origin_of(const Mesh& m, int e) {
    for (int c = 0; c < m.ncomp; ++c)
        if (e >= m.comp_first[c] && e < m.comp_first[c + 1])
            return v3(m.comp_origin[3 * c], m.comp_origin[3 * c + 1], m.comp_origin[3 * c + 2]);
    return v3(0, 0, 0);
}

// Body panels (Hydrodynamic_Solver.cpp:57-66) and their z-mirror images
// (Boundary_Base.cpp:51-85: global position with z negated, winding reversed,
// defined directly in the global frame).
static void build_panels(const Mesh& m, std::vector<Panel>& body, std::vector<Panel>& mirror) {
    body.resize(m.ne);
    mirror.resize(m.ne);
    for (int e = 0; e < m.ne; ++e) {
        const int* el = m.elems + 4 * e;
        int nv = el[3] < 0 ? 3 : 4;
        V3 org = comp_origin_of(m, e);
        V3 pl[4], pm[4];
        for (int k = 0; k < nv; ++k) pl[k] = node_local(m, el[k]);
        for (int k = 0; k < nv; ++k) {
            // Generate_Symmetry_Nodes: Position_Global with PR(2) *= -1.
            V3 g = add(pl[nv - 1 - k], org);
            g.z *= -1.0;
            pm[k] = g;
        }
        if (nv == 3) { tri_panel(pl, org, body[e]); tri_panel(pm, v3(0, 0, 0), mirror[e]); }
        else         { quad_panel(pl, org, body[e]); quad_panel(pm, v3(0, 0, 0), mirror[e]); }
    }
}

// FlatTriPanel/FlatQuadPanel::Inf_SourceKernel (Panel.cpp:17-78, 86-156):
// analytic constant-strength source S and dipole D of a flat panel at P.
static void inf_source_kernel(const Panel& p, V3 P, double& S, double& D) {
    const int n = p.nv;
    double lx[4], ly[4];
    for (int k = 0; k < n; ++k) {
        V3 d = sub(p.vtx[k], p.c);
        lx[k] = p.ex.x * d.x + p.ex.y * d.y + p.ex.z * d.z;
        ly[k] = p.ey.x * d.x + p.ey.y * d.y + p.ey.z * d.z;
    }
    V3 dp = sub(P, p.c);
    double PLx = p.ex.x * dp.x + p.ex.y * dp.y + p.ex.z * dp.z;
    double PLy = p.ey.x * dp.x + p.ey.y * dp.y + p.ey.z * dp.z;
    double PLz = p.ez.x * dp.x + p.ez.y * dp.y + p.ez.z * dp.z;
    double m[4], e[4], h[4], r[4], DX[4], DY[4];
    for (int k = 0; k < n; ++k) {
        int k1 = (k + 1) % n;
        m[k] = (ly[k1] - ly[k]) / (lx[k1] - lx[k]);
        DX[k] = PLx - lx[k];
        DY[k] = PLy - ly[k];
    }
    double Z2 = PLz * PLz;
    for (int k = 0; k < n; ++k) {
        e[k] = DX[k] * DX[k] + Z2;
        h[k] = DX[k] * DY[k];
        r[k] = std::sqrt(DX[k] * DX[k] + DY[k] * DY[k] + Z2);
    }
    double PhiDip = 0;
    for (int k = 0; k < n; ++k) {
        int k1 = (k + 1) % n;
        PhiDip += std::atan((m[k] * e[k] - h[k]) / (PLz * r[k])) -
                  std::atan((m[k] * e[k1] - h[k1]) / (PLz * r[k1]));
    }
    double sumBL = 0;
    for (int k = 0; k < n; ++k) {
        int k1 = (k + 1) % n;
        double ddx = lx[k1] - lx[k], ddy = ly[k1] - ly[k];
        double d = std::sqrt(ddx * ddx + ddy * ddy);
        double B = (DX[k] * ddy - DY[k] * ddx) / d;
        double L = std::log((r[k] + r[k1] + d) / (r[k] + r[k1] - d));
        sumBL += B * L;
    }
    D = PhiDip * FourPIinv;
    S = (PLz * PhiDip - sumBL) * FourPIinv;
}

// ---- Wave Green function, Kernels.cpp:31-412 (Liang/Wu/Noblesse) ----------
static double BesselJ0(double x) { return std::cyl_bessel_j(0.0, x); }
static double BesselJ1(double x) { return std::cyl_bessel_j(1.0, x); }
static double BesselY0(double x) { return std::cyl_neumann(0.0, x); }
static double BesselY1(double x) { return std::cyl_neumann(1.0, x); }

// Kernels.cpp:35-75
static double StruveH0(double xx) {
    double SH0;
    if (xx <= 3.0) {
        double yy = std::pow(xx / 3.0, 2);
        double P0 = +1.909859164, P1 = -1.909855001, P2 = +0.687514637,
               P3 = -0.126164557, P4 = +0.013828813, P5 = -0.000876918;
        SH0 = P0 + (P1 + (P2 + (P3 + (P4 + P5 * yy) * yy) * yy) * yy) * yy;
        SH0 *= xx / 3.0;
    } else {
        double yy = std::pow(3.0 / xx, 2);
        double a0 = 0.99999906, a1 = 4.77228920, a2 = 3.85542044, a3 = 0.32303607;
        double b1 = 4.88331068, b2 = 4.28957333, b3 = 0.52120508;
        double c1 = 2.0 * (a0 + (a1 + (a2 + a3 * yy) * yy) * yy);
        double c2 = PI_ * xx * (1.0 + (b1 + (b2 + b3 * yy) * yy) * yy);
        SH0 = c1 / c2 + BesselY0(xx);
    }
    return SH0;
}
// Kernels.cpp:76-116
static double StruveH1(double xx) {
    double SH1;
    if (xx <= 3.0) {
        double yy = std::pow(xx / 3.0, 2);
        double P1 = +1.909859286, P2 = -1.145914713, P3 = +0.294656958,
               P4 = -0.042070508, P5 = +0.003785727, P6 = -0.000207183;
        SH1 = (P1 + (P2 + (P3 + (P4 + (P5 + P6 * yy) * yy) * yy) * yy) * yy) * yy;
    } else {
        double yy = std::pow(3.0 / xx, 2);
        double a0 = 1.00000004, a1 = 3.92205313, a2 = 2.64893033, a3 = 0.27450895;
        double b1 = 3.81095112, b2 = 2.26216956, b3 = 0.10885141;
        double c1 = 2.0 * (a0 + (a1 + (a2 + a3 * yy) * yy) * yy);
        double c2 = PI_ * (1.0 + (b1 + (b2 + b3 * yy) * yy) * yy);
        SH1 = c1 / c2 + BesselY1(xx);
    }
    return SH1;
}

// Polynomials of Liang, Wu & Noblesse (2018) eq. 14a-c, 16a-c, in the
// reference's incremental-power form (Kernels.cpp:120-256).
static double poly_inc(const double* c, int n, double tt) {
    double S = c[0], t = tt;
    for (int i = 1; i < n; ++i) { S += c[i] * t; t *= tt; }
    return S;
}
const double cA[10] = {1.21, -13.328, 215.896, -1763.96, 8418.94, -24314.21, 42002.57, -41592.9, 21859.0, -4838.6};
const double cB[10] = {0.938, 5.737, -67.92, 796.534, -4780.77, 17137.74, -36618.81, 44894.06, -29030.24, 7671.22};
const double cC[8]  = {1.268, -9.747, 209.653, -1397.89, 5155.67, -9844.35, 9136.4, -3272.62};
const double cD[10] = {0.632, -40.97, 667.16, -6072.07, 31127.39, -96293.05, 181856.75, -205690.43, 128170.2, -33744.6};
const double dA[10] = {2.948, -24.53, 249.69, -754.85, -1187.71, 16370.75, -48811.41, 68220.87, -46688.0, 12622.25};
const double dB[10] = {1.11, 2.894, -76.765, 1565.35, -11336.19, 44270.15, -97014.11, 118879.26, -76209.82, 19923.28};
const double dC[6]  = {14.19, -148.24, 847.8, -2318.58, 3168.35, -1590.27};

// HavelockGF (Kernels.cpp:342-412) with GF_Func_L0/W/Ls/Wh (:258-338) inlined.
static void havelock_gf(double dx, double dy, double vv, cplx& GF, cplx& DGFX, cplx& DGFY, cplx& DGFZ) {
    double hh = std::sqrt(std::pow(dx, 2) + std::pow(dy, 2));
    double dd = std::sqrt(std::pow(hh, 2) + std::pow(vv, 2));
    double alpha = -vv / dd;
    double beta = hh / dd;
    double rho = dd / (1.0 + dd);
    // GF_Func_L0 (:258-282)
    double PP = std::log(0.5 * (dd - vv)) + EUL - 2.0 * std::pow(dd, 2);
    PP *= std::exp(vv);
    PP += std::pow(dd, 2) - vv;
    double A = poly_inc(cA, 10, rho), B = poly_inc(cB, 10, rho);
    double C = poly_inc(cC, 8, rho), D = poly_inc(cD, 10, rho);
    double RR = (1.0 - beta) * A;
    RR -= beta * B;
    RR -= alpha * C / (1.0 + 6.0 * alpha * rho * (1.0 - rho));
    RR += beta * (1.0 - beta) * D;
    double Lp = rho * std::pow(1.0 - rho, 3) * RR;
    double L0 = 2.0 * PP / (1.0 + std::pow(dd, 3)) + 2.0 * Lp;
    // GF_Func_W (:284-295)
    double H0 = StruveH0(hh), J0 = BesselJ0(hh);
    double E = 2.0 * PI_ * std::exp(vv);
    GF = cplx(L0, 0.0) + cplx(E * H0, -E * J0);
    // GF_Func_Ls (:297-325)
    double PS = (beta + hh) / (dd - vv);
    PS -= 2.0 * beta;
    PS += 2.0 * dd * std::exp(vv);
    PS -= hh;
    double QS = std::exp(-dd) * (1.0 - beta);
    QS *= 1.0 + dd / (1.0 + std::pow(dd, 3));
    double dAv = poly_inc(dA, 10, rho), dBv = poly_inc(dB, 10, rho), dCv = poly_inc(dC, 6, rho);
    double RS = beta * dAv;
    RS -= (1.0 - alpha) * dBv;
    RS += beta * (1.0 - beta) * rho * (1.0 - 2.0 * rho) * dCv;
    double Lsp = rho * std::pow(1.0 - rho, 3) * RS;
    double Ls = 2.0 * PS / (1.0 + std::pow(dd, 3)) - 4.0 * QS + 2.0 * Lsp;
    // GF_Func_Wh (:327-338)
    double H1 = StruveH1(hh), J1 = BesselJ1(hh);
    double E2 = 2.0 * PI_ * std::exp(vv);
    cplx GFh = cplx(Ls, 0.0) + cplx(E2 * (2.0 / PI_ - H1), E2 * J1);
    if (hh > 1.0e-6) {
        DGFX = GFh * dx / hh;
        DGFY = GFh * dy / hh;
    } else {
        DGFX = cplx(0.0, 0.0);
        DGFY = cplx(0.0, 0.0);
    }
    DGFZ = GF;
}

// FreeSurface_Wave_Kernel (Panel.cpp:601-636)
static void fs_wave_kernel(V3 Pg, V3 Ps, double K, cplx& G, cplx& dGX, cplx& dGY, cplx& dGZ) {
    if (K == 0.0) { G = dGX = dGY = dGZ = cplx(0, 0); return; }
    V3 R = sub(Pg, Ps);
    double XX = R.x * K, YY = R.y * K, V = R.z * K;
    havelock_gf(XX, YY, V, G, dGX, dGY, dGZ);
    G *= K * FourPIinv;
    dGX *= K * K * FourPIinv;
    dGY *= K * K * FourPIinv;
    dGZ *= K * K * FourPIinv;
}

// FlatWave{Tri,Quad}Panel::CInf_SingleDoubleLayerQuad (Panel.cpp:676-694, 776-794)
static void wave_panel_influence(const Panel& p, V3 P, double K, cplx& S, cplx& D) {
    cplx OS(0, 0), OD(0, 0);
    for (int i = 0; i < p.nq; ++i) {
        cplx G, dX, dY, dZ;
        fs_wave_kernel(P, p.qp[i], K, G, dX, dY, dZ);
        OS += p.qw[i] * G;
        OD += p.qw[i] * (dX * p.qn[i].x + dY * p.qn[i].y + dZ * p.qn[i].z);
    }
    S = OS;
    D = OD;
}

// y[j] -= l x[j] for j < m, in real arithmetic: the value std::complex's product
// gives for finite operands, without its NaN/inf recovery call in the inner loop.
static inline void axpy_neg(cplx l, const cplx* x, cplx* y, int m) {
    const double lr = l.real(), li = l.imag();
    const double* xs = reinterpret_cast<const double*>(x);
    double* ys = reinterpret_cast<double*>(y);
    for (int j = 0; j < m; ++j) {
        const double xr = xs[2 * j], xi = xs[2 * j + 1];
        ys[2 * j] -= lr * xr - li * xi;
        ys[2 * j + 1] -= lr * xi + li * xr;
    }
}

// Partial-pivot LU of a row-major complex matrix (stand-in for
// Eigen::PartialPivLU<MatrixXcd>, Solver_Base.h:85, Hydrodynamic_Solver.cpp:430).
// Pivot = first index of max |a_ik|.  Blocked right-looking, OpenMP over rows.
static void lu_factor(int n, cplx* a, int* piv) {
    const int nb = 64;
    for (int k0 = 0; k0 < n; k0 += nb) {
        int kb = std::min(nb, n - k0);
        for (int k = k0; k < k0 + kb; ++k) {
            int p = k;
            double best = std::abs(a[(size_t)k * n + k]);
            for (int i = k + 1; i < n; ++i) {
                double v = std::abs(a[(size_t)i * n + k]);
                if (v > best) { best = v; p = i; }
            }
            piv[k] = p;
            if (p != k)
                for (int j = 0; j < n; ++j) std::swap(a[(size_t)k * n + j], a[(size_t)p * n + j]);
            cplx inv = 1.0 / a[(size_t)k * n + k];
            #pragma omp parallel for schedule(static)
            for (int i = k + 1; i < n; ++i) {
                cplx* ri = a + (size_t)i * n;
                const cplx* rk = a + (size_t)k * n;
                cplx l = ri[k] * inv;
                ri[k] = l;
                axpy_neg(l, rk + k + 1, ri + k + 1, k0 + kb - k - 1);
            }
        }
        // U12 = L11^{-1} A12
        for (int k = k0; k < k0 + kb; ++k) {
            const cplx* rk = a + (size_t)k * n;
            #pragma omp parallel for schedule(static)
            for (int i = k + 1; i < k0 + kb; ++i) {
                cplx* ri = a + (size_t)i * n;
                axpy_neg(ri[k], rk + k0 + kb, ri + k0 + kb, n - k0 - kb);
            }
        }
        // A22 -= L21 U12
        #pragma omp parallel for schedule(static)
        for (int i = k0 + kb; i < n; ++i) {
            cplx* ri = a + (size_t)i * n;
            for (int k = k0; k < k0 + kb; ++k)
                axpy_neg(ri[k], a + (size_t)k * n + k0 + kb, ri + k0 + kb, n - k0 - kb);
        }
    }
}

// Solve with the factors; b is n x nr row-major (column j = one RHS).
static void lu_solve(int n, const cplx* a, const int* piv, int nr, cplx* b) {
    for (int k = 0; k < n; ++k)
        if (piv[k] != k)
            for (int j = 0; j < nr; ++j) std::swap(b[(size_t)k * nr + j], b[(size_t)piv[k] * nr + j]);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < i; ++k) {
            cplx l = a[(size_t)i * n + k];
            for (int j = 0; j < nr; ++j) b[(size_t)i * nr + j] -= l * b[(size_t)k * nr + j];
        }
    for (int i = n - 1; i >= 0; --i) {
        for (int k = i + 1; k < n; ++k) {
            cplx u = a[(size_t)i * n + k];
            for (int j = 0; j < nr; ++j) b[(size_t)i * nr + j] -= u * b[(size_t)k * nr + j];
        }
        cplx inv = 1.0 / a[(size_t)i * n + i];
        for (int j = 0; j < nr; ++j) b[(size_t)i * nr + j] *= inv;
    }
}

// 6x6 complex inverse by Gauss-Jordan with partial pivoting (Eigen's
// MatrixBase::inverse at Hydrodynamic_Solver.cpp:487 for a 6x6 uses PartialPivLU).
static bool inv6(const cplx* M, cplx* out) {
    cplx a[6][12];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 12; ++j) a[i][j] = j < 6 ? M[i * 6 + j] : cplx(i == j - 6 ? 1.0 : 0.0, 0.0);
    for (int k = 0; k < 6; ++k) {
        int p = k;
        for (int i = k + 1; i < 6; ++i) if (std::abs(a[i][k]) > std::abs(a[p][k])) p = i;
        if (p != k) for (int j = 0; j < 12; ++j) std::swap(a[k][j], a[p][j]);
        cplx inv = 1.0 / a[k][k];
        for (int j = 0; j < 12; ++j) a[k][j] *= inv;
        for (int i = 0; i < 6; ++i) {
            if (i == k) continue;
            cplx f = a[i][k];
            for (int j = 0; j < 12; ++j) a[i][j] -= f * a[k][j];
        }
    }
    for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) out[i * 6 + j] = a[i][j + 6];
    return true;
}

static Mesh make_mesh(int nn, const double* nodes, int ne, const int* elems, int ncomp,
                      const int* comp_first, const double* comp_origin) {
    Mesh m;
    m.nn = nn; m.nodes = nodes; m.ne = ne; m.elems = elems;
    m.ncomp = ncomp; m.comp_first = comp_first; m.comp_origin = comp_origin;
    return m;
}

static void pack_panel(const Panel& p, double* o) {
    // stride 56: nv, vtx[12], c[3], ex[3], ey[3], ez[3], area, nq, qp[12], qw[4], qn[12], pad
    std::memset(o, 0, 56 * sizeof(double));
    o[0] = p.nv;
    for (int k = 0; k < 4; ++k) { o[1 + 3 * k] = p.vtx[k].x; o[2 + 3 * k] = p.vtx[k].y; o[3 + 3 * k] = p.vtx[k].z; }
    o[13] = p.c.x; o[14] = p.c.y; o[15] = p.c.z;
    o[16] = p.ex.x; o[17] = p.ex.y; o[18] = p.ex.z;
    o[19] = p.ey.x; o[20] = p.ey.y; o[21] = p.ey.z;
    o[22] = p.ez.x; o[23] = p.ez.y; o[24] = p.ez.z;
    o[25] = p.area; o[26] = p.nq;
    for (int k = 0; k < 4; ++k) {
        o[27 + 3 * k] = p.qp[k].x; o[28 + 3 * k] = p.qp[k].y; o[29 + 3 * k] = p.qp[k].z;
        o[39 + k] = p.qw[k];
        o[43 + 3 * k] = p.qn[k].x; o[44 + 3 * k] = p.qn[k].y; o[45 + 3 * k] = p.qn[k].z;
    }
}

// Solver::Specify_BC_Positions (Solver_Base.cpp:71-83), BCF = 1e-5 (Solver_Base.h:55).
static std::vector<V3> collocation(const std::vector<Panel>& body) {
    std::vector<V3> x(body.size());
    for (size_t i = 0; i < body.size(); ++i) x[i] = add(body[i].c, scl(body[i].ez, 1.e-5));
    return x;
}

}  // namespace

extern "C" {

int orc_num_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

// ---- meshes ----------------------------------------------------------------
// Half_Cylinder::Generate_Nodes (Volume_of_Revolution.cpp:185-199) +
// Volume_of_Revolution::Generate_Nodes/Elements (:12-41, 92-109) +
// Generate_Aux_Nodes/Elements (:43-68, 111-130) with PiCosFac (Boundary_Base.h:39).
void orc_cylinder_sizes(int NA, int NR, int NV, int NRFS, int* nn, int* ne, int* nn_aux, int* ne_aux) {
    int NZ = NR + NV;
    *nn = 1 + NZ * NA;
    *ne = NA + (NZ - 1) * NA;
    *nn_aux = NRFS > 0 ? 1 + NRFS * NA : 0;
    *ne_aux = NRFS > 0 ? NA + (NRFS - 1) * NA : 0;
}

static inline double PiCosFac(int i, int itot) { return 0.5 * (1.0 - std::cos(i * PI_ / (itot - 1))); }

void orc_cylinder(double R, double draft, int NA, int NR, int NV, int NRFS, int cosine,
                  double* nodes, int* elems, double* aux_nodes, int* aux_elems) {
    double Z = -draft;
    std::vector<V3> per;
    if (cosine) {
        for (int i = 0; i < NR; ++i) { double f = PiCosFac(i, NR + 1); per.push_back(v3(R * f, 0, Z)); }
        for (int i = 0; i < NV + 1; ++i) { double f = PiCosFac(i, NV + 1); per.push_back(v3(R, 0, Z * (1.0 - f))); }
    } else {
        for (int i = 0; i < NR; ++i) per.push_back(v3(R * i / NR, 0, Z));
        for (int i = 0; i < NV + 1; ++i) per.push_back(v3(R, 0, Z * (1.0 - 1.0 * i / NV)));
    }
    int NZ = (int)per.size() - 1;
    int k = 0;
    for (int i = 0; i < NZ + 1; ++i) {
        int NAR = i == 0 ? 1 : NA;
        for (int j = 0; j < NAR; ++j) {
            double u = j * TwoPI / NAR;
            double r = per[i].x, z = per[i].z;
            nodes[3 * k] = r * std::cos(u); nodes[3 * k + 1] = r * std::sin(u); nodes[3 * k + 2] = z;
            ++k;
        }
    }
    auto nid = [&](int A, int Zr) {
        if (Zr == 0) return 0;
        if (A >= NA) return 1 + (Zr - 1) * NA + (A - NA);
        if (A < 0) return 1 + (Zr - 1) * NA + (A + NA);
        return 1 + (Zr - 1) * NA + A;
    };
    int e = 0;
    for (int i = 0; i < NA; ++i) {
        elems[4 * e] = nid(0, 0); elems[4 * e + 1] = nid(i + 1, 1); elems[4 * e + 2] = nid(i, 1); elems[4 * e + 3] = -1; ++e;
    }
    for (int z = 1; z < NZ; ++z)
        for (int i = 0; i < NA; ++i) {
            elems[4 * e] = nid(i, z); elems[4 * e + 1] = nid(i + 1, z);
            elems[4 * e + 2] = nid(i + 1, z + 1); elems[4 * e + 3] = nid(i, z + 1); ++e;
        }
    if (NRFS > 0 && aux_nodes && aux_elems) {
        k = 0;
        for (int i = 0; i < NRFS + 1; ++i) {
            double r = cosine ? R * PiCosFac(i, NRFS + 1) : R * i / NRFS;
            int NAR = i == 0 ? 1 : NA;
            for (int j = 0; j < NAR; ++j) {
                double u = j * TwoPI / NAR;
                aux_nodes[3 * k] = r * std::cos(u); aux_nodes[3 * k + 1] = r * std::sin(u); aux_nodes[3 * k + 2] = 0;
                ++k;
            }
        }
        e = 0;
        for (int i = 0; i < NA; ++i) {
            aux_elems[4 * e] = nid(0, 0); aux_elems[4 * e + 1] = nid(i, 1); aux_elems[4 * e + 2] = nid(i + 1, 1);
            aux_elems[4 * e + 3] = -1; ++e;
        }
        for (int z = 1; z < NRFS; ++z)
            for (int i = 0; i < NA; ++i) {
                aux_elems[4 * e] = nid(i, z + 1); aux_elems[4 * e + 1] = nid(i + 1, z + 1);
                aux_elems[4 * e + 2] = nid(i + 1, z); aux_elems[4 * e + 3] = nid(i, z); ++e;
            }
    }
}

// Barge (Barge.cpp:33-204): five faces, no lid; the interior waterplane grid is
// the auxiliary mesh.  The linear-spacing branch of Generate_Aux_Nodes uses
// i/NY for y (Barge.cpp:115); that is kept.
void orc_barge_sizes(int NX, int NY, int NZ, int* nn, int* ne, int* nn_aux, int* ne_aux) {
    *nn = 2 * (NY + 1) * (NZ + 1) + 2 * (NX + 1) * (NZ + 1) + (NX + 1) * (NY + 1);
    *ne = 2 * NY * NZ + 2 * NX * NZ + NX * NY;
    *nn_aux = (NX + 1) * (NY + 1);
    *ne_aux = NX * NY;
}

void orc_barge(double L, double W, double Dp, int NX, int NY, int NZ, int cosine,
               double* nodes, int* elems, double* aux_nodes, int* aux_elems) {
    int k = 0;
    auto put = [&](double x, double y, double z) { nodes[3 * k] = x; nodes[3 * k + 1] = y; nodes[3 * k + 2] = z; ++k; };
    int xf1 = 0, xf2 = (NY + 1) * (NZ + 1), yf1 = 2 * (NY + 1) * (NZ + 1);
    int yf2 = yf1 + (NX + 1) * (NZ + 1), zf = yf2 + (NX + 1) * (NZ + 1);
    std::vector<V3> X1, X2, Y1, Y2, ZF;
    for (int j = 0; j < NY + 1; ++j)
        for (int kk = 0; kk < NZ + 1; ++kk) {
            double y, z;
            if (cosine) { y = -0.5 * W + W * PiCosFac(j, NY + 1); z = -Dp + Dp * PiCosFac(kk, NZ + 1); }
            else { y = -0.5 * W + W * j / NY; z = -Dp + Dp * kk / NZ; }
            X1.push_back(v3(-0.5 * L, y, z)); X2.push_back(v3(0.5 * L, y, z));
        }
    for (int i = 0; i < NX + 1; ++i)
        for (int kk = 0; kk < NZ + 1; ++kk) {
            double x, z;
            if (cosine) { x = -0.5 * L + L * PiCosFac(i, NX + 1); z = -Dp + Dp * PiCosFac(kk, NZ + 1); }
            else { x = -0.5 * L + L * i / NX; z = -Dp + Dp * kk / NZ; }
            Y1.push_back(v3(x, -0.5 * W, z)); Y2.push_back(v3(x, 0.5 * W, z));
        }
    for (int i = 0; i < NX + 1; ++i)
        for (int j = 0; j < NY + 1; ++j) {
            double x, y;
            if (cosine) { x = -0.5 * L + L * PiCosFac(i, NX + 1); y = -0.5 * W + W * PiCosFac(j, NY + 1); }
            else { x = -0.5 * L + L * i / NX; y = -0.5 * W + W * j / NY; }
            ZF.push_back(v3(x, y, -Dp));
        }
    for (auto& p : X1) put(p.x, p.y, p.z);
    for (auto& p : X2) put(p.x, p.y, p.z);
    for (auto& p : Y1) put(p.x, p.y, p.z);
    for (auto& p : Y2) put(p.x, p.y, p.z);
    for (auto& p : ZF) put(p.x, p.y, p.z);
    int e = 0;
    auto quad = [&](int a, int b, int c, int d) { elems[4 * e] = a; elems[4 * e + 1] = b; elems[4 * e + 2] = c; elems[4 * e + 3] = d; ++e; };
    for (int j = 0; j < NY; ++j)
        for (int kk = 0; kk < NZ; ++kk) {
            quad(xf1 + j * (NZ + 1) + kk, xf1 + j * (NZ + 1) + kk + 1, xf1 + (j + 1) * (NZ + 1) + kk + 1, xf1 + (j + 1) * (NZ + 1) + kk);
            quad(xf2 + j * (NZ + 1) + kk, xf2 + (j + 1) * (NZ + 1) + kk, xf2 + (j + 1) * (NZ + 1) + kk + 1, xf2 + j * (NZ + 1) + kk + 1);
        }
    for (int i = 0; i < NX; ++i)
        for (int kk = 0; kk < NZ; ++kk) {
            quad(yf1 + i * (NZ + 1) + kk, yf1 + (i + 1) * (NZ + 1) + kk, yf1 + (i + 1) * (NZ + 1) + kk + 1, yf1 + i * (NZ + 1) + kk + 1);
            quad(yf2 + i * (NZ + 1) + kk, yf2 + i * (NZ + 1) + kk + 1, yf2 + (i + 1) * (NZ + 1) + kk + 1, yf2 + (i + 1) * (NZ + 1) + kk);
        }
    for (int i = 0; i < NX; ++i)
        for (int j = 0; j < NY; ++j)
            quad(zf + i * (NY + 1) + j, zf + i * (NY + 1) + j + 1, zf + (i + 1) * (NY + 1) + j + 1, zf + (i + 1) * (NY + 1) + j);
    if (aux_nodes && aux_elems) {
        k = 0;
        for (int i = 0; i < NX + 1; ++i)
            for (int j = 0; j < NY + 1; ++j) {
                double x, y;
                if (cosine) { x = -0.5 * L + L * PiCosFac(i, NX + 1); y = -0.5 * W + W * PiCosFac(j, NY + 1); }
                else { x = -0.5 * L + L * i / NX; y = -0.5 * W + W * i / NY; }
                aux_nodes[3 * k] = x; aux_nodes[3 * k + 1] = y; aux_nodes[3 * k + 2] = 0; ++k;
            }
        e = 0;
        for (int i = 0; i < NX; ++i)
            for (int j = 0; j < NY; ++j) {
                aux_elems[4 * e] = i * (NY + 1) + j; aux_elems[4 * e + 1] = (i + 1) * (NY + 1) + j;
                aux_elems[4 * e + 2] = (i + 1) * (NY + 1) + j + 1; aux_elems[4 * e + 3] = i * (NY + 1) + j + 1; ++e;
            }
    }
}

// ---- geometry ----------------------------------------------------------------
// Packed panel geometry, 56 doubles per panel (see pack_panel); mirror = 1 gives
// the z-reflected, winding-reversed panels of Boundary_Base.cpp:51-85.
void orc_panels(int nn, const double* nodes, int ne, const int* elems, int ncomp, const int* comp_first,
                const double* comp_origin, int mirror, double* out) {
    Mesh m = make_mesh(nn, nodes, ne, elems, ncomp, comp_first, comp_origin);
    std::vector<Panel> body, mir;
    build_panels(m, body, mir);
    const std::vector<Panel>& src = mirror ? mir : body;
    for (int i = 0; i < ne; ++i) pack_panel(src[i], out + 56 * i);
}

void orc_collocation(int nn, const double* nodes, int ne, const int* elems, int ncomp, const int* comp_first,
                     const double* comp_origin, double* out) {
    Mesh m = make_mesh(nn, nodes, ne, elems, ncomp, comp_first, comp_origin);
    std::vector<Panel> body, mir;
    build_panels(m, body, mir);
    std::vector<V3> x = collocation(body);
    for (int i = 0; i < ne; ++i) { out[3 * i] = x[i].x; out[3 * i + 1] = x[i].y; out[3 * i + 2] = x[i].z; }
}

// ---- kernels -----------------------------------------------------------------
void orc_havelock(int n, const double* x, const double* y, const double* v, double* out) {
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        cplx G, dx, dy, dz;
        havelock_gf(x[i], y[i], v[i], G, dx, dy, dz);
        double* o = out + 8 * i;
        o[0] = G.real(); o[1] = G.imag(); o[2] = dx.real(); o[3] = dx.imag();
        o[4] = dy.real(); o[5] = dy.imag(); o[6] = dz.real(); o[7] = dz.imag();
    }
}

// Analytic influence of packed panel `pp` at points P (n x 3) -> S, D.
void orc_source_kernel(const double* pp, int n, const double* P, double* S, double* D) {
    Panel p;
    p.nv = (int)pp[0];
    for (int k = 0; k < 4; ++k) p.vtx[k] = v3(pp[1 + 3 * k], pp[2 + 3 * k], pp[3 + 3 * k]);
    p.c = v3(pp[13], pp[14], pp[15]);
    p.ex = v3(pp[16], pp[17], pp[18]); p.ey = v3(pp[19], pp[20], pp[21]); p.ez = v3(pp[22], pp[23], pp[24]);
    for (int i = 0; i < n; ++i) inf_source_kernel(p, v3(P[3 * i], P[3 * i + 1], P[3 * i + 2]), S[i], D[i]);
}

// Prepare_Linear_System (Hydrodynamic_Solver.cpp:83-115).  Outputs are N x N
// row-major (row = receiver R, column = source S): s, sr, d, dr as the raw
// kernel values (the reference stores SSrc = -s, SSrcRefl = -sr, DSrc = d,
// DSrcRefl = dr) and reflnorm(S) = 2 n_z(S).
void orc_rankine(int nn, const double* nodes, int ne, const int* elems, int ncomp, const int* comp_first,
                 const double* comp_origin, double* s, double* sr, double* d, double* dr, double* reflnorm) {
    Mesh m = make_mesh(nn, nodes, ne, elems, ncomp, comp_first, comp_origin);
    std::vector<Panel> body, mir;
    build_panels(m, body, mir);
    std::vector<V3> x = collocation(body);
    int N = ne;
    #pragma omp parallel for schedule(dynamic, 4)
    for (int S = 0; S < N; ++S) {
        reflnorm[S] = body[S].ez.z * 2.0;
        for (int R = 0; R < N; ++R) {
            size_t o = (size_t)R * N + S;
            inf_source_kernel(body[S], x[R], s[o], d[o]);
            inf_source_kernel(mir[S], x[R], sr[o], dr[o]);
        }
    }
}

// Prepare_Linear_System_Wave_Terms (Hydrodynamic_Solver.cpp:177-203) without the
// Rankine K-term: ws, wd (N x N complex, interleaved re/im, row-major).
void orc_wave(int nn, const double* nodes, int ne, const int* elems, int ncomp, const int* comp_first,
              const double* comp_origin, double K, double* ws, double* wd) {
    Mesh m = make_mesh(nn, nodes, ne, elems, ncomp, comp_first, comp_origin);
    std::vector<Panel> body, mir;
    build_panels(m, body, mir);
    std::vector<V3> x = collocation(body);
    int N = ne;
    #pragma omp parallel for schedule(dynamic, 4)
    for (int S = 0; S < N; ++S)
        for (int R = 0; R < N; ++R) {
            cplx a, b;
            wave_panel_influence(mir[S], x[R], K, a, b);
            size_t o = 2 * ((size_t)R * N + S);
            ws[o] = a.real(); ws[o + 1] = a.imag();
            wd[o] = b.real(); wd[o + 1] = b.imag();
        }
}

// Wave influence of rows [r0, r1) only -- the bounded CPU-baseline sample.
void orc_wave_rows(int nn, const double* nodes, int ne, const int* elems, int ncomp, const int* comp_first,
                   const double* comp_origin, double K, int r0, int r1, double* ws, double* wd) {
    Mesh m = make_mesh(nn, nodes, ne, elems, ncomp, comp_first, comp_origin);
    std::vector<Panel> body, mir;
    build_panels(m, body, mir);
    std::vector<V3> x = collocation(body);
    int N = ne;
    #pragma omp parallel for schedule(dynamic, 1)
    for (int R = r0; R < r1; ++R)
        for (int S = 0; S < N; ++S) {
            cplx a, b;
            wave_panel_influence(mir[S], x[R], K, a, b);
            size_t o = 2 * ((size_t)(R - r0) * N + S);
            ws[o] = a.real(); ws[o + 1] = a.imag();
            wd[o] = b.real(); wd[o + 1] = b.imag();
        }
}

// Aerodynamic_Solver constant-panel steady solve (Aerodynamic_Solver.cpp:42-58,
// 126-180): G(R,S), H(R,S) = Inf_SingleDoubleLayer of the body panel S at the
// collocation point R (c + 1e-5 n, BCF = +1e-5 for constant panels, :134-137);
// BC(i) = V_i . n_i (Set_External_BC :150-166, sgnBCF = +1); X = H^-1 (G BC).
// vel: 3 doubles (uniform) if nvel == 1, else 3 N.  Outputs X (N) and BC (N).
void orc_aero(int nn, const double* nodes, int ne, const int* elems, int ncomp, const int* comp_first,
              const double* comp_origin, int nvel, const double* vel, double* X, double* BC) {
    Mesh m = make_mesh(nn, nodes, ne, elems, ncomp, comp_first, comp_origin);
    std::vector<Panel> body, mir;
    build_panels(m, body, mir);
    std::vector<V3> x = collocation(body);
    const int N = ne;
    std::vector<double> G((size_t)N * N), H((size_t)N * N);
    #pragma omp parallel for schedule(dynamic, 4)
    for (int S = 0; S < N; ++S)
        for (int R = 0; R < N; ++R) inf_source_kernel(body[S], x[R], G[(size_t)R * N + S], H[(size_t)R * N + S]);
    for (int i = 0; i < N; ++i) {
        const double* v = nvel == 1 ? vel : vel + 3 * (size_t)i;
        BC[i] = v[0] * body[i].ez.x + v[1] * body[i].ez.y + v[2] * body[i].ez.z;
    }
    std::vector<cplx> A((size_t)N * N), b(N);
    for (size_t k = 0; k < (size_t)N * N; ++k) A[k] = cplx(H[k], 0.0);
    #pragma omp parallel for schedule(static)
    for (int R = 0; R < N; ++R) {
        double acc = 0;
        for (int S = 0; S < N; ++S) acc += G[(size_t)R * N + S] * BC[S];
        b[R] = cplx(acc, 0.0);
    }
    std::vector<int> piv(N);
    lu_factor(N, A.data(), piv.data());
    lu_solve(N, A.data(), piv.data(), 1, b.data());
    for (int i = 0; i < N; ++i) X[i] = b[i].real();
}

// The steady solve with a trailing wake (the configuration the reference's
// Aerodynamic_Solver lacks, defined here): wake strip w is a constant-doublet panel
// (wake mesh element w, normal pointing down, i.e. away from the fluid above it) whose
// strength is the Kutta jump X[te_up[w]] - X[te_lo[w]] (Morino), so its dipole influence
// D_w(x_R) joins column te_up[w] of H with + and column te_lo[w] with -.  Otherwise as
// orc_aero: H X = G (V . n).
void orc_aero_wake(int nn, const double* nodes, int ne, const int* elems, int ncomp, const int* comp_first,
                   const double* comp_origin, int nwn, const double* wnodes, int nw, const int* welems,
                   const int* te_up, const int* te_lo, int nvel, const double* vel, double* X, double* BC) {
    Mesh m = make_mesh(nn, nodes, ne, elems, ncomp, comp_first, comp_origin);
    Mesh wm = make_mesh(nwn, wnodes, nw, welems, 0, nullptr, nullptr);
    std::vector<Panel> body, mir, wake, wmir;
    build_panels(m, body, mir);
    build_panels(wm, wake, wmir);
    std::vector<V3> x = collocation(body);
    const int N = ne;
    std::vector<double> G((size_t)N * N), H((size_t)N * N);
    #pragma omp parallel for schedule(dynamic, 4)
    for (int S = 0; S < N; ++S)
        for (int R = 0; R < N; ++R) inf_source_kernel(body[S], x[R], G[(size_t)R * N + S], H[(size_t)R * N + S]);
    #pragma omp parallel for schedule(static)
    for (int R = 0; R < N; ++R)
        for (int w = 0; w < nw; ++w) {
            double sw, dw;
            inf_source_kernel(wake[w], x[R], sw, dw);
            H[(size_t)R * N + te_up[w]] += dw;
            H[(size_t)R * N + te_lo[w]] -= dw;
        }
    for (int i = 0; i < N; ++i) {
        const double* v = nvel == 1 ? vel : vel + 3 * (size_t)i;
        BC[i] = v[0] * body[i].ez.x + v[1] * body[i].ez.y + v[2] * body[i].ez.z;
    }
    std::vector<cplx> A((size_t)N * N), b(N);
    for (size_t k = 0; k < (size_t)N * N; ++k) A[k] = cplx(H[k], 0.0);
    #pragma omp parallel for schedule(static)
    for (int R = 0; R < N; ++R) {
        double acc = 0;
        for (int S = 0; S < N; ++S) acc += G[(size_t)R * N + S] * BC[S];
        b[R] = cplx(acc, 0.0);
    }
    std::vector<int> piv(N);
    lu_factor(N, A.data(), piv.data());
    lu_solve(N, A.data(), piv.data(), 1, b.data());
    for (int i = 0; i < N; ++i) X[i] = b[i].real();
}

// Complex LU + solve (interleaved re/im, row-major), exposed for baselines/tests.
void orc_lu_solve(int n, double* a, int nr, double* b) {
    std::vector<int> piv(n);
    lu_factor(n, reinterpret_cast<cplx*>(a), piv.data());
    lu_solve(n, reinterpret_cast<cplx*>(a), piv.data(), nr, reinterpret_cast<cplx*>(b));
}
void orc_lu_factor(int n, double* a, int* piv) { lu_factor(n, reinterpret_cast<cplx*>(a), piv); }

// Calculate_Mass_Matrix (Hydrodynamic_Solver.cpp:300-339),
// Calculate_Hydrostatic_Stiffness_Matrix (:341-397, including the symmetry
// lines :394-396 that copy the zero lower entries over the upper ones),
// Calculate_Volume / Calculate_COB (Boundary_Base.cpp:177-224).
// params: rho, g, mass (0 -> V*Rho_wat), cog[3], gyr[9] (row-major).
// out: M[36], C[36], vol_cob[4] = {V, xb, yb, zb}.
void orc_mass_hydrostatics(int nn, const double* nodes, int ne, const int* elems, int ncomp, const int* comp_first,
                           const double* comp_origin, int nn_aux, const double* aux_nodes, int ne_aux,
                           const int* aux_elems, int ncomp_aux, const int* aux_comp_first, const double* aux_comp_origin,
                           double rho, double g, double mass, const double* cog, const double* gyr,
                           double* M, double* C, double* vol_cob) {
    Mesh m = make_mesh(nn, nodes, ne, elems, ncomp, comp_first, comp_origin);
    std::vector<Panel> body, mir;
    build_panels(m, body, mir);
    double Vx = 0, Vy = 0, Vz = 0, Xmin = 1e300, Xmax = -1e300, Ymin = 1e300, Ymax = -1e300, Zmin = 1e300, Zmax = -1e300;
    for (int e = 0; e < ne; ++e) {
        V3 n = body[e].ez, p = body[e].c;
        double A = body[e].area;
        Vx += -p.x * n.x * A; Vy += -p.y * n.y * A; Vz += -p.z * n.z * A;
    }
    double V = (Vx + Vy + Vz) / 3.0;
    for (int e = 0; e < ne; ++e) {
        // Calculate_GridParams (Boundary_Base.cpp:125-150) uses node positions;
        // element vertices cover the same node set.
        for (int k = 0; k < body[e].nv; ++k) {
            V3 q = body[e].vtx[k];
            Xmin = std::min(Xmin, q.x); Xmax = std::max(Xmax, q.x);
            Ymin = std::min(Ymin, q.y); Ymax = std::max(Ymax, q.y);
            Zmin = std::min(Zmin, q.z); Zmax = std::max(Zmax, q.z);
        }
    }
    double Max_Dim = 0;
    if (Xmax - Xmin > Max_Dim) Max_Dim = Xmax - Xmin;
    if (Ymax - Ymin > Max_Dim) Max_Dim = Ymax - Ymin;
    if (Zmax - Zmin > Max_Dim) Max_Dim = Zmax - Zmin;
    double cb[3] = {0, 0, 0};
    for (int e = 0; e < ne; ++e) {
        V3 n = body[e].ez, p = body[e].c;
        double A = body[e].area;
        cb[0] -= n.x * p.x * p.x * A; cb[1] -= n.y * p.y * p.y * A; cb[2] -= n.z * p.z * p.z * A;
    }
    for (int i = 0; i < 3; ++i) { cb[i] *= 0.5 / V; if (std::fabs(cb[i]) < Max_Dim * 1e-6) cb[i] = 0; }
    vol_cob[0] = V; vol_cob[1] = cb[0]; vol_cob[2] = cb[1]; vol_cob[3] = cb[2];
    double Mass = mass == 0 ? V * Rho_wat : mass;
    for (int i = 0; i < 36; ++i) { M[i] = 0; C[i] = 0; }
    auto Mi = [&](int i, int j) -> double& { return M[i * 6 + j]; };
    auto Ci = [&](int i, int j) -> double& { return C[i * 6 + j]; };
    Mi(0, 0) = Mass; Mi(1, 1) = Mass; Mi(2, 2) = Mass;
    Mi(0, 4) = Mass * cog[2]; Mi(1, 3) = -Mass * cog[2];
    Mi(0, 5) = -Mass * cog[1]; Mi(2, 3) = Mass * cog[1];
    Mi(1, 5) = Mass * cog[0]; Mi(2, 4) = -Mass * cog[0];
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) Mi(3 + i, j) = -Mi(i, 3 + j);
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) Mi(3 + i, 3 + j) = Mass * gyr[3 * i + j] * std::fabs(gyr[3 * i + j]);
    double AFS = 0, MOAx = 0, MOAy = 0, MOAxx = 0, MOAxy = 0, MOAyy = 0;
    if (ne_aux > 0) {
        Mesh ma = make_mesh(nn_aux, aux_nodes, ne_aux, aux_elems, ncomp_aux, aux_comp_first, aux_comp_origin);
        std::vector<Panel> ab, am;
        build_panels(ma, ab, am);
        for (int e = 0; e < ne_aux; ++e) {
            V3 p = ab[e].c; double A = ab[e].area;
            AFS += A; MOAy += A * p.y; MOAx += A * p.x; MOAxy += A * p.x * p.y;
            MOAxx += A * p.x * p.x; MOAyy += A * p.y * p.y;
        }
    }
    double rw = Rho_wat;
    Ci(2, 2) = rho * g * AFS;
    Ci(2, 3) = rho * g * MOAy;
    Ci(2, 4) = -rho * g * MOAx;
    Ci(3, 3) = rho * g * MOAyy + rw * g * V * cb[2] - Mass * g * cog[2];
    Ci(3, 4) = -rho * g * MOAxy;
    Ci(3, 5) = -rho * g * V * cb[0] + Mass * g * cog[0];
    Ci(4, 4) = rho * g * MOAxx + rw * g * V * cb[2] - Mass * g * cog[2];
    Ci(4, 5) = -rho * g * V * cb[1] + Mass * g * cog[1];
    Ci(2, 3) = Ci(3, 2);
    Ci(2, 4) = Ci(4, 2);
    Ci(3, 4) = Ci(4, 3);
}

// Hydrodynamic_Radiation_Solver::Solve (Hydrodynamic_Solver.cpp:400-487) for a
// list of internal angular frequencies Omega (the reference computes
// Omega = Frequency/(2 pi) at :405; callers pass Omega).  Per frequency f:
//   A[36f..], B[36f..] (row-major 6x6), FK/SC/F/RAO[2*6*nb*f..] (6 x nb complex,
//   row-major, interleaved), and optionally phiJ (N x 6) / phiS (N x nb) of the
//   last frequency.  M, C: 6x6 row-major mass and stiffness.
// RAO uses B_ijOm := Omega * B_ij (Hydrodynamic_Solver.h:57 leaves it unset).
// The frequency loop of Solve() over the system panels `body` (mirror images `mir`);
// forces integrate over the first NPA (hull) panels.  IFR (Create_Panels :45-55)
// appends the interior free-surface panels after the hull and solves a zero
// frequency at Omega = 1e-3 (:406).
// Optional stage clock of solve_panels (orc_solve_timed): [0] setup (Rankine
// matrices, N_k), then per frequency [1 + 3f] wave assembly + compose, [2 + 3f]
// LU, [3 + 3f] right-hand sides, solves and post; wall seconds.
static double* g_stage_clock = nullptr;

static void solve_panels(const std::vector<Panel>& body, const std::vector<Panel>& mir, int NPA, bool ifr,
                         int nfreq, const double* omegas, int nbeta, const double* betas, const double* Mmat,
                         const double* Cmat, double* A_out, double* B_out, double* FK_out, double* SC_out,
                         double* F_out, double* RAO_out, double* phiJ_out, double* phiS_out) {
    double* clk = g_stage_clock;
    double t0 = omp_get_wtime();
    std::vector<V3> x = collocation(body);
    const int N = (int)body.size(), NB = nbeta;
    std::vector<double> s((size_t)N * N), sr((size_t)N * N), d((size_t)N * N), dr((size_t)N * N), rn(N);
    #pragma omp parallel for schedule(dynamic, 4)
    for (int S = 0; S < N; ++S) {
        rn[S] = body[S].ez.z * 2.0;
        for (int R = 0; R < N; ++R) {
            size_t o = (size_t)R * N + S;
            inf_source_kernel(body[S], x[R], s[o], d[o]);
            inf_source_kernel(mir[S], x[R], sr[o], dr[o]);
        }
    }
    // Set_RHS_Mat (:117-138) and Prepare_PostProcessing_Mats (:140-175)
    std::vector<double> Nk((size_t)N * 6), area(N);
    for (int i = 0; i < N; ++i) {
        V3 P = body[i].c, Nn = body[i].ez, PCN = cross(P, Nn);
        double* r = &Nk[(size_t)i * 6];
        r[0] = Nn.x; r[1] = Nn.y; r[2] = Nn.z; r[3] = PCN.x; r[4] = PCN.y; r[5] = PCN.z;
        area[i] = body[i].area;
    }
    std::vector<cplx> Smat((size_t)N * N), Dmat((size_t)N * N);
    std::vector<int> piv(N);
    if (clk) clk[0] = omp_get_wtime() - t0;
    for (int f = 0; f < nfreq; ++f) {
        t0 = omp_get_wtime();
        double Omega = omegas[f];
        if (Omega == 0.0 && ifr) Omega = 1.0e-3;
        double Kappa = Omega * Omega / Gravity;  // :409 uses the global Gravity
        bool wave = Omega != 0.0;
        #pragma omp parallel for schedule(dynamic, 4)
        for (int S = 0; S < N; ++S)
            for (int R = 0; R < N; ++R) {
                size_t o = (size_t)R * N + S;
                cplx Sv(-s[o] - sr[o], 0.0), Dv(d[o] + dr[o], 0.0);
                if (wave) {
                    cplx ws, wd;
                    wave_panel_influence(mir[S], x[R], Kappa, ws, wd);
                    // SWave = -ws; DWave = wd + SSrcRefl*ReflNorm*Kappa  (:199-200)
                    Sv = cplx(-s[o], 0.0) + cplx(-sr[o], 0.0) + (-ws);
                    Dv = cplx(d[o], 0.0) + cplx(dr[o], 0.0) + (wd + cplx(-sr[o], 0.0) * rn[S] * Kappa);
                }
                Smat[o] = Sv;
                Dmat[o] = Dv;
            }
        double t1 = omp_get_wtime();
        if (clk) clk[1 + 3 * f] = t1 - t0;
        lu_factor(N, Dmat.data(), piv.data());
        t0 = omp_get_wtime();
        if (clk) clk[2 + 3 * f] = t0 - t1;
        // Set_Incident_Potential_Mats (:575-596), Calc_Phi_Incident (:544-573)
        std::vector<cplx> PhiI((size_t)N * NB), dPhiI((size_t)N * NB);
        for (int P = 0; P < N; ++P) {
            V3 pos = body[P].c, nrm = body[P].ez;
            for (int b = 0; b < NB; ++b) {
                double CB = std::cos(betas[b]), SB = std::sin(betas[b]);
                cplx Im(0.0, 1.0);
                cplx phiI = Im * Gravity / Omega * std::exp(Im * Kappa * (pos.x * CB + pos.y * SB));
                double Zf = std::exp(Kappa * pos.z);
                cplx pi_ = Zf * phiI;
                cplx dpx = Im * Kappa * CB * pi_, dpy = Im * Kappa * SB * pi_, dpz = Kappa * pi_;
                PhiI[(size_t)P * NB + b] = pi_;
                dPhiI[(size_t)P * NB + b] = nrm.x * dpx + nrm.y * dpy + nrm.z * dpz;
            }
        }
        // RHS = S * [N_k | -dPhiI .* area]   (:437, :445)
        const int NR = 6 + NB;
        std::vector<cplx> rhs((size_t)N * NR);
        #pragma omp parallel for schedule(static)
        for (int R = 0; R < N; ++R) {
            for (int j = 0; j < NR; ++j) {
                cplx acc(0, 0);
                for (int S = 0; S < N; ++S) {
                    cplx bv = j < 6 ? cplx(Nk[(size_t)S * 6 + j], 0.0)
                                    : -dPhiI[(size_t)S * NB + (j - 6)] * area[S];
                    acc += Smat[(size_t)R * N + S] * bv;
                }
                rhs[(size_t)R * NR + j] = acc;
            }
        }
        lu_solve(N, Dmat.data(), piv.data(), NR, rhs.data());
        // Post (:462-487) over the NPA hull panels (:452-457 cut the solutions)
        cplx AM[36];
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                cplx acc(0, 0);
                for (int p = 0; p < NPA; ++p) acc += (Nk[(size_t)p * 6 + i] * area[p]) * rhs[(size_t)p * NR + j];
                AM[i * 6 + j] = acc;
            }
        for (int i = 0; i < 36; ++i) { A_out[36 * f + i] = AM[i].real(); B_out[36 * f + i] = AM[i].imag(); }
        cplx Im(0.0, 1.0);
        std::vector<cplx> F(6 * NB);
        for (int i = 0; i < 6; ++i)
            for (int b = 0; b < NB; ++b) {
                cplx f1(0, 0), f2(0, 0);
                for (int p = 0; p < NPA; ++p) {
                    f1 += (Nk[(size_t)p * 6 + i] * area[p]) * PhiI[(size_t)p * NB + b];
                    f2 += rhs[(size_t)p * NR + i] * (dPhiI[(size_t)p * NB + b] * area[p]);
                }
                cplx FK = -Im * Omega * f1;
                cplx SC = Im * Omega * f2;
                cplx Fv = std::conj(FK + SC);
                if (Omega == 0.0) { FK = 0; Fv = 0; SC = 0; }
                size_t o = 2 * ((size_t)f * 6 * NB + i * NB + b);
                FK_out[o] = FK.real(); FK_out[o + 1] = FK.imag();
                SC_out[o] = SC.real(); SC_out[o + 1] = SC.imag();
                F_out[o] = Fv.real(); F_out[o + 1] = Fv.imag();
                F[i * NB + b] = Fv;
            }
        cplx LHS[36], LHSi[36];
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                double a = A_out[36 * f + i * 6 + j], bb = B_out[36 * f + i * 6 + j];
                LHS[i * 6 + j] = -Omega * Omega * (a + Mmat[i * 6 + j] / Rho_wat) + Omega * Im * (Omega * bb) +
                                 Cmat[i * 6 + j] / Rho_wat;
            }
        inv6(LHS, LHSi);
        for (int i = 0; i < 6; ++i)
            for (int b = 0; b < NB; ++b) {
                cplx acc(0, 0);
                for (int k = 0; k < 6; ++k) acc += LHSi[i * 6 + k] * F[k * NB + b];
                size_t o = 2 * ((size_t)f * 6 * NB + i * NB + b);
                RAO_out[o] = acc.real(); RAO_out[o + 1] = acc.imag();
            }
        if (f == nfreq - 1) {
            if (phiJ_out)
                for (int p = 0; p < NPA; ++p)
                    for (int j = 0; j < 6; ++j) {
                        phiJ_out[2 * ((size_t)p * 6 + j)] = rhs[(size_t)p * NR + j].real();
                        phiJ_out[2 * ((size_t)p * 6 + j) + 1] = rhs[(size_t)p * NR + j].imag();
                    }
            if (phiS_out)
                for (int p = 0; p < NPA; ++p)
                    for (int b = 0; b < NB; ++b) {
                        phiS_out[2 * ((size_t)p * NB + b)] = rhs[(size_t)p * NR + 6 + b].real();
                        phiS_out[2 * ((size_t)p * NB + b) + 1] = rhs[(size_t)p * NR + 6 + b].imag();
                    }
        }
        if (clk) clk[3 + 3 * f] = omp_get_wtime() - t0;
    }
}


void orc_solve(int nn, const double* nodes, int ne, const int* elems, int ncomp, const int* comp_first,
               const double* comp_origin, int nfreq, const double* omegas, int nbeta, const double* betas,
               double grav_unused, const double* Mmat, const double* Cmat,
               double* A_out, double* B_out, double* FK_out, double* SC_out, double* F_out, double* RAO_out,
               double* phiJ_out, double* phiS_out) {
    (void)grav_unused;
    Mesh m = make_mesh(nn, nodes, ne, elems, ncomp, comp_first, comp_origin);
    std::vector<Panel> body, mir;
    build_panels(m, body, mir);
    solve_panels(body, mir, ne, false, nfreq, omegas, nbeta, betas, Mmat, Cmat, A_out, B_out, FK_out, SC_out, F_out,
                 RAO_out, phiJ_out, phiS_out);
}

// orc_solve with the stage clock of solve_panels: clock receives 1 + 3 nfreq wall times.
void orc_solve_timed(int nn, const double* nodes, int ne, const int* elems, int ncomp, const int* comp_first,
                     const double* comp_origin, int nfreq, const double* omegas, int nbeta, const double* betas,
                     const double* Mmat, const double* Cmat, double* A_out, double* B_out, double* FK_out,
                     double* SC_out, double* F_out, double* RAO_out, double* clock) {
    g_stage_clock = clock;
    orc_solve(nn, nodes, ne, elems, ncomp, comp_first, comp_origin, nfreq, omegas, nbeta, betas, 9.81, Mmat, Cmat,
              A_out, B_out, FK_out, SC_out, F_out, RAO_out, nullptr, nullptr);
    g_stage_clock = nullptr;
}

// IFR: the hull mesh and the interior free-surface (aux) mesh.
void orc_solve_ifr(int nn, const double* nodes, int ne, const int* elems, int ncomp, const int* comp_first,
                   const double* comp_origin, int ann, const double* anodes, int ane, const int* aelems, int ancomp,
                   const int* acomp_first, const double* acomp_origin, int nfreq, const double* omegas, int nbeta,
                   const double* betas, const double* Mmat, const double* Cmat, double* A_out, double* B_out,
                   double* FK_out, double* SC_out, double* F_out, double* RAO_out, double* phiJ_out,
                   double* phiS_out) {
    Mesh m = make_mesh(nn, nodes, ne, elems, ncomp, comp_first, comp_origin);
    Mesh am = make_mesh(ann, anodes, ane, aelems, ancomp, acomp_first, acomp_origin);
    std::vector<Panel> body, mir, abody, amir;
    build_panels(m, body, mir);
    build_panels(am, abody, amir);
    body.insert(body.end(), abody.begin(), abody.end());
    mir.insert(mir.end(), amir.begin(), amir.end());
    solve_panels(body, mir, ne, true, nfreq, omegas, nbeta, betas, Mmat, Cmat, A_out, B_out, FK_out, SC_out, F_out,
                 RAO_out, phiJ_out, phiS_out);
}

// Exterior outputs of one frequency from given potentials Phi_J (N x 6) and
// Phi_S (N x nb), complex interleaved:
//   * free-surface elevation at nw points (Prepare_FS_Linear_System :205-231,
//     Prepare_FS_Linear_System_Wave_Terms :233-266, Solve :498-505)
//       ExtRad  = -i Omega/g ((Sext + Srefl + Swave) N_k   - (Dext + Drefl + Dwave) Phi_J)
//       ExtDiff = -i Omega/g ((Sext + Srefl + Swave) dPhiI  + (Dext + Drefl + Dwave) Phi_S)
//     with Swave = -ws, Dwave = wd + Srefl 2 n_z K;
//   * Kochin functions (Set_Kochin_Mats :598-642, Solve :492-494) at
//     theta_i = (i + 1/2) 2 pi / nk, with E = exp(K z + i K (x cos t + y sin t)) at the
//     panel centroids -- the reference reads an uninitialised E there (:626-627).
// Outputs: fs_rad [nw][6], fs_diff [nw][nb], k_rad [nk][6], k_diff [nk][nb].
void orc_exterior(int nn, const double* nodes, int ne, const int* elems, int ncomp, const int* comp_first,
                  const double* comp_origin, double Omega, int nbeta, const double* betas, const double* phiJ,
                  const double* phiS, int nw, const double* wpts, int nk, double* fs_rad, double* fs_diff,
                  double* k_rad, double* k_diff) {
    Mesh m = make_mesh(nn, nodes, ne, elems, ncomp, comp_first, comp_origin);
    std::vector<Panel> body, mir;
    build_panels(m, body, mir);
    const int N = ne, NB = nbeta;
    const double Kappa = Omega * Omega / Gravity;
    const cplx Im(0.0, 1.0);
    std::vector<double> Nk((size_t)N * 6);
    std::vector<cplx> dPhiI((size_t)N * NB), PJ((size_t)N * 6), PS((size_t)N * NB);
    for (int i = 0; i < N; ++i) {
        V3 P = body[i].c, Nn = body[i].ez, PCN = cross(P, Nn);
        double* r = &Nk[(size_t)i * 6];
        r[0] = Nn.x; r[1] = Nn.y; r[2] = Nn.z; r[3] = PCN.x; r[4] = PCN.y; r[5] = PCN.z;
        for (int j = 0; j < 6; ++j) PJ[(size_t)i * 6 + j] = cplx(phiJ[2 * (i * 6 + j)], phiJ[2 * (i * 6 + j) + 1]);
        for (int b = 0; b < NB; ++b) {
            PS[(size_t)i * NB + b] = cplx(phiS[2 * (i * NB + b)], phiS[2 * (i * NB + b) + 1]);
            if (Omega == 0.0) continue;  // k_incident: no incident wave at Omega = 0
            double CB = std::cos(betas[b]), SB = std::sin(betas[b]);
            cplx phi = Im * Gravity / Omega * std::exp(Im * Kappa * (P.x * CB + P.y * SB)) * std::exp(Kappa * P.z);
            cplx dpx = Im * Kappa * CB * phi, dpy = Im * Kappa * SB * phi, dpz = Kappa * phi;
            dPhiI[(size_t)i * NB + b] = Nn.x * dpx + Nn.y * dpy + Nn.z * dpz;
        }
    }
    #pragma omp parallel for schedule(dynamic, 1)
    for (int w = 0; w < nw; ++w) {
        V3 P = v3(wpts[3 * w], wpts[3 * w + 1], wpts[3 * w + 2]);
        std::vector<cplx> acc(6 + NB, cplx(0, 0));
        for (int S = 0; S < N; ++S) {
            double s, d, sr, dr;
            inf_source_kernel(body[S], P, s, d);
            inf_source_kernel(mir[S], P, sr, dr);
            cplx ws(0, 0), wd(0, 0);
            wave_panel_influence(mir[S], P, Kappa, ws, wd);
            const double rn = body[S].ez.z * 2.0;
            cplx WS = cplx(-s, 0.0) + cplx(-sr, 0.0) + (-ws);
            cplx WD = cplx(d, 0.0) + cplx(dr, 0.0) + (wd + cplx(-sr, 0.0) * rn * Kappa);
            for (int j = 0; j < 6; ++j) acc[j] += WS * Nk[(size_t)S * 6 + j] - WD * PJ[(size_t)S * 6 + j];
            for (int b = 0; b < NB; ++b) acc[6 + b] += WS * dPhiI[(size_t)S * NB + b] + WD * PS[(size_t)S * NB + b];
        }
        const cplx c = -Im * Omega / Gravity;
        for (int j = 0; j < 6; ++j) {
            cplx v = c * acc[j];
            fs_rad[2 * (w * 6 + j)] = v.real(); fs_rad[2 * (w * 6 + j) + 1] = v.imag();
        }
        for (int b = 0; b < NB; ++b) {
            cplx v = c * acc[6 + b];
            fs_diff[2 * (w * NB + b)] = v.real(); fs_diff[2 * (w * NB + b) + 1] = v.imag();
        }
    }
    for (int i = 0; i < nk; ++i) {
        double th = (0.5 + 1.0 * i) * TwoPI / nk, CTH = std::cos(th), STH = std::sin(th);
        std::vector<cplx> acc(6 + NB, cplx(0, 0));
        for (int p = 0; p < N; ++p) {
            V3 P = body[p].c, Nn = body[p].ez;
            cplx E = std::exp(cplx(Kappa * P.z, Kappa * (P.x * CTH + P.y * STH)));
            cplx dEdx = Im * Kappa * CTH * E, dEdy = Im * Kappa * STH * E, dEdz = Kappa * E;
            cplx KE = E * body[p].area;
            cplx KdE = (Nn.x * dEdx + Nn.y * dEdy + Nn.z * dEdz) * body[p].area;
            for (int j = 0; j < 6; ++j) acc[j] += KE * Nk[(size_t)p * 6 + j] - KdE * PJ[(size_t)p * 6 + j];
            for (int b = 0; b < NB; ++b) acc[6 + b] += KE * dPhiI[(size_t)p * NB + b] - KdE * PS[(size_t)p * NB + b];
        }
        for (int j = 0; j < 6; ++j) { k_rad[2 * (i * 6 + j)] = acc[j].real(); k_rad[2 * (i * 6 + j) + 1] = acc[j].imag(); }
        for (int b = 0; b < NB; ++b) {
            k_diff[2 * (i * NB + b)] = acc[6 + b].real();
            k_diff[2 * (i * NB + b) + 1] = acc[6 + b].imag();
        }
    }
}

}  // extern "C"
