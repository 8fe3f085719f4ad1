// green.cuh -- device forms of the infinite-depth wave Green function.
//
// HavelockGF of the reference (src/Kernels.cpp:342-412): the Liang/Wu/Noblesse
// global approximation of the free-surface term,
//   G    = L0(d, v, alpha, beta, rho) + 2 pi e^v (H0(h) - i J0(h))
//   dG/dh = Ls(...)                  + 2 pi e^v ((2/pi - H1(h)) + i J1(h))
//   dG/dx = dG/dh x/h, dG/dy = dG/dh y/h (0 for h <= 1e-6), dG/dz = G
// with h = sqrt(x^2+y^2), d = sqrt(h^2+v^2), alpha = -v/d, beta = h/d,
// rho = d/(1+d).  L0 and Ls use the polynomial fits of Liang, Wu & Noblesse,
// Appl. Ocean Res. 74 (2018), eq. 14a-c / 16a-c; H0/H1 the Struve fits of
// Kernels.cpp:35-116.  J0/J1/Y0/Y1 are CUDA's j0/j1/y0/y1 in FP64; in FP32
// they are the Abramowitz & Stegun 9.4.1-9.4.6 polynomial forms below
// (bessel_j01_small, bessel_large), not CUDA's j0f/j1f/y0f/y1f.
//
// gf64: FP64, same operation order as the reference (a common subexpression
//       e^v is computed once; the reference recomputes the same value).
// gf32: FP32.  The polynomials have coefficients up to 2e5 with alternating
//       signs, which cancel badly in FP32 around rho ~ 0.5; gf32 evaluates
//       each one re-expanded about rho = 1/2, which is the same polynomial; the
//       coefficients are compile-time literals (BEM_P32_*), so they stay instruction
//       operands rather than constant-memory loads.
#pragma once
#include <cuda_runtime.h>

namespace bem {

struct cd { double re, im; };
struct cf { float re, im; };

// Monomial coefficients, ascending powers of rho (Kernels.cpp:120-256).
#define BEM_POLY_TABLE(X)                                                                                     \
    X(A, 10, 1.21, -13.328, 215.896, -1763.96, 8418.94, -24314.21, 42002.57, -41592.9, 21859.0, -4838.6)      \
    X(B, 10, 0.938, 5.737, -67.92, 796.534, -4780.77, 17137.74, -36618.81, 44894.06, -29030.24, 7671.22)      \
    X(C, 8, 1.268, -9.747, 209.653, -1397.89, 5155.67, -9844.35, 9136.4, -3272.62)                           \
    X(D, 10, 0.632, -40.97, 667.16, -6072.07, 31127.39, -96293.05, 181856.75, -205690.43, 128170.2, -33744.6) \
    X(dA, 10, 2.948, -24.53, 249.69, -754.85, -1187.71, 16370.75, -48811.41, 68220.87, -46688.0, 12622.25)    \
    X(dB, 10, 1.11, 2.894, -76.765, 1565.35, -11336.19, 44270.15, -97014.11, 118879.26, -76209.82, 19923.28)  \
    X(dC, 6, 14.19, -148.24, 847.8, -2318.58, 3168.35, -1590.27)

// Incremental-power evaluation exactly as the reference writes it:
// S = c0; t = x; S += c_i t; t *= x.
__device__ __forceinline__ double poly_inc64(const double* c, int n, double x) {
    double S = c[0], t = x;
#pragma unroll
    for (int i = 1; i < 10; ++i) {
        if (i < n) { S += c[i] * t; t *= x; }
    }
    return S;
}

struct PolyCoef64 {
    double A[10], B[10], C[10], D[10], dA[10], dB[10], dC[10];
};

// Shifted-basis coefficients for FP32, ascending powers: p(rho) = sum_k s_k (rho - 1/2)^k,
// s_j = sum_{i >= j} c_i C(i, j) 2^-(i-j) from BEM_POLY_TABLE's c_i, rounded to float.
// BEM_P32_h1s, BEM_P32_h1d: the two forms of 2/pi - H1(x) that dG/dh needs (h1_gap32):
//   h1s: x <= 3, 2/pi - yy P(yy) (yy = (x/3)^2, P the series of BEM_H1_SMALL) re-expanded
//        about yy = 1/2 and rescaled to t = x^2 - 9/2 = 9 (yy - 1/2);
//   h1d: x > 3, 2 (c2_i - c1_i) of BEM_H1_C1 / BEM_H1_C2, leading terms cancelled.
// tests/test_poly32.py recomputes every value with rational arithmetic.
#define BEM_P32_A 1.671640635e+00f, 1.321628094e+01f, 9.012850189e+01f, 2.129387512e+02f, -2.447474976e+02f, -1.760199951e+03f, -1.364880005e+03f, 2.295699951e+03f, 8.530000305e+01f, -4.838600098e+03f
#define BEM_P32_B 3.298913956e+00f, -6.148437411e-02f, -3.370587540e+01f, 3.631500006e+00f, 3.526837463e+02f, 1.743025055e+02f, -2.153469971e+03f, -2.185919922e+03f, 5.490250000e+03f, 7.671220215e+03f
#define BEM_P32_C 5.853843689e+00f, 8.096312523e+00f, -4.139637375e+01f, -1.528125000e+01f, 4.885824890e+02f, 3.835950012e+02f, -2.317770020e+03f, -3.272620117e+03f
#define BEM_P32_D -6.455031395e+00f, -3.069187546e+01f, -2.602031326e+01f, 1.522068787e+02f, 3.372087402e+02f, 8.551174927e+02f, 4.813345215e+03f, 3.288969971e+03f, -2.368050000e+04f, -3.374460156e+04f
#define BEM_P32_dA 8.678410530e+00f, 1.629613304e+01f, -6.745562744e+01f, -1.360637512e+02f, 6.027931519e+02f, 6.803062744e+02f, -4.320740234e+03f, -4.930879883e+03f, 1.011212500e+04f, 1.262225000e+04f
#define BEM_P32_dB 8.081609726e+00f, 1.605587578e+01f, -6.992500305e+01f, -1.364287567e+02f, 6.629874878e+02f, 7.710250244e+02f, -5.211000000e+03f, -6.650500000e+03f, 1.344494043e+04f, 1.992327930e+04f
#define BEM_P32_dC 1.052343750e+01f, 4.784062576e+01f, 1.346174927e+02f, 4.244499969e+01f, -8.073250122e+02f, -1.590270020e+03f
#define BEM_P32_h1s -6.614897400e-02f, -1.072273552e-01f, 9.413545020e-03f, -3.010456858e-04f, 5.088115813e-06f, -5.358563371e-08f, 3.898513734e-10f
#define BEM_P32_h1d -7.999999951e-08f, -2.222040147e-01f, -7.735215425e-01f, -3.313150704e-01f

// Horner's rule on literal coefficients in ascending order: hornerc(u, c0, .., cn) =
// c0 + u (c1 + u (... + u cn)), each step one FMA (the order of horner32).
__device__ __forceinline__ float hornerc(float, float c0) { return c0; }
template <typename... T>
__device__ __forceinline__ float hornerc(float u, float c0, T... cs) {
    return fmaf(hornerc(u, cs...), u, c0);
}

// The reference's StruveH1 constants (Kernels.cpp:76-116): small-argument series
// coefficients and the large-argument rational c1 / c2.
#define BEM_H1_SMALL 1.909859286, -1.145914713, 0.294656958, -0.042070508, 0.003785727, -0.000207183
#define BEM_H1_C1 1.00000004, 3.92205313, 2.64893033, 0.27450895
#define BEM_H1_C2 1.0, 3.81095112, 2.26216956, 0.10885141

// ---- FP64 -----------------------------------------------------------------
__device__ __forceinline__ double struve_h0_64(double x, double y0x) {
    if (x <= 3.0) {
        double yy = (x / 3.0) * (x / 3.0);
        double s = 1.909859164 + (-1.909855001 + (0.687514637 + (-0.126164557 + (0.013828813 + -0.000876918 * yy) * yy) * yy) * yy) * yy;
        return s * (x / 3.0);
    }
    double yy = (3.0 / x) * (3.0 / x);
    double c1 = 2.0 * (0.99999906 + (4.77228920 + (3.85542044 + 0.32303607 * yy) * yy) * yy);
    double c2 = 3.14159265358979323846 * x * (1.0 + (4.88331068 + (4.28957333 + 0.52120508 * yy) * yy) * yy);
    return c1 / c2 + y0x;
}
__device__ __forceinline__ double struve_h1_64(double x, double y1x) {
    if (x <= 3.0) {
        double yy = (x / 3.0) * (x / 3.0);
        return (1.909859286 + (-1.145914713 + (0.294656958 + (-0.042070508 + (0.003785727 + -0.000207183 * yy) * yy) * yy) * yy) * yy) * yy;
    }
    double yy = (3.0 / x) * (3.0 / x);
    double c1 = 2.0 * (1.00000004 + (3.92205313 + (2.64893033 + 0.27450895 * yy) * yy) * yy);
    double c2 = 3.14159265358979323846 * (1.0 + (3.81095112 + (2.26216956 + 0.10885141 * yy) * yy) * yy);
    return c1 / c2 + y1x;
}

// Returns G and dG/dh (complex).  dx, dy only enter through h here.
__device__ __forceinline__ void gf64(const PolyCoef64& P, double hh, double vv, cd& G, cd& Gh) {
    const double PI = 3.14159265358979323846;
    const double EUL = 0.5772156649;
    double dd = sqrt(hh * hh + vv * vv);
    double alpha = -vv / dd;
    double beta = hh / dd;
    double rho = dd / (1.0 + dd);
    double ev = exp(vv);
    double d2 = dd * dd;
    double d3 = d2 * dd;
    // GF_Func_L0 (Kernels.cpp:258-282)
    double PP = log(0.5 * (dd - vv)) + EUL - 2.0 * d2;
    PP *= ev;
    PP += d2 - vv;
    double A = poly_inc64(P.A, 10, rho), B = poly_inc64(P.B, 10, rho);
    double C = poly_inc64(P.C, 8, rho), D = poly_inc64(P.D, 10, rho);
    double omr = 1.0 - rho;
    double RR = (1.0 - beta) * A;
    RR -= beta * B;
    RR -= alpha * C / (1.0 + 6.0 * alpha * rho * omr);
    RR += beta * (1.0 - beta) * D;
    double r3 = rho * (omr * omr * omr);
    double L0 = 2.0 * PP / (1.0 + d3) + 2.0 * (r3 * RR);
    // GF_Func_W (:284-295), GF_Func_Wh (:327-338)
    bool far = hh > 3.0;
    double j0v = j0(hh), j1v = j1(hh);
    double y0v = far ? y0(hh) : 0.0, y1v = far ? y1(hh) : 0.0;
    double H0 = struve_h0_64(hh, y0v), H1 = struve_h1_64(hh, y1v);
    double E = 2.0 * PI * ev;
    G.re = L0 + E * H0;
    G.im = -E * j0v;
    // GF_Func_Ls (:297-325)
    double PS = (beta + hh) / (dd - vv);
    PS -= 2.0 * beta;
    PS += 2.0 * dd * ev;
    PS -= hh;
    double QS = exp(-dd) * (1.0 - beta);
    QS *= 1.0 + dd / (1.0 + d3);
    double a2 = poly_inc64(P.dA, 10, rho), b2 = poly_inc64(P.dB, 10, rho), c2 = poly_inc64(P.dC, 6, rho);
    double RS = beta * a2;
    RS -= (1.0 - alpha) * b2;
    RS += beta * (1.0 - beta) * rho * (1.0 - 2.0 * rho) * c2;
    double Ls = 2.0 * PS / (1.0 + d3) - 4.0 * QS + 2.0 * (r3 * RS);
    Gh.re = Ls + E * (2.0 / PI - H1);
    Gh.im = E * j1v;
}

// ---- FP32 -----------------------------------------------------------------
// t3 = 3 / x (used for x > 3), computed once by the caller for all the x > 3 forms.
__device__ __forceinline__ float struve_h0_32(float x, float y0x, float t3) {
    if (x <= 3.0f) {
        float yy = (x * (1.0f / 3.0f)) * (x * (1.0f / 3.0f));
        float s = fmaf(fmaf(fmaf(fmaf(fmaf(-0.000876918f, yy, 0.013828813f), yy, -0.126164557f), yy, 0.687514637f), yy, -1.909855001f), yy, 1.909859164f);
        return s * (x * (1.0f / 3.0f));
    }
    float yy = t3 * t3;
    float c1 = 2.0f * fmaf(fmaf(fmaf(0.32303607f, yy, 3.85542044f), yy, 4.77228920f), yy, 0.99999906f);
    float c2 = 3.14159265f * x * fmaf(fmaf(fmaf(0.52120508f, yy, 4.28957333f), yy, 4.88331068f), yy, 1.0f);
    return __fdividef(c1, c2) + y0x;
}
// 2/pi - H1(x), which dG/dh multiplies by 2 pi e^v.  H1 tends to 2/pi, so the
// plain difference of two FP32 values loses several bits (about 1e-6 of dG/dh
// near h ~ 2.5 and h ~ 8).  The same function is evaluated without that
// cancellation: for x <= 3 the series 2/pi - yy P(yy), yy = (x/3)^2, re-expanded
// about yy = 1/2 with t = x^2 - 9/2 formed by one FMA; for x > 3,
// 2/pi - c1/c2 = ((2/pi) c2 - c1) / c2 with the numerator's coefficients
// subtracted exactly on the host, so only Y1 is added to a small, accurate term.
__device__ __forceinline__ float h1_gap32(float x, float y1x, float t3) {
    if (x <= 3.0f) {
        const float t = fmaf(x, x, -4.5f);
        return hornerc(t, BEM_P32_h1s);
    }
    const float yy = t3 * t3;
    const float num = hornerc(yy, BEM_P32_h1d);
    const float c2 = 3.14159265f * fmaf(fmaf(fmaf(0.10885141f, yy, 2.26216956f), yy, 3.81095112f), yy, 1.0f);
    return __fdividef(num, c2) - y1x;
}

// ---- FP32 Bessel functions J0, J1, Y0, Y1 -----------------------------------
// Polynomial approximations of Abramowitz & Stegun 9.4.1-9.4.6 (E. E. Allen):
// for 0 < x <= 3 power series in (x/3)^2; for x >= 3 the modulus/phase forms
//   J_n = x^-1/2 f_n(3/x) cos theta_n,  Y_n = x^-1/2 f_n(3/x) sin theta_n,
//   theta_0 = x - pi/4 + d_0(3/x),  theta_1 = x - 3 pi/4 + d_1(3/x),
// absolute errors ~1e-8 (x^-1/2 * 1e-7 for x >= 3).  The large-argument phase is
// reduced in double-float arithmetic from the argument as a float pair (xh, xl),
// so the oscillatory far field keeps ~1e-7 relative accuracy for x in the
// hundreds, where an FP32 argument alone would carry a phase error ~x * 6e-8.
__device__ __forceinline__ void bessel_j01_small(float x, float& j0, float& j1) {
    const float y = (x * (1.0f / 3.0f)) * (x * (1.0f / 3.0f));
    j0 = fmaf(y, fmaf(y, fmaf(y, fmaf(y, fmaf(y, fmaf(y, 0.0002100f, -0.0039444f), 0.0444479f), -0.3163866f),
                                1.2656208f), -2.2499997f), 1.0f);
    j1 = x * fmaf(y, fmaf(y, fmaf(y, fmaf(y, fmaf(y, fmaf(y, 0.00001109f, -0.00031761f), 0.00443319f), -0.03954289f),
                                  0.21093573f), -0.56249985f), 0.5f);
}

// sin and cos of a phase already reduced to about [-pi, pi] (|x| < 8 keeps the
// reduction exact): quadrant q = rint(2x / pi), r = x - q pi/2 by a two-constant
// Cody-Waite step, then the Taylor series of sin to r^9 and of cos to r^10 on
// |r| <= pi/4 (truncation below 3e-9), and the quadrant's swap and signs.  The
// general sincosf also handles arguments far outside this range, which the
// Bessel phase never is.
__device__ __forceinline__ void sincos_reduced(float x, float& sn, float& cs) {
    const float PIO2_H = 1.57079637f, PIO2_L = -4.37113883e-8f;  // pi / 2 = H + L
    const float q = rintf(x * 0.636619772f);
    float r = fmaf(-q, PIO2_H, x);
    r = fmaf(-q, PIO2_L, r);
    const float r2 = r * r;
    const float ps = r * fmaf(r2, fmaf(r2, fmaf(r2, fmaf(r2, 1.0f / 362880.0f, -1.0f / 5040.0f), 1.0f / 120.0f),
                                       -1.0f / 6.0f), 1.0f);
    const float pc = fmaf(r2, fmaf(r2, fmaf(r2, fmaf(r2, fmaf(r2, -1.0f / 3628800.0f, 1.0f / 40320.0f), -1.0f / 720.0f),
                                             1.0f / 24.0f), -0.5f), 1.0f);
    const int iq = (int)q;
    const bool swap = iq & 1;
    const float s0 = swap ? pc : ps, c0 = swap ? ps : pc;
    sn = (iq & 2) ? -s0 : s0;
    cs = ((iq + 1) & 2) ? -c0 : c0;
}

__device__ __forceinline__ void bessel_large(float xh, float xl, float t3, float& j0, float& j1, float& y0,
                                             float& y1) {
    const float TWOPI_H = 6.28318548f, TWOPI_L = -1.74845553e-7f;  // 2 pi = H + L
    const float PI4_H = 0.785398185f, PI4_L = -2.18556949e-8f;     // pi / 4 = H + L
    const float t = t3;
    const float f0 = fmaf(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, 0.00014476f, -0.00072805f), 0.00137237f),
                                                -0.00009512f), -0.00552740f), -0.00000077f), 0.79788456f);
    const float d0 = t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, 0.00013558f, -0.00029333f), -0.00054125f),
                                           0.00262573f), -0.00003954f), -0.04166397f);
    const float f1 = fmaf(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, -0.00020033f, 0.00113653f), -0.00249511f),
                                                0.00017105f), 0.01659667f), 0.00000156f), 0.79788456f);
    const float d1 = t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, fmaf(t, -0.00029166f, 0.00079824f), 0.00074348f),
                                           -0.00637879f), 0.00005650f), 0.12499612f);
    // theta_0 = x - pi/4 + d0 - 2 pi k, as a float pair (ph, pl)
    const float k = rintf((xh - PI4_H) * 0.159154943f);
    const float a = fmaf(-k, TWOPI_H, xh);  // exact: |a| < 8 and a is a multiple of ulp(TWOPI_H)
    const float s = a - PI4_H;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (-PI4_H - bb);
    float pl = e + (fmaf(-k, TWOPI_L, xl) - PI4_L + d0);
    const float ph = s + pl;
    pl -= ph - s;
    float sn, cs;
    sincos_reduced(ph, sn, cs);
    const float s0 = fmaf(cs, pl, sn), c0 = fmaf(-sn, pl, cs);  // sin, cos theta_0
    // theta_1 = theta_0 - pi/2 + (d1 - d0); |d1 - d0| < 0.17 for x >= 3, where the
    // Taylor series below are exact to ~1e-12
    const float dl = d1 - d0, dl2 = dl * dl;
    const float se = dl * fmaf(dl2, fmaf(dl2, fmaf(dl2, -1.0f / 5040.0f, 1.0f / 120.0f), -1.0f / 6.0f), 1.0f);
    const float ce = fmaf(dl2, fmaf(dl2, fmaf(dl2, fmaf(dl2, 1.0f / 40320.0f, -1.0f / 720.0f), 1.0f / 24.0f), -0.5f), 1.0f);
    const float sa = fmaf(s0, ce, c0 * se);   // sin(theta_0 + d1 - d0) =  cos theta_1
    const float ca = fmaf(c0, ce, -s0 * se);  // cos(theta_0 + d1 - d0) = -sin theta_1
    const float rs = rsqrtf(xh);
    j0 = rs * f0 * c0;
    y0 = rs * f0 * s0;
    j1 = rs * f1 * sa;
    y1 = -rs * f1 * ca;
}

// Horizontal wave-number distance h = K sqrt(dx^2 + dy^2) as a float pair from
// coordinate differences given as float pairs (K = kh + kl).
__device__ __forceinline__ void df_hdist(float dxh, float dxl, float dyh, float dyl, float kh, float kl, float& hh,
                                         float& hl) {
    const float p = dxh * dxh, q = dyh * dyh;
    const float ep = fmaf(dxh, dxh, -p) + 2.0f * dxh * dxl;
    const float eq = fmaf(dyh, dyh, -q) + 2.0f * dyh * dyl;
    const float r2 = p + q;
    const float bb = r2 - p;
    const float r2l = ((p - (r2 - bb)) + (q - bb)) + (ep + eq);
    // sqrt(r2) to about an ulp from the reciprocal square root; rl, formed from the exact
    // residual r2 - rh^2, makes (rh, rl) the square root to second order all the same
    const float rs = r2 > 0.0f ? rsqrtf(r2) : 0.0f;
    const float rh = r2 * rs;
    const float rl = (fmaf(-rh, rh, r2) + r2l) * (0.5f * rs);
    const float h = kh * rh;
    const float h2 = fmaf(kh, rh, -h) + fmaf(kh, rl, kl * rh);
    hh = h + h2;
    hl = h2 - (hh - h);
}

__device__ __forceinline__ void gf32(float hh, float vv, cf& G, cf& Gh) {
    const float PI = 3.14159265358979f;
    const float EUL = 0.5772156649f;
    float dd = sqrtf(fmaf(hh, hh, vv * vv));
    float inv_d = 1.0f / dd;
    float alpha = -vv * inv_d;
    float beta = hh * inv_d;
    float rho = dd / (1.0f + dd);
    float u = rho - 0.5f;
    float ev = expf(vv);
    float d2 = dd * dd;
    float d3 = d2 * dd;
    float inv_1d3 = 1.0f / (1.0f + d3);
    float dmv = dd - vv;
    float PP = logf(0.5f * dmv) + EUL - 2.0f * d2;
    PP = fmaf(PP, ev, d2 - vv);
    float A = hornerc(u, BEM_P32_A), B = hornerc(u, BEM_P32_B);
    float C = hornerc(u, BEM_P32_C), D = hornerc(u, BEM_P32_D);
    float omr = 1.0f - rho;
    float RR = (1.0f - beta) * A - beta * B;
    RR -= alpha * C / fmaf(6.0f * alpha * rho, omr, 1.0f);
    RR = fmaf(beta * (1.0f - beta), D, RR);
    float r3 = rho * (omr * omr * omr);
    float L0 = 2.0f * PP * inv_1d3 + 2.0f * (r3 * RR);
    bool far = hh > 3.0f;
    const float t3 = far ? 3.0f * __frcp_rn(hh) : 0.0f;
    float j0v, j1v, y0v = 0.0f, y1v = 0.0f;
    if (far) bessel_large(hh, 0.0f, t3, j0v, j1v, y0v, y1v);
    else bessel_j01_small(hh, j0v, j1v);
    float H0 = struve_h0_32(hh, y0v, t3), H1g = h1_gap32(hh, y1v, t3);
    float E = 2.0f * PI * ev;
    G.re = fmaf(E, H0, L0);
    G.im = -E * j0v;
    float PS = (beta + hh) / dmv;
    PS -= 2.0f * beta;
    PS = fmaf(2.0f * dd, ev, PS);
    PS -= hh;
    float QS = expf(-dd) * (1.0f - beta);
    QS *= 1.0f + dd * inv_1d3;
    float a2 = hornerc(u, BEM_P32_dA), b2 = hornerc(u, BEM_P32_dB), c2 = hornerc(u, BEM_P32_dC);
    float RS = beta * a2 - (1.0f - alpha) * b2;
    RS = fmaf(beta * (1.0f - beta) * rho * (1.0f - 2.0f * rho), c2, RS);
    float Ls = 2.0f * PS * inv_1d3 - 4.0f * QS + 2.0f * (r3 * RS);
    Gh.re = fmaf(E, H1g, Ls);
    Gh.im = E * j1v;
}

// ---- FP32 real parts + imaginary-part remainders ----------------------------
// Real parts of G and dG/dh (as gf32 computes them).
// y0v, y1v: Y0(hh), Y1(hh), t3 = 3 / hh (used when hh > 3).
// Gv: dG/dv ~ Gr - 2/d (to about 1 %: the infinite-depth wave term satisfies dG/dv = G
// up to the Rankine image's 2/d), used for the first-order correction of the rounding of v.
__device__ __forceinline__ void gf32_re(float hh, float vv, float ev, float y0v, float y1v,
                                        float t3, float& Gr, float& Ghr, float& Gv) {
    const float PI = 3.14159265358979f;
    const float EUL = 0.5772156649f;
    // d from the reciprocal square root and one Newton step (within about an ulp);
    // 1/d is the reciprocal square root itself.  Approximate reciprocals (about an ulp)
    // scale terms whose FP32 rounding is of the same size.
    const float d2s = fmaf(hh, hh, vv * vv);
    const float inv_d = rsqrtf(d2s);
    float dd = d2s * inv_d;
    dd = fmaf(fmaf(-dd, dd, d2s), 0.5f * inv_d, dd);
    float alpha = -vv * inv_d;
    float beta = hh * inv_d;
    float rho = __fdividef(dd, 1.0f + dd);
    float u = rho - 0.5f;
    float d2 = dd * dd;
    float d3 = d2 * dd;
    float inv_1d3 = __fdividef(1.0f, 1.0f + d3);
    float dmv = dd - vv;
    float PP = __logf(0.5f * dmv) + EUL - 2.0f * d2;  // fast log: ~4e-7 absolute, scaled by e^v / (1 + d^3)
    PP = fmaf(PP, ev, d2 - vv);
    float A = hornerc(u, BEM_P32_A), B = hornerc(u, BEM_P32_B);
    float C = hornerc(u, BEM_P32_C), D = hornerc(u, BEM_P32_D);
    float omr = 1.0f - rho;
    float RR = (1.0f - beta) * A - beta * B;
    RR -= __fdividef(alpha * C, fmaf(6.0f * alpha * rho, omr, 1.0f));
    RR = fmaf(beta * (1.0f - beta), D, RR);
    float r3 = rho * (omr * omr * omr);
    float L0 = 2.0f * PP * inv_1d3 + 2.0f * (r3 * RR);
    float H0 = struve_h0_32(hh, y0v, t3), H1g = h1_gap32(hh, y1v, t3);
    float E = 2.0f * PI * ev;
    Gr = fmaf(E, H0, L0);
    Gv = fmaf(-2.0f, inv_d, Gr);
    float PS = __fdividef(beta + hh, dmv);
    PS -= 2.0f * beta;
    PS = fmaf(2.0f * dd, ev, PS);
    PS -= hh;
    // e^-d with the fast exponential: its error is relative to |d| e^-d, small beside the
    // other terms at every d
    float QS = __expf(-dd) * (1.0f - beta);
    QS *= 1.0f + dd * inv_1d3;
    float a2 = hornerc(u, BEM_P32_dA), b2 = hornerc(u, BEM_P32_dB), c2 = hornerc(u, BEM_P32_dC);
    float RS = beta * a2 - (1.0f - alpha) * b2;
    RS = fmaf(beta * (1.0f - beta) * rho * (1.0f - 2.0f * rho), c2, RS);
    float Ls = 2.0f * PS * inv_1d3 - 4.0f * QS + 2.0f * (r3 * RS);
    Ghr = fmaf(E, H1g, Ls);
}

}  // namespace bem
