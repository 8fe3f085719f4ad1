// k_influence.cu -- influence-matrix assembly and hull integrations on sm_103a.
//
//   k_rankine      Prepare_Linear_System (Hydrodynamic_Solver.cpp:83-115) with
//                  FlatQuad/TriPanel::Inf_SourceKernel (Panel.cpp:17-156), FP64.
//   k_wave<T>      Prepare_Linear_System_Wave_Terms (Hydrodynamic_Solver.cpp:177-203),
//                  FlatWave*Panel::CInf_SingleDoubleLayerQuad (Panel.cpp:676-694,
//                  776-794), FreeSurface_Wave_Kernel (:601-636), composed with the
//                  Rankine part (Solve :415-429) and with the source matrix applied
//                  to the right-hand sides (Solve :437, :445) so that S is never stored.
//   k_incident     Calc_Phi_Incident / Set_Incident_Potential_Mats (:544-596).
//   (Ssrc + Srefl) * B, the Rankine half of S * B, is launch_matx (k_lu.cu).
//   k_post_*       AddedMassMat * Phi_J, AddedMassMat * Phi_I, Phi_J^T (dPhi_I .* A)
//                  (:462-476).
//
// Matrix layout: row-major, row = receiver (collocation point), column = source
// panel, leading dimension ld (a multiple of 128).  Complex matrices are planar
// (separate re and im arrays).
#include "bem_internal.h"
#include <algorithm>
#include "green.cuh"
#include "mlp_tc.cuh"

namespace bem {

__constant__ PolyCoef64 c_poly64;

static const double kFourPIinv = 0.25 / 3.14159265358979323846;

// ---------------------------------------------------------------------------
// K1: analytic constant-strength source and dipole of a flat panel.
// Panel record (RK_STRIDE doubles): nv, c[3], ex[3], ey[3], ez[3], lx[4], ly[4],
// m[4], d[4]; lx/ly are the vertices in the panel frame, m the edge slopes and d
// the edge lengths, precomputed on the host exactly as Inf_SourceKernel does.
__device__ __forceinline__ void source_kernel(const double* __restrict__ p, double Px, double Py, double Pz,
                                              double& S, double& D) {
    const int n = (int)p[0];
    double dx = Px - p[1], dy = Py - p[2], dz = Pz - p[3];
    double PLx = p[4] * dx + p[5] * dy + p[6] * dz;
    double PLy = p[7] * dx + p[8] * dy + p[9] * dz;
    double PLz = p[10] * dx + p[11] * dy + p[12] * dz;
    double Z2 = PLz * PLz;
    double DX[4], DY[4], e[4], h[4], r[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (k < n) {
            DX[k] = PLx - p[13 + k];
            DY[k] = PLy - p[17 + k];
            e[k] = DX[k] * DX[k] + Z2;
            h[k] = DX[k] * DY[k];
            r[k] = sqrt(DX[k] * DX[k] + DY[k] * DY[k] + Z2);
        }
    }
    double Phi = 0.0, sumBL = 0.0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (k < n) {
            int k1 = (k + 1 < n) ? k + 1 : 0;
            double m = p[21 + k];
            // atan(A0 / (z r0)) - atan(A1 / (z r1)) as one atan2: both angles lie in
            // (-pi/2, pi/2), so their difference is the angle of (z (A0 r1 - A1 r0),
            // z^2 r0 r1 + A0 A1) (both multiplied by z^2 r0 r1 > 0).  Half the arctangents
            // and none of the divisions; a vertical edge (infinite slope) keeps the two terms.
            const double A0 = m * e[k] - h[k], A1 = m * e[k1] - h[k1];
            if (isfinite(m))
                Phi += atan2(PLz * (A0 * r[k1] - A1 * r[k]), Z2 * r[k] * r[k1] + A0 * A1);
            else
                Phi += atan(A0 / (PLz * r[k])) - atan(A1 / (PLz * r[k1]));
            double ddx = p[13 + k1] - p[13 + k], ddy = p[17 + k1] - p[17 + k];
            double d = p[25 + k];
            double B = (DX[k] * ddy - DY[k] * ddx) / d;
            double L = log((r[k] + r[k1] + d) / (r[k] + r[k1] - d));
            sumBL += B * L;
        }
    }
    D = Phi * kFourPIinv;
    S = (PLz * Phi - sumBL) * kFourPIinv;
}

// mode 0: RS = -(s + sr), RD = d + dr, RSR = -sr * 2 n_z(S)  (composed, ld stride)
// mode 1: o0 = s, o1 = sr, o2 = d, o3 = dr                    (raw, ld stride)
// mode 2: o0 = s, o1 = d of the body panels only               (aero G and H)
__global__ void __launch_bounds__(256) k_rankine(int N, int ld, const double* __restrict__ rec,
                                                 const double* __restrict__ xr, const double* __restrict__ rn,
                                                 int mode, double* __restrict__ o0, double* __restrict__ o1,
                                                 double* __restrict__ o2, double* __restrict__ o3) {
    int s = blockIdx.x * 32 + threadIdx.x;
    int r = blockIdx.y * 8 + threadIdx.y;
    if (s >= N || r >= N) return;
    double Px = xr[r], Py = xr[N + r], Pz = xr[2 * N + r];
    double sd, dd, sm, dm;
    source_kernel(rec + (size_t)s * RK_STRIDE, Px, Py, Pz, sd, dd);
    size_t o = (size_t)r * ld + s;
    if (mode == 2) {  // aero: G = s, H = d of the body panels only (Aerodynamic_Solver.cpp:49-54)
        o0[o] = sd;
        o1[o] = dd;
        return;
    }
    source_kernel(rec + ((size_t)N + s) * RK_STRIDE, Px, Py, Pz, sm, dm);
    if (mode == 0) {
        o0[o] = (-sd) + (-sm);
        o1[o] = dd + dm;
        o2[o] = (-sm) * rn[s];
    } else {
        o0[o] = sd; o1[o] = sm; o2[o] = dd; o3[o] = dm;
    }
}

// Trailing wake of the steady solve: wake strip w (Rankine record rec_w + w RK_STRIDE) is a
// constant-doublet panel of strength X[te_up[w]] - X[te_lo[w]] (the Kutta condition), so its
// dipole influence at collocation point r joins H[r][te_up[w]] with + and H[r][te_lo[w]] with -.
__global__ void k_wake_fold(int N, int ld, int W, const double* __restrict__ rec_w, const double* __restrict__ xr,
                            const int* __restrict__ te_up, const int* __restrict__ te_lo, double* __restrict__ H) {
    const int w = blockIdx.y;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N || w >= W) return;
    double sw, dw;
    source_kernel(rec_w + (size_t)w * RK_STRIDE, xr[r], xr[N + r], xr[2 * N + r], sw, dw);
    atomicAdd(H + (size_t)r * ld + te_up[w], dw);
    atomicAdd(H + (size_t)r * ld + te_lo[w], -dw);
}

void launch_wake_fold(cudaStream_t st, int N, int ld, int W, const double* rec_w, const double* xr, const int* te_up,
                      const int* te_lo, double* H) {
    if (W <= 0) return;
    BEM_LAUNCH(k_wake_fold<<<dim3((N + 127) / 128, W), 128, 0, st>>>(N, ld, W, rec_w, xr, te_up, te_lo, H));
}

// ---------------------------------------------------------------------------
// K2: wave term.  One warp per receiver row, lanes over source panels; the
// eight warps of a CTA sweep the same source tiles so those come from L1.
template <typename T> struct WaveMath;
template <> struct WaveMath<double> {
    typedef cd C;
    static __device__ __forceinline__ void gf(double h, double v, cd& G, cd& Gh) { gf64(c_poly64, h, v, G, Gh); }
};
template <> struct WaveMath<float> {
    typedef cf C;
    static __device__ __forceinline__ void gf(float h, float v, cf& G, cf& Gh) { gf32(h, v, G, Gh); }
};

// Influence (ws, wd) of mirrored wave panel s at receiver point (xr, yr, zr).
template <typename T>
__device__ __forceinline__ void wave_pair(const WaveArgs& a, int s, double X, double Y, double Z, T& wsr, T& wsi,
                                          T& wdr, T& wdi) {
    const int N = a.N;
    const int nq = a.nq[s];
    const T K = (T)a.K;
    const T c1 = (T)(a.K * kFourPIinv);
    const T c2 = (T)(a.K * a.K * kFourPIinv);
    wsr = wsi = wdr = wdi = (T)0;
    if (a.K == 0.0) return;  // FreeSurface_Wave_Kernel returns zero for K == 0 (Panel.cpp:607-614)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (q < nq) {
            const double* g = a.gq + (size_t)q * N + s;  // field stride 4N
            double qx = g[0], qy = g[(size_t)4 * N], qz = g[(size_t)8 * N];
            T w = (T)g[(size_t)12 * N];
            T nx = (T)g[(size_t)16 * N], ny = (T)g[(size_t)20 * N], nz = (T)g[(size_t)24 * N];
            T XX = (T)(X - qx) * K, YY = (T)(Y - qy) * K, VV = (T)(Z - qz) * K;
            T hh = sqrt(XX * XX + YY * YY);
            typename WaveMath<T>::C G, Gh;
            WaveMath<T>::gf(hh, VV, G, Gh);
            T gxr = 0, gxi = 0, gyr = 0, gyi = 0;
            if (hh > (T)1.0e-6) {
                gxr = Gh.re * XX / hh; gxi = Gh.im * XX / hh;
                gyr = Gh.re * YY / hh; gyi = Gh.im * YY / hh;
            }
            // FreeSurface_Wave_Kernel scaling: G *= K/(4 pi), dG *= K^2/(4 pi)
            T Gr = G.re * c1, Gi = G.im * c1;
            T dxr = gxr * c2, dxi = gxi * c2, dyr = gyr * c2, dyi = gyi * c2;
            T dzr = G.re * c2, dzi = G.im * c2;
            wsr += w * Gr;
            wsi += w * Gi;
            wdr += w * (dxr * nx + dyr * ny + dzr * nz);
            wdi += w * (dxi * nx + dyi * ny + dzi * nz);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_wave(WaveArgs a) {
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (r >= a.N) return;
    const int N = a.N, R = a.R;
    const double X = a.xr[r], Y = a.xr[N + r], Z = a.xr[2 * N + r];
    T acc_re[MAX_RHS], acc_im[MAX_RHS];
#pragma unroll
    for (int j = 0; j < MAX_RHS; ++j) { acc_re[j] = 0; acc_im[j] = 0; }
    const size_t row = (size_t)r * a.ld;
    for (int s = lane; s < N; s += 32) {
        T wsr, wsi, wdr, wdi;
        wave_pair<T>(a, s, X, Y, Z, wsr, wsi, wdr, wdi);
        if (a.mode == 1) {
            size_t o = 2 * ((size_t)r * N + s);
            a.ws_out[o] = (double)wsr; a.ws_out[o + 1] = (double)wsi;
            a.wd_out[o] = (double)wdr; a.wd_out[o + 1] = (double)wdi;
            continue;
        }
        // D = (d + dr) + (wd + (-sr) 2 n_z K): Solve (:428) with DWave (:200)
        double dre = a.RD[row + s] + ((double)wdr + a.RSR[row + s] * a.K);
        double dim = (double)wdi;
        a.D64r[row + s] = dre;
        a.D64i[row + s] = dim;
        if (a.D32r) { a.D32r[row + s] = (float)dre; a.D32i[row + s] = (float)dim; }
        // S = Ssrc + Srefl - ws; the (-ws) part times the RHS block B (N x R).
        const double* b = a.Bm + (size_t)s * 2 * R;
#pragma unroll
        for (int j = 0; j < MAX_RHS; ++j) {
            if (j < R) {
                T br = (T)b[2 * j], bi = (T)b[2 * j + 1];
                acc_re[j] -= wsr * br - wsi * bi;
                acc_im[j] -= wsr * bi + wsi * br;
            }
        }
    }
    if (a.mode == 1) return;
#pragma unroll
    for (int j = 0; j < MAX_RHS; ++j) {
        if (j < R) {
            T vr = acc_re[j], vi = acc_im[j];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                vr += __shfl_xor_sync(0xffffffffu, vr, off);
                vi += __shfl_xor_sync(0xffffffffu, vi, off);
            }
            if (lane == 0) {
                a.Y[2 * ((size_t)r * R + j)] += (double)vr;
                a.Y[2 * ((size_t)r * R + j) + 1] += (double)vi;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// One receiver of the mixed assembly: the collocation point as float pairs.
struct Recv32 {
    float xh, yh, zh, xl, yl, zl;
};
__device__ __forceinline__ Recv32 load_recv32(const WaveArgs& a, int r) {
    const int N = a.N;
    return Recv32{a.xr32[r], a.xr32[N + r], a.xr32[2 * N + r], a.xr32[3 * N + r], a.xr32[4 * N + r],
                  a.xr32[5 * N + r]};
}

// Geometry of one (receiver, Gauss point) pair of the mixed assembly: coordinate
// differences as float pairs, K (x, y) and the nondimensional h = (hh, hl), v = (VV, vl)
// as float pairs.
struct GaussGeo {
    float sx, lx, sy, ly, sz, ez;  // dimensional differences receiver - Gauss point (hi, lo)
    float XX, YY;                  // K dx, K dy
    float hh, hl, VV, vl;
    float inv_h;                   // 1 / hh: the x > 3 Bessel/Struve forms and dG/dx, dG/dy
};

__device__ __forceinline__ GaussGeo gauss_geo32(const Recv32& R, float gx, float gy, float gz, float gxl, float gyl,
                                                float gzl, float Kh, float Kl) {
    GaussGeo o;
    const float K = Kh;
    // coordinate differences as float pairs (two-differences of the hi parts + lo parts)
    o.sx = R.xh - gx;
    o.sy = R.yh - gy;
    const float bx = o.sx - R.xh, by = o.sy - R.yh;
    o.lx = ((R.xh - (o.sx - bx)) - (gx + bx)) + (R.xl - gxl);
    o.ly = ((R.yh - (o.sy - by)) - (gy + by)) + (R.yl - gyl);
    // v = K (z_r - z_q) as a float pair (VV, vl), like h = (hh, hl)
    o.sz = R.zh - gz;
    const float bz = o.sz - R.zh;
    o.ez = ((R.zh - (o.sz - bz)) - (gz + bz)) + (R.zl - gzl);
    const float vh = o.sz * Kh;
    const float vlo = fmaf(o.sz, Kh, -vh) + fmaf(o.sz, Kl, o.ez * Kh);
    o.VV = vh + vlo;
    o.vl = vlo - (o.VV - vh);
    o.XX = (o.sx + o.lx) * K;
    o.YY = (o.sy + o.ly) * K;
    df_hdist(o.sx, o.lx, o.sy, o.ly, Kh, Kl, o.hh, o.hl);
    o.inv_h = __fdividef(1.0f, o.hh);
    return o;
}

// HavelockGF at the pair by the FP32 closed form: Re/Im of G and of dG/dh.
__device__ __forceinline__ void gauss_G32(const GaussGeo& o, float& Gr, float& Gi, float& Ghr, float& Ghi) {
    const float twopi = 6.28318530717959f;
    // e^v by the fast exponential (ex2 of v log2 e): its error, about |v| 1e-7 of e^v, is at
    // most ~4e-8 in absolute terms (at v = -1), the size of the FP32 rounding of the terms
    const float ev = __expf(o.VV);
    float j0v, j1v, y0v = 0.0f, y1v = 0.0f;
    const float t3 = 3.0f * o.inv_h;
    if (o.hh > 3.0f) bessel_large(o.hh, o.hl, t3, j0v, j1v, y0v, y1v);
    else bessel_j01_small(o.hh, j0v, j1v);
    float Gv;
    gf32_re(o.hh, o.VV, ev, y0v, y1v, t3, Gr, Ghr, Gv);
    // G at the unrounded (h, v): the first-order terms of the float pairs' low parts.
    // The radiation damping is a small difference of terms that each carry this
    // rounding, so without it B loses ~1e-6 at the highest frequencies.
    Gr = fmaf(Ghr, o.hl, fmaf(Gv, o.vl, Gr));
    Ghi = twopi * ev * j1v;
    Gi = -twopi * ev * j0v;
}

// The pair's terms of ws and wd from G and dG/dh at one Gauss point (normal n, weights
// wc1 = w K/4pi, wc2 = w K^2/4pi): FreeSurface_Wave_Kernel and
// CInf_SingleDoubleLayerQuad (Panel.cpp:601-636, 776-794).
__device__ __forceinline__ void gauss_accum32(const GaussGeo& o, float Gr, float Gi, float Ghr, float Ghi, float nx,
                                              float ny, float nz, float wc1, float wc2, float& wsr, float& wsi,
                                              float& wdr, float& wdi) {
    const float proj = fmaf(o.XX, nx, o.YY * ny);
    float dgr = 0.f, dgi = 0.f;
    if (o.hh > 1.0e-6f) {
        dgr = Ghr * proj * o.inv_h;
        dgi = Ghi * proj * o.inv_h;
    }
    wsr = fmaf(wc1, Gr, wsr);
    wsi = fmaf(wc1, Gi, wsi);
    wdr = fmaf(wc2, fmaf(Gr, nz, dgr), wdr);
    wdi = fmaf(wc2, fmaf(Gi, nz, dgi), wdi);
}

// One Gauss point of a mirrored wave panel (coordinates as float pairs g*, g*l; normal n;
// weights wc1 = w K/4pi, wc2 = w K^2/4pi) at receiver R: adds its FP32 terms of ws and wd.
__device__ __forceinline__ void gauss_eval32(const Recv32& R, float gx, float gy, float gz, float gxl, float gyl,
                                             float gzl, float nx, float ny, float nz, float wc1, float wc2, float Kh,
                                             float Kl, float& wsr, float& wsi, float& wdr, float& wdi) {
    const GaussGeo o = gauss_geo32(R, gx, gy, gz, gxl, gyl, gzl, Kh, Kl);
    float Gr, Gi, Ghr, Ghi;
    gauss_G32(o, Gr, Gi, Ghr, Ghi);
    gauss_accum32(o, Gr, Gi, Ghr, Ghi, nx, ny, nz, wc1, wc2, wsr, wsi, wdr, wdi);
}

// Re D = RD + K RSR + wd_re in double-float arithmetic (RD, RSR stored as float pairs):
// FMA-exact products and Knuth two-sums keep ~48 bits, as the refinement residual needs.
__device__ __forceinline__ void redf_store(const WaveArgs& a, size_t o, float rdh, float rdl, float rsh, float rsl,
                                           float wdr, float wdi) {
    const float Kh = a.kh, Kl = a.kl;
    const float ph = Kh * rsh;
    const float pe = fmaf(Kh, rsl, fmaf(Kl, rsh, fmaf(Kh, rsh, -ph)));
    const float sh = rdh + ph;
    float bb = sh - rdh;
    const float se = ((rdh - (sh - bb)) + (ph - bb)) + (rdl + pe);
    const float th = sh + wdr;
    bb = th - sh;
    const float te = ((sh - (th - bb)) + (wdr - bb)) + se;
    const float hi = th + te;
    a.Dhi[o] = hi;
    a.Dlo[o] = te - (hi - th);
    a.D32r[o] = hi;
    a.D32i[o] = wdi;
}

// Admission of a persistent assembly CTA (see WaveArgs): returns false if it should leave.
__device__ __forceinline__ bool wave_admit(const WaveArgs& a, uint32_t& smid, int* s_admit) {
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    if (smid >= (uint32_t)WAVE_SM_SLOTS) smid = WAVE_SM_SLOTS - 1;  // only the admission policy shares a slot
    if (threadIdx.x == 0) {
        // The first WAVE_ALWAYS CTAs to start always work, wherever they land, so that a
        // launch whose CTAs all find room only on reserved SMs (the GPU full of other work)
        // still assembles the frequency; later CTAs stay only on unreserved SMs with room.
        const int arrival = atomicAdd(a.sm_ctr + WAVE_SM_SLOTS, 1);
        const int here = atomicAdd(a.sm_ctr + smid, 1);
        int ok = 1;
        if (arrival >= WAVE_ALWAYS && ((int)smid < a.reserve || here >= a.per_sm)) {
            atomicSub(a.sm_ctr + smid, 1);
            ok = 0;
        }
        *s_admit = ok;
    }
    __syncthreads();
    return *s_admit != 0;
}

// K2, mixed precision.  Every term of G and dG in FP32; the FP64 operator
// gets the real part (Rankine FP64 + wave FP32) and the LU copy gets both parts
// in FP32.  The imaginary part of the operator and of S*B is not taken from
// here: it is applied exactly, in FP64, by the plane-wave kernels below
// (k_pw_*), because the radiation damping at low K is a small difference of
// O(K) imaginary terms and amplifies FP32 rounding in them up to ~200x.
template <int RM>
__global__ void __launch_bounds__(256, 3) k_wave_mixed(WaveArgs a) {
    const int lane = threadIdx.x & 31;
    __shared__ int s_admit;
    uint32_t smid;
    if (!wave_admit(a, smid, &s_admit)) return;
    // work item = one receiver row x one of a.split source ranges, so the last items
    // are short and the tail of the launch leaves few SMs idle
    const int split = a.split > 0 ? a.split : WAVE_SPLIT;
    const int chunk = ((a.N + split - 1) / split + 31) & ~31;
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(a.row_ctr, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= a.N * split) break;
        const int r = item / split, s_begin = (item % split) * chunk;
        const int s_end = min(a.N, s_begin + chunk);
        const int N = a.N, R = a.R;
        const Recv32 Rv = load_recv32(a, r);
        const float Kh = a.kh, Kl = a.kl;
        const float c1 = a.c1f, c2 = a.c2f;
        float acc_re[RM], acc_im[RM];
    #pragma unroll
        for (int j = 0; j < RM; ++j) { acc_re[j] = 0.f; acc_im[j] = 0.f; }
        const size_t row = (size_t)r * a.ld;
        const bool live = a.live != 0;
        for (int s = s_begin + lane; s < s_end; s += 32) {
            float wsr = 0.f, wsi = 0.f, wdr = 0.f, wdi = 0.f;
            // the pair's Rankine float pairs come from HBM: issued first, so that their latency
            // overlaps the Green-function arithmetic below
            float rdh = 0.f, rdl = 0.f, rsh = 0.f, rsl = 0.f;
            if (a.mode != 1) {
                rdh = __ldcs(a.RDhi + row + s); rdl = __ldcs(a.RDlo + row + s);
                rsh = __ldcs(a.RSRhi + row + s); rsl = __ldcs(a.RSRlo + row + s);
            }
            const int nq = live ? __ldg(a.nq + s) : 0;
    #pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (q < nq) {
                    // source data is read by every row: read-only path, three 16-byte loads
                    const float4* gv = a.gq32v + (size_t)q * 3 * N + s;
                    const float4 g0 = __ldg(gv), g1 = __ldg(gv + N), g2 = __ldg(gv + 2 * N);
                    gauss_eval32(Rv, g0.x, g0.y, g0.z, g1.w, g2.x, g2.y, g1.x, g1.y, g1.z, g0.w * c1, g0.w * c2, Kh,
                                 Kl, wsr, wsi, wdr, wdi);
                }
            }
            if (a.mode == 1) {
                size_t o = 2 * ((size_t)r * N + s);
                a.ws_out[o] = (double)wsr; a.ws_out[o + 1] = (double)wsi;
                a.wd_out[o] = (double)wdr; a.wd_out[o + 1] = (double)wdi;
                continue;
            }
            redf_store(a, row + s, rdh, rdl, rsh, rsl, wdr, wdi);
            // the real part of S = Ssrc + Srefl - ws applied to B: -ws_re * B
            const float* b = a.Bm32 + (size_t)s * 2 * R;
    #pragma unroll
            for (int j = 0; j < RM; ++j) {
                if (j < R) {
                    acc_re[j] = fmaf(-wsr, __ldg(b + 2 * j), acc_re[j]);
                    acc_im[j] = fmaf(-wsr, __ldg(b + 2 * j + 1), acc_im[j]);
                }
            }
        }
        if (a.mode == 1) continue;
    #pragma unroll
        for (int j = 0; j < RM; ++j) {
            if (j < R) {
                float vr = acc_re[j], vi = acc_im[j];
    #pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    vr += __shfl_xor_sync(0xffffffffu, vr, off);
                    vi += __shfl_xor_sync(0xffffffffu, vi, off);
                }
                if (lane == 0) {
                    atomicAdd(a.Y + 2 * ((size_t)r * R + j), (double)vr);
                    atomicAdd(a.Y + 2 * ((size_t)r * R + j) + 1, (double)vi);
                }
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) atomicSub(a.sm_ctr + smid, 1);
}


// ---------------------------------------------------------------------------
// K2, surrogate form.  Work item = a receiver row x SUR_SB blocks of 32 source panels; a
// warpgroup takes items from the counter and runs one 128-sample tile per block: thread
// t = 4 p + q is Gauss point q of panel s0 + p.  Far pairs inside the network's domain
// take G and dG/dh from the tensor-core network (mlp_tc.cuh), scaled back by the
// envelope the network was trained on:
//   G:      2 / (d + 0.05) + w,   dG/dh: 2 h / (d^2 (1 + d)) + w,   Im parts: w,
//   w = 2 pi e^v / sqrt(1 + h), d = sqrt(h^2 + v^2);
// near pairs (a Gauss point of the mirrored panel nearer than sqrt(near2) panel
// diameters), out-of-domain pairs and the judged sample take the FP32 closed form
// (gauss_G32).  A tile whose pairs all take the closed form skips the network.  The
// imaginary parts of the operator and of S B still come from the plane waves (exact);
// the network's imaginary parts only reach the FP32 copy that is factorised.
constexpr int SUR_SB = 8;

__device__ __forceinline__ bool wg_any(int g, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred pi, po;\n\t"
        "setp.ne.u32 pi, %1, 0;\n\t"
        "barrier.cta.red.or.pred po, %2, 128, pi;\n\t"
        "selp.u32 %0, 1, 0, po;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(1 + g)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ uint32_t pair_hash(uint32_t r, uint32_t s, uint32_t seed) {
    uint32_t h = (r * 2654435761u) ^ (s * 2246822519u) ^ seed;
    h ^= h >> 15;
    h *= 0x2c1b3c6du;
    h ^= h >> 12;
    h *= 0x297a2d39u;
    h ^= h >> 15;
    return h;
}

__global__ void __launch_bounds__(mlptc::THREADS, 1) k_wave_surrogate(WaveArgs a, SurArgs sa) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_admit;
    __shared__ int s_item[2];
    uint32_t smid;
    if (!wave_admit(a, smid, &s_admit)) return;
    const mlptc::Smem m = mlptc::smem_layout(smem_raw);
    const uint32_t tmem = mlptc::cta_setup(m, sa.img, sa.fw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = warp >> 2, t = threadIdx.x & 127;
    const uint32_t acc = tmem + (uint32_t)g * 128;
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    const uint32_t tile = m.s_tile0 + (uint32_t)g * mlptc::TILE_BYTES;
    uint32_t phase = 0;
    const int p = t >> 2, q = t & 3;
    const int N = a.N;
    const int nblk = (N + 31) / 32, ipr = (nblk + SUR_SB - 1) / SUR_SB;
    const long long nitems = (long long)N * ipr;
    const size_t fs = (size_t)4 * N;
    const float Kh = a.kh, Kl = a.kl, c1 = a.c1f, c2 = a.c2f;
    const float twopi = 6.28318530717959f;
    unsigned long long n_mlp = 0, n_cf = 0, n_judge = 0;
    float jerr = 0.f;
    for (;;) {
        if (t == 0) s_item[g] = atomicAdd(a.row_ctr, 1);
        mlptc::wg_sync(g);
        const int item = s_item[g];
        mlptc::wg_sync(g);  // read by every thread before thread 0 draws the next item
        if (item >= nitems) break;
        const int r = item / ipr, b0 = (item % ipr) * SUR_SB;
        const Recv32 Rv = load_recv32(a, r);
        const size_t row = (size_t)r * a.ld;
        for (int b = b0; b < min(b0 + SUR_SB, nblk); ++b) {
            const int s = b * 32 + p;
            const bool valid = s < N;
            const int nq = (valid && a.live) ? __ldg(a.nq + s) : 0;
            const bool active = q < nq;
            GaussGeo o{};
            float nx = 0.f, ny = 0.f, nz = 0.f, w = 0.f;
            bool okq = true;
            if (active) {
                const float* gp = a.gq32 + (size_t)q * N + s;
                w = __ldg(gp + 3 * fs);
                nx = __ldg(gp + 4 * fs);
                ny = __ldg(gp + 5 * fs);
                nz = __ldg(gp + 6 * fs);
                o = gauss_geo32(Rv, __ldg(gp), __ldg(gp + fs), __ldg(gp + 2 * fs), __ldg(gp + 7 * fs),
                                __ldg(gp + 8 * fs), __ldg(gp + 9 * fs), Kh, Kl);
                const float dx = o.sx + o.lx, dy = o.sy + o.ly, dz = o.sz + o.ez;
                const float dia = __ldg(sa.pdiam + s);
                okq = fmaf(dx, dx, fmaf(dy, dy, dz * dz)) >= sa.near2 * dia * dia && o.hh >= sa.kr_min &&
                      o.hh <= sa.kr_max && o.VV >= sa.kz_min;
            }
            // a pair is far when all its Gauss points are (lanes 4 p .. 4 p + 3 of one warp)
            const unsigned bal = __ballot_sync(0xffffffffu, okq);
            const bool far = valid && a.live && ((bal >> (lane & ~3)) & 0xFu) == 0xFu;
            const bool judged =
                far && sa.judge_mod != 0u && pair_hash((uint32_t)r, (uint32_t)s, sa.judge_seed) % sa.judge_mod == 0u;
            const bool use_net = active && far && !judged;
            float out[mlptc::NOUT];
#pragma unroll
            for (int j = 0; j < mlptc::NOUT; ++j) out[j] = 0.f;
            if (wg_any(g, far)) {
                const bool in = far && active;  // a triangle's fourth lane has no Gauss point
                const float x0 = in ? (log10f(o.hh) - sa.in_shift[0]) / sa.in_scale[0] : 0.f;
                const float x1 = in ? (o.VV - sa.in_shift[1]) / sa.in_scale[1] : 0.f;
                mlptc::layer0(m, tile, t, x0, x1);
                mlptc::layers(m, tile, acc, lane_base, g, t, phase, sa.gflags, out);
            }
            float wsr = 0.f, wsi = 0.f, wdr = 0.f, wdi = 0.f;
            if (active) {
                float nGr = 0.f, nGi = 0.f, nGhr = 0.f, nGhi = 0.f, eg = 1.f, er = 1.f;
                if (far) {
                    const float d = sqrtf(fmaf(o.hh, o.hh, o.VV * o.VV));
                    const float wv = twopi * expf(o.VV) * rsqrtf(1.0f + o.hh);
                    eg = 2.0f / (d + 0.05f) + wv;
                    er = 2.0f * o.hh / fmaf(d * d, 1.0f + d, 1e-12f) + wv;
                    nGr = fmaf(out[0], sa.out_scale[0], sa.out_shift[0]) * eg;
                    nGi = fmaf(out[1], sa.out_scale[1], sa.out_shift[1]) * wv;
                    nGhr = fmaf(out[2], sa.out_scale[2], sa.out_shift[2]) * er;
                    nGhi = fmaf(out[3], sa.out_scale[3], sa.out_shift[3]) * wv;
                }
                float Gr, Gi, Ghr, Ghi;
                if (use_net) {
                    Gr = nGr; Gi = nGi; Ghr = nGhr; Ghi = nGhi;
                    ++n_mlp;
                } else {
                    gauss_G32(o, Gr, Gi, Ghr, Ghi);
                    ++n_cf;
                    if (judged) jerr = fmaxf(jerr, fmaxf(fabsf(nGr - Gr) / eg, fabsf(nGhr - Ghr) / er));
                }
                gauss_accum32(o, Gr, Gi, Ghr, Ghi, nx, ny, nz, w * c1, w * c2, wsr, wsi, wdr, wdi);
            }
            // sums over the pair's Gauss points (its four lanes)
#pragma unroll
            for (int off = 1; off <= 2; off <<= 1) {
                wsr += __shfl_xor_sync(0xffffffffu, wsr, off);
                wsi += __shfl_xor_sync(0xffffffffu, wsi, off);
                wdr += __shfl_xor_sync(0xffffffffu, wdr, off);
                wdi += __shfl_xor_sync(0xffffffffu, wdi, off);
            }
            if (q == 0 && valid) {
                if (judged) ++n_judge;
                if (a.mode == 1) {
                    const size_t o2 = 2 * ((size_t)r * N + s);
                    a.ws_out[o2] = (double)wsr; a.ws_out[o2 + 1] = (double)wsi;
                    a.wd_out[o2] = (double)wdr; a.wd_out[o2 + 1] = (double)wdi;
                } else {
                    redf_store(a, row + s, __ldcs(a.RDhi + row + s), __ldcs(a.RDlo + row + s),
                               __ldcs(a.RSRhi + row + s), __ldcs(a.RSRlo + row + s), wdr, wdi);
                    sa.ws32[row + s] = wsr;
                }
            }
        }
    }
    // counts and the largest judged error (non-negative floats order like their bits)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        n_mlp += __shfl_xor_sync(0xffffffffu, n_mlp, off);
        n_cf += __shfl_xor_sync(0xffffffffu, n_cf, off);
        n_judge += __shfl_xor_sync(0xffffffffu, n_judge, off);
        jerr = fmaxf(jerr, __shfl_xor_sync(0xffffffffu, jerr, off));
    }
    if (lane == 0) {
        atomicAdd(sa.stats, n_mlp);
        atomicAdd(sa.stats + 1, n_cf);
        atomicAdd(sa.stats + 2, n_judge);
        atomicMax(sa.stats + 3, (unsigned long long)__float_as_uint(jerr));
    }
    mlptc::cta_teardown(tmem);
    __syncthreads();
    if (threadIdx.x == 0) atomicSub(a.sm_ctr + smid, 1);
}

int launch_wave_surrogate(cudaStream_t st, const WaveArgs& a, const SurArgs& sa) {
    WaveArgs b = a;
    set_wave_f32_constants(b);
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_wave_surrogate, cudaFuncAttributeMaxDynamicSharedMemorySize, mlptc::SMEM_BYTES) !=
            cudaSuccess)
            return 1;
        attr = true;
    }
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    b.per_sm = 1;  // one CTA fits per SM (shared memory)
    cudaMemsetAsync(a.row_ctr, 0, sizeof(int) * (2 + WAVE_SM_SLOTS), st);
    BEM_LAUNCH(k_wave_surrogate<<<nsm, mlptc::THREADS, mlptc::SMEM_BYTES, st>>>(b, sa));
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 1;
}

// ---------------------------------------------------------------------------
// Exact FP64 imaginary parts by plane waves.  With Bessel's integral
// J0(h) = (1/2pi) int exp(i h cos(t - phi)) dt, the imaginary parts of the wave
// influence separate over M equispaced angles t_m (trapezoid rule; exact to
// rounding once M > 1.3 K D + 30, D the largest horizontal distance):
//   e^v J0(h)              = (1/M) sum_m E_r(m) F_q(m)
//   e^v J1(h)/h (X nx + Y ny) = -(1/M) sum_m i (cos t nx + sin t ny) E_r F_q
// with E_r(m) = exp(K z_r + i K (x_r cos t_m + y_r sin t_m)) at the receiver and
// F_q(m) = exp(-K z_q - i K (x_q cos t_m + y_q sin t_m)) at the Gauss point, so
//   Im ws(r,s) = -(2 pi c1 / M) Re sum_m E_r(m) Vs_s(m),  Vs_s = sum_q w_q F_q
//   Im wd(r,s) = -(2 pi c2 / M) Re sum_m E_r(m) Wd_s(m),  Wd_s = sum_q w_q (nz + i(cos t nx + sin t ny)) F_q
// (c1 = K/4pi, c2 = K^2/4pi; Panel.cpp:632-634).  The operator products then
// cost O(N M R) instead of O(N^2).
__device__ __forceinline__ float4 df_pack(double re, double im) {
    const float rh = (float)re, ih = (float)im;
    return make_float4(rh, (float)(re - (double)rh), ih, (float)(im - (double)ih));
}

// Factors are stored as float pairs per component: float4 = (re hi, re lo, im hi, im lo).
__global__ void k_pw_build(int N, int M, double K, const double* __restrict__ xr, const double* __restrict__ gq,
                           const int* __restrict__ nq, float4* __restrict__ E, float4* __restrict__ V,
                           float4* __restrict__ W) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.y;
    if (i >= N) return;
    double st, ct;
    sincospi(2.0 * m / M, &st, &ct);
    // receiver factor
    {
        double ph = K * (xr[i] * ct + xr[N + i] * st);
        double amp = exp(K * xr[2 * N + i]);
        double sp, cp;
        sincos(ph, &sp, &cp);
        E[(size_t)m * N + i] = df_pack(amp * cp, amp * sp);
    }
    // source panel i: sums over its Gauss points
    double vr = 0, vi = 0, wr = 0, wi = 0;
    const int n = nq[i];
    for (int q = 0; q < 4; ++q) {
        if (q < n) {
            const double* g = gq + (size_t)q * N + i;
            const size_t fs = (size_t)4 * N;
            double x = g[0], y = g[fs], z = g[2 * fs], w = g[3 * fs];
            double nx = g[4 * fs], ny = g[5 * fs], nz = g[6 * fs];
            double amp = w * exp(-K * z);
            double sp, cp;
            sincos(-K * (x * ct + y * st), &sp, &cp);
            double fr = amp * cp, fi = amp * sp;
            vr += fr; vi += fi;
            double tr = nz, ti = ct * nx + st * ny;  // nz + i (cos t nx + sin t ny)
            wr += tr * fr - ti * fi;
            wi += tr * fi + ti * fr;
        }
    }
    V[(size_t)m * N + i] = df_pack(vr, vi);
    W[(size_t)m * N + i] = df_pack(wr, wi);
}

// Double-float helpers: a * b ~ p + e (e from an FMA), (s, c) += p + e with Knuth's two-sum.
__device__ __forceinline__ void pw_prod(float ah, float al, float bh, float bl, float& p, float& e) {
    p = ah * bh;
    e = fmaf(ah, bl, fmaf(al, bh, fmaf(ah, bh, -p)));
}
__device__ __forceinline__ void pw_acc(float& s, float& c, float p, float e) {
    const float t = s + p, z = t - s;
    c += ((s - (t - z)) + (p - z)) + e;
    s = t;
}

// T[m][j] += {T1.re, T1.im, T2.re, T2.im} with T1 = sum_s P_s(m) Z[s][j], T2 = sum_s conj(P_s(m)) Z[s][j]
// (Z: N x R complex as float pairs).  CTA (m, chunk of PW_CHUNK panels); double-float
// sums per thread, FP64 across the CTA and FP64 atomics across chunks (T zeroed first).
constexpr int PW_CHUNK = 1024, PW_THREADS = 128;

template <int RR>
__global__ void __launch_bounds__(PW_THREADS) k_pw_project(int N, const float4* __restrict__ P,
                                                           const float4* __restrict__ Z, double* __restrict__ T) {
    extern __shared__ double pw_red[];  // [4 RR][PW_THREADS + 1]
    const int m = blockIdx.x, s0 = blockIdx.y * PW_CHUNK, t = threadIdx.x;
    float as[4 * RR], ac[4 * RR];
#pragma unroll
    for (int k = 0; k < 4 * RR; ++k) { as[k] = 0.f; ac[k] = 0.f; }
    const float4* pm = P + (size_t)m * N;
    const int s1 = min(N, s0 + PW_CHUNK);
    for (int s = s0 + t; s < s1; s += PW_THREADS) {
        const float4 p = pm[s];
        const float4* z = Z + (size_t)s * RR;
#pragma unroll
        for (int j = 0; j < RR; ++j) {
            const float4 zz = z[j];
            float Ap, Ae, Bp, Be, Cp, Ce, Dp, De;
            pw_prod(p.x, p.y, zz.x, zz.y, Ap, Ae);  // pr zr
            pw_prod(p.z, p.w, zz.z, zz.w, Bp, Be);  // pi zi
            pw_prod(p.x, p.y, zz.z, zz.w, Cp, Ce);  // pr zi
            pw_prod(p.z, p.w, zz.x, zz.y, Dp, De);  // pi zr
            pw_acc(as[4 * j], ac[4 * j], Ap, Ae);          // T1.re = pr zr - pi zi
            pw_acc(as[4 * j], ac[4 * j], -Bp, -Be);
            pw_acc(as[4 * j + 1], ac[4 * j + 1], Cp, Ce);  // T1.im = pr zi + pi zr
            pw_acc(as[4 * j + 1], ac[4 * j + 1], Dp, De);
            pw_acc(as[4 * j + 2], ac[4 * j + 2], Ap, Ae);  // T2.re = pr zr + pi zi
            pw_acc(as[4 * j + 2], ac[4 * j + 2], Bp, Be);
            pw_acc(as[4 * j + 3], ac[4 * j + 3], Cp, Ce);  // T2.im = pr zi - pi zr
            pw_acc(as[4 * j + 3], ac[4 * j + 3], -Dp, -De);
        }
    }
#pragma unroll
    for (int k = 0; k < 4 * RR; ++k) pw_red[k * (PW_THREADS + 1) + t] = (double)as[k] + (double)ac[k];
    __syncthreads();
    for (int k = t; k < 4 * RR; k += PW_THREADS) {
        double v = 0.0;
        for (int i = 0; i < PW_THREADS; ++i) v += pw_red[k * (PW_THREADS + 1) + i];
        atomicAdd(T + (size_t)m * RR * 4 + k, v);
    }
}

// out[r][j] += i * scale * sum_m (E_r(m) T1[m][j] + conj(E_r(m)) T2[m][j]), one thread per (r, j).
// With T1 = a + ib, T2 = c + id and E = er + i ei the sum is
//   er (a + c) + ei (d - b)  +  i (er (b + d) + ei (a - c)),
// formed per (m, j) once in shared memory as float pairs.
__global__ void __launch_bounds__(256) k_pw_apply(int N, int M, int R, double scale, const float4* __restrict__ E,
                                                  const double* __restrict__ T, double* __restrict__ out) {
    extern __shared__ float4 U[];  // [M * R][2]: (s1 hi, s1 lo, s2 hi, s2 lo), (s3 .., s4 ..)
    for (int k = threadIdx.x; k < M * R; k += blockDim.x) {
        const double* tt = T + (size_t)k * 4;
        const double a = tt[0], b = tt[1], c = tt[2], d = tt[3];
        U[2 * k] = df_pack(a + c, d - b);
        U[2 * k + 1] = df_pack(b + d, a - c);
    }
    __syncthreads();
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N * R) return;
    const int r = idx / R, j = idx % R;
    float rs = 0.f, rc = 0.f, is = 0.f, ic = 0.f;
    for (int m = 0; m < M; ++m) {
        const float4 e = E[(size_t)m * N + r];
        const float4 u0 = U[2 * (m * R + j)], u1 = U[2 * (m * R + j) + 1];
        float p, q;
        pw_prod(e.x, e.y, u0.x, u0.y, p, q); pw_acc(rs, rc, p, q);  // er s1
        pw_prod(e.z, e.w, u0.z, u0.w, p, q); pw_acc(rs, rc, p, q);  // ei s2
        pw_prod(e.x, e.y, u1.x, u1.y, p, q); pw_acc(is, ic, p, q);  // er s3
        pw_prod(e.z, e.w, u1.z, u1.w, p, q); pw_acc(is, ic, p, q);  // ei s4
    }
    const double ar = (double)rs + (double)rc, ai = (double)is + (double)ic;
    // i * scale * (ar + i ai) = -scale ai + i scale ar
    out[2 * (size_t)idx] += -scale * ai;
    out[2 * (size_t)idx + 1] += scale * ar;
}

// Padding rows/columns of the working matrices: identity (so the padded LU
// factors the block diagonal [D, 0; 0, I]).
__global__ void k_pad_identity(int N, int ld, double* D64r, double* D64i, float* D32r, float* D32i) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int total = ld - N;
    if (total <= 0) return;
    // rows N..ld-1 (full) and columns N..ld-1 of rows 0..N-1
    for (size_t idx = i; idx < (size_t)ld * ld; idx += (size_t)gridDim.x * blockDim.x) {
        int r = (int)(idx / ld), c = (int)(idx % ld);
        if (r < N && c < N) continue;
        double v = (r == c) ? 1.0 : 0.0;
        if (D64r) { D64r[idx] = v; D64i[idx] = 0.0; }
        if (D32r) { D32r[idx] = (float)v; D32i[idx] = 0.0f; }
    }
}

// ---------------------------------------------------------------------------
// Incident wave (infinite depth, Calc_Phi_Incident :544-561) at the panel
// centroids and the diffraction right-hand sides -dPhi_I/dn .* area (:445).
__global__ void k_incident(int N, int NB, int R, const double* __restrict__ betas, double K, double Omega,
                           const double* __restrict__ cen, const double* __restrict__ nrm,
                           const double* __restrict__ area, double* __restrict__ phiI, double* __restrict__ dphiI,
                           double* __restrict__ Bm) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= N) return;
    const double g = 9.81;
    double x = cen[p], y = cen[N + p], z = cen[2 * N + p];
    double nx = nrm[p], ny = nrm[N + p], nz = nrm[2 * N + p];
    for (int b = 0; b < NB; ++b) {
        double pr = 0, pi = 0, dr = 0, di = 0;
        if (Omega != 0.0) {
            double CB = cos(betas[b]), SB = sin(betas[b]);
            // Phi_I = (i g / Omega) exp(i K (x cos b + y sin b)); Phi_i = e^{K z} Phi_I
            double arg = K * (x * CB + y * SB);
            double sa, ca;
            sincos(arg, &sa, &ca);
            double a = g / Omega;          // Im*Gravity/Omega = (0, g/Omega)
            double Pr = -a * sa, Pi = a * ca;  // (0 + i a)(ca + i sa)
            double Zf = exp(K * z);
            pr = Zf * Pr; pi = Zf * Pi;
            // dPhi/dx = i K CB Phi, dPhi/dy = i K SB Phi, dPhi/dz = K Phi
            double kx = K * CB, ky = K * SB;
            double dxr = -kx * pi, dxi = kx * pr;
            double dyr = -ky * pi, dyi = ky * pr;
            double dzr = K * pr, dzi = K * pi;
            dr = nx * dxr + ny * dyr + nz * dzr;
            di = nx * dxi + ny * dyi + nz * dzi;
        }
        size_t o = 2 * ((size_t)p * NB + b);
        phiI[o] = pr; phiI[o + 1] = pi;
        dphiI[o] = dr; dphiI[o + 1] = di;
        size_t ob = 2 * ((size_t)p * R + 6 + b);
        Bm[ob] = -(dr * area[p]);
        Bm[ob + 1] = -(di * area[p]);
    }
}

// ---------------------------------------------------------------------------
// Hull integrations (Hydrodynamic_Solver.cpp:462-476).  X = solution (N x R,
// interleaved complex; columns 0..5 = Phi_J).  Outputs per CTA (POST_PANELS panels, so
// each thread's FP64 sum is a short dependent chain) partial sums of
//   AM[i][j]  = sum_p Nk[p][i] A_p X[p][j]          (36 complex)
//   F1[i][b]  = sum_p Nk[p][i] A_p PhiI[p][b]       (6 NB complex)
//   F2[i][b]  = sum_p X[p][i] dPhiI[p][b] A_p       (6 NB complex)
constexpr int POST_PANELS = 32;

__global__ void __launch_bounds__(256) k_post_partial(int N, int NB, int R, const double* __restrict__ X,
                                                      const double* __restrict__ Nk, const double* __restrict__ area,
                                                      const double* __restrict__ phiI,
                                                      const double* __restrict__ dphiI, double* __restrict__ part) {
    const int nout = 36 + 12 * NB;
    const int p0 = blockIdx.x * POST_PANELS;
    const int pend = min(N, p0 + POST_PANELS);
    for (int t = threadIdx.x; t < nout; t += blockDim.x) {
        double sr = 0, si = 0;
        if (t < 36) {
            int i = t / 6, j = t % 6;
            for (int p = p0; p < pend; ++p) {
                double w = Nk[(size_t)p * 6 + i] * area[p];
                sr += w * X[2 * ((size_t)p * R + j)];
                si += w * X[2 * ((size_t)p * R + j) + 1];
            }
        } else if (t < 36 + 6 * NB) {
            int u = t - 36, i = u / NB, b = u % NB;
            for (int p = p0; p < pend; ++p) {
                double w = Nk[(size_t)p * 6 + i] * area[p];
                sr += w * phiI[2 * ((size_t)p * NB + b)];
                si += w * phiI[2 * ((size_t)p * NB + b) + 1];
            }
        } else {
            int u = t - 36 - 6 * NB, i = u / NB, b = u % NB;
            for (int p = p0; p < pend; ++p) {
                double xr = X[2 * ((size_t)p * R + i)], xi = X[2 * ((size_t)p * R + i) + 1];
                double gr = dphiI[2 * ((size_t)p * NB + b)] * area[p], gi = dphiI[2 * ((size_t)p * NB + b) + 1] * area[p];
                sr += xr * gr - xi * gi;
                si += xr * gi + xi * gr;
            }
        }
        part[2 * ((size_t)blockIdx.x * nout + t)] = sr;
        part[2 * ((size_t)blockIdx.x * nout + t) + 1] = si;
    }
}

__global__ void k_post_reduce(int nblk, int nout, const double* __restrict__ part, double* __restrict__ out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nout) return;
    double sr = 0, si = 0;
    for (int b = 0; b < nblk; ++b) {
        sr += part[2 * ((size_t)b * nout + t)];
        si += part[2 * ((size_t)b * nout + t) + 1];
    }
    out[2 * t] = sr;
    out[2 * t + 1] = si;
}

// ---------------------------------------------------------------------------
// Exterior free-surface elevation (Hydrodynamic_Solver.cpp:205-266, 498-505).
// One warp per wave point w, lanes over body panels s.  Per pair the Rankine
// source/dipole of the body panel and of its mirror image (Prepare_FS_Linear_System)
// and the wave term of the mirrored panel (Prepare_FS_Linear_System_Wave_Terms):
//     WS = -s - sr - ws                      (SMatExt + SMatReflExt + SWaveMatExt)
//     WD = d + dr + wd + (-sr) 2 n_z(s) K    (DMatExt + DMatReflExt + DWaveMatExt)
// then, with X = [Phi_J | Phi_S] (N x R),
//     ExtRad  = -i Omega / g (WS N_k   - WD Phi_J)      (:503)
//     ExtDiff = -i Omega / g (WS dPhiI/dn + WD Phi_S)  (:504)
// g is the global Gravity = 9.81.  Sources are the nsrc hull panels (with IFR the
// interior free-surface panels follow them and are not sources here, :218-229).
// out: [NW][R] complex interleaved.
__global__ void __launch_bounds__(256) k_fs_elevation(WaveArgs a, int nsrc, int NW, const double* __restrict__ wp,
                                                      const double* __restrict__ rec, const double* __restrict__ rn,
                                                      double Omega, int NB, const double* __restrict__ Nk,
                                                      const double* __restrict__ dphiI, const double* __restrict__ X,
                                                      double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (w >= NW) return;
    const int N = a.N, R = 6 + NB;
    const double Px = wp[w], Py = wp[NW + w], Pz = wp[2 * NW + w];
    double ar[MAX_RHS], ai[MAX_RHS];
#pragma unroll
    for (int j = 0; j < MAX_RHS; ++j) { ar[j] = 0; ai[j] = 0; }
    for (int s = lane; s < nsrc; s += 32) {
        double sd, dd, sm, dm, wsr, wsi, wdr, wdi;
        source_kernel(rec + (size_t)s * RK_STRIDE, Px, Py, Pz, sd, dd);
        source_kernel(rec + ((size_t)N + s) * RK_STRIDE, Px, Py, Pz, sm, dm);
        wave_pair<double>(a, s, Px, Py, Pz, wsr, wsi, wdr, wdi);
        const double WSr = (-sd) + (-sm) + (-wsr), WSi = -wsi;
        const double WDr = dd + dm + (wdr + (-sm) * rn[s] * a.K), WDi = wdi;
        const double* x = X + (size_t)s * 2 * R;
#pragma unroll
        for (int j = 0; j < MAX_RHS; ++j) {
            if (j < R) {
                double ur, ui;
                if (j < 6) { ur = Nk[(size_t)s * 6 + j]; ui = 0.0; }
                else { ur = dphiI[2 * ((size_t)s * NB + j - 6)]; ui = dphiI[2 * ((size_t)s * NB + j - 6) + 1]; }
                const double sg = j < 6 ? -1.0 : 1.0;
                const double xr = x[2 * j], xi = x[2 * j + 1];
                ar[j] += (WSr * ur - WSi * ui) + sg * (WDr * xr - WDi * xi);
                ai[j] += (WSr * ui + WSi * ur) + sg * (WDr * xi + WDi * xr);
            }
        }
    }
    const double c = Omega / 9.81;
#pragma unroll
    for (int j = 0; j < MAX_RHS; ++j) {
        if (j < R) {
            double vr = ar[j], vi = ai[j];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                vr += __shfl_xor_sync(0xffffffffu, vr, off);
                vi += __shfl_xor_sync(0xffffffffu, vi, off);
            }
            if (lane == 0) {  // -i c (vr + i vi) = c vi - i c vr
                out[2 * ((size_t)w * R + j)] = c * vi;
                out[2 * ((size_t)w * R + j) + 1] = -c * vr;
            }
        }
    }
}

// Kochin functions (Set_Kochin_Mats, Hydrodynamic_Solver.cpp:598-642, and :492-494)
// at theta_i = (i + 1/2) 2 pi / NK.  The reference reads an uninitialised E
// (:626-627); this computes the evident intent E = exp(K z + i K (x cos t + y sin t))
// at the panel centroids, so that
//     KochinRad(i, j)  = sum_P A_P (E N_k(P, j)     - dE/dn Phi_J(P, j))
//     KochinDiff(i, b) = sum_P A_P (E dPhiI/dn(P, b) - dE/dn Phi_S(P, b))
// with dE/dn = (i K (n_x cos t + n_y sin t) + K n_z) E, over the nsrc hull panels
// (N is the stride of cen / nrm).  One warp per angle.
__global__ void __launch_bounds__(256) k_kochin(int N, int nsrc, int NK, int NB, double K, const double* __restrict__ cen,
                                                const double* __restrict__ nrm, const double* __restrict__ area,
                                                const double* __restrict__ Nk, const double* __restrict__ dphiI,
                                                const double* __restrict__ X, double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (i >= NK) return;
    const int R = 6 + NB;
    const double th = (0.5 + (double)i) * 6.283185307179586 / NK;
    double st, ct;
    sincos(th, &st, &ct);
    double ar[MAX_RHS], ai[MAX_RHS];
#pragma unroll
    for (int j = 0; j < MAX_RHS; ++j) { ar[j] = 0; ai[j] = 0; }
    for (int p = lane; p < nsrc; p += 32) {
        const double x = cen[p], y = cen[N + p], z = cen[2 * N + p];
        const double nx = nrm[p], ny = nrm[N + p], nz = nrm[2 * N + p];
        double sa, ca;
        sincos(K * (x * ct + y * st), &sa, &ca);
        const double m = exp(K * z) * area[p];
        const double Er = m * ca, Ei = m * sa;
        const double tr = K * nz, ti = K * (nx * ct + ny * st);  // dE/dn = (tr + i ti) E
        const double Gr = tr * Er - ti * Ei, Gi = tr * Ei + ti * Er;
        const double* xp = X + (size_t)p * 2 * R;
#pragma unroll
        for (int j = 0; j < MAX_RHS; ++j) {
            if (j < R) {
                double ur, ui;
                if (j < 6) { ur = Nk[(size_t)p * 6 + j]; ui = 0.0; }
                else { ur = dphiI[2 * ((size_t)p * NB + j - 6)]; ui = dphiI[2 * ((size_t)p * NB + j - 6) + 1]; }
                const double xr = xp[2 * j], xi = xp[2 * j + 1];
                ar[j] += (Er * ur - Ei * ui) - (Gr * xr - Gi * xi);
                ai[j] += (Er * ui + Ei * ur) - (Gr * xi + Gi * xr);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < MAX_RHS; ++j) {
        if (j < R) {
            double vr = ar[j], vi = ai[j];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                vr += __shfl_xor_sync(0xffffffffu, vr, off);
                vi += __shfl_xor_sync(0xffffffffu, vi, off);
            }
            if (lane == 0) {
                out[2 * ((size_t)i * R + j)] = vr;
                out[2 * ((size_t)i * R + j) + 1] = vi;
            }
        }
    }
}

// Batch HavelockGF (Kernels.cpp:342-412) for the C ABI and tests.
template <typename T>
__global__ void k_havelock(int n, const double* __restrict__ x, const double* __restrict__ y,
                           const double* __restrict__ v, double* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T dx = (T)x[i], dy = (T)y[i], vv = (T)v[i];
    T hh = sqrt(dx * dx + dy * dy);
    typename WaveMath<T>::C G, Gh;
    WaveMath<T>::gf(hh, vv, G, Gh);
    double* o = out + 8 * (size_t)i;
    o[0] = G.re; o[1] = G.im;
    if (hh > (T)1.0e-6) {
        o[2] = (double)(Gh.re * dx / hh); o[3] = (double)(Gh.im * dx / hh);
        o[4] = (double)(Gh.re * dy / hh); o[5] = (double)(Gh.im * dy / hh);
    } else {
        o[2] = o[3] = o[4] = o[5] = 0.0;
    }
    o[6] = G.re; o[7] = G.im;
}

// ---------------------------------------------------------------------------
// Host launchers
static bool g_poly_ready[64] = {false};

// FP32 FMA throughput probe (the roofline denominator of the FP32-bound assembly):
// every thread runs 8 independent FMA chains of `iters` steps, x <- x a + b, with
// a, b chosen so the values stay bounded.  The result is stored only when it
// equals `never`, which it does not, so the chains cannot be removed.
__global__ void __launch_bounds__(256) k_ffma_peak(int iters, float a, float b, float never, float* out) {
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = (float)(threadIdx.x + k) * 1e-3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
#pragma unroll
            for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], a, b);
        }
    }
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) sum += x[k];
    if (sum == never) out[blockIdx.x * blockDim.x + threadIdx.x] = sum;
}

double ffma_peak_tflops(int device) {
    if (cudaSetDevice(device) != cudaSuccess) return -1.0;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    float* out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * 256 * 8 * (size_t)nsm) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int iters = 4096, grid = 8 * nsm;
    BEM_LAUNCH(k_ffma_peak<<<grid, 256>>>(iters, 0.9999f, 1e-4f, -12345.f, out));  // warm-up
    cudaEventRecord(e0);
    for (int r = 0; r < 5; ++r) BEM_LAUNCH(k_ffma_peak<<<grid, 256>>>(iters, 0.9999f, 1e-4f, -12345.f, out));
    cudaEventRecord(e1);
    float ms = 0.f;
    const bool ok = cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    cudaGetLastError();
    if (!ok || ms <= 0.f) return -1.0;
    const double flops = 5.0 * 2.0 * 8.0 * 16.0 * iters * (double)grid * 256.0;
    return flops / (ms * 1e-3) / 1e12;
}

cudaError_t upload_poly_constants(int device) {
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    if (g_poly_ready[device]) return cudaSuccess;
    // the FP64 monomial coefficients of the reference (the FP32 path uses the shifted
    // literals BEM_P32_* compiled into its kernels)
    PolyCoef64 p64;
    memset(&p64, 0, sizeof(p64));
    double* dst64[7] = {p64.A, p64.B, p64.C, p64.D, p64.dA, p64.dB, p64.dC};
    int k = 0;
#define BEM_FILL(name, n, ...)                         \
    {                                                   \
        const double c[] = {__VA_ARGS__};               \
        for (int i = 0; i < n; ++i) dst64[k][i] = c[i]; \
        ++k;                                            \
    }
    BEM_POLY_TABLE(BEM_FILL)
#undef BEM_FILL
    const cudaError_t e = cudaMemcpyToSymbol(c_poly64, &p64, sizeof(p64));
    if (e == cudaSuccess) g_poly_ready[device] = true;
    return e;
}

void launch_rankine(cudaStream_t st, int N, int ld, const double* rec, const double* xr, const double* rn, int mode,
                    double* o0, double* o1, double* o2, double* o3) {
    dim3 blk(32, 8), grd((N + 31) / 32, (N + 7) / 8);
    BEM_LAUNCH(k_rankine<<<grd, blk, 0, st>>>(N, ld, rec, xr, rn, mode, o0, o1, o2, o3));
}

void set_wave_f32_constants(WaveArgs& a) {
    a.kh = (float)a.K;
    a.kl = (float)(a.K - (double)a.kh);
    a.c1f = (float)(a.K * kFourPIinv);
    a.c2f = (float)(a.K * a.K * kFourPIinv);
    a.live = a.K != 0.0 ? 1 : 0;
}

void launch_wave(cudaStream_t st, const WaveArgs& a, bool fp32) {
    if (fp32) {
        WaveArgs b = a;
        set_wave_f32_constants(b);
        // persistent: three CTAs per SM when the GPU is free (the occupancy limit)
        int dev = 0, nsm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaMemsetAsync(a.row_ctr, 0, sizeof(int) * (2 + WAVE_SM_SLOTS), st);
        // the S*B accumulators are sized for the right-hand sides at hand: with 16 of them the
        // kernel spills at its 80-register bound (three CTAs per SM), with 8 or 10 it does not
        const int grid = std::min(3 * nsm, (b.N + 7) / 8);
        if (b.R <= 8) BEM_LAUNCH(k_wave_mixed<8><<<grid, 256, 0, st>>>(b));
        else if (b.R <= 10) BEM_LAUNCH(k_wave_mixed<10><<<grid, 256, 0, st>>>(b));
        else BEM_LAUNCH(k_wave_mixed<MAX_RHS><<<grid, 256, 0, st>>>(b));
    } else {
        BEM_LAUNCH(k_wave<double><<<(a.N + 7) / 8, 256, 0, st>>>(a));
    }
}

void launch_pw_build(cudaStream_t st, int N, int M, double K, const double* xr, const double* gq, const int* nq,
                     float4* E, float4* V, float4* W) {
    dim3 grd((N + 127) / 128, M);
    BEM_LAUNCH(k_pw_build<<<grd, 128, 0, st>>>(N, M, K, xr, gq, nq, E, V, W));
}

template <int RR>
static void pw_project_rr(cudaStream_t st, int N, int M, const float4* P, const float4* Z, double* T) {
    const size_t smem = sizeof(double) * 4 * RR * (PW_THREADS + 1);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(k_pw_project<RR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    BEM_LAUNCH(k_pw_project<RR><<<dim3(M, (N + PW_CHUNK - 1) / PW_CHUNK), PW_THREADS, smem, st>>>(N, P, Z, T));
}

void launch_pw_correct(cudaStream_t st, int N, int M, int R, double scale, const float4* P, const float4* E,
                       const float4* Zdf, double* T, double* out) {
    cudaMemsetAsync(T, 0, sizeof(double) * 4 * (size_t)M * R, st);
    switch (R) {
        case 1: pw_project_rr<1>(st, N, M, P, Zdf, T); break;
        case 2: pw_project_rr<2>(st, N, M, P, Zdf, T); break;
        case 3: pw_project_rr<3>(st, N, M, P, Zdf, T); break;
        case 4: pw_project_rr<4>(st, N, M, P, Zdf, T); break;
        case 5: pw_project_rr<5>(st, N, M, P, Zdf, T); break;
        case 6: pw_project_rr<6>(st, N, M, P, Zdf, T); break;
        case 7: pw_project_rr<7>(st, N, M, P, Zdf, T); break;
        case 8: pw_project_rr<8>(st, N, M, P, Zdf, T); break;
        case 9: pw_project_rr<9>(st, N, M, P, Zdf, T); break;
        case 10: pw_project_rr<10>(st, N, M, P, Zdf, T); break;
        case 11: pw_project_rr<11>(st, N, M, P, Zdf, T); break;
        case 12: pw_project_rr<12>(st, N, M, P, Zdf, T); break;
        case 13: pw_project_rr<13>(st, N, M, P, Zdf, T); break;
        case 14: pw_project_rr<14>(st, N, M, P, Zdf, T); break;
        case 15: pw_project_rr<15>(st, N, M, P, Zdf, T); break;
        default: pw_project_rr<16>(st, N, M, P, Zdf, T); break;
    }
    const size_t smem = sizeof(float4) * 2 * (size_t)M * R;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_pw_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int total = N * R;
    BEM_LAUNCH(k_pw_apply<<<(total + 255) / 256, 256, smem, st>>>(N, M, R, scale, E, T, out));
}

void launch_pad_identity(cudaStream_t st, int N, int ld, double* D64r, double* D64i, float* D32r, float* D32i) {
    if (ld <= N) return;
    BEM_LAUNCH(k_pad_identity<<<1024, 256, 0, st>>>(N, ld, D64r, D64i, D32r, D32i));
}

void launch_incident(cudaStream_t st, int N, int NB, int R, const double* betas, double K, double Omega,
                     const double* cen, const double* nrm, const double* area, double* phiI, double* dphiI,
                     double* Bm) {
    BEM_LAUNCH(k_incident<<<(N + 127) / 128, 128, 0, st>>>(N, NB, R, betas, K, Omega, cen, nrm, area, phiI, dphiI, Bm));
}

int post_blocks(int N) { return (N + POST_PANELS - 1) / POST_PANELS; }

void launch_post(cudaStream_t st, int N, int NB, int R, const double* X, const double* Nk, const double* area,
                 const double* phiI, const double* dphiI, double* part, double* out) {
    int nblk = post_blocks(N);
    int nout = 36 + 12 * NB;
    BEM_LAUNCH(k_post_partial<<<nblk, 256, 0, st>>>(N, NB, R, X, Nk, area, phiI, dphiI, part));
    BEM_LAUNCH(k_post_reduce<<<(nout + 127) / 128, 128, 0, st>>>(nblk, nout, part, out));
}

void launch_fs_elevation(cudaStream_t st, const WaveArgs& a, int nsrc, int NW, const double* wp, const double* rec,
                         const double* rn, double Omega, int NB, const double* Nk, const double* dphiI,
                         const double* X, double* out) {
    if (NW <= 0) return;
    BEM_LAUNCH(k_fs_elevation<<<(NW + 7) / 8, 256, 0, st>>>(a, nsrc, NW, wp, rec, rn, Omega, NB, Nk, dphiI, X,
                                                           out));
}

void launch_kochin(cudaStream_t st, int N, int nsrc, int NK, int NB, double K, const double* cen, const double* nrm,
                   const double* area, const double* Nk, const double* dphiI, const double* X, double* out) {
    if (NK <= 0) return;
    BEM_LAUNCH(k_kochin<<<(NK + 7) / 8, 256, 0, st>>>(N, nsrc, NK, NB, K, cen, nrm, area, Nk, dphiI, X, out));
}

void launch_havelock(cudaStream_t st, int n, const double* x, const double* y, const double* v, double* out,
                     bool fp32) {
    int g = (n + 127) / 128;
    if (fp32) BEM_LAUNCH(k_havelock<float><<<g, 128, 0, st>>>(n, x, y, v, out));
    else BEM_LAUNCH(k_havelock<double><<<g, 128, 0, st>>>(n, x, y, v, out));
}

}  // namespace bem
