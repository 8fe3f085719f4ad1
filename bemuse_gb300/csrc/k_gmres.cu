// k_gmres.cu -- FP64 vector kernels of the flexible GMRES refinement (host loop in
// host_api.cpp::refine_gmres).
//
// All vectors are Np x R complex blocks, interleaved (re, im), row-major with R
// columns (one column per right-hand side): the layout of the solution and residual
// blocks.  A set of nvec vectors is stored back to back, vstride doubles apart.
// Every reduction is two-phase with a fixed summation order, so results do not
// depend on scheduling.
//
// Reference: the linear solve of Hydrodynamic_Solver.cpp:430-446 (Eigen
// PartialPivLU::solve); GMRES replaces the direct solve's accuracy with FP64
// refinement against the FP64-accurate operator.
#include "bem_internal.h"

namespace bem {

constexpr int GM_ROWS = 64;   // rows per partial sum
constexpr int GM_LANES = 16;  // columns per CTA row (R <= MAX_RHS = 16)

size_t gm_part_doubles(int Np, int nvec) {
    return (size_t)2 * nvec * ((Np + GM_ROWS - 1) / GM_ROWS) * GM_LANES;
}

// part[v][chunk][r] = sum over the chunk's rows n of conj(V_v[n][r]) * w[n][r]
__global__ void __launch_bounds__(256) k_gm_dots(int Np, int R, const double* __restrict__ V, size_t vstride,
                                                 const double* __restrict__ w, double* __restrict__ part) {
    __shared__ double red[16][GM_LANES][2];
    const int v = blockIdx.y, r = threadIdx.x % GM_LANES, rr = threadIdx.x / GM_LANES;
    const double* Vv = V + (size_t)v * vstride;
    double sr = 0.0, si = 0.0;
    if (r < R) {
        const int n1 = min(Np, (int)(blockIdx.x + 1) * GM_ROWS);
        for (int n = blockIdx.x * GM_ROWS + rr; n < n1; n += 16) {
            const size_t o = 2 * ((size_t)n * R + r);
            const double a = Vv[o], b = Vv[o + 1], c = w[o], d = w[o + 1];
            sr = fma(a, c, fma(b, d, sr));
            si = fma(a, d, fma(-b, c, si));
        }
    }
    red[rr][r][0] = sr;
    red[rr][r][1] = si;
    __syncthreads();
    if (rr == 0) {
        double tr = 0.0, ti = 0.0;
        for (int k = 0; k < 16; ++k) { tr += red[k][r][0]; ti += red[k][r][1]; }
        double* p = part + 2 * (((size_t)v * gridDim.x + blockIdx.x) * GM_LANES + r);
        p[0] = tr;
        p[1] = ti;
    }
}

// h[v][r] = sum over chunks of part[v][chunk][r], chunk order fixed
__global__ void k_gm_sum(int nvec, int nchunk, int R, const double* __restrict__ part, double* __restrict__ h) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nvec * R) return;
    const int v = i / R, r = i % R;
    double tr = 0.0, ti = 0.0;
    for (int c = 0; c < nchunk; ++c) {
        const double* p = part + 2 * (((size_t)v * nchunk + c) * GM_LANES + r);
        tr += p[0];
        ti += p[1];
    }
    h[2 * i] = tr;
    h[2 * i + 1] = ti;
}

// out[n][r] = beta out[n][r] + sign sum_v c[v][r] V_v[n][r]   (complex, no conjugation)
__global__ void k_gm_combine(int Np, int R, int nvec, const double* __restrict__ V, size_t vstride,
                             const double* __restrict__ c, double sign, double beta, double* __restrict__ out) {
    const size_t tot = (size_t)Np * R;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(i % R);
        double xr = 0.0, xi = 0.0;
        if (beta != 0.0) { xr = beta * out[2 * i]; xi = beta * out[2 * i + 1]; }
        for (int v = 0; v < nvec; ++v) {
            const double* Vv = V + (size_t)v * vstride + 2 * i;
            const double cr = sign * c[2 * (v * R + r)], ci = sign * c[2 * (v * R + r) + 1];
            xr = fma(cr, Vv[0], fma(-ci, Vv[1], xr));
            xi = fma(cr, Vv[1], fma(ci, Vv[0], xi));
        }
        out[2 * i] = xr;
        out[2 * i + 1] = xi;
    }
}

// out = w / sqrt(nrm2[r].re) per column (0 where the norm vanishes: the column has converged)
__global__ void k_gm_scale(int Np, int R, const double* __restrict__ w, const double* __restrict__ nrm2,
                           double* __restrict__ out) {
    const size_t tot = (size_t)Np * R;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < tot; i += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(i % R);
        const double s = nrm2[2 * r];
        const double f = s > 1e-300 ? 1.0 / sqrt(s) : 0.0;
        out[2 * i] = w[2 * i] * f;
        out[2 * i + 1] = w[2 * i + 1] * f;
    }
}

__global__ void k_f32_to_f64(size_t n, const float* __restrict__ s, double* __restrict__ d) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        d[i] = (double)s[i];
}

void launch_gm_dots(cudaStream_t st, int Np, int R, int nvec, const double* V, size_t vstride, const double* w,
                    double* part, double* h) {
    const int nchunk = (Np + GM_ROWS - 1) / GM_ROWS;
    BEM_LAUNCH(k_gm_dots<<<dim3(nchunk, nvec), 256, 0, st>>>(Np, R, V, vstride, w, part));
    BEM_LAUNCH(k_gm_sum<<<(nvec * R + 127) / 128, 128, 0, st>>>(nvec, nchunk, R, part, h));
}
void launch_gm_combine(cudaStream_t st, int Np, int R, int nvec, const double* V, size_t vstride, const double* c,
                       double sign, double beta, double* out) {
    BEM_LAUNCH(k_gm_combine<<<1024, 256, 0, st>>>(Np, R, nvec, V, vstride, c, sign, beta, out));
}
void launch_gm_scale(cudaStream_t st, int Np, int R, const double* w, const double* nrm2, double* out) {
    BEM_LAUNCH(k_gm_scale<<<1024, 256, 0, st>>>(Np, R, w, nrm2, out));
}
void launch_f32_to_f64(cudaStream_t st, size_t n, const float* src, double* dst) {
    BEM_LAUNCH(k_f32_to_f64<<<1024, 256, 0, st>>>(n, src, dst));
}

// The convergence test of one classic refinement sweep, on the device: the decision the
// host loop of factor_and_solve makes after reading the sweep's residual norms, so that
// the sweeps can repeat inside a graph (a conditional while node on handle h) without a
// round trip to the host.  One thread; the loop continues while it sets h to 1.
__global__ void k_refine_step(int R, const unsigned long long* __restrict__ nrm, const int* __restrict__ flags,
                              double tol, int max_iter, int coarse_first, int gmres_switch, RefineState* st,
                              cudaGraphConditionalHandle h) {
    RefineState v = *st;
    v.iters += 1;
    v.flags = *flags;
    unsigned int go = 0;
    if (v.flags & FLAG_TIMEOUT) {
        v.status = REFINE_TIMEOUT;
    } else {
        double resid = 0.0;
        for (int j = 0; j < R; ++j) {
            const double rn = __longlong_as_double((long long)nrm[j]);
            const double yn = __longlong_as_double((long long)nrm[R + j]);
            const double rel = yn > 0 ? rn / yn : rn;
            if (resid < rel) resid = rel;
        }
        v.resid = resid;
        // the coarse first residual (high words of Re D only) never certifies convergence
        const bool full = !(v.iters == 1 && coarse_first);
        if (full) {
            if (v.prev_full > 0.0) v.contraction = resid / v.prev_full;
            v.prev_full = resid;
        }
        if (resid <= tol && full) {
            v.status = REFINE_CONVERGED;
        } else if (v.iters >= max_iter || !(resid < 1e300)) {
            v.status = REFINE_FAILED;
        } else if (gmres_switch && v.iters >= 2 && resid > 0.05 * v.prev) {
            v.status = REFINE_STALLED;  // a sweep that gained less than 20x: flexible GMRES takes over
        } else {
            v.prev = resid;
            go = 1;
        }
    }
    *st = v;
    cudaGraphSetConditional(h, go);
}

void launch_refine_step(cudaStream_t st, int R, const unsigned long long* nrm, const int* flags, double tol,
                        int max_iter, int coarse_first, int gmres_switch, RefineState* state,
                        cudaGraphConditionalHandle h) {
    BEM_LAUNCH(k_refine_step<<<1, 1, 0, st>>>(R, nrm, flags, tol, max_iter, coarse_first, gmres_switch, state, h));
}

}  // namespace bem
