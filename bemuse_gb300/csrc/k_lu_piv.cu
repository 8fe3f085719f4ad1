// k_lu_piv.cu -- complex LU with partial pivoting (FP64), the factorisation of
// Eigen::PartialPivLU<MatrixXcd> (Solver_Base.h:85; compute / solve at
// Hydrodynamic_Solver.cpp:430, 438, 446): at step j the pivot is the first row i >= j
// of largest |a_ij| (the magnitude of the complex entry), rows j and i are exchanged
// over the whole matrix, the column below the pivot is divided by it and the trailing
// matrix takes the rank-1 update.  Right-looking and unblocked: on this GPU the FP64
// rate, not the memory traffic of the rank-1 updates, bounds a blocked factorization
// as well.  The no-exchange blocked LU (k_lu.cu) stays the fast path; this one is the
// fallback of bem_dense_solve for matrices that need row exchanges.
//
// Matrix: planar complex (re and im arrays), row-major, leading dimension ld.
#include <cuda_runtime.h>

#include "bem_internal.h"

namespace bem {

namespace {

constexpr int PV_THREADS = 1024;

// piv[j] = first row i >= j of largest |a_ij|; a zero (or non-finite) pivot sets FLAG_ZERO_PIVOT.
__global__ void __launch_bounds__(PV_THREADS) k_piv_find(int n, int j, CMat<double> A, int* piv, int* flags) {
    __shared__ double sv[PV_THREADS];
    __shared__ int si[PV_THREADS];
    double best = -1.0;
    int bi = n;
    for (int i = j + threadIdx.x; i < n; i += PV_THREADS) {
        const double v = hypot(A.re[(size_t)i * A.ld + j], A.im[(size_t)i * A.ld + j]);
        if (v > best) { best = v; bi = i; }  // rows visited in increasing order: the first max stays
    }
    sv[threadIdx.x] = best;
    si[threadIdx.x] = bi;
    __syncthreads();
    for (int w = PV_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            const double v2 = sv[threadIdx.x + w];
            const int i2 = si[threadIdx.x + w];
            if (v2 > sv[threadIdx.x] || (v2 == sv[threadIdx.x] && i2 < si[threadIdx.x])) {
                sv[threadIdx.x] = v2;
                si[threadIdx.x] = i2;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const bool bad = !(sv[0] > 0.0) || !isfinite(sv[0]);
        piv[j] = bad ? j : si[0];
        if (bad) atomicOr(flags, FLAG_ZERO_PIVOT);
    }
}

// Exchanges rows j and piv[j] over all columns.
__global__ void k_piv_swap(int n, int j, CMat<double> A, const int* __restrict__ piv) {
    const int p = piv[j];
    if (p == j) return;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        double* r1 = A.re + (size_t)j * A.ld + c;
        double* r2 = A.re + (size_t)p * A.ld + c;
        double* i1 = A.im + (size_t)j * A.ld + c;
        double* i2 = A.im + (size_t)p * A.ld + c;
        const double tr = *r1, ti = *i1;
        *r1 = *r2; *i1 = *i2;
        *r2 = tr; *i2 = ti;
    }
}

// l_ij = a_ij / a_jj below the pivot (the multipliers, stored in place).
__global__ void k_piv_scale(int n, int j, CMat<double> A) {
    const double pr = A.re[(size_t)j * A.ld + j], pi = A.im[(size_t)j * A.ld + j];
    const double den = pr * pr + pi * pi;
    for (int i = j + 1 + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const size_t o = (size_t)i * A.ld + j;
        const double ar = A.re[o], ai = A.im[o];
        A.re[o] = (ar * pr + ai * pi) / den;
        A.im[o] = (ai * pr - ar * pi) / den;
    }
}

// a_ik -= l_ij u_jk for i, k > j (32 x 8 threads per block of the trailing matrix).
__global__ void k_piv_rank1(int n, int j, CMat<double> A) {
    const int k = j + 1 + blockIdx.x * 32 + threadIdx.x;
    const int i = j + 1 + blockIdx.y * 8 + threadIdx.y;
    if (k >= n || i >= n) return;
    const double lr = A.re[(size_t)i * A.ld + j], li = A.im[(size_t)i * A.ld + j];
    const double ur = A.re[(size_t)j * A.ld + k], ui = A.im[(size_t)j * A.ld + k];
    const size_t o = (size_t)i * A.ld + k;
    A.re[o] -= lr * ur - li * ui;
    A.im[o] -= lr * ui + li * ur;
}

// X (n x R complex interleaved): rows exchanged as the factorization exchanged them,
// then forward substitution with the unit-lower L and back substitution with U.
// One CTA per right-hand side.
__global__ void __launch_bounds__(256) k_piv_solve(int n, CMat<double> A, const int* __restrict__ piv, int R,
                                                   double* __restrict__ X) {
    const int r = blockIdx.x;
    if (r >= R) return;
    if (threadIdx.x == 0)
        for (int j = 0; j < n; ++j) {
            const int p = piv[j];
            if (p != j) {
                double* a = X + 2 * ((size_t)j * R + r);
                double* b = X + 2 * ((size_t)p * R + r);
                const double t0 = a[0], t1 = a[1];
                a[0] = b[0]; a[1] = b[1];
                b[0] = t0; b[1] = t1;
            }
        }
    __syncthreads();
    for (int j = 0; j < n; ++j) {
        const double xr = X[2 * ((size_t)j * R + r)], xi = X[2 * ((size_t)j * R + r) + 1];
        for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x) {
            const double lr = A.re[(size_t)i * A.ld + j], li = A.im[(size_t)i * A.ld + j];
            X[2 * ((size_t)i * R + r)] -= lr * xr - li * xi;
            X[2 * ((size_t)i * R + r) + 1] -= lr * xi + li * xr;
        }
        __syncthreads();
    }
    for (int j = n - 1; j >= 0; --j) {
        if (threadIdx.x == 0) {
            const double ur = A.re[(size_t)j * A.ld + j], ui = A.im[(size_t)j * A.ld + j];
            const double den = ur * ur + ui * ui;
            double* x = X + 2 * ((size_t)j * R + r);
            const double xr = x[0], xi = x[1];
            x[0] = (xr * ur + xi * ui) / den;
            x[1] = (xi * ur - xr * ui) / den;
        }
        __syncthreads();
        const double xr = X[2 * ((size_t)j * R + r)], xi = X[2 * ((size_t)j * R + r) + 1];
        for (int i = threadIdx.x; i < j; i += blockDim.x) {
            const double ur = A.re[(size_t)i * A.ld + j], ui = A.im[(size_t)i * A.ld + j];
            X[2 * ((size_t)i * R + r)] -= ur * xr - ui * xi;
            X[2 * ((size_t)i * R + r) + 1] -= ur * xi + ui * xr;
        }
        __syncthreads();
    }
}

}  // namespace

int lu_piv_factor_f64(cudaStream_t st, int n, CMat<double> A, int* piv, int* flags) {
    for (int j = 0; j < n; ++j) {
        BEM_LAUNCH(k_piv_find<<<1, PV_THREADS, 0, st>>>(n, j, A, piv, flags));
        BEM_LAUNCH(k_piv_swap<<<(n + 255) / 256, 256, 0, st>>>(n, j, A, piv));
        if (j + 1 < n) {
            BEM_LAUNCH(k_piv_scale<<<(n - j + 255) / 256, 256, 0, st>>>(n, j, A));
            const dim3 grd((n - j - 1 + 31) / 32, (n - j - 1 + 7) / 8);
            BEM_LAUNCH(k_piv_rank1<<<grd, dim3(32, 8), 0, st>>>(n, j, A));
        }
    }
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 1;
}

int lu_piv_solve_f64(cudaStream_t st, int n, CMat<double> A, const int* piv, int R, double* X) {
    BEM_LAUNCH(k_piv_solve<<<R, 256, 0, st>>>(n, A, piv, R, X));
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace bem
