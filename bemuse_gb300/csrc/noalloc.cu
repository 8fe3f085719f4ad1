// noalloc.cu -- dense complex solve that allocates no memory.
//
// bem_dense_solve_noalloc() is the FP64 dense solve of bem_dense_solve() (blocked
// LU k_lu_diag / k_cgemm / k_copy_back and the cooperative triangular solve
// k_trsv_coop) for callers that cannot call cudaMalloc: code inside an
// application that hands all device memory to its own pool allocator, or a loop
// where cudaMalloc's implicit device-wide synchronization and latency are not
// acceptable.  Every buffer the solve needs (the padded planar matrix, its
// staging copy, LU workspaces, diagonal-block inverses, solution scratch, flags)
// lives in one file-scope __device__ array of fixed size, so the library holds
// it on every GPU that loads the library until the process exits.
#include <cuda_runtime.h>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/bemgpu.h"
#include "bem_internal.h"

namespace bem {
namespace {

constexpr int NA_MAX_N = BEM_NOALLOC_MAX_N;   // largest order accepted
constexpr int NA_NB = 64;                      // FP64 LU block width
constexpr int NA_NP = NA_MAX_N;                // padded order (multiple of 128)
constexpr size_t NA_MAT = (size_t)NA_NP * NA_NP;             // one planar plane
constexpr size_t NA_STAGE = (size_t)2 * NA_MAX_N * NA_MAX_N;  // interleaved upload
constexpr size_t NA_INV = (size_t)(NA_NP / NA_NB) * 2 * NA_NB * NA_NB;
constexpr size_t NA_WL = (size_t)2 * NA_NP * NA_NB;
constexpr size_t NA_X = (size_t)4 * NA_NP * MAX_RHS;
constexpr size_t NA_Y = (size_t)2 * NA_NP * MAX_RHS;
// layout (doubles): Dr | Di | stage | inv_r | inv_i | wl | wu | X | Y | ints
constexpr size_t OFF_DR = 0, OFF_DI = OFF_DR + NA_MAT, OFF_ST = OFF_DI + NA_MAT, OFF_IR = OFF_ST + NA_STAGE,
                 OFF_II = OFF_IR + NA_INV, OFF_WL = OFF_II + NA_INV, OFF_WU = OFF_WL + NA_WL, OFF_X = OFF_WU + NA_WL,
                 OFF_Y = OFF_X + NA_X, OFF_INT = OFF_Y + NA_Y;
constexpr size_t NA_INTS = 1 + NA_NP / NA_NB;  // flags + block-ready flags
constexpr size_t NA_TOTAL = OFF_INT + (NA_INTS + 1) / 2 + 1;

}  // namespace
}  // namespace bem

// The scratch array.  In host code this name is only a host-side stand-in for
// the symbol; its device address comes from cudaGetSymbolAddress (below).
static __device__ __align__(256) double g_noalloc_scratch[bem::NA_TOTAL];

namespace bem {
namespace {

// Padded planar copy: D[i][j] = A[i][j] for i, j < n, identity elsewhere.
__global__ void k_na_planar(int n, int np, const double* __restrict__ stage, double* __restrict__ Dr,
                            double* __restrict__ Di) {
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < (size_t)np * np;
         idx += (size_t)gridDim.x * blockDim.x) {
        int i = (int)(idx / np), j = (int)(idx % np);
        double re = 0.0, im = 0.0;
        if (i < n && j < n) {
            re = stage[2 * ((size_t)i * n + j)];
            im = stage[2 * ((size_t)i * n + j) + 1];
        } else if (i == j) {
            re = 1.0;
        }
        Dr[idx] = re;
        Di[idx] = im;
    }
}

// X = [Y; 0] (n x R rows of the right-hand sides, zero padding rows).
__global__ void k_na_rhs(int n, int np, int R, const double* __restrict__ Y, double* __restrict__ X) {
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < (size_t)2 * np * R;
         idx += (size_t)gridDim.x * blockDim.x)
        X[idx] = idx < (size_t)2 * n * R ? Y[idx] : 0.0;
}

std::mutex g_na_mutex;
double* g_na_ptr[64] = {nullptr};

// Errors go to the message bem_last_error(NULL) returns.
bem_status na_fail(bem_status s, const std::string& m) {
    set_static_error(("bem_dense_solve_noalloc: " + m).c_str());
    return s;
}

}  // namespace
}  // namespace bem

extern "C" {

bem_status bem_dense_solve_noalloc(int device, int n, const double* A, int nrhs, double* B) {
    using namespace bem;
    if (n < 1 || n > NA_MAX_N)
        return na_fail(BEM_ERR_ARG, "order n = " + std::to_string(n) + " outside [1, " +
                                        std::to_string(NA_MAX_N) + "] (the fixed scratch holds n <= " +
                                        std::to_string(NA_MAX_N) + ")");
    if (nrhs < 1 || nrhs > MAX_RHS)
        return na_fail(BEM_ERR_ARG, "nrhs = " + std::to_string(nrhs) + " outside [1, 16]");
    if (!A || !B) return na_fail(BEM_ERR_ARG, "null matrix or right-hand side");
    if (device < 0 || device >= 64) return na_fail(BEM_ERR_ARG, "device index out of range");
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return na_fail(BEM_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    double* base = nullptr;
    {
        // Set-up, once per device, with that device current: the device address
        // of the scratch symbol (the host-side name is not a device pointer).
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na_ptr[device]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess)
                return na_fail(BEM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_na_ptr[device] = static_cast<double*>(p);
        }
        base = g_na_ptr[device];
    }
    const int np = (n + 127) / 128 * 128;
    double* Dr = base + OFF_DR;
    double* Di = base + OFF_DI;
    double* stage = base + OFF_ST;
    double* invr = base + OFF_IR;
    double* invi = base + OFF_II;
    double* wl = base + OFF_WL;
    double* wu = base + OFF_WU;
    double* X = base + OFF_X;
    double* Y = base + OFF_Y;
    int* flags = reinterpret_cast<int*>(base + OFF_INT);
    int* ready = flags + 1;
    cudaStream_t st = 0;
    // The scratch keeps the previous call's contents: clear the flags that must
    // start at zero; everything else is overwritten before it is read.
    e = cudaMemsetAsync(flags, 0, sizeof(int) * NA_INTS, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(stage, A, sizeof(double) * 2 * (size_t)n * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(Y, B, sizeof(double) * 2 * (size_t)n * nrhs, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return na_fail(BEM_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
    BEM_LAUNCH(k_na_planar<<<256, 256, 0, st>>>(n, np, stage, Dr, Di));
    BEM_LAUNCH(k_na_rhs<<<64, 256, 0, st>>>(n, np, nrhs, Y, X));
    CMat<double> M{Dr, Di, np};
    lu_factor_f64(st, np, M, invr, invi, wl, wu, flags);
    if (lu_solve_f64(st, np, M, invr, invi, nrhs, X, ready, 1, flags))
        return na_fail(BEM_ERR_CUDA, "cooperative triangular-solve launch failed");
    e = cudaGetLastError();
    int hflags = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hflags, flags, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(B, X, sizeof(double) * 2 * (size_t)n * nrhs, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return na_fail(BEM_ERR_CUDA, cudaGetErrorString(e));
    // the same status codes as bem_dense_solve: an expired device wait is a CUDA-side
    // failure, a zero pivot a numeric one
    if (hflags & FLAG_TIMEOUT)
        return na_fail(BEM_ERR_CUDA, "a device-side wait in the triangular solve expired");
    if (hflags & FLAG_ZERO_PIVOT) return na_fail(BEM_ERR_NUMERIC, "zero or non-finite pivot in the LU");
    if (hflags & FLAG_PIVOT)
        return na_fail(BEM_ERR_NUMERIC, "a multiplier |l_ik| > 1: partial pivoting would exchange rows");
    return BEM_OK;
}

}  // extern "C"
