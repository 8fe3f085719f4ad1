// host_cusolver.cu -- cuSOLVER's complex LU (zgetrf, partial pivoting) timed on the
// device, as the library figure beside the plain FP64 path's own LU.  Measurement only:
// nothing on the solve path calls it.  cuSOLVER is opened at run time (dlopen), so the
// library has no link-time dependency on it; where it is absent the call reports
// BEM_ERR_UNSUPPORTED.
#include <cuComplex.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/bemgpu.h"
#include "bem_internal.h"

namespace {

// A[i][j] = (u1 + i u2) * 0.2 / sqrt(n) + 0.5 delta_ij with u1, u2 uniform on [-1, 1)
// from a counter-based hash of (i, j): a well-conditioned dense complex matrix.
__global__ void k_fill_zrand(int n, cuDoubleComplex* A, double scale) {
    const size_t total = (size_t)n * n;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
        uint64_t h = k * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
        h ^= h >> 31;
        h *= 0xBF58476D1CE4E5B9ull;
        h ^= h >> 27;
        h *= 0x94D049BB133111EBull;
        h ^= h >> 33;
        const double u1 = (double)(h >> 40) * (1.0 / 8388608.0) - 1.0;
        const double u2 = (double)(h & 0xFFFFFFull) * (1.0 / 8388608.0) - 1.0;
        const size_t i = k / n, j = k % n;
        A[k] = make_cuDoubleComplex(u1 * scale + (i == j ? 0.5 : 0.0), u2 * scale);
    }
}

using PfnCreate = cusolverStatus_t (*)(cusolverDnHandle_t*);
using PfnDestroy = cusolverStatus_t (*)(cusolverDnHandle_t);
using PfnSetStream = cusolverStatus_t (*)(cusolverDnHandle_t, cudaStream_t);
using PfnZgetrfBuf = cusolverStatus_t (*)(cusolverDnHandle_t, int, int, cuDoubleComplex*, int, int*);
using PfnZgetrf = cusolverStatus_t (*)(cusolverDnHandle_t, int, int, cuDoubleComplex*, int, cuDoubleComplex*, int*,
                                       int*);

bem_status cs_fail(bem_status s, const std::string& msg) {
    bem::set_static_error(("bem_cusolver_zgetrf_ms: " + msg).c_str());
    return s;
}

}  // namespace

extern "C" bem_status bem_cusolver_zgetrf_ms(int device, int n, double* ms) {
    if (n < 1 || n > 32768 || !ms) return cs_fail(BEM_ERR_ARG, "n outside [1, 32768] or null output");
    void* lib = dlopen("libcusolver.so.12", RTLD_NOW | RTLD_LOCAL);
    if (!lib) lib = dlopen("libcusolver.so", RTLD_NOW | RTLD_LOCAL);
    if (!lib) return cs_fail(BEM_ERR_UNSUPPORTED, "libcusolver not found");
    const auto create = reinterpret_cast<PfnCreate>(dlsym(lib, "cusolverDnCreate"));
    const auto destroy = reinterpret_cast<PfnDestroy>(dlsym(lib, "cusolverDnDestroy"));
    const auto set_stream = reinterpret_cast<PfnSetStream>(dlsym(lib, "cusolverDnSetStream"));
    const auto getrf_buf = reinterpret_cast<PfnZgetrfBuf>(dlsym(lib, "cusolverDnZgetrf_bufferSize"));
    const auto getrf = reinterpret_cast<PfnZgetrf>(dlsym(lib, "cusolverDnZgetrf"));
    if (!create || !destroy || !set_stream || !getrf_buf || !getrf) {
        dlclose(lib);
        return cs_fail(BEM_ERR_UNSUPPORTED, "libcusolver lacks the zgetrf entry points");
    }
    int prev_device = 0;
    cudaGetDevice(&prev_device);
    bem_status st = BEM_OK;
    std::string why;
    cudaStream_t s = nullptr;
    cusolverDnHandle_t h = nullptr;
    cuDoubleComplex *A = nullptr, *work = nullptr;
    int *ipiv = nullptr, *info = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int lwork = 0;
    float best = 1e30f;
    const double scale = 0.2 / std::sqrt((double)n);
    auto ck = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess && st == BEM_OK) {
            st = e == cudaErrorMemoryAllocation ? BEM_ERR_NOMEM : BEM_ERR_CUDA;
            why = std::string(what) + ": " + cudaGetErrorString(e);
        }
        return st == BEM_OK;
    };
    auto cks = [&](cusolverStatus_t e, const char* what) {
        if (e != CUSOLVER_STATUS_SUCCESS && st == BEM_OK) {
            st = BEM_ERR_CUDA;
            why = std::string(what) + " failed (cusolver status " + std::to_string((int)e) + ")";
        }
        return st == BEM_OK;
    };
    if (ck(cudaSetDevice(device), "cudaSetDevice") && ck(cudaStreamCreate(&s), "cudaStreamCreate") &&
        ck(cudaEventCreate(&e0), "cudaEventCreate") && ck(cudaEventCreate(&e1), "cudaEventCreate") &&
        ck(cudaMalloc(&A, sizeof(cuDoubleComplex) * (size_t)n * n), "cudaMalloc") &&
        ck(cudaMalloc(&ipiv, sizeof(int) * (size_t)n), "cudaMalloc") && ck(cudaMalloc(&info, sizeof(int)), "cudaMalloc") &&
        cks(create(&h), "cusolverDnCreate") && cks(set_stream(h, s), "cusolverDnSetStream") &&
        cks(getrf_buf(h, n, n, A, n, &lwork), "cusolverDnZgetrf_bufferSize") &&
        ck(cudaMalloc(&work, sizeof(cuDoubleComplex) * (size_t)std::max(lwork, 1)), "cudaMalloc")) {
        // one warm-up factorization, then the best of two timed ones, each of a fresh matrix
        for (int rep = 0; rep < 3 && st == BEM_OK; ++rep) {
            BEM_LAUNCH(k_fill_zrand<<<1024, 256, 0, s>>>(n, A, scale));
            if (!ck(cudaGetLastError(), "fill kernel")) break;
            if (!ck(cudaEventRecord(e0, s), "cudaEventRecord")) break;
            if (!cks(getrf(h, n, n, A, n, work, ipiv, info), "cusolverDnZgetrf")) break;
            if (!ck(cudaEventRecord(e1, s), "cudaEventRecord") || !ck(cudaStreamSynchronize(s), "synchronize")) break;
            float t = 0.f;
            if (!ck(cudaEventElapsedTime(&t, e0, e1), "cudaEventElapsedTime")) break;
            int hinfo = 0;
            if (!ck(cudaMemcpy(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy")) break;
            if (hinfo != 0) {
                st = BEM_ERR_NUMERIC;
                why = "zgetrf reported info = " + std::to_string(hinfo);
                break;
            }
            if (rep > 0 && t < best) best = t;
        }
    }
    if (h) destroy(h);
    cudaFree(work);
    cudaFree(info);
    cudaFree(ipiv);
    cudaFree(A);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    dlclose(lib);
    cudaSetDevice(prev_device);  // the caller's current device is left as it was
    if (st != BEM_OK) return cs_fail(st, why);
    *ms = (double)best;
    return BEM_OK;
}
