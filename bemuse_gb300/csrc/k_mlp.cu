// k_mlp.cu -- MLP surrogate of the wave Green function (HavelockGF, Kernels.cpp:342-412):
// inputs (log10 KR, KZ), 4 hidden layers of width 128 with SiLU, 6 outputs
// (Re/Im of G, dG/dR, dG/dZ).  Weights are kept as an FP32 master copy and
// used as BF16 (round-to-nearest) in every product; all sums accumulate in
// FP32.  Training is plain mini-batch Adam on the mean squared error of the
// normalised outputs, with this file's own forward and backward kernels:
//   k_gemm        C = A B (+ beta C), either operand transposed, BF16 or FP32 operands
//   k_bias_act    Z += b, A = SiLU(Z) (hidden layers) or A = Z (output layer)
//   k_act_back    dZ = dA * SiLU'(Z)
//   k_colsum      db = column sums of dZ
//   k_mse         dY = 2 (Y - T) / (B * 6), loss partial sums
//   k_adam        Adam step on the master weights, then the BF16 copy
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/bemgpu.h"
#include "bem_internal.h"

namespace {

constexpr int NL = 5;                                 // linear layers
constexpr int DIMS[NL + 1] = {2, 128, 128, 128, 128, 6};
constexpr int GT = 64, GK = 16;                       // GEMM tile (m, n) and k-chunk

constexpr int w_off(int l) {
    int o = 0;
    for (int i = 0; i < l; ++i) o += DIMS[i + 1] * DIMS[i] + DIMS[i + 1];
    return o;
}
constexpr int N_PARAMS = w_off(NL);

__device__ __forceinline__ float ld_f(const float* p) { return *p; }
__device__ __forceinline__ float ld_f(const __nv_bfloat16* p) { return __bfloat162float(*p); }

// C[m][n] = sum_k A(m, k) B(k, n) + beta C[m][n];  A(m, k) = ta ? A[k lda + m] : A[m lda + k],
// B(k, n) = tb ? B[n ldb + k] : B[k ldb + n].  64 x 64 tiles, 256 threads, 4 x 4 outputs each.
template <typename TA, typename TB>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const TA* __restrict__ A, int lda, int ta,
                                              const TB* __restrict__ B, int ldb, int tb, float* __restrict__ C,
                                              int ldc, float beta) {
    __shared__ float As[GK][GT + 4];
    __shared__ float Bs[GK][GT + 4];
    const int m0 = blockIdx.y * GT, n0 = blockIdx.x * GT;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int k0 = 0; k0 < K; k0 += GK) {
        for (int e = threadIdx.x; e < GT * GK; e += 256) {
            int mm, kk;
            if (ta) { kk = e / GT; mm = e % GT; } else { mm = e / GK; kk = e % GK; }
            const int m = m0 + mm, k = k0 + kk;
            float v = 0.f;
            if (m < M && k < K) v = ta ? ld_f(A + (size_t)k * lda + m) : ld_f(A + (size_t)m * lda + k);
            As[kk][mm] = v;
        }
        for (int e = threadIdx.x; e < GT * GK; e += 256) {
            int nn, kk;
            if (tb) { nn = e / GK; kk = e % GK; } else { kk = e / GT; nn = e % GT; }
            const int n = n0 + nn, k = k0 + kk;
            float v = 0.f;
            if (n < N && k < K) v = tb ? ld_f(B + (size_t)n * ldb + k) : ld_f(B + (size_t)k * ldb + n);
            Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty * 4 + i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tx * 4 + j;
            if (n >= N) continue;
            float* c = C + (size_t)m * ldc + n;
            *c = beta != 0.f ? fmaf(beta, *c, acc[i][j]) : acc[i][j];
        }
    }
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_d(float z) {
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

__global__ void k_bias_act(int B, int OUT, float* Z, float* A, const float* __restrict__ bias, int act) {
    const size_t n = (size_t)B * OUT;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float z = Z[i] + bias[i % OUT];
        Z[i] = z;
        A[i] = act ? silu(z) : z;
    }
}

__global__ void k_act_back(size_t n, const float* __restrict__ dA, const float* __restrict__ Z, float* dZ) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dZ[i] = dA[i] * silu_d(Z[i]);
}

// db[o] = sum_b dZ[b][o]: one CTA per output column.
__global__ void k_colsum(int B, int OUT, const float* __restrict__ dZ, float* db) {
    __shared__ float red[256];
    const int o = blockIdx.x;
    float s = 0.f;
    for (int b = threadIdx.x; b < B; b += blockDim.x) s += dZ[(size_t)b * OUT + o];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[o] = red[0];
}

// dY = 2 (Y - T) / (B NO);  loss += sum (Y - T)^2 / (B NO)
__global__ void k_mse(int B, int NO, const float* __restrict__ Y, const float* __restrict__ T, float* dY,
                      double* loss) {
    __shared__ double red[256];
    const size_t n = (size_t)B * NO;
    const float inv = 1.0f / (float)n;
    double s = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float d = Y[i] - T[i];
        dY[i] = 2.0f * d * inv;
        s += (double)d * d;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0] / (double)n);
}

__global__ void k_adam(int n, float* w, float* m, float* v, const float* __restrict__ g, __nv_bfloat16* wb, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    w[i] = wi;
    wb[i] = __float2bfloat16_rn(wi);
}

__global__ void k_to_bf16(int n, const float* __restrict__ w, __nv_bfloat16* wb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

}  // namespace

struct bem_mlp {
    int device = 0;
    cudaStream_t st = nullptr;
    float* w = nullptr;            // FP32 master weights
    __nv_bfloat16* wb = nullptr;   // BF16 copy used by the products
    float *m = nullptr, *v = nullptr, *g = nullptr;
    int adam_t = 0;
    double in_shift[2] = {0, 0}, in_scale[2] = {1, 1}, out_shift[6] = {0, 0, 0, 0, 0, 0},
           out_scale[6] = {1, 1, 1, 1, 1, 1};
    int cap = 0;                   // batch capacity of the activation buffers
    float* Z[NL] = {};             // pre-activations [cap][DIMS[l+1]]
    float* A[NL + 1] = {};         // activations; A[0] = normalised input
    float *dA = nullptr, *dZ = nullptr, *T = nullptr;
    double* d_loss = nullptr;
    // tensor-core inference (k_mlp_tc.cu): operand image of the BF16 weights, rebuilt
    // when the weights change (version counts set_params / train calls)
    uint8_t* tc_img = nullptr;
    float* tc_f = nullptr;
    int* tc_flags = nullptr;
    float *tc_x = nullptr, *tc_y = nullptr;
    int tc_cap = 0;
    long version = 0, tc_version = -1;
    std::string err;
};

namespace {

bem_status mlp_fail(bem_mlp* p, const std::string& msg, bem_status s = BEM_ERR_CUDA) {
    if (p) p->err = msg;
    return s;
}

#define MK(call)                                                                            \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return mlp_fail(p, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename TA, typename TB>
void gemm(cudaStream_t st, int M, int N, int K, const TA* A, int lda, int ta, const TB* B, int ldb, int tb, float* C,
          int ldc, float beta) {
    dim3 grd((N + GT - 1) / GT, (M + GT - 1) / GT);
    BEM_LAUNCH(k_gemm<TA, TB><<<grd, 256, 0, st>>>(M, N, K, A, lda, ta, B, ldb, tb, C, ldc, beta));
}

bem_status ensure_cap(bem_mlp* p, int B) {
    if (B <= p->cap) return BEM_OK;
    for (int l = 0; l < NL; ++l) { cudaFree(p->Z[l]); p->Z[l] = nullptr; }
    for (int l = 0; l <= NL; ++l) { cudaFree(p->A[l]); p->A[l] = nullptr; }
    cudaFree(p->dA); cudaFree(p->dZ); cudaFree(p->T);
    p->dA = p->dZ = p->T = nullptr;
    for (int l = 0; l < NL; ++l) MK(cudaMalloc(&p->Z[l], sizeof(float) * (size_t)B * DIMS[l + 1]));
    for (int l = 0; l <= NL; ++l) MK(cudaMalloc(&p->A[l], sizeof(float) * (size_t)B * DIMS[l]));
    MK(cudaMalloc(&p->dA, sizeof(float) * (size_t)B * 128));
    MK(cudaMalloc(&p->dZ, sizeof(float) * (size_t)B * 128));
    MK(cudaMalloc(&p->T, sizeof(float) * (size_t)B * DIMS[NL]));
    p->cap = B;
    return BEM_OK;
}

void forward(bem_mlp* p, int B) {
    for (int l = 0; l < NL; ++l) {
        const int in = DIMS[l], out = DIMS[l + 1];
        const __nv_bfloat16* W = p->wb + w_off(l);
        gemm(p->st, B, out, in, p->A[l], in, 0, W, in, 1, p->Z[l], out, 0.f);  // Z = A W^T
        const size_t n = (size_t)B * out;
        BEM_LAUNCH(k_bias_act<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, p->st>>>(
            B, out, p->Z[l], p->A[l + 1], p->w + w_off(l) + out * in, l < NL - 1));
    }
}

// Gradients of the loss against T (p->T) into p->g; the loss is added into *d_loss.
void backward(bem_mlp* p, int B) {
    const int no = DIMS[NL];
    BEM_LAUNCH(k_mse<<<256, 256, 0, p->st>>>(B, no, p->A[NL], p->T, p->dZ, p->d_loss));
    for (int l = NL - 1; l >= 0; --l) {
        const int in = DIMS[l], out = DIMS[l + 1];
        // p->dZ holds dL/dZ_l  [B][out]
        float* gW = p->g + w_off(l);
        gemm(p->st, out, in, B, p->dZ, out, 1, p->A[l], in, 0, gW, in, 0.f);  // dW = dZ^T A_l
        BEM_LAUNCH(k_colsum<<<out, 256, 0, p->st>>>(B, out, p->dZ, gW + out * in));
        if (l == 0) break;
        const __nv_bfloat16* W = p->wb + w_off(l);
        gemm(p->st, B, in, out, p->dZ, out, 0, W, in, 0, p->dA, in, 0.f);  // dA_l = dZ W
        const size_t n = (size_t)B * in;
        BEM_LAUNCH(k_act_back<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, p->st>>>(
            n, p->dA, p->Z[l - 1], p->dZ));
    }
}

void upload_inputs(bem_mlp* p, int B, const double* x, const double* y, std::vector<float>& hx,
                   std::vector<float>& hy) {
    hx.resize((size_t)B * 2);
    for (int i = 0; i < B; ++i)
        for (int c = 0; c < 2; ++c) hx[2 * i + c] = (float)((x[2 * i + c] - p->in_shift[c]) / p->in_scale[c]);
    cudaMemcpyAsync(p->A[0], hx.data(), hx.size() * 4, cudaMemcpyHostToDevice, p->st);
    if (y) {
        hy.resize((size_t)B * 6);
        for (int i = 0; i < B; ++i)
            for (int c = 0; c < 6; ++c) hy[6 * i + c] = (float)((y[6 * i + c] - p->out_shift[c]) / p->out_scale[c]);
        cudaMemcpyAsync(p->T, hy.data(), hy.size() * 4, cudaMemcpyHostToDevice, p->st);
    }
}

// The tensor-core operand image of the current weights and n samples of I/O space.
bem_status ensure_tc(bem_mlp* p, int n) {
    if (!bem::tc_gemm_supported(p->device))
        return mlp_fail(p, "tensor-core inference needs an sm_103 GPU", BEM_ERR_UNSUPPORTED);
    if (!p->tc_img) {
        MK(cudaMalloc(&p->tc_img, bem::mlp_tc_image_bytes()));
        MK(cudaMalloc(&p->tc_f, sizeof(float) * bem::mlp_tc_param_floats()));
        MK(cudaMalloc(&p->tc_flags, sizeof(int)));
    }
    if (n > p->tc_cap) {
        cudaFree(p->tc_x);
        cudaFree(p->tc_y);
        p->tc_x = p->tc_y = nullptr;
        p->tc_cap = 0;
        MK(cudaMalloc(&p->tc_x, sizeof(float) * 2 * (size_t)n));
        MK(cudaMalloc(&p->tc_y, sizeof(float) * 6 * (size_t)n));
        p->tc_cap = n;
    }
    if (p->tc_version != p->version) {
        bem::mlp_tc_build_image(p->st, p->w, p->tc_img, p->tc_f);
        p->tc_version = p->version;
    }
    MK(cudaMemsetAsync(p->tc_flags, 0, sizeof(int), p->st));
    return BEM_OK;
}

bem_status tc_flags_ok(bem_mlp* p) {
    int hf = 0;
    MK(cudaMemcpyAsync(&hf, p->tc_flags, sizeof(int), cudaMemcpyDeviceToHost, p->st));
    MK(cudaStreamSynchronize(p->st));
    if (hf & bem::FLAG_TIMEOUT) return mlp_fail(p, "a device-side wait of the tensor-core forward expired");
    return BEM_OK;
}

}  // namespace

int bem::mlp_tc_ref(bem_mlp* p, bem::MlpTcRef* out) {
    if (!p || !out) return 1;
    if (cudaSetDevice(p->device) != cudaSuccess) return 1;
    if (ensure_tc(p, 1) != BEM_OK) return 1;
    if (cudaStreamSynchronize(p->st) != cudaSuccess) {
        p->err = "building the tensor-core operand image failed";
        return 1;
    }
    out->img = p->tc_img;
    out->fw = p->tc_f;
    memcpy(out->in_shift, p->in_shift, sizeof(out->in_shift));
    memcpy(out->in_scale, p->in_scale, sizeof(out->in_scale));
    memcpy(out->out_shift, p->out_shift, sizeof(out->out_shift));
    memcpy(out->out_scale, p->out_scale, sizeof(out->out_scale));
    out->device = p->device;
    return 0;
}

extern "C" {

int bem_mlp_num_params(void) { return N_PARAMS; }

bem_status bem_mlp_eval_tc(bem_mlp* p, int n, const double* x, double* y) {
    if (!p || n < 0 || (n > 0 && (!x || !y))) return BEM_ERR_ARG;
    MK(cudaSetDevice(p->device));
    if (n == 0) return BEM_OK;
    bem_status s = ensure_tc(p, n);
    if (s != BEM_OK) return s;
    std::vector<float> hx((size_t)n * 2), hy((size_t)n * 6);
    for (int i = 0; i < n; ++i)
        for (int c = 0; c < 2; ++c) hx[2 * (size_t)i + c] = (float)((x[2 * (size_t)i + c] - p->in_shift[c]) / p->in_scale[c]);
    MK(cudaMemcpyAsync(p->tc_x, hx.data(), hx.size() * 4, cudaMemcpyHostToDevice, p->st));
    if (bem::mlp_tc_forward(p->st, n, p->tc_x, p->tc_y, p->tc_img, p->tc_f, p->tc_flags))
        return mlp_fail(p, "tensor-core forward launch failed");
    MK(cudaMemcpyAsync(hy.data(), p->tc_y, hy.size() * 4, cudaMemcpyDeviceToHost, p->st));
    s = tc_flags_ok(p);
    if (s != BEM_OK) return s;
    for (size_t i = 0; i < (size_t)n; ++i)
        for (int c = 0; c < 6; ++c) y[6 * i + c] = hy[6 * i + c] * p->out_scale[c] + p->out_shift[c];
    return BEM_OK;
}

bem_status bem_mlp_throughput_tc(bem_mlp* p, int n, double* evals_per_s) {
    if (!p || n <= 0 || !evals_per_s) return BEM_ERR_ARG;
    MK(cudaSetDevice(p->device));
    bem_status s = ensure_tc(p, n);
    if (s != BEM_OK) return s;
    MK(cudaMemsetAsync(p->tc_x, 0, sizeof(float) * 2 * (size_t)n, p->st));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    bem::mlp_tc_forward(p->st, n, p->tc_x, p->tc_y, p->tc_img, p->tc_f, p->tc_flags);  // warm-up
    cudaEventRecord(e0, p->st);
    const int reps = 5;
    for (int r = 0; r < reps; ++r) bem::mlp_tc_forward(p->st, n, p->tc_x, p->tc_y, p->tc_img, p->tc_f, p->tc_flags);
    cudaEventRecord(e1, p->st);
    cudaError_t ce = cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ce != cudaSuccess) return mlp_fail(p, cudaGetErrorString(ce));
    s = tc_flags_ok(p);
    if (s != BEM_OK) return s;
    *evals_per_s = (double)n * reps / (ms / 1000.0);
    return BEM_OK;
}

bem_status bem_mlp_create(bem_mlp** out, int device, unsigned long long seed) {
    if (!out) return BEM_ERR_ARG;
    *out = nullptr;
    bem_mlp* p = new bem_mlp();
    p->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&p->st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete p;
        bem::set_static_error("bem_mlp_create: CUDA device unavailable");
        return BEM_ERR_CUDA;
    }
    // Xavier-uniform weights, zero biases
    std::vector<float> h(N_PARAMS, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < NL; ++l) {
        const int in = DIMS[l], outd = DIMS[l + 1];
        const double a = std::sqrt(6.0 / (in + outd));
        std::uniform_real_distribution<double> U(-a, a);
        for (int i = 0; i < in * outd; ++i) h[w_off(l) + i] = (float)U(rng);
    }
    bem_status s = BEM_OK;
    if (cudaMalloc(&p->w, 4 * N_PARAMS) || cudaMalloc(&p->wb, 2 * N_PARAMS) || cudaMalloc(&p->m, 4 * N_PARAMS) ||
        cudaMalloc(&p->v, 4 * N_PARAMS) || cudaMalloc(&p->g, 4 * N_PARAMS) || cudaMalloc(&p->d_loss, 8))
        s = BEM_ERR_NOMEM;
    if (s == BEM_OK) {
        cudaMemcpy(p->w, h.data(), 4 * N_PARAMS, cudaMemcpyHostToDevice);
        cudaMemset(p->m, 0, 4 * N_PARAMS);
        cudaMemset(p->v, 0, 4 * N_PARAMS);
        BEM_LAUNCH(k_to_bf16<<<(N_PARAMS + 255) / 256, 256, 0, p->st>>>(N_PARAMS, p->w, p->wb));
        if (cudaStreamSynchronize(p->st) != cudaSuccess) s = BEM_ERR_CUDA;
    }
    if (s != BEM_OK) {
        cudaGetLastError();
        bem::set_static_error("bem_mlp_create: device allocation failed");
        *out = p;
        return s;
    }
    *out = p;
    return BEM_OK;
}

void bem_mlp_destroy(bem_mlp* p) {
    if (!p) return;
    cudaSetDevice(p->device);
    if (p->st) cudaStreamSynchronize(p->st);
    for (int l = 0; l < NL; ++l) cudaFree(p->Z[l]);
    for (int l = 0; l <= NL; ++l) cudaFree(p->A[l]);
    cudaFree(p->dA); cudaFree(p->dZ); cudaFree(p->T);
    cudaFree(p->w); cudaFree(p->wb); cudaFree(p->m); cudaFree(p->v); cudaFree(p->g); cudaFree(p->d_loss);
    cudaFree(p->tc_img); cudaFree(p->tc_f); cudaFree(p->tc_flags); cudaFree(p->tc_x); cudaFree(p->tc_y);
    if (p->st) cudaStreamDestroy(p->st);
    delete p;
}

const char* bem_mlp_last_error(const bem_mlp* p) { return p ? p->err.c_str() : ""; }

bem_status bem_mlp_set_normalization(bem_mlp* p, const double* in_shift, const double* in_scale,
                                     const double* out_shift, const double* out_scale) {
    if (!p || !in_shift || !in_scale || !out_shift || !out_scale) return BEM_ERR_ARG;
    for (int c = 0; c < 2; ++c)
        if (!(in_scale[c] != 0.0)) return mlp_fail(p, "zero input scale", BEM_ERR_ARG);
    for (int c = 0; c < 6; ++c)
        if (!(out_scale[c] != 0.0)) return mlp_fail(p, "zero output scale", BEM_ERR_ARG);
    memcpy(p->in_shift, in_shift, sizeof(p->in_shift));
    memcpy(p->in_scale, in_scale, sizeof(p->in_scale));
    memcpy(p->out_shift, out_shift, sizeof(p->out_shift));
    memcpy(p->out_scale, out_scale, sizeof(p->out_scale));
    return BEM_OK;
}

bem_status bem_mlp_get_params(bem_mlp* p, double* w) {
    if (!p || !w) return BEM_ERR_ARG;
    MK(cudaSetDevice(p->device));
    std::vector<float> h(N_PARAMS);
    MK(cudaMemcpyAsync(h.data(), p->w, 4 * N_PARAMS, cudaMemcpyDeviceToHost, p->st));
    MK(cudaStreamSynchronize(p->st));
    for (int i = 0; i < N_PARAMS; ++i) w[i] = h[i];
    return BEM_OK;
}

bem_status bem_mlp_set_params(bem_mlp* p, const double* w) {
    if (!p || !w) return BEM_ERR_ARG;
    MK(cudaSetDevice(p->device));
    std::vector<float> h(N_PARAMS);
    for (int i = 0; i < N_PARAMS; ++i) h[i] = (float)w[i];
    MK(cudaMemcpyAsync(p->w, h.data(), 4 * N_PARAMS, cudaMemcpyHostToDevice, p->st));
    BEM_LAUNCH(k_to_bf16<<<(N_PARAMS + 255) / 256, 256, 0, p->st>>>(N_PARAMS, p->w, p->wb));
    MK(cudaStreamSynchronize(p->st));
    ++p->version;
    p->adam_t = 0;
    MK(cudaMemsetAsync(p->m, 0, 4 * N_PARAMS, p->st));
    MK(cudaMemsetAsync(p->v, 0, 4 * N_PARAMS, p->st));
    return BEM_OK;
}

bem_status bem_mlp_eval(bem_mlp* p, int n, const double* x, double* y) {
    if (!p || n < 0 || (n > 0 && (!x || !y))) return BEM_ERR_ARG;
    MK(cudaSetDevice(p->device));
    const int chunk = 1 << 16;
    std::vector<float> hx, hy, ho((size_t)chunk * 6);
    for (int s0 = 0; s0 < n; s0 += chunk) {
        const int B = std::min(chunk, n - s0);
        bem_status s = ensure_cap(p, B);
        if (s != BEM_OK) return s;
        upload_inputs(p, B, x + 2 * (size_t)s0, nullptr, hx, hy);
        forward(p, B);
        MK(cudaMemcpyAsync(ho.data(), p->A[NL], sizeof(float) * 6 * (size_t)B, cudaMemcpyDeviceToHost, p->st));
        MK(cudaStreamSynchronize(p->st));
        for (int i = 0; i < B; ++i)
            for (int c = 0; c < 6; ++c)
                y[6 * ((size_t)s0 + i) + c] = ho[6 * (size_t)i + c] * p->out_scale[c] + p->out_shift[c];
    }
    MK(cudaGetLastError());
    return BEM_OK;
}

bem_status bem_mlp_grad(bem_mlp* p, int n, const double* x, const double* y, double* grad, double* loss) {
    if (!p || n <= 0 || !x || !y || !grad) return BEM_ERR_ARG;
    MK(cudaSetDevice(p->device));
    bem_status s = ensure_cap(p, n);
    if (s != BEM_OK) return s;
    std::vector<float> hx, hy, hg(N_PARAMS);
    upload_inputs(p, n, x, y, hx, hy);
    MK(cudaMemsetAsync(p->d_loss, 0, 8, p->st));
    forward(p, n);
    backward(p, n);
    double l = 0;
    MK(cudaMemcpyAsync(hg.data(), p->g, 4 * N_PARAMS, cudaMemcpyDeviceToHost, p->st));
    MK(cudaMemcpyAsync(&l, p->d_loss, 8, cudaMemcpyDeviceToHost, p->st));
    MK(cudaStreamSynchronize(p->st));
    for (int i = 0; i < N_PARAMS; ++i) grad[i] = hg[i];
    if (loss) *loss = l;
    return BEM_OK;
}

bem_status bem_mlp_train(bem_mlp* p, int n, const double* x, const double* y, int epochs, int batch, double lr,
                         unsigned long long seed, double* loss_per_epoch) {
    if (!p || n <= 0 || !x || !y || epochs < 0 || batch <= 0) return BEM_ERR_ARG;
    MK(cudaSetDevice(p->device));
    bem_status s = ensure_cap(p, batch);
    if (s != BEM_OK) return s;
    // normalised data set resident on the device
    std::vector<float> hx((size_t)n * 2), hy((size_t)n * 6);
    for (int i = 0; i < n; ++i) {
        for (int c = 0; c < 2; ++c) hx[2 * (size_t)i + c] = (float)((x[2 * (size_t)i + c] - p->in_shift[c]) / p->in_scale[c]);
        for (int c = 0; c < 6; ++c) hy[6 * (size_t)i + c] = (float)((y[6 * (size_t)i + c] - p->out_shift[c]) / p->out_scale[c]);
    }
    float *dx = nullptr, *dy = nullptr;
    MK(cudaMalloc(&dx, hx.size() * 4));
    if (cudaMalloc(&dy, hy.size() * 4) != cudaSuccess) { cudaFree(dx); return mlp_fail(p, "cudaMalloc", BEM_ERR_NOMEM); }
    cudaMemcpyAsync(dx, hx.data(), hx.size() * 4, cudaMemcpyHostToDevice, p->st);
    cudaMemcpyAsync(dy, hy.data(), hy.size() * 4, cudaMemcpyHostToDevice, p->st);
    std::mt19937_64 rng(seed);
    const int nb = n / batch;
    std::vector<int> order(std::max(nb, 1));
    for (int i = 0; i < (int)order.size(); ++i) order[i] = i;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int e = 0; e < epochs; ++e) {
        std::shuffle(order.begin(), order.end(), rng);
        cudaMemsetAsync(p->d_loss, 0, 8, p->st);
        for (int k = 0; k < nb; ++k) {
            const size_t s0 = (size_t)order[k] * batch;
            cudaMemcpyAsync(p->A[0], dx + 2 * s0, sizeof(float) * 2 * batch, cudaMemcpyDeviceToDevice, p->st);
            cudaMemcpyAsync(p->T, dy + 6 * s0, sizeof(float) * 6 * batch, cudaMemcpyDeviceToDevice, p->st);
            forward(p, batch);
            backward(p, batch);
            ++p->adam_t;
            const float c1 = 1.0f / (1.0f - std::pow(b1, (float)p->adam_t));
            const float c2 = 1.0f / (1.0f - std::pow(b2, (float)p->adam_t));
            BEM_LAUNCH(k_adam<<<(N_PARAMS + 255) / 256, 256, 0, p->st>>>(N_PARAMS, p->w, p->m, p->v, p->g, p->wb,
                                                                         (float)lr, b1, b2, eps, c1, c2));
        }
        if (loss_per_epoch) {
            double l = 0;
            cudaMemcpyAsync(&l, p->d_loss, 8, cudaMemcpyDeviceToHost, p->st);
            cudaStreamSynchronize(p->st);
            loss_per_epoch[e] = nb > 0 ? l / nb : 0.0;
        }
    }
    cudaError_t ce = cudaStreamSynchronize(p->st);
    cudaFree(dx);
    cudaFree(dy);
    ++p->version;
    if (ce != cudaSuccess) return mlp_fail(p, std::string("training: ") + cudaGetErrorString(ce));
    return BEM_OK;
}

// Device time of a batched forward pass of n samples (inputs resident), and of the
// FP32 closed-form HavelockGF on the same number of points, both per second.
bem_status bem_mlp_throughput(bem_mlp* p, int n, double* mlp_evals_per_s) {
    if (!p || n <= 0 || !mlp_evals_per_s) return BEM_ERR_ARG;
    MK(cudaSetDevice(p->device));
    bem_status s = ensure_cap(p, n);
    if (s != BEM_OK) return s;
    MK(cudaMemsetAsync(p->A[0], 0, sizeof(float) * 2 * (size_t)n, p->st));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    forward(p, n);  // warm-up
    cudaEventRecord(e0, p->st);
    const int reps = 5;
    for (int r = 0; r < reps; ++r) forward(p, n);
    cudaEventRecord(e1, p->st);
    cudaError_t ce = cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ce != cudaSuccess) return mlp_fail(p, cudaGetErrorString(ce));
    *mlp_evals_per_s = (double)n * reps / (ms / 1000.0);
    return BEM_OK;
}

}  // extern "C"
