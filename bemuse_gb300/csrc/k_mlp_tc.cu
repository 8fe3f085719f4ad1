// k_mlp_tc.cu -- tensor-core (tcgen05, BF16 operands, FP32 accumulation in TMEM)
// inference of the Green-function surrogate network of k_mlp.cu:
//   (log10 KR, KZ) -> 128 -> 128 -> 128 -> 128 -> 6, SiLU on the hidden layers.
//
// Layout.  Each CTA holds the network in shared memory once: layer 0 (2 -> 128)
// as FP32 values of its BF16 weights (it runs on the CUDA cores: K = 2 is too
// short for an MMA), layers 1-3 (128 x 128) and the output layer (padded to 16
// rows) as BF16 images in the K-major, 128-byte-swizzle operand layout of
// tcgen05.mma, prepared once on the device (k_mlp_tc_image).  A tile is 128
// samples: thread t of a warpgroup owns sample t, i.e. row t of the A operand
// and lane t of the TMEM accumulator.
//
// Per tile and hidden layer: the warpgroup's threads write their activation rows
// (BF16) into the A operand, one elected thread issues eight MMAs (K = 16 each)
// into the warpgroup's 128 TMEM columns and commits them to an mbarrier, then
// every warp reads its 32 lanes back (tcgen05.ld), adds the bias, applies SiLU
// (x/2 (1 + tanh(x/2)) with the hardware tanh) and writes the next A operand.
// Two warpgroups per CTA work on different tiles, so one's epilogue (CUDA
// cores) overlaps the other's MMAs.  Every mbarrier wait has an iteration limit
// (FLAG_TIMEOUT); the CTA then stops and frees its TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "bem_internal.h"
#include "tc_ptx.cuh"

namespace bem {

namespace {

using namespace tcp;

constexpr int H = 128;                                // hidden width
constexpr int NOUT = 6, NOUT_PAD = 16;                // outputs (the MMA needs N % 16 == 0 at M = 128)
constexpr int LAYER_BYTES = 2 * H * 128;              // 128 rows x 128 bf16: two 64-wide swizzle atoms
constexpr int OUT_BYTES = 2 * NOUT_PAD * 128;         // 16 rows x 128 bf16
constexpr int IMG_BYTES = 3 * LAYER_BYTES + OUT_BYTES;
constexpr int TILE_BYTES = 2 * H * 128;               // A operand of one 128-sample tile
constexpr int TAIL_FLOATS = 256 + 4 * H + NOUT_PAD;     // W0 and the biases in FP32
constexpr int SMEM_BYTES = 1024 + IMG_BYTES + 2 * TILE_BYTES + 4 * TAIL_FLOATS + 64;
constexpr int THREADS = 256;                          // two warpgroups

// byte offset of element (row, k) of a K-major bf16 operand with 128-byte swizzle whose
// 64-wide k atoms are `atom_bytes` apart: row r at r * 128 within its atom, 16-byte chunks
// permuted by r mod 8
__host__ __device__ constexpr uint32_t sw128_offset(int row, int k, uint32_t atom_bytes) {
    return (uint32_t)(k >> 6) * atom_bytes + (uint32_t)row * 128u +
           ((((uint32_t)(k & 63) >> 3) ^ ((uint32_t)row & 7u)) << 4) + (uint32_t)(k & 7) * 2u;
}

// Instruction descriptor: kind::f16, D = F32, A = B = BF16, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float silu_tc(float z) {
    const float h = 0.5f * z;
    return fmaf(h, tanh_fast(h), h);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// Writes activations v[0..31] (columns c0 .. c0 + 31) of row `row` into the A operand at `tile`.
__device__ __forceinline__ void store_row32(uint32_t tile, int row, int c0, const float* v) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint32_t addr = tile + sw128_offset(row, c0 + 8 * q, H * 128);
        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(pack_bf16(v[8 * q], v[8 * q + 1])),
                     "r"(pack_bf16(v[8 * q + 2], v[8 * q + 3])), "r"(pack_bf16(v[8 * q + 4], v[8 * q + 5])),
                     "r"(pack_bf16(v[8 * q + 6], v[8 * q + 7]))
                     : "memory");
    }
}

__device__ __forceinline__ void wg_sync(int g) {
    asm volatile("bar.sync %0, 128;" ::"r"(1 + g) : "memory");
}

}  // namespace

// The weight image (k_mlp_tc_image) of the master parameters w (k_mlp.cu order: W0 (128 x 2),
// b0, W1 (128 x 128), b1, W2, b2, W3, b3, W4 (6 x 128), b4; W row-major [out][in]): img holds
// layers 1-3 and the padded output layer as swizzled BF16 operands; f holds W0 (as the values
// of its BF16 rounding) and the biases in FP32: [W0 256][b0 128][b1 128][b2 128][b3 128][b4 16].
__global__ void k_mlp_tc_image(const float* __restrict__ w, uint8_t* __restrict__ img, float* __restrict__ f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int o_W0 = 0, o_b0 = 256, o_W1 = o_b0 + 128, stride = H * H + H;
    const int o_W4 = o_W1 + 3 * stride, o_b4 = o_W4 + NOUT * H;
    if (i < 3 * H * H) {
        const int l = i / (H * H), r = (i / H) % H, k = i % H;
        const __nv_bfloat16 b = __float2bfloat16_rn(w[o_W1 + l * stride + r * H + k]);
        *reinterpret_cast<__nv_bfloat16*>(img + l * LAYER_BYTES + sw128_offset(r, k, H * 128)) = b;
    } else if (i < 3 * H * H + NOUT_PAD * H) {
        const int j = i - 3 * H * H, r = j / H, k = j % H;
        const float v = r < NOUT ? w[o_W4 + r * H + k] : 0.0f;
        *reinterpret_cast<__nv_bfloat16*>(img + 3 * LAYER_BYTES + sw128_offset(r, k, NOUT_PAD * 128)) =
            __float2bfloat16_rn(v);
    } else if (i < 3 * H * H + NOUT_PAD * H + 256) {
        const int j = i - 3 * H * H - NOUT_PAD * H;
        f[j] = __bfloat162float(__float2bfloat16_rn(w[o_W0 + j]));
    } else if (i < 3 * H * H + NOUT_PAD * H + 256 + 4 * H) {
        const int j = i - 3 * H * H - NOUT_PAD * H - 256, l = j / H, c = j % H;
        f[256 + j] = l == 0 ? w[o_b0 + c] : w[o_W1 + (l - 1) * stride + H * H + c];
    } else if (i < 3 * H * H + NOUT_PAD * H + 256 + 4 * H + NOUT_PAD) {
        const int c = i - 3 * H * H - NOUT_PAD * H - 256 - 4 * H;
        f[256 + 4 * H + c] = c < NOUT ? w[o_b4 + c] : 0.0f;
    }
}

// y[s][0..5] = network(x[s][0..1]) for s < n (normalised inputs and outputs, FP32).
__global__ void __launch_bounds__(THREADS, 1)
    k_mlp_tc_forward(int n, const float2* __restrict__ x, float* __restrict__ y, const uint8_t* __restrict__ img,
                     const float* __restrict__ fw, int* gflags) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char* gbase = smem_raw + (base - raw);
    const uint32_t s_img = base, s_tile0 = base + IMG_BYTES;
    float* s_f = reinterpret_cast<float*>(gbase + IMG_BYTES + 2 * TILE_BYTES);  // W0, biases (256 + 4H + 16 floats)
    uint64_t* bars = reinterpret_cast<uint64_t*>(s_f + TAIL_FLOATS);
    volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(bars + 2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 3);
    const int warp = threadIdx.x >> 5;
    const int g = warp >> 2, t = threadIdx.x & 127;  // warpgroup, sample row in the tile
    // weight image and FP32 parameters into shared memory
    {
        const uint4* src = reinterpret_cast<const uint4*>(img);
        uint4* dst = reinterpret_cast<uint4*>(gbase);
        for (int i = threadIdx.x; i < IMG_BYTES / 16; i += THREADS) dst[i] = src[i];
        for (int i = threadIdx.x; i < TAIL_FLOATS; i += THREADS) s_f[i] = fw[i];
    }
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(bars), 1);
        mbar_init(smem_u32(bars + 1), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32((void*)tmem_slot)),
                     "r"(256));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the image is read by the tensor cores
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t acc = tmem + (uint32_t)g * 128;                     // this warpgroup's 128 columns
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;     // the warp's 32 TMEM lanes
    const uint32_t tile = s_tile0 + (uint32_t)g * TILE_BYTES;
    const uint32_t bar = smem_u32(bars + g);
    uint32_t phase = 0;
    bool ok = true;
    const int ntiles = (n + 127) / 128;
    for (int tt = blockIdx.x * 2 + g; tt < ntiles && ok; tt += gridDim.x * 2) {
        const int s = tt * 128 + t;
        const float2 xi = s < n ? x[s] : make_float2(0.f, 0.f);
        // layer 0 on the CUDA cores: 128 outputs of 2 inputs each
#pragma unroll 1
        for (int c0 = 0; c0 < H; c0 += 32) {
            float v[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int c = c0 + j;
                v[j] = silu_tc(fmaf(s_f[2 * c], xi.x, fmaf(s_f[2 * c + 1], xi.y, s_f[256 + c])));
            }
            store_row32(tile, t, c0, v);
        }
        for (int l = 0; l < 4 && ok; ++l) {
            const bool last = l == 3;
            // the A operand written by this warpgroup's threads, then read by the tensor cores
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            wg_sync(g);
            if (t == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t wl = s_img + (uint32_t)l * LAYER_BYTES;
                const uint32_t atom_b = last ? NOUT_PAD * 128 : H * 128;
                const uint32_t id = idesc_bf16(last ? NOUT_PAD : H);
#pragma unroll
                for (int kk = 0; kk < H / 16; ++kk) {
                    const uint32_t koff = (uint32_t)(kk & 3) * 32u;  // 16 bf16 = 32 bytes inside the atom
                    const uint64_t ad = smem_desc_sw128(tile + (uint32_t)(kk >> 2) * (H * 128) + koff);
                    const uint64_t bd = smem_desc_sw128(wl + (uint32_t)(kk >> 2) * atom_b + koff);
                    mma_bf16(acc, ad, bd, id, kk > 0 ? 1u : 0u);
                }
                mma_commit(bar);
            }
            __syncwarp();
            const bool have = mbar_wait(bar, phase, abort_flag, gflags);
            phase ^= 1u;
            if (!__all_sync(0xffffffffu, have)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (!last) {
                const float* bias = s_f + 256 + (l + 1) * H;
#pragma unroll 1
                for (int c0 = 0; c0 < H; c0 += 32) {
                    float v[32];
                    tmem_ld32(acc + lane_base + (uint32_t)c0, v);
#pragma unroll
                    for (int j = 0; j < 32; ++j) v[j] = silu_tc(v[j] + bias[c0 + j]);
                    store_row32(tile, t, c0, v);
                }
            } else {
                float v[16];
                tmem_ld16(acc + lane_base, v);
                if (s < n) {
                    const float* bias = s_f + 256 + 4 * H;
#pragma unroll
                    for (int j = 0; j < NOUT; ++j) y[(size_t)s * NOUT + j] = v[j] + bias[j];
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256));
    }
}

int mlp_tc_image_bytes() { return IMG_BYTES; }
int mlp_tc_param_floats() { return TAIL_FLOATS; }

void mlp_tc_build_image(cudaStream_t st, const float* w, uint8_t* img, float* fw) {
    const int total = 3 * H * H + NOUT_PAD * H + 256 + 4 * H + NOUT_PAD;
    BEM_LAUNCH(k_mlp_tc_image<<<(total + 255) / 256, 256, 0, st>>>(w, img, fw));
}

int mlp_tc_forward(cudaStream_t st, int n, const float* x, float* y, const uint8_t* img, const float* fw, int* flags) {
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(k_mlp_tc_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) !=
            cudaSuccess)
            return 1;
        attr = true;
    }
    if (n <= 0) return 0;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int tiles = (n + 127) / 128;
    const int grid = std::min(nsm, (tiles + 1) / 2);
    BEM_LAUNCH(k_mlp_tc_forward<<<grid, THREADS, SMEM_BYTES, st>>>(n, reinterpret_cast<const float2*>(x), y, img, fw,
                                                                   flags));
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace bem
