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
#include "mlp_tc.cuh"

namespace bem {

using namespace mlptc;

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
    const Smem m = smem_layout(smem_raw);
    const int warp = threadIdx.x >> 5;
    const int g = warp >> 2, t = threadIdx.x & 127;  // warpgroup, sample row in the tile
    const uint32_t tmem = cta_setup(m, img, fw);
    const uint32_t acc = tmem + (uint32_t)g * 128;                  // this warpgroup's 128 columns
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;  // the warp's 32 TMEM lanes
    const uint32_t tile = m.s_tile0 + (uint32_t)g * TILE_BYTES;
    uint32_t phase = 0;
    const int ntiles = (n + 127) / 128;
    for (int tt = blockIdx.x * 2 + g; tt < ntiles; tt += gridDim.x * 2) {
        const int s = tt * 128 + t;
        const float2 xi = s < n ? x[s] : make_float2(0.f, 0.f);
        layer0(m, tile, t, xi.x, xi.y);
        float out[NOUT];
        layers(m, tile, acc, lane_base, g, t, phase, gflags, out);
        if (s < n)
#pragma unroll
            for (int j = 0; j < NOUT; ++j) y[(size_t)s * NOUT + j] = out[j];
    }
    cta_teardown(tmem);
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
