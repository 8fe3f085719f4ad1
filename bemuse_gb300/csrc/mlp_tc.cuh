// mlp_tc.cuh -- the tensor-core (tcgen05) forward pass of the Green-function surrogate
// network, as device functions shared by the batched inference kernel (k_mlp_tc.cu)
// and the fused far-field assembly kernel (k_influence.cu).
//
// Network: (log10 KR, KZ) -> 128 -> 128 -> 128 -> 128 -> 6, SiLU on the hidden layers.
// Each CTA holds it in shared memory once: layer 0 (2 -> 128) as FP32 values of its
// BF16 weights (it runs on the CUDA cores: K = 2 is too short for an MMA), layers 1-3
// (128 x 128) and the output layer (padded to 16 rows) as BF16 images in the K-major,
// 128-byte-swizzle operand layout of tcgen05.mma (built by k_mlp_tc_image).  A tile is
// 128 samples: thread t of a warpgroup owns sample t, i.e. row t of the A operand and
// lane t of the warpgroup's TMEM accumulator (128 columns).  Per hidden layer the
// threads write their activation rows (BF16) into the A operand, one elected thread
// issues eight MMAs (K = 16 each, kind::f16, FP32 accumulation) and commits them to
// the warpgroup's mbarrier, then every warp reads its 32 lanes back (tcgen05.ld), adds
// the bias, applies SiLU = x/2 (1 + tanh(x/2)) with the hardware tanh and writes the
// next operand.  Every mbarrier wait has an iteration limit; after one expires
// (FLAG_TIMEOUT) the warpgroup keeps its barrier sequence but issues and waits no more.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "bem_internal.h"
#include "tc_ptx.cuh"

namespace bem {
namespace mlptc {

using namespace tcp;

constexpr int H = 128;                                  // hidden width
constexpr int NOUT = 6, NOUT_PAD = 16;                  // outputs (the MMA needs N % 16 == 0 at M = 128)
constexpr int LAYER_BYTES = 2 * H * 128;                // 128 rows x 128 bf16: two 64-wide swizzle atoms
constexpr int OUT_BYTES = 2 * NOUT_PAD * 128;           // 16 rows x 128 bf16
constexpr int IMG_BYTES = 3 * LAYER_BYTES + OUT_BYTES;
constexpr int TILE_BYTES = 2 * H * 128;                 // A operand of one 128-sample tile
constexpr int TAIL_FLOATS = 256 + 4 * H + NOUT_PAD;     // W0 and the biases in FP32
constexpr int SMEM_BYTES = 1024 + IMG_BYTES + 2 * TILE_BYTES + 4 * TAIL_FLOATS + 64;
constexpr int THREADS = 256;                            // two warpgroups

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

// Shared-memory layout of a CTA: [image][tile 0][tile 1][FP32 tail][2 mbarriers][TMEM
// address][abort flag of each warpgroup], the image 1024-byte aligned.  Each warpgroup
// sets and reads only its own abort flag, and reads it only after its own barrier, so
// all its threads agree on it.
struct Smem {
    unsigned char* gbase;
    uint32_t s_img, s_tile0;
    float* s_f;
    uint64_t* bars;
    volatile uint32_t* tmem_slot;
    volatile int* abort_flag;
};

__device__ __forceinline__ Smem smem_layout(unsigned char* smem_raw) {
    Smem m;
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    m.gbase = smem_raw + (base - raw);
    m.s_img = base;
    m.s_tile0 = base + IMG_BYTES;
    m.s_f = reinterpret_cast<float*>(m.gbase + IMG_BYTES + 2 * TILE_BYTES);
    m.bars = reinterpret_cast<uint64_t*>(m.s_f + TAIL_FLOATS);
    m.tmem_slot = reinterpret_cast<volatile uint32_t*>(m.bars + 2);
    m.abort_flag = reinterpret_cast<volatile int*>(m.bars + 3);
    return m;
}

// Every thread of the CTA: network into shared memory, mbarriers, 256 TMEM columns (two
// warpgroups x 128).  Returns the TMEM base address.
__device__ __forceinline__ uint32_t cta_setup(const Smem& m, const uint8_t* __restrict__ img,
                                              const float* __restrict__ fw) {
    const uint4* src = reinterpret_cast<const uint4*>(img);
    uint4* dst = reinterpret_cast<uint4*>(m.gbase);
    for (int i = threadIdx.x; i < IMG_BYTES / 16; i += blockDim.x) dst[i] = src[i];
    for (int i = threadIdx.x; i < TAIL_FLOATS; i += blockDim.x) m.s_f[i] = fw[i];
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(m.bars), 1);
        mbar_init(smem_u32(m.bars + 1), 1);
        m.abort_flag[0] = 0;
        m.abort_flag[1] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if ((threadIdx.x >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32((void*)m.tmem_slot)),
                     "r"(256));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the image is read by the tensor cores
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    return *m.tmem_slot;
}

// Every thread of the CTA, after its last layer: frees the TMEM columns.
__device__ __forceinline__ void cta_teardown(uint32_t tmem) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(256));
    }
}

// Layer 0 of sample t from its normalised inputs (x0, x1) into the A operand `tile`.
__device__ __forceinline__ void layer0(const Smem& m, uint32_t tile, int t, float x0, float x1) {
#pragma unroll 1
    for (int c0 = 0; c0 < H; c0 += 32) {
        float v[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const int c = c0 + j;
            v[j] = silu_tc(fmaf(m.s_f[2 * c], x0, fmaf(m.s_f[2 * c + 1], x1, m.s_f[256 + c])));
        }
        store_row32(tile, t, c0, v);
    }
}

// Layers 1-4 of warpgroup g's tile (layer 0 already in its A operand): out[0..5] receive
// the thread's sample's normalised outputs (zeros after an expired wait).  phase is the
// warpgroup's mbarrier phase, kept by the caller across tiles.  Every thread of the
// warpgroup calls this.
__device__ __forceinline__ void layers(const Smem& m, uint32_t tile, uint32_t acc, uint32_t lane_base, int g, int t,
                                       uint32_t& phase, int* gflags, float* out) {
    const uint32_t bar = smem_u32(m.bars + g);
    volatile int* abort_flag = m.abort_flag + g;
#pragma unroll
    for (int j = 0; j < NOUT; ++j) out[j] = 0.f;
#pragma unroll 1
    for (int l = 0; l < 4; ++l) {
        const bool last = l == 3;
        // the A operand written by this warpgroup's threads, then read by the tensor cores
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        wg_sync(g);
        const bool live = *abort_flag == 0;
        if (t == 0 && live) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t wl = m.s_img + (uint32_t)l * LAYER_BYTES;
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
        bool have = false;
        if (live) {
            have = mbar_wait(bar, phase, abort_flag, gflags);
            phase ^= 1u;
        }
        // a warp whose wait expired skips the accumulator but keeps the barrier sequence
        have = __all_sync(0xffffffffu, have);
        if (have) asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (!last) {
            const float* bias = m.s_f + 256 + (l + 1) * H;
#pragma unroll 1
            for (int c0 = 0; c0 < H; c0 += 32) {
                float v[32];
                if (have) {
                    tmem_ld32(acc + lane_base + (uint32_t)c0, v);
                } else {
#pragma unroll
                    for (int j = 0; j < 32; ++j) v[j] = 0.f;
                }
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = silu_tc(v[j] + bias[c0 + j]);
                store_row32(tile, t, c0, v);
            }
        } else if (have) {
            float v[16];
            tmem_ld16(acc + lane_base, v);
            const float* bias = m.s_f + 256 + 4 * H;
#pragma unroll
            for (int j = 0; j < NOUT; ++j) out[j] = v[j] + bias[j];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

}  // namespace mlptc
}  // namespace bem
