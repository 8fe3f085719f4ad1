// k_tc_gemm.cu -- tcgen05 TF32 trailing update of the complex LU:
//     A22 -= L21 * U12      (planar complex, FP32 storage, FP32 accumulation)
//
// One CTA computes a 128 x 256 tile of A22.  The complex product is four real
// TF32 MMAs into two TMEM accumulators:
//     Cr = Lr Ur^T - Li Ui^T        (the minus via the instruction's negate-A bit)
//     Ci = Lr Ui^T + Li Ur^T
// L21 (K-major, ld = nb) and U12^T (K-major, written by the LU's copy-back) are
// brought into shared memory by TMA with 128-byte swizzle, in a two-stage
// mbarrier pipeline over the nb = 128 contraction (four 32-wide k-blocks).
// Warp 0 lane 0 issues TMA, warp 1 lane 0 issues tcgen05.mma; all four warps
// run the epilogue (tcgen05.ld from TMEM, C -= acc in global memory).
// Every mbarrier wait has an iteration limit; on expiry the CTA sets
// FLAG_TIMEOUT, skips the rest of its work, frees its TMEM and exits.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include "bem_internal.h"

namespace bem {

namespace {

constexpr int BM = 128, BN = 256, BK = 32, STAGES = 2;
constexpr int L_TILE = BM * BK * 4;          // 16 KB
constexpr int U_TILE = BN * BK * 4;          // 32 KB
constexpr int STAGE_BYTES = 2 * L_TILE + 2 * U_TILE;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr uint32_t TMEM_COLS = 512;          // Cr: cols [0,256), Ci: [256,512)
constexpr long WAIT_LIMIT = 1L << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false (and the abort flag set) if the phase never completes.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, int* gflags) {
    for (long i = 0; i < WAIT_LIMIT; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 255) == 255 && *abort_flag) return false;
    }
    *abort_flag = 1;
    atomicOr(gflags, FLAG_TIMEOUT);
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle,
// 8-row core-matrix groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);        // start address
    d |= (uint64_t)1 << 16;                       // leading byte offset (unused for SW128 K-major)
    d |= (uint64_t)(1024 >> 4) << 32;             // stride byte offset
    d |= (uint64_t)1 << 46;                       // descriptor version (tcgen05)
    d |= (uint64_t)2 << 61;                       // SWIZZLE_128B
    return d;
}

// Instruction descriptor: kind::tf32, D = F32, A = B = TF32, K-major, M = 128, N = 256.
__host__ __device__ constexpr uint32_t idesc_tf32(bool neg_a) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((neg_a ? 1u : 0u) << 13) | ((uint32_t)(BN >> 3) << 17) |
           ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace

__global__ void __launch_bounds__(128, 1)
    k_tc_trailing(const __grid_constant__ CUtensorMap mapL, const __grid_constant__ CUtensorMap mapU, int n, int M,
                  int Nc, float* __restrict__ Cr, float* __restrict__ Ci, int ldc, int* gflags) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // 1024-byte aligned tile area
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char* tiles = smem_raw + (base - raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(tiles + STAGES * STAGE_BYTES);  // full[2], empty[2], done
    volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(bars + 8);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 9);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + 2), done = smem_u32(bars + 4);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) { mbar_init(full0 + 8 * s, 1); mbar_init(empty0 + 8 * s, 1); }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapL)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapU)) : "memory");
    }
    __syncwarp();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32((void*)tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const int KB = 128 / BK;  // nb = 128

    if (warp == 0 && lane == 0) {
        // TMA producer
        for (int kb = 0; kb < KB; ++kb) {
            const int s = kb % STAGES, use = kb / STAGES;
            if (kb >= STAGES && !mbar_wait(empty0 + 8 * s, (use - 1) & 1, abort_flag, gflags)) break;
            const uint32_t st = base + s * STAGE_BYTES;
            mbar_expect_tx(full0 + 8 * s, STAGE_BYTES);
            tma_load_2d(st, &mapL, kb * BK, m0, full0 + 8 * s);
            tma_load_2d(st + L_TILE, &mapL, kb * BK, n + m0, full0 + 8 * s);
            tma_load_2d(st + 2 * L_TILE, &mapU, kb * BK, n0, full0 + 8 * s);
            tma_load_2d(st + 2 * L_TILE + U_TILE, &mapU, kb * BK, n + n0, full0 + 8 * s);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t id_pos = idesc_tf32(false), id_neg = idesc_tf32(true);
        const uint32_t accR = tmem, accI = tmem + 256;
        bool ok = true;
        for (int kb = 0; kb < KB && ok; ++kb) {
            const int s = kb % STAGES, use = kb / STAGES;
            if (!mbar_wait(full0 + 8 * s, use & 1, abort_flag, gflags)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t st = base + s * STAGE_BYTES;
#pragma unroll
            for (int kk = 0; kk < BK / 8; ++kk) {
                const uint32_t off = kk * 32;  // 8 tf32 = 32 bytes along K inside the swizzle atom
                const uint64_t aR = smem_desc_sw128(st + off), aI = smem_desc_sw128(st + L_TILE + off);
                const uint64_t bR = smem_desc_sw128(st + 2 * L_TILE + off);
                const uint64_t bI = smem_desc_sw128(st + 2 * L_TILE + U_TILE + off);
                const uint32_t first = (kb == 0 && kk == 0) ? 0u : 1u;
                mma_tf32(accR, aR, bR, id_pos, first);
                mma_tf32(accR, aI, bI, id_neg, 1u);
                mma_tf32(accI, aR, bI, id_pos, first);
                mma_tf32(accI, aI, bR, id_pos, 1u);
            }
            mma_commit(empty0 + 8 * s);
        }
        if (ok) mma_commit(done);
    }
    __syncwarp();
    // Epilogue: all 128 threads; thread owns tile row 32*warp + lane.
    bool have = mbar_wait(done, 0, abort_flag, gflags);
    __syncwarp();
    have = __all_sync(0xffffffffu, have);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (have) {
        const int row = m0 + warp * 32 + lane;
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
        float vr[32], vi[32];
        for (int cb = 0; cb < BN / 32; ++cb) {
            tmem_ld32(tmem + lane_base + cb * 32, vr);
            tmem_ld32(tmem + lane_base + 256 + cb * 32, vi);
            const int col = n0 + cb * 32;
            if (row < M && col < Nc) {
                float* pr = Cr + (size_t)row * ldc + col;
                float* pi = Ci + (size_t)row * ldc + col;
#pragma unroll
                for (int j = 0; j < 32; j += 4) {
                    float4 a = *reinterpret_cast<float4*>(pr + j);
                    float4 b = *reinterpret_cast<float4*>(pi + j);
                    a.x -= vr[j]; a.y -= vr[j + 1]; a.z -= vr[j + 2]; a.w -= vr[j + 3];
                    b.x -= vi[j]; b.y -= vi[j + 1]; b.z -= vi[j + 2]; b.w -= vi[j + 3];
                    *reinterpret_cast<float4*>(pr + j) = a;
                    *reinterpret_cast<float4*>(pi + j) = b;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn get_encode() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// 2D FP32 tensor of 2n rows x 128 columns (rows [0,n) real part, [n,2n) imaginary).
static bool make_map(CUtensorMap* m, const float* base, int n, int box_rows) {
    EncodeTiledFn enc = get_encode();
    if (!enc) return false;
    cuuint64_t dims[2] = {128, (cuuint64_t)2 * n};
    cuuint64_t strides[1] = {128 * sizeof(float)};
    cuuint32_t box[2] = {BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int tc_gemm_supported(int device) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return 0;
    if (!(p.major == 10 && p.minor == 3)) return 0;
    return get_encode() != nullptr ? 1 : 0;
}

// A22 -= L21 U12 for LU step k0 (nb = 128).  wl = [2][n][128] (L21 rows from 0),
// wut = [2][n][128] (U12^T rows from 0).
bool tc_trailing_update(cudaStream_t st, int n, int k0, int nb, CMat<float> A, const float* wl, const float* wut,
                        int* flags) {
    const int rem = n - k0 - nb;
    if (rem <= 0) return true;
    if (nb != 128) return false;
    CUtensorMap mL, mU;
    if (!make_map(&mL, wl, n, BM) || !make_map(&mU, wut, n, BN)) return false;
    cudaFuncSetAttribute(k_tc_trailing, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    float* Cr = A.re + (size_t)(k0 + nb) * A.ld + k0 + nb;
    float* Ci = A.im + (size_t)(k0 + nb) * A.ld + k0 + nb;
    dim3 grid((rem + BN - 1) / BN, rem / BM);
    BEM_LAUNCH(k_tc_trailing<<<grid, 128, SMEM_BYTES, st>>>(mL, mU, n, rem, rem, Cr, Ci, A.ld, flags));
    return true;
}

}  // namespace bem
