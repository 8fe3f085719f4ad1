// k_tc_gemm.cu -- tcgen05 TF32 products of the complex block LU:
//     A22 -= L21 * U12      (trailing update; planar complex, FP32 storage and accumulation)
//     W21  = A21 * D^-1     (block-column multipliers, stored to two places)
//     U   <- U * D^-1       (column blocks of U, for the backward solve)
//     the pair fold of both factors after the factorization (tc_pair_fold)
//
// Persistent, warp-specialised kernel over 128 x 128 tiles of A22 (or of any
// tile-aligned rectangle of it).  The complex product is four real TF32 MMAs
// into two TMEM accumulators:
//     Cr = Lr Ur^T - Li Ui^T        (the minus via the instruction's negate-A bit)
//     Ci = Lr Ui^T + Li Ur^T
//   warp 0      TMA producer: L21 (K-major, ld = 128) and U12^T (K-major) tiles,
//               128-byte swizzle, three-stage mbarrier ring over the 128-deep
//               contraction (four 32-wide k-blocks per tile, continuing across tiles)
//   warp 1      tcgen05.mma issuer; two TMEM accumulator buffers (Cr | Ci, 256
//               columns each), so the epilogue of tile i overlaps the MMAs of i+1
//   warps 2-5   epilogue: tcgen05.ld of a 32-row x 32-column slice into a swizzled
//               shared-memory box, then either a TMA reduce-add of -acc into A22
//               (cp.reduce.async.bulk.tensor ... .add: C is never loaded by the SM)
//               or TMA stores of +acc into two destinations (the W21 product).
// Every mbarrier wait has an iteration limit; on expiry the CTA sets
// FLAG_TIMEOUT, stops issuing work, drains its bulk copies, frees TMEM and exits.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include "bem_internal.h"
#include "tc_ptx.cuh"

namespace bem {

namespace {

using namespace tcp;

constexpr int BM = 128, BN = 128, BK = 32, STAGES = 3, KB = 128 / BK;
constexpr int L_TILE = BM * BK * 4;                     // 16 KB
constexpr int U_TILE = BN * BK * 4;                     // 16 KB
constexpr int STAGE_BYTES = 2 * L_TILE + 2 * U_TILE;    // 64 KB
constexpr int EPI_WARPS = 4;
constexpr int SLOT_BYTES = 32 * 32 * 4;                 // one 32 x 32 FP32 box
constexpr int EPI_BYTES = EPI_WARPS * 2 * SLOT_BYTES;   // 32 KB
constexpr int BAR_BYTES = 256;
constexpr int SMEM_BYTES = 1024 + STAGES * STAGE_BYTES + EPI_BYTES + BAR_BYTES;
constexpr int NTHREADS = 64 + 32 * EPI_WARPS;
constexpr uint32_t TMEM_COLS = 512;                     // 2 buffers x (Cr 128 | Ci 128)



__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}
// global[box at (x, y)] += shared box (element-wise FP32 add performed by the TMA unit)
__device__ __forceinline__ void tma_reduce_add_2d(const CUtensorMap* map, int x, int y, uint32_t src) {
    asm volatile("cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];"
                 ::"l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(src)
                 : "memory");
}
__device__ __forceinline__ void prefetch_map(const CUtensorMap* m) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(m)) : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, uint32_t src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];"
                 ::"l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(src)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }


// Instruction descriptor: kind::tf32, D = F32, A = B = TF32, K-major, M = 128, N = 128.
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



}  // namespace

// Tile rectangle and destination of one k_tc_update launch.
struct TcTiles {
    int lr0, ur0, Mt, Nt, lw, lskip, crow0, ccol0, mode, c2row0, c2col0;
    int npair, lr0b, ur0b;  // second operand pair (npair = 2): L rows from lr0b, U rows from ur0b
    int fold, nblk;         // pair fold of the triangular factors (1: L, 2: U; nblk 128-blocks)
};

// Tiles (tm, tn), tm < Mt, tn < Nt, of the rectangle whose L rows start at lr0
// (rows of mapLr / mapLi) and U rows at ur0 (rows of mapUr / mapUi); lw > 0 keeps
// only the L of width lw (tile columns < lw, then tile rows < lw), without its first
// lskip tiles.  With npair = 2 the product also sums the second pair of operands
// (mapL2*, rows from lr0b; mapU2*, rows from ur0b): K = 256, two elimination steps
// applied in one pass over C.  mode 0: the tile's -acc is reduce-added into
// mapCr / mapCi at rows crow0 + tm*128, columns ccol0 + tn*128.  mode 1: +acc is
// stored there and at c2row0 + tm*128, c2col0 + tn*128 of mapC2r / mapC2i.  mode 2:
// +acc is stored there, rounded to TF32 (nearest).  fold = 1 / 2 (pair fold, Mt tiles
// in all, Nt = 1): tile t is tile m of pair p, p = 0, 1, .. in turn:
//   fold 1 (m < nblk - 2p - 2): C = block (2p+2+m, 2p), L operand = block (2p+2+m, 2p+1)
//   fold 2 (m < 2p):            C = block (m, 2p+1),   L operand = block (m, 2p)
// of the matrix behind mapLr / mapLi / mapCr / mapCi, U operand = rows 128 p of mapUr /
// mapUi; mode 0 (C -= L_op * U_op).
__global__ void __launch_bounds__(NTHREADS, 1)
    k_tc_update(const __grid_constant__ CUtensorMap mapLr, const __grid_constant__ CUtensorMap mapLi,
                const __grid_constant__ CUtensorMap mapUr, const __grid_constant__ CUtensorMap mapUi,
                const __grid_constant__ CUtensorMap mapCr, const __grid_constant__ CUtensorMap mapCi,
                const __grid_constant__ CUtensorMap mapC2r, const __grid_constant__ CUtensorMap mapC2i,
                const __grid_constant__ CUtensorMap mapL2r, const __grid_constant__ CUtensorMap mapL2i,
                const __grid_constant__ CUtensorMap mapU2r, const __grid_constant__ CUtensorMap mapU2i,
                const TcTiles a, int* gflags) {
    // a kernel launched after this one as its programmatic dependent (the block inverse after
    // the corner update) may be scheduled now; it waits for this grid's completion itself
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;  // 1024-byte aligned (128-byte swizzle atoms)
    unsigned char* gbase = smem_raw + (base - raw);
    const uint32_t epi_base = base + STAGES * STAGE_BYTES;
    uint64_t* bars = reinterpret_cast<uint64_t*>(gbase + STAGES * STAGE_BYTES + EPI_BYTES);
    // bars: full[3] | empty[3] | tfull[2] | tempty[2] | TMEM address | abort flag
    volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(bars + 10);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 11);
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + 3);
    const uint32_t tfull0 = smem_u32(bars + 6), tempty0 = smem_u32(bars + 8);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // rectangle: Mt x Nt tiles; an L of width lw: tile columns < lw (Mt lw tiles), then
    // tile rows < lw right of them (lw (Nt - lw) tiles), the first lskip tiles dropped
    const int Mt = a.Mt, Nt = a.Nt, lw = a.lw;
    const int ncol = Mt * lw, nrow = lw * max(Nt - lw, 0);
    const int ntiles = lw ? ncol + nrow - a.lskip : Mt * Nt;
    auto tile_of = [&](int t, int& tm, int& tn) {
        if (lw) {
            t += a.lskip;
            if (t < ncol) {
                tm = t / lw; tn = t % lw;
            } else {
                t -= ncol;
                tm = t / (Nt - lw); tn = lw + t % (Nt - lw);
            }
        } else {
            tm = t / Nt; tn = t % Nt;
        }
    };
    const int KBT = KB * a.npair;
    // tile t -> first rows of its L and U operands, the L operand's first column, and C
    auto place = [&](int t, int& lrow, int& lx, int& urow, int& crow, int& ccol) {
        if (a.fold) {
            int p = 0;
            for (;; ++p) {
                const int c = a.fold == 1 ? a.nblk - 2 * p - 2 : 2 * p;
                if (t < c) break;
                t -= c;
            }
            crow = (a.fold == 1 ? 2 * p + 2 + t : t) * BM;
            ccol = (a.fold == 1 ? 2 * p : 2 * p + 1) * BN;
            lrow = crow;
            lx = (a.fold == 1 ? 2 * p + 1 : 2 * p) * BN;
            urow = p * BN;
        } else {
            int tm, tn;
            tile_of(t, tm, tn);
            lrow = a.lr0 + tm * BM;
            lx = 0;
            urow = a.ur0 + tn * BN;
            crow = a.crow0 + tm * BM;
            ccol = a.ccol0 + tn * BN;
        }
    };

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) { mbar_init(full0 + 8 * s, 1); mbar_init(empty0 + 8 * s, 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(tfull0 + 8 * b, 1); mbar_init(tempty0 + 8 * b, EPI_WARPS); }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        prefetch_map(&mapLr); prefetch_map(&mapLi); prefetch_map(&mapUr); prefetch_map(&mapUi);
        prefetch_map(&mapCr); prefetch_map(&mapCi);
        if (a.mode == 1) { prefetch_map(&mapC2r); prefetch_map(&mapC2i); }
        if (a.npair == 2) { prefetch_map(&mapL2r); prefetch_map(&mapL2i); prefetch_map(&mapU2r); prefetch_map(&mapU2i); }
    }
    __syncwarp();
    // launched as a programmatic dependent (the first W21 tile after the block inverse): the
    // set-up above overlaps the inverse; the TMEM allocation and every read of its results
    // come after this wait, so a waiting CTA holds no tensor memory (a no-op for an
    // ordinary launch)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32((void*)tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // TMA producer
            uint32_t it = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                int lrow1, lx, urow1, crow, ccol;
                place(t, lrow1, lx, urow1, crow, ccol);
                for (int kb = 0; kb < KBT; ++kb, ++it) {
                    const uint32_t s = it % STAGES, u = it / STAGES;
                    if (u > 0 && !mbar_wait(empty0 + 8 * s, (u - 1) & 1, abort_flag, gflags)) { ok = false; break; }
                    const uint32_t st = base + s * STAGE_BYTES;
                    const bool second = kb >= KB;
                    const int x = (second ? kb - KB : kb) * BK;
                    // the second operand pair sits at the same tile offsets from lr0b / ur0b
                    const int lrow = second ? lrow1 - a.lr0 + a.lr0b : lrow1;
                    const int urow = second ? urow1 - a.ur0 + a.ur0b : urow1;
                    mbar_expect_tx(full0 + 8 * s, STAGE_BYTES);
                    tma_load_2d(st, second ? &mapL2r : &mapLr, lx + x, lrow, full0 + 8 * s);
                    tma_load_2d(st + L_TILE, second ? &mapL2i : &mapLi, lx + x, lrow, full0 + 8 * s);
                    tma_load_2d(st + 2 * L_TILE, second ? &mapU2r : &mapUr, x, urow, full0 + 8 * s);
                    tma_load_2d(st + 2 * L_TILE + U_TILE, second ? &mapU2i : &mapUi, x, urow, full0 + 8 * s);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer
            const uint32_t id_pos = idesc_tf32(false), id_neg = idesc_tf32(true);
            uint32_t it = 0, local = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++local) {
                const uint32_t buf = local & 1, u = local >> 1;
                if (u > 0 && !mbar_wait(tempty0 + 8 * buf, (u - 1) & 1, abort_flag, gflags)) { ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t accR = tmem + buf * 256, accI = accR + 128;
                for (int kb = 0; kb < KBT; ++kb, ++it) {
                    const uint32_t s = it % STAGES, su = it / STAGES;
                    if (!mbar_wait(full0 + 8 * s, su & 1, abort_flag, gflags)) { ok = false; break; }
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
                if (ok) mma_commit(tfull0 + 8 * buf);
            }
        }
    } else {
        // Epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 = tile rows q*32 + lane.
        const int q = warp & 3;
        const uint32_t lane_base = (uint32_t)(q * 32) << 16;
        const uint32_t slot0 = epi_base + (uint32_t)(warp - 2) * 2 * SLOT_BYTES;
        uint32_t local = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++local) {
            int lrow1, lx, urow1, crow, ccol;
            place(t, lrow1, lx, urow1, crow, ccol);
            const uint32_t buf = local & 1, u = local >> 1;
            bool have = mbar_wait(tfull0 + 8 * buf, u & 1, abort_flag, gflags);
            if (!__all_sync(0xffffffffu, have)) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int row = crow + q * 32, row2 = a.c2row0 + (crow - a.crow0) + q * 32;
            const float sgn = a.mode ? 1.f : -1.f;
#pragma unroll 1
            for (int c = 0; c < BN / 32; ++c) {
#pragma unroll 1
                for (int p = 0; p < 2; ++p) {
                    float v[32];
                    tmem_ld32(tmem + lane_base + buf * 256 + p * 128 + c * 32, v);
                    const uint32_t slot = slot0 + p * SLOT_BYTES;
                    if (lane == 0) bulk_wait_read1();  // the previous box from this slot has been read
                    __syncwarp();
                    const uint32_t rowaddr = slot + lane * 128;
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const uint32_t sa = rowaddr + ((uint32_t)(j ^ (lane & 7)) << 4);
                        float o0 = sgn * v[4 * j], o1 = sgn * v[4 * j + 1], o2 = sgn * v[4 * j + 2],
                              o3 = sgn * v[4 * j + 3];
                        if (a.mode) {  // W21 is the L operand of later updates, U D^-1 of the pair fold:
                                       // round it once, to nearest
                            o0 = tf32_rn(o0); o1 = tf32_rn(o1); o2 = tf32_rn(o2); o3 = tf32_rn(o3);
                        }
                        asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(sa), "f"(o0), "f"(o1),
                                     "f"(o2), "f"(o3)
                                     : "memory");
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) {
                        const int col = ccol + c * 32;
                        if (a.mode) {
                            tma_store_2d(p ? &mapCi : &mapCr, col, row, slot);
                            if (a.mode == 1)
                                tma_store_2d(p ? &mapC2i : &mapC2r, a.c2col0 + (ccol - a.ccol0) + c * 32, row2, slot);
                        } else {
                            tma_reduce_add_2d(p ? &mapCi : &mapCr, col, row, slot);
                        }
                        bulk_commit();
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty0 + 8 * buf);
        }
        if (lane == 0) bulk_wait_all();
        __syncwarp();
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        __syncwarp();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn get_encode() {
    static const EncodeTiledFn fn = [] {  // resolved once, thread-safe
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<EncodeTiledFn>(p);
        return (EncodeTiledFn) nullptr;
    }();
    return fn;
}

// FP32 operand of rows x cols columns (row stride ld floats), 32-column x
// box_rows boxes, 128-byte swizzle: one plane of an L or U operand.
static bool make_map(CUtensorMap* m, const float* base, int rows, int ld, int box_rows, int cols = 128) {
    EncodeTiledFn enc = get_encode();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
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

// FP32 matrix of rows x cols (row stride ld floats), 32 x 32 boxes, 128-byte swizzle:
// the target of the epilogue's TMA reduce-add or store.
static bool make_map_c(CUtensorMap* m, const float* base, int rows, int cols, int ld) {
    EncodeTiledFn enc = get_encode();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
    cuuint32_t box[2] = {32, 32};
    cuuint32_t estr[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static int tc_grid(int ntiles, int max_ctas) {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(k_tc_update, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (max_ctas < 0) return (ntiles + (-max_ctas) - 1) / (-max_ctas);
    int grid = ntiles;
    if (max_ctas > 0 && grid > max_ctas) grid = max_ctas;
    return grid > nsm ? nsm : grid;
}

// Tile rectangle of the step-k0 update (nb = 128): L21 rows [lr0, lr0 + 128 Mt) of
// wl, U12^T rows [ur0, ur0 + 128 Nt) of wut, landing at A[k0+128+lr0.., k0+128+ur0..].
// wl = [2][n][128] (L21 rows from 0), wut = [2][n][128] (U12^T rows from 0).
// max_ctas > 0 caps the persistent grid at that many CTAs; max_ctas < 0 launches
// ceil(tiles / -max_ctas) CTAs of about -max_ctas tiles each, so CTAs retire
// while the update runs and a higher-priority stream can take the freed SMs.
// lshape 1: only tile column 0 (Mt tiles) and tile row 0 (Nt tiles) of the rectangle;
// lshape 2: the same without the corner tile (0, 0).
bool tc_update_rect(cudaStream_t st, int n, int k0, CMat<float> A, const float* wl, const float* wut, int lr0,
                    int ur0, int Mt, int Nt, int max_ctas, int* flags, int lshape) {
    if (Mt <= 0 || Nt <= 0) return true;
    if (n % 128 || k0 % 128 || lr0 % 128 || ur0 % 128 || A.ld % 4) return false;
    if (k0 + 128 + lr0 + 128 * Mt > n || k0 + 128 + ur0 + 128 * Nt > n) return false;
    CUtensorMap mLr, mLi, mUr, mUi, mCr, mCi;
    const size_t plane = (size_t)n * 128;
    if (!make_map(&mLr, wl, n, 128, BM) || !make_map(&mLi, wl + plane, n, 128, BM) ||
        !make_map(&mUr, wut, n, 128, BN) || !make_map(&mUi, wut + plane, n, 128, BN) ||
        !make_map_c(&mCr, A.re, n, n, A.ld) || !make_map_c(&mCi, A.im, n, n, A.ld))
        return false;
    const int ntiles = lshape ? Mt + Nt - lshape : Mt * Nt;
    if (ntiles <= 0) return true;
    const TcTiles a{lr0, ur0, Mt, Nt, lshape ? 1 : 0, lshape == 2 ? 1 : 0, k0 + 128 + lr0, k0 + 128 + ur0, 0, 0, 0,
                    1, 0, 0};
    BEM_LAUNCH(k_tc_update<<<tc_grid(ntiles, max_ctas), NTHREADS, SMEM_BYTES, st>>>(
        mLr, mLi, mUr, mUi, mCr, mCi, mCr, mCi, mLr, mLi, mUr, mUi, a, flags));
    return true;
}

// W21 = A21 D^-1 for the block column at k0 (nb = 128, rem = n - k0 - 128 rows):
// A21 is read in place from A, D^-1 as its transpose dT ([2][128][128], row j =
// column j of D^-1); the product is stored into w ([2][n][128], rows from 0)
// and over A21 in A.  Each tile reads its A21 rows before it overwrites them.
// Row tiles t0 .. t0 + count - 1 of A21 (count < 0: all from t0).
bool tc_w21(cudaStream_t st, int n, int k0, CMat<float> A, const float* dT, float* w, int* flags, int t0,
            int count, int pdl) {
    const int rem = n - k0 - 128;
    if (rem <= 0) return true;
    if (n % 128 || k0 % 128 || A.ld % 4) return false;
    CUtensorMap mLr, mLi, mUr, mUi, mCr, mCi, mC2r, mC2i;
    const size_t plane = (size_t)n * 128;
    if (!make_map(&mLr, A.re + k0, n, A.ld, BM) || !make_map(&mLi, A.im + k0, n, A.ld, BM) ||
        !make_map(&mUr, dT, 128, 128, BN) || !make_map(&mUi, dT + 128 * 128, 128, 128, BN) ||
        !make_map_c(&mCr, w, n, 128, 128) || !make_map_c(&mCi, w + plane, n, 128, 128) ||
        !make_map_c(&mC2r, A.re, n, n, A.ld) || !make_map_c(&mC2i, A.im, n, n, A.ld))
        return false;
    const int mt = std::min(rem / 128 - t0, count < 0 ? rem / 128 : count);
    if (t0 < 0 || mt <= 0) return true;
    const TcTiles a{k0 + 128 + 128 * t0, 0, mt, 1, 0, 0, 128 * t0, 0, 1, k0 + 128 + 128 * t0, k0, 1, 0, 0};
    if (pdl) {
        // a programmatic dependent of the kernel before it on this stream (the block inverse)
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(tc_grid(mt, 0));
        cfg.blockDim = dim3(NTHREADS);
        cfg.dynamicSmemBytes = SMEM_BYTES;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        BEM_LAUNCH(cudaLaunchKernelEx(&cfg, k_tc_update, mLr, mLi, mUr, mUi, mCr, mCi, mC2r, mC2i, mLr, mLi, mUr,
                                      mUi, a, flags));
        return cudaPeekAtLastError() == cudaSuccess;
    }
    BEM_LAUNCH(k_tc_update<<<tc_grid(mt, 0), NTHREADS, SMEM_BYTES, st>>>(mLr, mLi, mUr, mUi, mCr, mCi, mC2r, mC2i,
                                                                        mLr, mLi, mUr, mUi, a, flags));
    return true;
}

// U_{0:c, c} <- U_{0:c, c} D_cc^-1 in place for the column block at c0 (c0 / 128 row
// tiles above the diagonal), dT = D_cc^-1 transposed ([2][128][128]).  Each tile reads
// its rows before it overwrites them.
bool tc_ucol(cudaStream_t st, int n, int c0, CMat<float> A, const float* dT, int max_ctas, int* flags) {
    if (c0 <= 0) return true;
    if (n % 128 || c0 % 128 || A.ld % 4) return false;
    CUtensorMap mLr, mLi, mUr, mUi, mCr, mCi;
    if (!make_map(&mLr, A.re + c0, n, A.ld, BM) || !make_map(&mLi, A.im + c0, n, A.ld, BM) ||
        !make_map(&mUr, dT, 128, 128, BN) || !make_map(&mUi, dT + 128 * 128, 128, 128, BN) ||
        !make_map_c(&mCr, A.re, n, n, A.ld) || !make_map_c(&mCi, A.im, n, n, A.ld))
        return false;
    const int mt = c0 / 128;
    const TcTiles a{0, 0, mt, 1, 0, 0, 0, c0, 2, 0, 0, 1, 0, 0};
    BEM_LAUNCH(k_tc_update<<<tc_grid(mt, max_ctas), NTHREADS, SMEM_BYTES, st>>>(
        mLr, mLi, mUr, mUi, mCr, mCi, mCr, mCi, mLr, mLi, mUr, mUi, a, flags));
    return true;
}

// C -= W_a U_a [+ W_b U_b] over tiles of the Mt x Nt block rectangle whose first element
// is A[row0][col0] (both multiples of 128): W_a rows (of wl_a, [2][n][128]) start at
// lr_a for the rectangle's first row, U_a^T rows (of wut_a) at ur_a for its first
// column, and likewise for the optional second step b (wl_b != nullptr: K = 256, both
// steps applied in one pass over C).  lw > 0: only the L of width lw, first lskip tiles
// dropped (see k_tc_update).
bool tc_update_pair(cudaStream_t st, int n, CMat<float> A, int row0, int col0, int Mt, int Nt, int lw, int lskip,
                    int max_ctas, int* flags, const float* wl_a, const float* wut_a, int lr_a, int ur_a,
                    const float* wl_b, const float* wut_b, int lr_b, int ur_b) {
    if (Mt <= 0 || Nt <= 0) return true;
    if (n % 128 || row0 % 128 || col0 % 128 || lr_a % 128 || ur_a % 128 || A.ld % 4) return false;
    if (row0 + 128 * Mt > n || col0 + 128 * Nt > n || lr_a < 0 || ur_a < 0) return false;
    if (lr_a + 128 * Mt > n || ur_a + 128 * Nt > n) return false;
    if (wl_b && (lr_b % 128 || ur_b % 128 || lr_b < 0 || ur_b < 0 || lr_b + 128 * Mt > n || ur_b + 128 * Nt > n))
        return false;
    const int ntiles = lw ? Mt * lw + lw * std::max(Nt - lw, 0) - lskip : Mt * Nt;
    if (ntiles <= 0) return true;
    CUtensorMap mLr, mLi, mUr, mUi, mCr, mCi, mL2r, mL2i, mU2r, mU2i;
    const size_t plane = (size_t)n * 128;
    if (!make_map(&mLr, wl_a, n, 128, BM) || !make_map(&mLi, wl_a + plane, n, 128, BM) ||
        !make_map(&mUr, wut_a, n, 128, BN) || !make_map(&mUi, wut_a + plane, n, 128, BN) ||
        !make_map_c(&mCr, A.re, n, n, A.ld) || !make_map_c(&mCi, A.im, n, n, A.ld))
        return false;
    const int npair = wl_b ? 2 : 1;
    if (wl_b) {
        if (!make_map(&mL2r, wl_b, n, 128, BM) || !make_map(&mL2i, wl_b + plane, n, 128, BM) ||
            !make_map(&mU2r, wut_b, n, 128, BN) || !make_map(&mU2i, wut_b + plane, n, 128, BN))
            return false;
    } else {
        mL2r = mLr; mL2i = mLi; mU2r = mUr; mU2i = mUi;
    }
    const TcTiles a{lr_a, ur_a, Mt, Nt, lw, lskip, row0, col0, 0, 0, 0, npair, lr_b, ur_b};
    BEM_LAUNCH(k_tc_update<<<tc_grid(ntiles, max_ctas), NTHREADS, SMEM_BYTES, st>>>(
        mLr, mLi, mUr, mUi, mCr, mCi, mCr, mCi, mL2r, mL2i, mU2r, mU2i, a, flags));
    return true;
}

// Pair fold of the block-unit triangular factors left in A by the LU (which = 1: the
// block-lower L, which = 2: the block-upper U D^-1), over the pairs of 128-blocks
// (2p, 2p+1):
//   which 1:  L_{r,2p}   -= L_{r,2p+1} L_{2p+1,2p}     block rows r >= 2p + 2
//   which 2:  U_{r,2p+1} -= U_{r,2p}   U_{2p,2p+1}     block rows r <  2p
// T: the transposed pair blocks, [2 planes][np][128][128] (T[p][j][i] = L_{2p+1,2p}[i][j],
// resp. U_{2p,2p+1}[i][j]).  Each launch reads only blocks it does not write.
bool tc_pair_fold(cudaStream_t st, int n, CMat<float> A, const float* T, int which, int* flags) {
    if (n % 128 || A.ld % 4 || (which != 1 && which != 2)) return false;
    const int nblk = n / 128, np = nblk / 2;
    long long ntiles = 0;
    for (int p = 0; p < np; ++p) ntiles += which == 1 ? nblk - 2 * p - 2 : 2 * p;
    if (ntiles <= 0) return true;
    if (ntiles > (1LL << 30)) return false;
    CUtensorMap mLr, mLi, mUr, mUi, mCr, mCi;
    const size_t plane = (size_t)np * 128 * 128;
    if (!make_map(&mLr, A.re, n, A.ld, BM, n) || !make_map(&mLi, A.im, n, A.ld, BM, n) ||
        !make_map(&mUr, T, np * 128, 128, BN) || !make_map(&mUi, T + plane, np * 128, 128, BN) ||
        !make_map_c(&mCr, A.re, n, n, A.ld) || !make_map_c(&mCi, A.im, n, n, A.ld))
        return false;
    const TcTiles a{0, 0, (int)ntiles, 1, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, which, nblk};
    BEM_LAUNCH(k_tc_update<<<tc_grid((int)ntiles, 0), NTHREADS, SMEM_BYTES, st>>>(
        mLr, mLi, mUr, mUi, mCr, mCi, mCr, mCi, mLr, mLi, mUr, mUi, a, flags));
    return true;
}

// A22 -= L21 U12 over the whole trailing matrix of step k0.
bool tc_trailing_update(cudaStream_t st, int n, int k0, int nb, CMat<float> A, const float* wl, const float* wut,
                        int* flags) {
    const int rem = n - k0 - nb;
    if (rem <= 0) return true;
    if (nb != 128) return false;
    return tc_update_rect(st, n, k0, A, wl, wut, 0, 0, rem / 128, rem / 128, 0, flags, 0);
}

// ---------------------------------------------------------------------------
// Probe of k_tc_update in one tile mode on caller data (bem_tc_probe): every
// operand and the destination are copied to the device, the product runs once,
// and the destination (and for the W21 mode its second destination) comes back.
int tc_probe(int device, int mode, int n, float* C, const float* Wa, const float* Ua, const float* Wb,
             const float* Ub, const float* T, float* Wout, char* err, int err_len) {
    auto fail = [&](const char* m) {
        snprintf(err, err_len, "%s", m);
        return -1;
    };
    if (mode < 0 || mode > 6) return fail("mode outside 0..6");
    if (n < 512 || n % 256 != 0 || n > 8192) return fail("n must be a multiple of 256 in [512, 8192]");
    if (!C) return fail("null destination");
    const bool pair_op = mode <= 2;
    if (pair_op && (!Wa || !Ua || (mode >= 1 && (!Wb || !Ub)))) return fail("null operand");
    if (!pair_op && !T) return fail("null operand");
    if (mode == 3 && !Wout) return fail("null second destination");
    if (cudaSetDevice(device) != cudaSuccess || !tc_gemm_supported(device)) return fail("no sm_103 device");
    const size_t nn = (size_t)n * n, nw = (size_t)2 * n * 128;
    const size_t nt = mode >= 5 ? (size_t)2 * (n / 256) * 128 * 128 : (size_t)2 * 128 * 128;
    float *dC = nullptr, *dWa = nullptr, *dUa = nullptr, *dWb = nullptr, *dUb = nullptr, *dT = nullptr,
          *dW = nullptr;
    int* flags = nullptr;
    int rc = 0;
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaMalloc(&dC, 2 * nn * 4) ||
        cudaMalloc(&dWa, nw * 4) || cudaMalloc(&dUa, nw * 4) || cudaMalloc(&dWb, nw * 4) ||
        cudaMalloc(&dUb, nw * 4) || cudaMalloc(&dT, nt * 4) || cudaMalloc(&dW, nw * 4) || cudaMalloc(&flags, 4)) {
        rc = fail("device allocation failed");
    } else {
        cudaMemcpy(dC, C, 2 * nn * 4, cudaMemcpyHostToDevice);
        if (pair_op) {
            cudaMemcpy(dWa, Wa, nw * 4, cudaMemcpyHostToDevice);
            cudaMemcpy(dUa, Ua, nw * 4, cudaMemcpyHostToDevice);
            if (mode >= 1) {
                cudaMemcpy(dWb, Wb, nw * 4, cudaMemcpyHostToDevice);
                cudaMemcpy(dUb, Ub, nw * 4, cudaMemcpyHostToDevice);
            }
        } else {
            cudaMemcpy(dT, T, nt * 4, cudaMemcpyHostToDevice);
        }
        cudaMemset(dW, 0, nw * 4);
        cudaMemset(flags, 0, 4);
        CMat<float> A{dC, dC + nn, n};
        const int mt = n / 128 - 1;
        bool ok = false;
        switch (mode) {
            case 0: ok = tc_update_pair(st, n, A, 128, 128, mt, mt, 0, 0, 0, flags, dWa, dUa, 0, 0, nullptr, nullptr, 0, 0); break;
            case 1: ok = tc_update_pair(st, n, A, 128, 128, mt, mt, 0, 0, 0, flags, dWa, dUa, 0, 0, dWb, dUb, 0, 0); break;
            case 2: ok = tc_update_pair(st, n, A, 128, 128, mt, mt, 2, 1, 0, flags, dWa, dUa, 0, 0, dWb, dUb, 0, 0); break;
            case 3: ok = tc_w21(st, n, 0, A, dT, dW, flags, 0, -1, 0); break;
            case 4: ok = tc_ucol(st, n, n - 128, A, dT, 0, flags); break;
            default: ok = tc_pair_fold(st, n, A, dT, mode - 4, flags); break;
        }
        int hf = 0;
        cudaError_t e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = cudaMemcpy(&hf, flags, 4, cudaMemcpyDeviceToHost);
        if (!ok) rc = fail("tensor map or launch set-up failed");
        else if (e != cudaSuccess) rc = fail(cudaGetErrorString(e));
        else if (hf & FLAG_TIMEOUT) rc = fail("a device-side wait expired");
        else {
            cudaMemcpy(C, dC, 2 * nn * 4, cudaMemcpyDeviceToHost);
            if (mode == 3) cudaMemcpy(Wout, dW, nw * 4, cudaMemcpyDeviceToHost);
        }
    }
    cudaGetLastError();
    cudaFree(dC); cudaFree(dWa); cudaFree(dUa); cudaFree(dWb); cudaFree(dUb); cudaFree(dT); cudaFree(dW);
    cudaFree(flags);
    if (st) cudaStreamDestroy(st);
    return rc;
}

}  // namespace bem
