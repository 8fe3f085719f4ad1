// k_lu.cu -- blocked complex LU, triangular solves and the FP64 residual.
//
// Replaces Eigen::PartialPivLU<CMatrix> (Hydrodynamic_Solver.cpp:430, 438, 446).
// The BIE matrix D = (1/2) I + K has |D_kk| >= |D_ik| at every elimination step
// on the meshes this solver targets, so partial pivoting never exchanges rows;
// the factorization here performs no exchanges and flags FLAG_PIVOT whenever a
// multiplier has |l_ik| > 1 (+1e-6), i.e. whenever partial pivoting *would*
// have exchanged rows.  With no flag raised, L and U are those of partial
// pivoting with the identity permutation.
//
// Step k0 (block width nb), block LU:
//   k_gj_inv       one CTA inverts the diagonal block D11 (Gauss-Jordan, shared memory)
//   k_cgemm        W21 = A21 D11^-1 (into a workspace), k_copy_back stores it in place
//   k_cgemm / tc   A22 -= W21 A12 (SIMT complex GEMM; tcgen05 TF32 in k_tc_gemm.cu)
// Solves (k_trsv_coop) use the stored off-diagonal blocks and the diagonal-block inverses.
#include "bem_internal.h"
#include <cstdio>
#include <cstring>
#include <algorithm>

namespace bem {

bool tc_trailing_update(cudaStream_t st, int n, int k0, int nb, CMat<float> A, const float* wl, const float* wut,
                        int* flags);
bool tc_update_rect(cudaStream_t st, int n, int k0, CMat<float> A, const float* wl, const float* wut, int lr0,
                    int ur0, int Mt, int Nt, int max_ctas, int* flags, int lshape);
bool tc_w21(cudaStream_t st, int n, int k0, CMat<float> A, const float* dT, float* w, int* flags, int t0,
            int count, int pdl = 0);
bool tc_ucol(cudaStream_t st, int n, int c0, CMat<float> A, const float* dT, int max_ctas, int* flags);
bool tc_pair_fold(cudaStream_t st, int n, CMat<float> A, const float* T, int which, int* flags);
bool tc_update_pair(cudaStream_t st, int n, CMat<float> A, int row0, int col0, int Mt, int Nt, int lw, int lskip,
                    int max_ctas, int* flags, const float* wl_a, const float* wut_a, int lr_a, int ur_a,
                    const float* wl_b, const float* wut_b, int lr_b, int ur_b);

template <typename T> __device__ __forceinline__ bool finite_(T x) { return isfinite(x); }

// ---------------------------------------------------------------------------
// In-place Gauss-Jordan inverse of the nb x nb diagonal block (the current Schur
// complement block), no row exchanges; written to inv[blk].  1024 threads hold
// the block in registers, thread (ty, tx) owning rows ty + 32 a and columns
// tx + 32 b; per pivot, the owners publish row k and column k through shared
// memory (double-buffered, one barrier per pivot) and every thread updates its
// own elements.  Multipliers |a_ik / a_kk| > 1 below the pivot raise FLAG_PIVOT
// (partial pivoting would have exchanged rows inside the block); a zero or
// non-finite pivot raises FLAG_ZERO_PIVOT.
template <typename T, int NB>
__global__ void __launch_bounds__(1024) k_gj_inv(int k0, CMat<T> A, T* invr, T* invi, int* flags) {
    constexpr int G = NB / 32;  // row / column groups per thread
    __shared__ T rowr[2][NB], rowi[2][NB], colr[2][NB], coli[2][NB];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const size_t ld = A.ld;
    T vr[G][G], vi[G][G];
#pragma unroll
    for (int a = 0; a < G; ++a)
#pragma unroll
        for (int b = 0; b < G; ++b) {
            size_t g = (size_t)(k0 + ty + 32 * a) * ld + k0 + tx + 32 * b;
            vr[a][b] = A.re[g];
            vi[a][b] = A.im[g];
        }
    int local_flags = 0;
    for (int k = 0; k < NB; ++k) {
        const int buf = k & 1;
        const int ka = k >> 5, kt = k & 31;
        // publish row k (owners: ty == kt) and column k (owners: tx == kt)
        if (ty == kt) {
#pragma unroll
            for (int a = 0; a < G; ++a)
                if (a == ka) {
#pragma unroll
                    for (int b = 0; b < G; ++b) { rowr[buf][tx + 32 * b] = vr[a][b]; rowi[buf][tx + 32 * b] = vi[a][b]; }
                }
        }
        if (tx == kt) {
#pragma unroll
            for (int b = 0; b < G; ++b)
                if (b == ka) {
#pragma unroll
                    for (int a = 0; a < G; ++a) { colr[buf][ty + 32 * a] = vr[a][b]; coli[buf][ty + 32 * a] = vi[a][b]; }
                }
        }
        __syncthreads();
        const T pr = colr[buf][k], pi = coli[buf][k];
        const T den = pr * pr + pi * pi;
        if (threadIdx.x == 0 && (!(den > (T)0) || !isfinite(den))) local_flags |= FLAG_ZERO_PIVOT;
        const T qr = pr / den, qi = -pi / den;  // 1 / pivot
        // new row k: a_kj / p for j != k, 1/p at j == k
        T nr[G], ni[G];
#pragma unroll
        for (int b = 0; b < G; ++b) {
            const int j = tx + 32 * b;
            T xr = (j == k) ? (T)1 : rowr[buf][j], xi = (j == k) ? (T)0 : rowi[buf][j];
            nr[b] = xr * qr - xi * qi;
            ni[b] = xr * qi + xi * qr;
        }
#pragma unroll
        for (int a = 0; a < G; ++a) {
            const int i = ty + 32 * a;
            if (i == k) {
#pragma unroll
                for (int b = 0; b < G; ++b) { vr[a][b] = nr[b]; vi[a][b] = ni[b]; }
            } else {
                const T cr = colr[buf][i], ci = coli[buf][i];
                if (tx == kt && i > k) {
                    T lr = cr * qr - ci * qi, li = cr * qi + ci * qr;
                    if (lr * lr + li * li > (T)(1.000002)) local_flags |= FLAG_PIVOT;
                    if (lr * lr + li * li > (T)256) local_flags |= FLAG_GROWTH;
                }
#pragma unroll
                for (int b = 0; b < G; ++b) {
                    const int j = tx + 32 * b;
                    T ur = nr[b], ui = ni[b];
                    if (j == k) {
                        vr[a][b] = -(cr * ur - ci * ui);
                        vi[a][b] = -(cr * ui + ci * ur);
                    } else {
                        vr[a][b] -= cr * ur - ci * ui;
                        vi[a][b] -= cr * ui + ci * ur;
                    }
                }
            }
        }
    }
    const int blk = k0 / NB;
    T* Mr = invr + (size_t)blk * NB * NB;
    T* Mi = invi + (size_t)blk * NB * NB;
#pragma unroll
    for (int a = 0; a < G; ++a)
#pragma unroll
        for (int b = 0; b < G; ++b) {
            size_t o = (size_t)(ty + 32 * a) * NB + tx + 32 * b;
            Mr[o] = vr[a][b];
            Mi[o] = vi[a][b];
        }
    if (local_flags) atomicOr(flags, local_flags);
}

// ---------------------------------------------------------------------------
// 128 x 128 FP32 block inverse (the tensor-core LU's diagonal blocks), one CTA
// of 256 threads, Gauss-Jordan without row exchanges, block held in registers:
// thread (rg, cg) owns rows 8 rg .. 8 rg + 7 and columns 8 cg .. 8 cg + 7.
// Each pivot step is branch-free.  For pivot k with value p the owners of row k
// publish n_j = r_j / p, where r is the row with r_k replaced by p + 1, and the
// owners of column k publish c_i = a_ik with c_k replaced by p - 1; then
//     a_ij <- a_ij - c_i n_j
// is exactly the in-place Gauss-Jordan update for every (i, j): for j = k it
// gives -a_ik / p, for i = k it gives a_kj / p, and a_kk becomes 1 / p.  The
// p +- 1 substitution costs a factor ~max(1, |p|) in rounding on row and column
// k, irrelevant for a TF32 preconditioner.  The published row and column are
// stored chunk-major (16-byte chunk q of thread group g at [q][g]), so the
// per-pivot shared loads are free of bank conflicts; the pivot-row owners (one
// half-warp) compute 1/p once.  A zero or non-finite pivot raises
// FLAG_ZERO_PIVOT.  Multipliers are not checked here: this factorization only
// preconditions the FP64 refinement, which decides success.
constexpr int IV_THREADS = 256;

__global__ void __launch_bounds__(IV_THREADS, 1) k_inv128(int k0, CMat<float> A, float* invr, float* invi,
                                                          float* dT, int* flags) {
    __shared__ __align__(16) float4 nrow[2][4 * 16];  // [buffer][chunk q][column group]
    __shared__ __align__(16) float4 ccol[2][4 * 16];  // [buffer][chunk q][row group]
    const int t = threadIdx.x, cg = t & 15, rg = t >> 4, lane = t & 31;
    float2 v[8][8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const size_t g = (size_t)(k0 + 8 * rg + m) * A.ld + k0 + 8 * cg;
        const float4 r0 = *reinterpret_cast<const float4*>(A.re + g);
        const float4 r1 = *reinterpret_cast<const float4*>(A.re + g + 4);
        const float4 i0 = *reinterpret_cast<const float4*>(A.im + g);
        const float4 i1 = *reinterpret_cast<const float4*>(A.im + g + 4);
        v[m][0] = make_float2(r0.x, i0.x); v[m][1] = make_float2(r0.y, i0.y);
        v[m][2] = make_float2(r0.z, i0.z); v[m][3] = make_float2(r0.w, i0.w);
        v[m][4] = make_float2(r1.x, i1.x); v[m][5] = make_float2(r1.y, i1.y);
        v[m][6] = make_float2(r1.z, i1.z); v[m][7] = make_float2(r1.w, i1.w);
    }
    int lf = 0;
    // Publish pivot kp (row and column kp = 8 g + m1, g = kp >> 3) into buffer b.
    auto publish = [&](int kp, int m1, int b) {
        const int g = kp >> 3;
        if ((rg >> 1) == (g >> 1)) {  // the warp holding row kp
            const float2 pv = v[m1][m1];
            const int src = ((g & 1) << 4) | g;
            const float px = __shfl_sync(0xffffffffu, pv.x, src), py = __shfl_sync(0xffffffffu, pv.y, src);
            if (rg == g) {
                const float den = px * px + py * py;
                if (cg == g && (!(den > 0.f) || !isfinite(den))) lf |= FLAG_ZERO_PIVOT;
                const float rc = __frcp_rn(den), qr = px * rc, qi = -py * rc;
                float o[16];
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    float rx = v[m1][c].x, ry = v[m1][c].y;
                    if (c == m1 && cg == g) rx = px + 1.f;
                    o[2 * c] = rx * qr - ry * qi;
                    o[2 * c + 1] = rx * qi + ry * qr;
                }
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    nrow[b][q * 16 + cg] = make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
            }
        }
        if (cg == g) {
            float o[16];
#pragma unroll
            for (int m = 0; m < 8; ++m) {
                o[2 * m] = v[m][m1].x - ((m == m1 && rg == g) ? 1.f : 0.f);
                o[2 * m + 1] = v[m][m1].y;
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
                ccol[b][q * 16 + rg] = make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
        }
    };
    publish(0, 0, 0);
    __syncthreads();
#pragma unroll 1
    for (int kq = 0; kq < 16; ++kq) {
#pragma unroll
        for (int kr = 0; kr < 8; ++kr) {
            const int k = 8 * kq + kr, b = kr & 1;
            float2 n[8], cm[8];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float4 x = nrow[b][q * 16 + cg];
                n[2 * q] = make_float2(x.x, x.y);
                n[2 * q + 1] = make_float2(x.z, x.w);
                const float4 y = ccol[b][q * 16 + rg];
                cm[2 * q] = make_float2(y.x, y.y);
                cm[2 * q + 1] = make_float2(y.z, y.w);
            }
#pragma unroll
            for (int m = 0; m < 8; ++m)
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    v[m][c].x = fmaf(-cm[m].x, n[c].x, fmaf(cm[m].y, n[c].y, v[m][c].x));
                    v[m][c].y = fmaf(-cm[m].x, n[c].y, fmaf(-cm[m].y, n[c].x, v[m][c].y));
                }
            if (k < 127) publish(k + 1, (kr + 1) & 7, b ^ 1);
            __syncthreads();
        }
    }
    float* Or = invr + (size_t)(k0 / 128) * 128 * 128;
    float* Oi = invi + (size_t)(k0 / 128) * 128 * 128;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const size_t g = (size_t)(8 * rg + m) * 128 + 8 * cg;
        *reinterpret_cast<float4*>(Or + g) = make_float4(v[m][0].x, v[m][1].x, v[m][2].x, v[m][3].x);
        *reinterpret_cast<float4*>(Or + g + 4) = make_float4(v[m][4].x, v[m][5].x, v[m][6].x, v[m][7].x);
        *reinterpret_cast<float4*>(Oi + g) = make_float4(v[m][0].y, v[m][1].y, v[m][2].y, v[m][3].y);
        *reinterpret_cast<float4*>(Oi + g + 4) = make_float4(v[m][4].y, v[m][5].y, v[m][6].y, v[m][7].y);
    }
    if (dT) {  // the transpose, [2][128][128], TF32-rounded: the K-major B operand of W21 = A21 D^-1
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const size_t g = (size_t)(8 * cg + c) * 128 + 8 * rg;
            auto rn4 = [](float a, float b, float c_, float d) {
                return make_float4(tf32_rn(a), tf32_rn(b), tf32_rn(c_), tf32_rn(d));
            };
            *reinterpret_cast<float4*>(dT + g) = rn4(v[0][c].x, v[1][c].x, v[2][c].x, v[3][c].x);
            *reinterpret_cast<float4*>(dT + g + 4) = rn4(v[4][c].x, v[5][c].x, v[6][c].x, v[7][c].x);
            *reinterpret_cast<float4*>(dT + 16384 + g) = rn4(v[0][c].y, v[1][c].y, v[2][c].y, v[3][c].y);
            *reinterpret_cast<float4*>(dT + 16384 + g + 4) = rn4(v[4][c].y, v[5][c].y, v[6][c].y, v[7][c].y);
        }
    }
    if (lf) atomicOr(flags, lf);
}


// ---------------------------------------------------------------------------
// The same inverse on a cluster of CL CTAs (CL = 2, 4 or 8), split by rows: CTA q
// owns rows RPC q .. RPC q + RPC - 1 of the block (RPC = 128 / CL; thread (rg, cg):
// rows RPT rg .. RPT rg + RPT - 1 with RPT = RPC / 16, columns 8 cg .. 8 cg + 7), so
// each pivot costs each SM 1 / CL of the FMAs.  The pivot rows of RPC consecutive
// pivots belong to one CTA, which normalises them (the p + 1 substitution above) and
// writes each one both into its own shared memory and, by st.async, into every
// peer's, completing a per-pivot mbarrier there.  Every pivot row has its own 1 KB
// slot, so the owner never waits for the others; they follow one remote-store
// latency behind and the roles pass on every RPC pivots.  The column of each pivot
// is local to each CTA.  Waits on a peer give up at a 2 s deadline (FLAG_TIMEOUT);
// every CTA always reaches the final cluster barrier.  Launched with the cluster
// size as a launch attribute (inv128_cluster).
constexpr int IC_THREADS = 256;
constexpr int IC_SMEM = 128 * 64 * 16       // pivot rows [128][chunk q][column group] float4
                        + 2 * 32 * 16       // pivot-column values [buffer][row group][RPT <= 4] float2
                        + 128 * 8;          // one mbarrier per pivot row

__device__ __forceinline__ uint32_t ic_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t ic_peer_addr(uint32_t local, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}
__device__ __forceinline__ void ic_cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Bounded wait for a pivot row written by the peer (acquire at cluster scope).
__device__ __forceinline__ bool ic_wait(uint32_t bar, unsigned long long deadline) {
    for (int i = 0;; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], 0;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar)
            : "memory");
        if (done) return true;
        if ((i & 255) == 255) {  // a %globaltimer read costs far more than a poll
            unsigned long long t;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
            if (t > deadline) return false;
        }
    }
}

template <int CL>
__global__ void __launch_bounds__(IC_THREADS, 1)
    k_inv128c(int k0, CMat<float> A, float* invr, float* invi, float* dT, int* flags) {
    // launched as a programmatic dependent of the update that produced this block: wait
    // for its completion before reading A (returns at once for an ordinary launch); the
    // first W21 tile after it may be scheduled now and waits for this grid in turn
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    constexpr int RPC = 128 / CL, RPT = RPC / 16;
    static_assert(CL == 2 || CL == 4 || CL == 8, "cluster of 2, 4 or 8 CTAs");
    extern __shared__ __align__(16) float4 ic_smem[];
    float4* nrow = ic_smem;                                                   // [128][4 * 16]
    float2* ccol = reinterpret_cast<float2*>(nrow + 128 * 64);                // [2][16][RPT]
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(nrow + 128 * 64 + 2 * 32);  // [128]
    const uint32_t rank = ic_rank();
    const int t = threadIdx.x, cg = t & 15, rg = t >> 4;
    const uint32_t nrow_s = (uint32_t)__cvta_generic_to_shared(nrow);
    const uint32_t bars_s = (uint32_t)__cvta_generic_to_shared(bars);
    float2 v[RPT][8];
    const int row_base = RPC * (int)rank + RPT * rg;
#pragma unroll
    for (int m = 0; m < RPT; ++m) {
        const size_t g = (size_t)(k0 + row_base + m) * A.ld + k0 + 8 * cg;
        const float4 r0 = *reinterpret_cast<const float4*>(A.re + g);
        const float4 r1 = *reinterpret_cast<const float4*>(A.re + g + 4);
        const float4 i0 = *reinterpret_cast<const float4*>(A.im + g);
        const float4 i1 = *reinterpret_cast<const float4*>(A.im + g + 4);
        v[m][0] = make_float2(r0.x, i0.x); v[m][1] = make_float2(r0.y, i0.y);
        v[m][2] = make_float2(r0.z, i0.z); v[m][3] = make_float2(r0.w, i0.w);
        v[m][4] = make_float2(r1.x, i1.x); v[m][5] = make_float2(r1.y, i1.y);
        v[m][6] = make_float2(r1.z, i1.z); v[m][7] = make_float2(r1.w, i1.w);
    }
    if (t < 128) {
        // rows this CTA receives: one arrival now, completed by 1 KB of the owner's stores
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bars_s + 8 * t) : "memory");
        if (t / RPC != (int)rank)
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], 1024;" ::"r"(bars_s + 8 * t)
                         : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    ic_cluster_sync();
    unsigned long long deadline;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(deadline));
    deadline += 2000000000ull;
    int lf = 0;
    bool dead = false;
    // Publish pivot kp: m1 = its row inside an RPT-row tile, c1 = its column inside an 8-column tile.
    auto publish = [&](int kp, int m1, int c1, int b) {
        const int kl = kp % RPC, grow = kl / RPT, gcol = kp >> 3;
        const bool mine = kp / RPC == (int)rank;
        if (mine && (rg >> 1) == (grow >> 1)) {  // the warp holding row kp
            const float2 pv = v[m1][c1];
            const int src = ((grow & 1) << 4) | gcol;
            const float px = __shfl_sync(0xffffffffu, pv.x, src), py = __shfl_sync(0xffffffffu, pv.y, src);
            if (rg == grow) {
                const float den = px * px + py * py;
                if (cg == gcol && (!(den > 0.f) || !isfinite(den))) lf |= FLAG_ZERO_PIVOT;
                const float rc = __frcp_rn(den), qr = px * rc, qi = -py * rc;
                float o[16];
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    float rx = v[m1][c].x, ry = v[m1][c].y;
                    if (c == c1 && cg == gcol) rx = px + 1.f;
                    o[2 * c] = rx * qr - ry * qi;
                    o[2 * c + 1] = rx * qi + ry * qr;
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float4 w = make_float4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
                    const uint32_t off = (uint32_t)((kp * 64 + q * 16 + cg) * 16);
                    nrow[kp * 64 + q * 16 + cg] = w;
#pragma unroll
                    for (int p = 1; p < CL; ++p) {
                        const uint32_t peer = (rank + (uint32_t)p) % CL;
                        const uint32_t dst = ic_peer_addr(nrow_s + off, peer), bar = ic_peer_addr(bars_s + 8 * kp, peer);
                        asm volatile(
                            "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, "
                            "[%5];" ::"r"(dst), "f"(w.x), "f"(w.y), "f"(w.z), "f"(w.w), "r"(bar)
                            : "memory");
                    }
                }
            }
        }
        if (cg == gcol) {
#pragma unroll
            for (int m = 0; m < RPT; ++m)
                ccol[(b * 16 + rg) * RPT + m] =
                    make_float2(v[m][c1].x - ((mine && m == m1 && rg == grow) ? 1.f : 0.f), v[m][c1].y);
        }
    };
    // Thread 0 alone waits for a pivot row written by a peer; the CTA barrier that
    // follows orders every thread's reads of it after that acquire.
    auto await_row = [&](int kp) {
        if (t == 0 && kp / RPC != (int)rank && !dead && !ic_wait(bars_s + 8 * kp, deadline)) dead = true;
    };
    publish(0, 0, 0, 0);
    await_row(0);
    __syncthreads();
#pragma unroll 1
    for (int kq = 0; kq < 16; ++kq) {
#pragma unroll
        for (int kr = 0; kr < 8; ++kr) {
            const int k = 8 * kq + kr, b = kr & 1;
            float2 n[8], cm[RPT];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float4 x = nrow[k * 64 + q * 16 + cg];
                n[2 * q] = make_float2(x.x, x.y);
                n[2 * q + 1] = make_float2(x.z, x.w);
            }
#pragma unroll
            for (int m = 0; m < RPT; ++m) cm[m] = ccol[(b * 16 + rg) * RPT + m];
#pragma unroll
            for (int m = 0; m < RPT; ++m)
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    v[m][c].x = fmaf(-cm[m].x, n[c].x, fmaf(cm[m].y, n[c].y, v[m][c].x));
                    v[m][c].y = fmaf(-cm[m].x, n[c].y, fmaf(-cm[m].y, n[c].x, v[m][c].y));
                }
            if (k < 127) {
                publish(k + 1, (kr + 1) % RPT, (kr + 1) & 7, b ^ 1);
                await_row(k + 1);
            }
            __syncthreads();
        }
    }
    if (dead) lf |= FLAG_TIMEOUT;
    float* Or = invr + (size_t)(k0 / 128) * 128 * 128;
    float* Oi = invi + (size_t)(k0 / 128) * 128 * 128;
#pragma unroll
    for (int m = 0; m < RPT; ++m) {
        const size_t g = (size_t)(row_base + m) * 128 + 8 * cg;
        *reinterpret_cast<float4*>(Or + g) = make_float4(v[m][0].x, v[m][1].x, v[m][2].x, v[m][3].x);
        *reinterpret_cast<float4*>(Or + g + 4) = make_float4(v[m][4].x, v[m][5].x, v[m][6].x, v[m][7].x);
        *reinterpret_cast<float4*>(Oi + g) = make_float4(v[m][0].y, v[m][1].y, v[m][2].y, v[m][3].y);
        *reinterpret_cast<float4*>(Oi + g + 4) = make_float4(v[m][4].y, v[m][5].y, v[m][6].y, v[m][7].y);
    }
    if (dT) {
        // the transpose, [2][128][128], TF32-rounded: the K-major B operand of W21 = A21 D^-1.
        // Staged through the (now free) panel-row buffer as [2][128 columns][RPC + 4 rows] so
        // that each CTA writes its RPC-row stripe of every dT row with float4 stores.
        constexpr int SL = RPC + 4;
        float* st = reinterpret_cast<float*>(nrow);
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 8; ++c)
#pragma unroll
            for (int m = 0; m < RPT; ++m) {
                st[(8 * cg + c) * SL + RPT * rg + m] = tf32_rn(v[m][c].x);
                st[128 * SL + (8 * cg + c) * SL + RPT * rg + m] = tf32_rn(v[m][c].y);
            }
        __syncthreads();
        constexpr int V = RPC / 4;  // float4 per stripe row
        for (int idx = t; idx < 2 * 128 * V; idx += IC_THREADS) {
            const int pl = idx / (128 * V), col = (idx / V) % 128, f = idx % V;
            const float4 w = *reinterpret_cast<const float4*>(st + pl * 128 * SL + col * SL + 4 * f);
            *reinterpret_cast<float4*>(dT + pl * 16384 + col * 128 + RPC * (int)rank + 4 * f) = w;
        }
    }
    if (lf) atomicOr(flags, lf);
    ic_cluster_sync();  // no CTA leaves while another may still address its shared memory
}

// Blocked form of the same Gauss-Jordan inverse on a cluster of CL CTAs, with the
// rows split as in k_inv128c: the 128 pivots are taken 8 at a time (16 panels), so
// the CTAs synchronise 16 times instead of 128.  Panel p (pivot rows / columns
// P = 8p .. 8p + 7) belongs to the CTA owning those rows, which
//   1. inverts the 8 x 8 pivot block D = M[P][P] in one warp (in-place Gauss-Jordan,
//      the p + 1 substitution, shuffles only): X = D^-1;
//   2. forms the panel row R = X M[P][:] with R[:, P] = X (8 x 128; a warp reads the
//      staged rows as contiguous 16-byte words) in its own shared memory and sends it to
//      every peer as one 8 KB bulk copy (cp.async.bulk, shared::cta -> shared::cluster),
//      completing one mbarrier per panel there;
// then every CTA updates its other rows i: M[i][j] <- M[i][j] [j not in P] - M[i][P] R[:, j]
// and the owner copies R into rows P.  This is the composition of the 8 single-pivot
// steps.  Waits on a peer give up at a 2 s deadline (FLAG_TIMEOUT); every CTA always
// reaches the final cluster barrier.
constexpr int IB_SMEM = 128 * 64 * 16      // panel rows R, [128][4][16] float4 as in k_inv128c
                        + 64 * 8 * 8       // M[i][P] of this CTA's rows, [<= 64][8] float2
                        + 8 * 128 * 8      // the owner's rows P, [8][128] float2
                        + 64 * 8           // X, [8][8] float2
                        + 16 * 8;          // one mbarrier per panel

template <int CL>
__global__ void __launch_bounds__(IC_THREADS, 1)
    k_inv128b(int k0, CMat<float> A, float* invr, float* invi, float* dT, int* flags) {
    // launched as a programmatic dependent of the update that produced this block: wait
    // for its completion before reading A (returns at once for an ordinary launch); the
    // first W21 tile after it may be scheduled now and waits for this grid in turn
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    constexpr int RPC = 128 / CL, RPT = RPC / 16;
    static_assert(CL == 2 || CL == 4 || CL == 8, "cluster of 2, 4 or 8 CTAs");
    extern __shared__ __align__(16) float4 ib_smem[];
    float4* nrow = ib_smem;                                              // [128][4][16]
    float2* ccol = reinterpret_cast<float2*>(nrow + 128 * 64);           // [RPC][8]
    float2* prow = ccol + 64 * 8;                                        // [8][128]
    float2* xblk = prow + 8 * 128;                                       // [8][8]
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(xblk + 64);  // [16]
    const uint32_t rank = ic_rank();
    const int t = threadIdx.x, cg = t & 15, rg = t >> 4, warp = t >> 5, lane = t & 31;
    const uint32_t nrow_s = (uint32_t)__cvta_generic_to_shared(nrow);
    const uint32_t bars_s = (uint32_t)__cvta_generic_to_shared(bars);
    float2 v[RPT][8];
    const int row_base = RPC * (int)rank + RPT * rg;
#pragma unroll
    for (int m = 0; m < RPT; ++m) {
        const size_t g = (size_t)(k0 + row_base + m) * A.ld + k0 + 8 * cg;
        const float4 r0 = *reinterpret_cast<const float4*>(A.re + g);
        const float4 r1 = *reinterpret_cast<const float4*>(A.re + g + 4);
        const float4 i0 = *reinterpret_cast<const float4*>(A.im + g);
        const float4 i1 = *reinterpret_cast<const float4*>(A.im + g + 4);
        v[m][0] = make_float2(r0.x, i0.x); v[m][1] = make_float2(r0.y, i0.y);
        v[m][2] = make_float2(r0.z, i0.z); v[m][3] = make_float2(r0.w, i0.w);
        v[m][4] = make_float2(r1.x, i1.x); v[m][5] = make_float2(r1.y, i1.y);
        v[m][6] = make_float2(r1.z, i1.z); v[m][7] = make_float2(r1.w, i1.w);
    }
    if (t < 16) {
        // panels this CTA receives: one arrival now, completed by the owner's 8 KB
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bars_s + 8 * t) : "memory");
        if ((8 * t) / RPC != (int)rank)
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], 8192;" ::"r"(bars_s + 8 * t)
                         : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    ic_cluster_sync();
    unsigned long long deadline;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(deadline));
    deadline += 2000000000ull;
    int lf = 0;
    bool dead = false;
#pragma unroll 1
    for (int p = 0; p < 16; ++p) {
        const bool owner = (8 * p) / RPC == (int)rank;
        const int lp = 8 * p - RPC * (int)rank;  // first local row of P (owner only)
        // M[i][P] of this CTA's rows: the threads holding column group p
        if (cg == p) {
#pragma unroll
            for (int m = 0; m < RPT; ++m)
#pragma unroll
                for (int j = 0; j < 8; ++j) ccol[(RPT * rg + m) * 8 + j] = v[m][j];
        }
        if (owner) {
#pragma unroll
            for (int m = 0; m < RPT; ++m) {
                const int li = RPT * rg + m - lp;
                if (li >= 0 && li < 8)
#pragma unroll
                    for (int c = 0; c < 8; ++c) prow[li * 128 + 8 * cg + c] = v[m][c];
            }
            __syncthreads();
            if (warp == 0) {
                // X = D^-1: lane (i, q) = (lane / 4, lane % 4) holds D[i][q] and D[i][q + 4]
                const int i = lane >> 2, q = lane & 3;
                float2 a0 = ccol[(lp + i) * 8 + q], a1 = ccol[(lp + i) * 8 + q + 4];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int kc = k & 3;
                    const float2 s0 = k < 4 ? a0 : a1;  // this lane's value in column k
                    const float px = __shfl_sync(0xffffffffu, s0.x, k * 4 + kc);
                    const float py = __shfl_sync(0xffffffffu, s0.y, k * 4 + kc);
                    const float den = px * px + py * py;
                    if (lane == 0 && (!(den > 0.f) || !isfinite(den))) lf |= FLAG_ZERO_PIVOT;
                    const float rc = __frcp_rn(den), qr = px * rc, qi = -py * rc;
                    // pivot row k, this lane's columns q and q + 4 (column k carries p + 1)
                    float2 n0 = make_float2(__shfl_sync(0xffffffffu, a0.x, k * 4 + q),
                                            __shfl_sync(0xffffffffu, a0.y, k * 4 + q));
                    float2 n1 = make_float2(__shfl_sync(0xffffffffu, a1.x, k * 4 + q),
                                            __shfl_sync(0xffffffffu, a1.y, k * 4 + q));
                    if (q == kc) {
                        if (k < 4) n0.x += 1.f;
                        else n1.x += 1.f;
                    }
                    const float2 m0 = make_float2(n0.x * qr - n0.y * qi, n0.x * qi + n0.y * qr);
                    const float2 m1 = make_float2(n1.x * qr - n1.y * qi, n1.x * qi + n1.y * qr);
                    // column k of row i (minus 1 on the pivot row)
                    float cx = __shfl_sync(0xffffffffu, s0.x, i * 4 + kc);
                    const float cy = __shfl_sync(0xffffffffu, s0.y, i * 4 + kc);
                    if (i == k) cx -= 1.f;
                    a0.x = fmaf(-cx, m0.x, fmaf(cy, m0.y, a0.x));
                    a0.y = fmaf(-cx, m0.y, fmaf(-cy, m0.x, a0.y));
                    a1.x = fmaf(-cx, m1.x, fmaf(cy, m1.y, a1.x));
                    a1.y = fmaf(-cx, m1.y, fmaf(-cy, m1.x, a1.y));
                }
                xblk[i * 8 + q] = a0;
                xblk[i * 8 + q + 4] = a1;
            }
            __syncthreads();
            {
                // R[i0 + ii][c0 + cc] (ii, cc < 2) for c0 = 2 (t % 64), i0 = 2 (t / 64); R[:, P] = X.
                // A warp reads each staged pivot row as contiguous 16-byte words (no bank conflicts).
                const int c0 = 2 * (t & 63), i0 = 2 * (t >> 6);
                float2 r[2][2];
                if ((c0 >> 3) == p) {
#pragma unroll
                    for (int ii = 0; ii < 2; ++ii)
#pragma unroll
                        for (int cc = 0; cc < 2; ++cc) r[ii][cc] = xblk[(i0 + ii) * 8 + (c0 & 7) + cc];
                } else {
#pragma unroll
                    for (int ii = 0; ii < 2; ++ii) { r[ii][0] = make_float2(0.f, 0.f); r[ii][1] = make_float2(0.f, 0.f); }
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const float4 y = *reinterpret_cast<const float4*>(prow + j * 128 + c0);
#pragma unroll
                        for (int ii = 0; ii < 2; ++ii) {
                            const float2 x = xblk[(i0 + ii) * 8 + j];
                            r[ii][0].x = fmaf(x.x, y.x, fmaf(-x.y, y.y, r[ii][0].x));
                            r[ii][0].y = fmaf(x.x, y.y, fmaf(x.y, y.x, r[ii][0].y));
                            r[ii][1].x = fmaf(x.x, y.z, fmaf(-x.y, y.w, r[ii][1].x));
                            r[ii][1].y = fmaf(x.x, y.w, fmaf(x.y, y.z, r[ii][1].y));
                        }
                    }
                }
                const int qq = (c0 & 7) >> 1, cgc = c0 >> 3;
#pragma unroll
                for (int ii = 0; ii < 2; ++ii)
                    nrow[(8 * p + i0 + ii) * 64 + qq * 16 + cgc] =
                        make_float4(r[ii][0].x, r[ii][0].y, r[ii][1].x, r[ii][1].y);
                // the panel row goes to the peers as one 8 KB bulk copy each (async proxy)
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            }
            __syncthreads();
            if (t == 0) {
                const uint32_t src = nrow_s + 16u * (uint32_t)(8 * p * 64);
#pragma unroll
                for (int pp = 1; pp < CL; ++pp) {
                    const uint32_t peer = (rank + (uint32_t)pp) % CL;
                    asm volatile(
                        "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], 8192, [%2];"
                        ::"r"(ic_peer_addr(src, peer)), "r"(src), "r"(ic_peer_addr(bars_s + 8u * (uint32_t)p, peer))
                        : "memory");
                }
                asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            }
        } else {
            if (t == 0 && !dead && !ic_wait(bars_s + 8 * p, deadline)) dead = true;
            __syncthreads();
        }
        // rows of this CTA: M[i][j] <- M[i][j] [j not in P] - M[i][P] R[:, j]; rows P <- R
        bool inP[RPT];
        float2 cm[RPT][8];
#pragma unroll
        for (int m = 0; m < RPT; ++m) {
            const int li = RPT * rg + m - lp;
            inP[m] = owner && li >= 0 && li < 8;
#pragma unroll
            for (int j = 0; j < 8; ++j) cm[m][j] = ccol[(RPT * rg + m) * 8 + j];
#pragma unroll
            for (int c = 0; c < 8; ++c)
                if (inP[m] || cg == p) v[m][c] = make_float2(0.f, 0.f);
            if (inP[m]) {
#pragma unroll
                for (int j = 0; j < 8; ++j) cm[m][j] = make_float2(j == li ? -1.f : 0.f, 0.f);
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            float2 rr[8];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float4 x = nrow[(8 * p + j) * 64 + q * 16 + cg];
                rr[2 * q] = make_float2(x.x, x.y);
                rr[2 * q + 1] = make_float2(x.z, x.w);
            }
#pragma unroll
            for (int m = 0; m < RPT; ++m)
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    v[m][c].x = fmaf(-cm[m][j].x, rr[c].x, fmaf(cm[m][j].y, rr[c].y, v[m][c].x));
                    v[m][c].y = fmaf(-cm[m][j].x, rr[c].y, fmaf(-cm[m][j].y, rr[c].x, v[m][c].y));
                }
        }
        __syncthreads();  // ccol, prow and xblk are rewritten for the next panel
    }
    if (dead) lf |= FLAG_TIMEOUT;
    float* Or = invr + (size_t)(k0 / 128) * 128 * 128;
    float* Oi = invi + (size_t)(k0 / 128) * 128 * 128;
#pragma unroll
    for (int m = 0; m < RPT; ++m) {
        const size_t g = (size_t)(row_base + m) * 128 + 8 * cg;
        *reinterpret_cast<float4*>(Or + g) = make_float4(v[m][0].x, v[m][1].x, v[m][2].x, v[m][3].x);
        *reinterpret_cast<float4*>(Or + g + 4) = make_float4(v[m][4].x, v[m][5].x, v[m][6].x, v[m][7].x);
        *reinterpret_cast<float4*>(Oi + g) = make_float4(v[m][0].y, v[m][1].y, v[m][2].y, v[m][3].y);
        *reinterpret_cast<float4*>(Oi + g + 4) = make_float4(v[m][4].y, v[m][5].y, v[m][6].y, v[m][7].y);
    }
    // the bulk copies out of the panel rows have read their sources before the shared
    // memory is reused or released
    if (t == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    if (dT) {
        // the transpose, [2][128][128], TF32-rounded: the K-major B operand of W21 = A21 D^-1.
        // Staged through the (now free) panel-row buffer as [2][128 columns][RPC + 4 rows] so
        // that each CTA writes its RPC-row stripe of every dT row with float4 stores.
        constexpr int SL = RPC + 4;
        float* st = reinterpret_cast<float*>(nrow);
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 8; ++c)
#pragma unroll
            for (int m = 0; m < RPT; ++m) {
                st[(8 * cg + c) * SL + RPT * rg + m] = tf32_rn(v[m][c].x);
                st[128 * SL + (8 * cg + c) * SL + RPT * rg + m] = tf32_rn(v[m][c].y);
            }
        __syncthreads();
        constexpr int V = RPC / 4;  // float4 per stripe row
        for (int idx = t; idx < 2 * 128 * V; idx += IC_THREADS) {
            const int pl = idx / (128 * V), col = (idx / V) % 128, f = idx % V;
            const float4 w = *reinterpret_cast<const float4*>(st + pl * 128 * SL + col * SL + 4 * f);
            *reinterpret_cast<float4*>(dT + pl * 16384 + col * 128 + RPC * (int)rank + 4 * f) = w;
        }
    }
    if (lf) atomicOr(flags, lf);
    ic_cluster_sync();  // no CTA leaves while another may still address its shared memory
}

// The blocked cluster inverse with the next panel's chain taken ahead of the bulk of each
// rank-8 update.  The CTA has a ninth warp (the pivot warp) that holds no rows.  For panel
// q the owner of panel q+1 first applies R_q to its 8 pivot rows of q+1 and stages their
// 8 x 8 pivot block and 8 x 128 panel rows; then the pivot warp inverts that block while
// the 256 row threads apply R_q to every other row; then the row threads form R_{q+1}
// and send it.  The chain per panel is the pivot-row update, the 8 x 8 inverse and the
// panel row; the bulk update runs beside the inverse.  Same arithmetic as k_inv128b.
constexpr int IL_THREADS = IC_THREADS + 32;
constexpr int IL_SMEM = 128 * 64 * 16       // panel rows R, [128][4][16] float4
                        + 2 * 64 * 8 * 8    // M[i][P] of this CTA's rows, two buffers [2][<= 64][8] float2
                        + 8 * 128 * 8       // staged pivot rows of the next panel, [8][128] float2
                        + 64 * 8            // X, [8][8] float2
                        + 64 * 8            // next pivot block, [8][8] float2
                        + 16 * 8;           // one mbarrier per panel

template <int CL>
__global__ void __launch_bounds__(IL_THREADS, 1)
    k_inv128l(int k0, CMat<float> A, float* invr, float* invi, float* dT, int* flags) {
    // launched as a programmatic dependent of the update that produced this block: wait
    // for its completion before reading A (returns at once for an ordinary launch); the
    // first W21 tile after it may be scheduled now and waits for this grid in turn
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    constexpr int RPC = 128 / CL, RPT = RPC / 16;
    static_assert(CL == 2 || CL == 4 || CL == 8, "cluster of 2, 4 or 8 CTAs");
    extern __shared__ __align__(16) float4 il_smem[];
    float4* nrow = il_smem;                                              // [128][4][16]
    float2* ccol = reinterpret_cast<float2*>(nrow + 128 * 64);           // [2][64][8]
    float2* prow = ccol + 2 * 64 * 8;                                    // [8][128]
    float2* xblk = prow + 8 * 128;                                       // [8][8]
    float2* dblk = xblk + 64;                                            // [8][8]
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(dblk + 64);  // [16]
    const uint32_t rank = ic_rank();
    const int t = threadIdx.x, cg = t & 15, rg = (t >> 4) & 15, warp = t >> 5, lane = t & 31;
    const bool rowthr = t < IC_THREADS;  // warp 8 is the pivot warp
    const uint32_t nrow_s = (uint32_t)__cvta_generic_to_shared(nrow);
    const uint32_t bars_s = (uint32_t)__cvta_generic_to_shared(bars);
    float2 v[RPT][8];
    const int row_base = RPC * (int)rank + RPT * rg;
    if (rowthr) {
#pragma unroll
        for (int m = 0; m < RPT; ++m) {
            const size_t g = (size_t)(k0 + row_base + m) * A.ld + k0 + 8 * cg;
            const float4 r0 = *reinterpret_cast<const float4*>(A.re + g);
            const float4 r1 = *reinterpret_cast<const float4*>(A.re + g + 4);
            const float4 i0 = *reinterpret_cast<const float4*>(A.im + g);
            const float4 i1 = *reinterpret_cast<const float4*>(A.im + g + 4);
            v[m][0] = make_float2(r0.x, i0.x); v[m][1] = make_float2(r0.y, i0.y);
            v[m][2] = make_float2(r0.z, i0.z); v[m][3] = make_float2(r0.w, i0.w);
            v[m][4] = make_float2(r1.x, i1.x); v[m][5] = make_float2(r1.y, i1.y);
            v[m][6] = make_float2(r1.z, i1.z); v[m][7] = make_float2(r1.w, i1.w);
        }
    }
    if (t < 16) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bars_s + 8 * t) : "memory");
        if ((8 * t) / RPC != (int)rank)
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], 8192;" ::"r"(bars_s + 8 * t)
                         : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    ic_cluster_sync();
    unsigned long long deadline;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(deadline));
    deadline += 2000000000ull;
    int lf = 0;
    bool dead = false;
    auto owns = [&](int q) { return (8 * q) / RPC == (int)rank; };
    // rows (local index RPT rg + m - 8 q + RPC rank) of panel q held by this thread
    auto in_panel = [&](int q, int m) {
        const int li = RPT * rg + m - (8 * q - RPC * (int)rank);
        return li >= 0 && li < 8;
    };
    // this thread's M[i][P_q] into ccol buffer q & 1 (threads of column group q)
    auto put_ccol = [&](int q) {
        if (rowthr && cg == q) {
#pragma unroll
            for (int m = 0; m < RPT; ++m)
#pragma unroll
                for (int j = 0; j < 8; ++j) ccol[((q & 1) * 64 + RPT * rg + m) * 8 + j] = v[m][j];
        }
    };
    // the owner's pivot rows of panel q into prow, their 8 x 8 pivot block into dblk
    auto stage = [&](int q) {
        if (rowthr) {
#pragma unroll
            for (int m = 0; m < RPT; ++m) {
                if (!in_panel(q, m)) continue;
                const int li = RPT * rg + m - (8 * q - RPC * (int)rank);
#pragma unroll
                for (int c = 0; c < 8; ++c) prow[li * 128 + 8 * cg + c] = v[m][c];
                if (cg == q) {
#pragma unroll
                    for (int c = 0; c < 8; ++c) dblk[li * 8 + c] = v[m][c];
                }
            }
        }
    };
    // X = D^-1 of the staged pivot block (pivot warp; lane (i, c) = (lane / 4, lane % 4)
    // holds D[i][c] and D[i][c + 4]; in-place Gauss-Jordan with the p + 1 substitution)
    auto pivot_inverse = [&]() {
        const int i = lane >> 2, q = lane & 3;
        float2 a0 = dblk[i * 8 + q], a1 = dblk[i * 8 + q + 4];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int kc = k & 3;
            const float2 s0 = k < 4 ? a0 : a1;
            const float px = __shfl_sync(0xffffffffu, s0.x, k * 4 + kc);
            const float py = __shfl_sync(0xffffffffu, s0.y, k * 4 + kc);
            const float den = px * px + py * py;
            if (lane == 0 && (!(den > 0.f) || !isfinite(den))) lf |= FLAG_ZERO_PIVOT;
            const float rc = __frcp_rn(den), qr = px * rc, qi = -py * rc;
            float2 n0 = make_float2(__shfl_sync(0xffffffffu, a0.x, k * 4 + q), __shfl_sync(0xffffffffu, a0.y, k * 4 + q));
            float2 n1 = make_float2(__shfl_sync(0xffffffffu, a1.x, k * 4 + q), __shfl_sync(0xffffffffu, a1.y, k * 4 + q));
            if (q == kc) {
                if (k < 4) n0.x += 1.f;
                else n1.x += 1.f;
            }
            const float2 m0 = make_float2(n0.x * qr - n0.y * qi, n0.x * qi + n0.y * qr);
            const float2 m1 = make_float2(n1.x * qr - n1.y * qi, n1.x * qi + n1.y * qr);
            float cx = __shfl_sync(0xffffffffu, s0.x, i * 4 + kc);
            const float cy = __shfl_sync(0xffffffffu, s0.y, i * 4 + kc);
            if (i == k) cx -= 1.f;
            a0.x = fmaf(-cx, m0.x, fmaf(cy, m0.y, a0.x));
            a0.y = fmaf(-cx, m0.y, fmaf(-cy, m0.x, a0.y));
            a1.x = fmaf(-cx, m1.x, fmaf(cy, m1.y, a1.x));
            a1.y = fmaf(-cx, m1.y, fmaf(-cy, m1.x, a1.y));
        }
        xblk[i * 8 + q] = a0;
        xblk[i * 8 + q + 4] = a1;
    };
    // R_q = X prow with R[:, P_q] = X (row threads), into nrow; then one bulk copy per peer
    auto form_and_send = [&](int q) {
        if (rowthr) {
            const int c0 = 2 * (t & 63), i0 = 2 * (t >> 6);
            float2 r[2][2];
            if ((c0 >> 3) == q) {
#pragma unroll
                for (int ii = 0; ii < 2; ++ii)
#pragma unroll
                    for (int cc = 0; cc < 2; ++cc) r[ii][cc] = xblk[(i0 + ii) * 8 + (c0 & 7) + cc];
            } else {
#pragma unroll
                for (int ii = 0; ii < 2; ++ii) { r[ii][0] = make_float2(0.f, 0.f); r[ii][1] = make_float2(0.f, 0.f); }
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const float4 y = *reinterpret_cast<const float4*>(prow + j * 128 + c0);
#pragma unroll
                    for (int ii = 0; ii < 2; ++ii) {
                        const float2 x = xblk[(i0 + ii) * 8 + j];
                        r[ii][0].x = fmaf(x.x, y.x, fmaf(-x.y, y.y, r[ii][0].x));
                        r[ii][0].y = fmaf(x.x, y.y, fmaf(x.y, y.x, r[ii][0].y));
                        r[ii][1].x = fmaf(x.x, y.z, fmaf(-x.y, y.w, r[ii][1].x));
                        r[ii][1].y = fmaf(x.x, y.w, fmaf(x.y, y.z, r[ii][1].y));
                    }
                }
            }
            const int qq = (c0 & 7) >> 1, cgc = c0 >> 3;
#pragma unroll
            for (int ii = 0; ii < 2; ++ii)
                nrow[(8 * q + i0 + ii) * 64 + qq * 16 + cgc] = make_float4(r[ii][0].x, r[ii][0].y, r[ii][1].x, r[ii][1].y);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        __syncthreads();
        if (t == 0) {
            const uint32_t src = nrow_s + 16u * (uint32_t)(8 * q * 64);
#pragma unroll
            for (int pp = 1; pp < CL; ++pp) {
                const uint32_t peer = (rank + (uint32_t)pp) % CL;
                asm volatile(
                    "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], 8192, [%2];"
                    ::"r"(ic_peer_addr(src, peer)), "r"(src), "r"(ic_peer_addr(bars_s + 8u * (uint32_t)q, peer))
                    : "memory");
            }
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        }
    };
    // apply R_q to this thread's rows (rows of P_q become R_q; rows already done are skipped)
    auto update = [&](int q, bool skip_next) {
        if (!rowthr) return;
#pragma unroll
        for (int m = 0; m < RPT; ++m) {
            if (skip_next && in_panel(q + 1, m)) continue;
            const bool inP = owns(q) && in_panel(q, m);
            const int li = RPT * rg + m - (8 * q - RPC * (int)rank);
            float2 cm[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)
                cm[j] = inP ? make_float2(j == li ? -1.f : 0.f, 0.f) : ccol[((q & 1) * 64 + RPT * rg + m) * 8 + j];
            if (inP || cg == q) {
#pragma unroll
                for (int c = 0; c < 8; ++c) v[m][c] = make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                float2 rr[8];
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) {
                    const float4 x = nrow[(8 * q + j) * 64 + qq * 16 + cg];
                    rr[2 * qq] = make_float2(x.x, x.y);
                    rr[2 * qq + 1] = make_float2(x.z, x.w);
                }
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    v[m][c].x = fmaf(-cm[j].x, rr[c].x, fmaf(cm[j].y, rr[c].y, v[m][c].x));
                    v[m][c].y = fmaf(-cm[j].x, rr[c].y, fmaf(-cm[j].y, rr[c].x, v[m][c].y));
                }
            }
        }
    };
    // panel 0
    put_ccol(0);
    if (owns(0)) {
        stage(0);
        __syncthreads();
        if (warp == 8) pivot_inverse();
        __syncthreads();
        form_and_send(0);
    }
    __syncthreads();
#pragma unroll 1
    for (int q = 0; q < 16; ++q) {
        if (!owns(q)) {
            if (t == 0 && !dead && !ic_wait(bars_s + 8 * q, deadline)) dead = true;
        }
        __syncthreads();  // R_q in nrow (local or received); ccol buffer q & 1 complete
        const bool next = q + 1 < 16, own_next = next && owns(q + 1);
        if (own_next) {
            // the pivot rows of panel q+1 first, then their block and panel rows
            if (rowthr) {
#pragma unroll
                for (int m = 0; m < RPT; ++m) {
                    if (!in_panel(q + 1, m)) continue;
                    const bool inP = owns(q) && in_panel(q, m);  // never: panels are disjoint
                    (void)inP;
                    float2 cm[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) cm[j] = ccol[((q & 1) * 64 + RPT * rg + m) * 8 + j];
                    if (cg == q) {
#pragma unroll
                        for (int c = 0; c < 8; ++c) v[m][c] = make_float2(0.f, 0.f);
                    }
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        float2 rr[8];
#pragma unroll
                        for (int qq = 0; qq < 4; ++qq) {
                            const float4 x = nrow[(8 * q + j) * 64 + qq * 16 + cg];
                            rr[2 * qq] = make_float2(x.x, x.y);
                            rr[2 * qq + 1] = make_float2(x.z, x.w);
                        }
#pragma unroll
                        for (int c = 0; c < 8; ++c) {
                            v[m][c].x = fmaf(-cm[j].x, rr[c].x, fmaf(cm[j].y, rr[c].y, v[m][c].x));
                            v[m][c].y = fmaf(-cm[j].x, rr[c].y, fmaf(-cm[j].y, rr[c].x, v[m][c].y));
                        }
                    }
                }
            }
            stage(q + 1);
            __syncthreads();
            if (warp == 8) pivot_inverse();
        }
        update(q, own_next);
        if (next) put_ccol(q + 1);
        __syncthreads();  // every row updated by R_q; X of panel q+1 ready
        if (own_next) form_and_send(q + 1);
    }
    if (dead) lf |= FLAG_TIMEOUT;
    // the bulk copies out of the panel rows have read their sources before the shared
    // memory is reused or released
    if (t == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    float* Or = invr + (size_t)(k0 / 128) * 128 * 128;
    float* Oi = invi + (size_t)(k0 / 128) * 128 * 128;
    if (rowthr) {
#pragma unroll
        for (int m = 0; m < RPT; ++m) {
            const size_t g = (size_t)(row_base + m) * 128 + 8 * cg;
            *reinterpret_cast<float4*>(Or + g) = make_float4(v[m][0].x, v[m][1].x, v[m][2].x, v[m][3].x);
            *reinterpret_cast<float4*>(Or + g + 4) = make_float4(v[m][4].x, v[m][5].x, v[m][6].x, v[m][7].x);
            *reinterpret_cast<float4*>(Oi + g) = make_float4(v[m][0].y, v[m][1].y, v[m][2].y, v[m][3].y);
            *reinterpret_cast<float4*>(Oi + g + 4) = make_float4(v[m][4].y, v[m][5].y, v[m][6].y, v[m][7].y);
        }
    }
    if (dT) {
        // the transpose, TF32-rounded, staged through the panel-row buffer as in k_inv128b
        constexpr int SL = RPC + 4;
        float* stg = reinterpret_cast<float*>(nrow);
        __syncthreads();
        if (rowthr) {
#pragma unroll
            for (int c = 0; c < 8; ++c)
#pragma unroll
                for (int m = 0; m < RPT; ++m) {
                    stg[(8 * cg + c) * SL + RPT * rg + m] = tf32_rn(v[m][c].x);
                    stg[128 * SL + (8 * cg + c) * SL + RPT * rg + m] = tf32_rn(v[m][c].y);
                }
        }
        __syncthreads();
        constexpr int V = RPC / 4;
        for (int idx = t; idx < 2 * 128 * V; idx += IL_THREADS) {
            const int pl = idx / (128 * V), col = (idx / V) % 128, f = idx % V;
            const float4 w = *reinterpret_cast<const float4*>(stg + pl * 128 * SL + col * SL + 4 * f);
            *reinterpret_cast<float4*>(dT + pl * 16384 + col * 128 + RPC * (int)rank + 4 * f) = w;
        }
    }
    if (lf) atomicOr(flags, lf);
    ic_cluster_sync();  // no CTA leaves while another may still address its shared memory
}

// One cluster of cl CTAs (2, 4 or 8) inverting the diagonal block at k0.
static void inv128_cluster(cudaStream_t st, int cl, int blocked, int k0, CMat<float> A, float* invr, float* invi,
                           float* dT, int* flags, int pdl = 0) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cl);
    cfg.blockDim = dim3(IC_THREADS);
    cfg.dynamicSmemBytes = blocked == 2 ? IL_SMEM : blocked ? IB_SMEM : IC_SMEM;
    if (blocked == 2) cfg.blockDim = dim3(IL_THREADS);
    cfg.stream = st;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    // programmatic dependent launch: the inverse's CTAs may be scheduled once the kernel
    // before it on this stream has signalled (griddepcontrol.launch_dependents); they wait
    // for that kernel's completion and memory (griddepcontrol.wait) before reading A
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 2 : 1;
    if (blocked == 2) {
        switch (cl) {
            case 2: BEM_LAUNCH(cudaLaunchKernelEx(&cfg, k_inv128l<2>, k0, A, invr, invi, dT, flags)); break;
            case 4: BEM_LAUNCH(cudaLaunchKernelEx(&cfg, k_inv128l<4>, k0, A, invr, invi, dT, flags)); break;
            default: BEM_LAUNCH(cudaLaunchKernelEx(&cfg, k_inv128l<8>, k0, A, invr, invi, dT, flags)); break;
        }
        return;
    }
    if (blocked) {
        switch (cl) {
            case 2: BEM_LAUNCH(cudaLaunchKernelEx(&cfg, k_inv128b<2>, k0, A, invr, invi, dT, flags)); break;
            case 4: BEM_LAUNCH(cudaLaunchKernelEx(&cfg, k_inv128b<4>, k0, A, invr, invi, dT, flags)); break;
            default: BEM_LAUNCH(cudaLaunchKernelEx(&cfg, k_inv128b<8>, k0, A, invr, invi, dT, flags)); break;
        }
        return;
    }
    switch (cl) {
        case 2: BEM_LAUNCH(cudaLaunchKernelEx(&cfg, k_inv128c<2>, k0, A, invr, invi, dT, flags)); break;
        case 4: BEM_LAUNCH(cudaLaunchKernelEx(&cfg, k_inv128c<4>, k0, A, invr, invi, dT, flags)); break;
        default: BEM_LAUNCH(cudaLaunchKernelEx(&cfg, k_inv128c<8>, k0, A, invr, invi, dT, flags)); break;
    }
}
static void inv128_cluster_setup() {
    cudaFuncSetAttribute(k_inv128l<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, IL_SMEM);
    cudaFuncSetAttribute(k_inv128l<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, IL_SMEM);
    cudaFuncSetAttribute(k_inv128l<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, IL_SMEM);
    cudaFuncSetAttribute(k_inv128b<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, IB_SMEM);
    cudaFuncSetAttribute(k_inv128b<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, IB_SMEM);
    cudaFuncSetAttribute(k_inv128b<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, IB_SMEM);
    cudaFuncSetAttribute(k_inv128c<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, IC_SMEM);
    cudaFuncSetAttribute(k_inv128c<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, IC_SMEM);
    cudaFuncSetAttribute(k_inv128c<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, IC_SMEM);
}

// ---------------------------------------------------------------------------
// C = beta C + sgn * A B, planar complex, row-major.  M, N multiples of 64,
// K multiple of 16.  256 threads, 64x64 tile, 4x4 outputs per thread.
template <typename T>
__global__ void __launch_bounds__(256) k_cgemm(int M, int N, int K, CMat<T> A, CMat<T> B, CMat<T> C, T sgn,
                                               int beta) {
    __shared__ T Asr[16][64], Asi[16][64], Bsr[16][64], Bsi[16][64];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    T cr[4][4], ci[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) { cr[i][j] = 0; ci[i][j] = 0; }
    for (int k0 = 0; k0 < K; k0 += 16) {
        // A tile: 64 rows x 16 k  (stored transposed As[k][m])
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            int idx = tid + t * 256;
            int m = idx >> 4, k = idx & 15;
            size_t g = (size_t)(m0 + m) * A.ld + k0 + k;
            Asr[k][m] = A.re[g];
            Asi[k][m] = A.im[g];
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            int idx = tid + t * 256;
            int k = idx >> 6, n = idx & 63;
            size_t g = (size_t)(k0 + k) * B.ld + n0 + n;
            Bsr[k][n] = B.re[g];
            Bsi[k][n] = B.im[g];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            T ar_[4], ai_[4], br_[4], bi_[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) { ar_[i] = Asr[k][ty * 4 + i]; ai_[i] = Asi[k][ty * 4 + i]; }
#pragma unroll
            for (int j = 0; j < 4; ++j) { br_[j] = Bsr[k][tx * 4 + j]; bi_[j] = Bsi[k][tx * 4 + j]; }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    cr[i][j] = fma(ar_[i], br_[j], cr[i][j]);
                    cr[i][j] = fma(-ai_[i], bi_[j], cr[i][j]);
                    ci[i][j] = fma(ar_[i], bi_[j], ci[i][j]);
                    ci[i][j] = fma(ai_[i], br_[j], ci[i][j]);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            size_t g = (size_t)(m0 + ty * 4 + i) * C.ld + n0 + tx * 4 + j;
            T vr = sgn * cr[i][j], vi = sgn * ci[i][j];
            if (beta) { vr += C.re[g]; vi += C.im[g]; }
            C.re[g] = vr;
            C.im[g] = vi;
        }
}

// Copy a panel workspace (rows x cols, ld = wld) into the matrix block at
// (r0, c0); optionally check |x| <= 1 (L21 multipliers) and write a transposed
// copy (for the tensor-core B operand).
template <typename T>
__global__ void k_copy_back(int rows, int cols, const T* wr, const T* wi, int wld, CMat<T> A, int r0, int c0,
                            int check, T* tr, T* ti, int tld, int* flags) {
    size_t total = (size_t)rows * cols;
    int bad = 0;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total; idx += (size_t)gridDim.x * blockDim.x) {
        int i = (int)(idx / cols), j = (int)(idx % cols);
        T vr = wr[(size_t)i * wld + j], vi = wi[(size_t)i * wld + j];
        size_t g = (size_t)(r0 + i) * A.ld + c0 + j;
        A.re[g] = vr;
        A.im[g] = vi;
        if (check && vr * vr + vi * vi > (T)(1.000002)) bad = 1;
        if (tr) { tr[(size_t)j * tld + i] = vr; ti[(size_t)j * tld + i] = vi; }
    }
    if (bad) atomicOr(flags, FLAG_PIVOT);
}

// Block LU without row exchanges: for each diagonal block (order nb),
//   D11^-1 (Gauss-Jordan),  W21 = A21 D11^-1  (stored in place of A21),
//   A22 -= W21 A12          (A12 is the block-upper factor, kept in place).
// Then D = L U with L = I + (strictly lower blocks W), U = block upper with the
// diagonal blocks D_bb, whose inverses are kept in inv[blk].
template <typename T, int NB>
static int lu_factor_t(cudaStream_t st, int n, CMat<T> A, T* invr, T* invi, T* wl, int* flags) {
    T* wlr = wl; T* wli = wl + (size_t)n * NB;
    for (int k0 = 0; k0 < n; k0 += NB) {
        BEM_LAUNCH(k_gj_inv<T, NB><<<1, 1024, 0, st>>>(k0, A, invr, invi, flags));
        const int rem = n - k0 - NB;
        if (rem <= 0) break;
        const int blk = k0 / NB;
        CMat<T> Dinv{invr + (size_t)blk * NB * NB, invi + (size_t)blk * NB * NB, NB};
        CMat<T> A21{A.re + (size_t)(k0 + NB) * A.ld + k0, A.im + (size_t)(k0 + NB) * A.ld + k0, A.ld};
        CMat<T> A12{A.re + (size_t)k0 * A.ld + k0 + NB, A.im + (size_t)k0 * A.ld + k0 + NB, A.ld};
        CMat<T> WL{wlr, wli, NB};
        // W21 = A21 D11^-1  (rem x NB)
        BEM_LAUNCH(k_cgemm<T><<<dim3(NB / 64, rem / 64), 256, 0, st>>>(rem, NB, NB, A21, Dinv, WL, (T)1, 0));
        int nblk = (int)(((size_t)rem * NB + 255) / 256);
        if (nblk > 4096) nblk = 4096;
        BEM_LAUNCH(k_copy_back<T><<<nblk, 256, 0, st>>>(rem, NB, wlr, wli, NB, A, k0 + NB, k0, 0, (T*)nullptr,
                                                        (T*)nullptr, 0, flags));
        CMat<T> A22{A.re + (size_t)(k0 + NB) * A.ld + k0 + NB, A.im + (size_t)(k0 + NB) * A.ld + k0 + NB, A.ld};
        BEM_LAUNCH(k_cgemm<T><<<dim3(rem / 64, rem / 64), 256, 0, st>>>(rem, rem, NB, WL, A12, A22, (T)-1, 1));
    }
    return 0;
}

// wut[j][i] = A[r0 + i][c0 + j] for i < 128, j < cols (both planes; wut rows of 128 floats).
__global__ void k_panel_transpose(int cols, CMat<float> A, int r0, int c0, float* wtr, float* wti) {
    __shared__ float tr[32][33], ti[32][33];
    const int j0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int j = j0 + threadIdx.x;
        const size_t g = (size_t)(r0 + i0 + y) * A.ld + c0 + j;
        tr[y][threadIdx.x] = j < cols ? A.re[g] : 0.f;
        ti[y][threadIdx.x] = j < cols ? A.im[g] : 0.f;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const int j = j0 + y;
        if (j < cols) {
            wtr[(size_t)j * 128 + i0 + threadIdx.x] = tf32_rn(tr[threadIdx.x][y]);
            wti[(size_t)j * 128 + i0 + threadIdx.x] = tf32_rn(ti[threadIdx.x][y]);
        }
    }
}

// T[which][plane][p][j][i] = B_p[i][j] for the off-diagonal blocks of the 128-block pairs
// (2p, 2p+1): which 0: B_p = L_{2p+1,2p}, which 1: B_p = (U D^-1)_{2p,2p+1}; rounded to
// TF32 (nearest).  Grid (4, 4, 2 np), 32 x 8 threads.
__global__ void k_pair_transpose(int np, CMat<float> A, float* T) {
    __shared__ float tr[32][33], ti[32][33];
    const int p = blockIdx.z % np, which = blockIdx.z / np;
    const size_t r0 = (size_t)(which == 0 ? 2 * p + 1 : 2 * p) * 128, c0 = (size_t)(which == 0 ? 2 * p : 2 * p + 1) * 128;
    const int j0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const size_t g = (r0 + i0 + y) * A.ld + c0 + j0 + threadIdx.x;
        tr[y][threadIdx.x] = A.re[g];
        ti[y][threadIdx.x] = A.im[g];
    }
    __syncthreads();
    const size_t plane = (size_t)np * 128 * 128;
    float* Tr = T + 2 * which * plane + (size_t)p * 128 * 128;
    float* Ti = Tr + plane;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
        const size_t o = (size_t)(j0 + y) * 128 + i0 + threadIdx.x;
        Tr[o] = tf32_rn(tr[threadIdx.x][y]);
        Ti[o] = tf32_rn(ti[threadIdx.x][y]);
    }
}

// Pair fold: with P = blockdiag([I 0; L_{2p+1,2p} I]) and Q = blockdiag([I U_{2p,2p+1}; 0 I])
// over the 128-block pairs, L = L'' P and U D^-1 = U'' Q, where L'' and U'' have identity
// diagonal blocks of 256 rows.  A forward solve is then a chain of n / 256 steps over L''
// followed by x = P^-1 y (one independent 128 x 128 product per pair), and likewise the
// backward solve; see k_trsv_tk and k_pair_apply.  L'' and U'' replace L and U D^-1 in A
// (the pair blocks themselves are kept).  T: 4 np 128 128 floats.
int lu_pair_fold(cudaStream_t st, int n, CMat<float> A, float* T, int* flags) {
    const int np = n / 256;
    if (np == 0) return 0;
    if (!T) return 1;
    BEM_LAUNCH(k_pair_transpose<<<dim3(4, 4, 2 * np), dim3(32, 8), 0, st>>>(np, A, T));
    const size_t plane = (size_t)np * 128 * 128;
    if (!tc_pair_fold(st, n, A, T, 1, flags)) return 1;
    if (!tc_pair_fold(st, n, A, T + 2 * plane, 2, flags)) return 1;
    return 0;
}

int lu_factor_f32_lookahead(cudaStream_t st, const LuStreams& ls, int n, CMat<float> A, float* invr, float* invi,
                            float* wl2, float* wut2, int* flags) {
    constexpr int NB = 128;
    const int nblk = n / NB;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    // reserve_sms > 0: persistent rest update on nsm - reserve_sms CTAs; 0: CTAs of about
    // four tiles each, which retire during the update and hand SMs to the panel stream
    const int rest_ctas = ls.reserve_sms > 0 ? std::max(1, nsm - ls.reserve_sms) : -std::max(1, ls.rest_tiles);
    auto wlb = [&](int k) { return wl2 + (size_t)(k & 1) * 2 * n * NB; };
    auto wutb = [&](int k) { return wut2 + (size_t)(k & 1) * 2 * n * NB; };
    cudaStream_t sp = ls.panel;
    if (ls.cluster_inverse >= 2) inv128_cluster_setup();
    // Panel k on the panel stream: D_kk^-1, W21 = A21 D_kk^-1 (into wl and A21), U12^T
    // (into wut); ev_panel marks the operands of the step-k updates ready.
    // timeline (optional): per step k, [0] cross update start, [1] cross done (main stream),
    // [2] inverse of block k+1 done, [3] W21 done, [4] panel k+1 ready (panel stream), [5] rest done
    auto mark = [&](int k, int slot, cudaStream_t s) {
        if (ls.timeline && k >= 0 && k < nblk) cudaEventRecord(ls.timeline[6 * k + slot], s);
    };
    // D_kk^-1 transposed, [nblk][2][128][128]: block k's copy feeds W21 of step k and the
    // U-column transform, which runs on its own stream behind the panel chain
    auto dTb = [&](int k) { return wut2 + (size_t)4 * n * NB + (size_t)k * 2 * NB * NB; };
    // Panel k+1 on the panel stream: the inverse of block k+1 (after its own update by
    // step k, the single corner tile, also run on this stream), then W21 and the
    // transpose, which need the rest of block column / row k+1 (the main stream's
    // L-shaped update of step k).  Only their first tiles (block (k+2, k+1) of W21 and
    // block (k+1, k+2) of U) feed the next corner tile and so the next inverse; with
    // ls.panel_tail the other tiles run on that second stream, off the inverse chain.
    auto inverse = [&](int k) {
        const int k0 = k * NB;
        if (ls.cluster_inverse >= 2)
            inv128_cluster(sp, ls.cluster_inverse, ls.block_inverse, k0, A, invr, invi, dTb(k), flags, ls.pdl);
        else
            BEM_LAUNCH(k_inv128<<<1, IV_THREADS, 0, sp>>>(k0, A, invr, invi, dTb(k), flags));
        mark(k - 1, 2, sp);
    };
    cudaStream_t sq = ls.panel_tail ? ls.panel_tail : sp;
    auto w21 = [&](int k) {
        const int k0 = k * NB, rem = n - k0 - NB;
        // W21 = A21 D^-1 on the tensor cores, into wl and over A21 (for the solves), and
        // U12^T into wut, for row / column tiles t0 .. t0 + count - 1 (count < 0: to the end)
        auto w21_tiles = [&](cudaStream_t s, int t0, int count, int pdl = 0) {
            return tc_w21(s, n, k0, A, dTb(k), wlb(k), flags, t0, count, pdl);
        };
        auto tr_tiles = [&](cudaStream_t s, int t0, int count) {
            const int c0 = t0 * NB, cols = std::min(rem - c0, count < 0 ? rem : count * NB);
            if (cols <= 0) return;
            float* wtr = wutb(k) + (size_t)c0 * NB;
            BEM_LAUNCH(k_panel_transpose<<<dim3((cols + 31) / 32, NB / 32), dim3(32, 8), 0, s>>>(
                cols, A, k0, k0 + NB + c0, wtr, wtr + (size_t)n * NB));
        };
        if (ls.panel_tail) {
            // the first U tile needs only the cross update, not the inverse: transposed on
            // the tail stream while the inverse runs
            cudaStreamWaitEvent(sq, ls.ev_cross, 0);
            tr_tiles(sq, 0, 1);
            cudaEventRecord(ls.ev_t0, sq);
            if (!w21_tiles(sp, 0, 1)) return false;
            cudaStreamWaitEvent(sp, ls.ev_t0, 0);
            cudaEventRecord(ls.ev_head, sp);
            cudaStreamWaitEvent(sq, ls.ev_head, 0);
        } else {
            if (!w21_tiles(sp, 0, 1)) return false;
            tr_tiles(sp, 0, 1);
        }
        if (!w21_tiles(sq, 1, -1)) return false;
        tr_tiles(sq, 1, -1);
        mark(k - 1, 3, sq);
        cudaEventRecord(ls.ev_panel, sq);
        mark(k - 1, 4, sq);
        if (k > 0) {
            // U_{0:k, k} <- U_{0:k, k} D_kk^-1 (the backward solve's operator); those rows are
            // final and no longer read by the factorization
            if (ls.ucol_own) cudaStreamWaitEvent(ls.ucol, ls.ev_panel, 0);
            if (!tc_ucol(ls.ucol_own ? ls.ucol : sq, n, k0, A, dTb(k), ls.ucol_ctas, flags)) return false;
        }
        return true;
    };
    cudaEventRecord(ls.ev_cross, st);
    cudaStreamWaitEvent(sp, ls.ev_cross, 0);
    inverse(0);
    if (!w21(0)) return 1;
    cudaEventRecord(ls.ev_rest, st);
    for (int k = 0; k < nblk; ++k) {
        cudaStreamWaitEvent(st, ls.ev_panel, 0);
        const int k0 = k * NB, rem = n - k0 - NB;
        if (rem <= 0) break;
        const int mt = rem / NB;
        mark(k, 0, st);
        // panel stream: block (k+1, k+1) needs the rest update of step k-1 and step k's
        // operands, then its inverse
        cudaStreamWaitEvent(sp, ls.ev_rest, 0);
        if (!tc_update_rect(sp, n, k0, A, wlb(k), wutb(k), 0, 0, 1, 1, 0, flags, 0)) return 1;
        inverse(k + 1);
        // main stream: the rest of block column k+1 and block row k+1 (one L-shaped launch)
        if (!tc_update_rect(st, n, k0, A, wlb(k), wutb(k), 0, 0, mt, mt, 0, flags, 2)) return 1;
        cudaEventRecord(ls.ev_cross, st);
        mark(k, 1, st);
        cudaStreamWaitEvent(sp, ls.ev_cross, 0);
        if (!w21(k + 1)) return 1;
        if (mt > 1 &&
            !tc_update_rect(st, n, k0, A, wlb(k), wutb(k), NB, NB, mt - 1, mt - 1, rest_ctas, flags, 0))
            return 1;
        cudaEventRecord(ls.ev_rest, st);
        mark(k, 5, st);
    }
    // the last W21 stores and U-column transforms precede the solves
    cudaEventRecord(ls.ev_panel, sp);
    cudaStreamWaitEvent(st, ls.ev_panel, 0);
    if (ls.panel_tail) {
        cudaEventRecord(ls.ev_panel, sq);
        cudaStreamWaitEvent(st, ls.ev_panel, 0);
    }
    if (nblk > 1 && ls.ucol_own) {
        cudaEventRecord(ls.ev_ucol, ls.ucol);
        cudaStreamWaitEvent(st, ls.ev_ucol, 0);
    }
    return lu_pair_fold(st, n, A, ls.pair_t, flags);
}

// The same factorization with the trailing updates of two consecutive steps applied
// in one pass over the trailing matrix (K = 256), which halves the HBM traffic of the
// update-bound first half of the LU.  Per pair of steps (k, k+1), k even:
//   main stream:  L1(k): block column / row k+1 by step k (width-1 L, corner excluded);
//                 L2(k): block columns / rows k+2, k+3 by steps k and k+1 (width-2 L,
//                 corner (k+2, k+2) excluded), once the previous pair's rest is done;
//   panel stream: corner (k+1, k+1) by step k, inverse k+1, first W21 tile of k+1;
//                 then corner (k+2, k+2) by steps k and k+1, inverse k+2, first tile of k+2;
//   tail stream:  the other W21 / U^T tiles of each panel;
//   rest stream:  blocks >= k+4 by steps k and k+1, beside L1(k+2) and panel k+3.
// Operand buffers rotate over four slots (step k uses slot k & 3): a slot is rewritten
// by panel k+4, which follows L2(k+2), which waits for the rest of pair (k, k+1).
// wl4: 4 [2][n][128] buffers (8 n 128 floats); wut4: the same plus the transposed
// block inverses (8 n 128 + 256 n floats).
int lu_factor_f32_paired(cudaStream_t st, const LuStreams& ls, int n, CMat<float> A, float* invr, float* invi,
                         float* wl4, float* wut4, int* flags) {
    constexpr int NB = 128;
    const int nblk = n / NB;
    if (!ls.panel_tail || !ls.rest || !ls.ucol_own) return 1;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int rest_ctas = ls.reserve_sms > 0 ? std::max(1, nsm - ls.reserve_sms) : -std::max(1, ls.rest_tiles);
    auto wlb = [&](int k) { return wl4 + (size_t)(k & 3) * 2 * n * NB; };
    auto wutb = [&](int k) { return wut4 + (size_t)(k & 3) * 2 * n * NB; };
    auto dTb = [&](int k) { return wut4 + (size_t)8 * n * NB + (size_t)k * 2 * NB * NB; };
    cudaStream_t sp = ls.panel, sq = ls.panel_tail, sr = ls.rest;
    cudaEvent_t ev_pan[2] = {ls.ev_panel, ls.ev_panel2};
    if (ls.cluster_inverse >= 2) inv128_cluster_setup();
    auto inverse = [&](int k) {
        const int k0 = k * NB;
        if (ls.cluster_inverse >= 2)
            inv128_cluster(sp, ls.cluster_inverse, ls.block_inverse, k0, A, invr, invi, dTb(k), flags, ls.pdl);
        else
            BEM_LAUNCH(k_inv128<<<1, IV_THREADS, 0, sp>>>(k0, A, invr, invi, dTb(k), flags));
    };
    // panel k after the update that completed block column / row k (event ready; sp has
    // waited for it): first W21 tile on sp, first U^T tile on sq, the rest on sq
    auto panel = [&](int k, cudaEvent_t ready) -> bool {
        const int k0 = k * NB, rem = n - k0 - NB;
        auto w21_tiles = [&](cudaStream_t s, int t0, int count, int pdl = 0) {
            return tc_w21(s, n, k0, A, dTb(k), wlb(k), flags, t0, count, pdl);
        };
        auto tr_tiles = [&](cudaStream_t s, int t0, int count) {
            const int c0 = t0 * NB, cols = std::min(rem - c0, count < 0 ? rem : count * NB);
            if (cols <= 0) return;
            float* wtr = wutb(k) + (size_t)c0 * NB;
            BEM_LAUNCH(k_panel_transpose<<<dim3((cols + 31) / 32, NB / 32), dim3(32, 8), 0, s>>>(
                cols, A, k0, k0 + NB + c0, wtr, wtr + (size_t)n * NB));
        };
        cudaStreamWaitEvent(sq, ready, 0);
        tr_tiles(sq, 0, 1);
        cudaEventRecord(ls.ev_t0, sq);
        if (!w21_tiles(sp, 0, 1, ls.pdl)) return false;
        cudaStreamWaitEvent(sp, ls.ev_t0, 0);
        cudaEventRecord(ls.ev_head, sp);
        cudaStreamWaitEvent(sq, ls.ev_head, 0);
        if (!w21_tiles(sq, 1, -1)) return false;
        tr_tiles(sq, 1, -1);
        cudaEventRecord(ev_pan[k & 1], sq);
        if (k > 0) {
            cudaStreamWaitEvent(ls.ucol, ev_pan[k & 1], 0);
            if (!tc_ucol(ls.ucol, n, k0, A, dTb(k), ls.ucol_ctas, flags)) return false;
        }
        return true;
    };
    bool rest_used = false;
    cudaEventRecord(ls.ev_cross, st);
    cudaEventRecord(ls.ev_rest, st);
    cudaStreamWaitEvent(sp, ls.ev_cross, 0);
    inverse(0);
    if (!panel(0, ls.ev_cross)) return 1;
    for (int k = 0; k <= nblk - 2; k += 2) {
        const bool pair = k + 1 <= nblk - 2;
        const int mt = nblk - k - 1;
        // step k on block column / row k+1
        cudaStreamWaitEvent(st, ev_pan[k & 1], 0);
        if (!tc_update_pair(st, n, A, (k + 1) * NB, (k + 1) * NB, mt, mt, 1, 1, 0, flags, wlb(k), wutb(k), 0, 0,
                            nullptr, nullptr, 0, 0))
            return 1;
        cudaEventRecord(ls.ev_cross, st);
        if (!tc_update_pair(sp, n, A, (k + 1) * NB, (k + 1) * NB, 1, 1, 0, 0, 0, flags, wlb(k), wutb(k), 0, 0,
                            nullptr, nullptr, 0, 0))
            return 1;
        inverse(k + 1);
        cudaStreamWaitEvent(sp, ls.ev_cross, 0);
        if (!panel(k + 1, ls.ev_cross)) return 1;
        if (!pair) break;
        // steps k and k+1 on block columns / rows k+2, k+3
        const int o = k + 2, nr = nblk - o, w = std::min(2, nr);
        cudaStreamWaitEvent(st, ev_pan[(k + 1) & 1], 0);
        cudaStreamWaitEvent(st, ls.ev_rest, 0);
        if (!tc_update_pair(st, n, A, o * NB, o * NB, nr, nr, w, 1, 0, flags, wlb(k), wutb(k), NB, NB, wlb(k + 1),
                            wutb(k + 1), 0, 0))
            return 1;
        cudaEventRecord(ls.ev_cross2, st);
        cudaStreamWaitEvent(sp, ls.ev_rest, 0);
        cudaStreamWaitEvent(sp, ev_pan[k & 1], 0);
        if (!tc_update_pair(sp, n, A, o * NB, o * NB, 1, 1, 0, 0, 0, flags, wlb(k), wutb(k), NB, NB, wlb(k + 1),
                            wutb(k + 1), 0, 0))
            return 1;
        inverse(o);
        cudaStreamWaitEvent(sp, ls.ev_cross2, 0);
        if (!panel(o, ls.ev_cross2)) return 1;
        // steps k and k+1 on blocks >= k+4
        if (nr > 2) {
            cudaStreamWaitEvent(sr, ev_pan[(k + 1) & 1], 0);
            if (!tc_update_pair(sr, n, A, (o + 2) * NB, (o + 2) * NB, nr - 2, nr - 2, 0, 0, rest_ctas, flags, wlb(k),
                                wutb(k), 3 * NB, 3 * NB, wlb(k + 1), wutb(k + 1), 2 * NB, 2 * NB))
                return 1;
            cudaEventRecord(ls.ev_rest, sr);
            rest_used = true;
        }
    }
    // join every stream back into st: the last W21 stores, transforms and updates precede the solves
    cudaEventRecord(ls.ev_cross, sp);
    cudaStreamWaitEvent(st, ls.ev_cross, 0);
    cudaEventRecord(ls.ev_cross2, sq);
    cudaStreamWaitEvent(st, ls.ev_cross2, 0);
    if (rest_used) cudaStreamWaitEvent(st, ls.ev_rest, 0);
    if (nblk > 1) {
        cudaEventRecord(ls.ev_ucol, ls.ucol);
        cudaStreamWaitEvent(st, ls.ev_ucol, 0);
    }
    return lu_pair_fold(st, n, A, ls.pair_t, flags);
}

int lu_factor_f64(cudaStream_t st, int n, CMat<double> A, double* invr, double* invi, double* wl, double* wu,
                  int* flags) {
    (void)wu;
    return lu_factor_t<double, 64>(st, n, A, invr, invi, wl, flags);
}

// ---------------------------------------------------------------------------
// Cooperative block triangular solve: one CTA per diagonal block (rounds if the
// grid is smaller than the block count).  CTA b accumulates
//     z_b = y_b - sum_{c before b} A_bc x_c
// taking the x_c as soon as their CTAs publish them (epoch flags with release /
// acquire ordering).  Forward (which = 0): block-unit-lower L (blocks W), c < b,
// x_b = z_b.  Backward (which = 1): block-upper U, c > b, x_b = D_bb^-1 z_b.  The
// launch is cooperative, so every CTA is resident and every wait is on a CTA
// that is running or finished; the waits are bounded all the same and record
// FLAG_TIMEOUT if they expire.
template <typename T, int NB, int TPR>
__global__ void __launch_bounds__(NB * TPR) k_trsv_coop(int nblk, int R, CMat<T> A, const T* __restrict__ invr,
                                                        const T* __restrict__ invi, int which,
                                                        const T* __restrict__ Yin, T* __restrict__ Xout,
                                                        int* __restrict__ ready, int epoch, int* __restrict__ gflags) {
    constexpr int NT = NB * TPR;
    constexpr int JPT = (MAX_RHS + TPR - 1) / TPR;  // RHS columns per thread
    constexpr int LP = NB + 16 / (int)sizeof(T);    // padded tile row (16-byte aligned)
    constexpr int CH = 16 / (int)sizeof(T);         // elements per 16-byte chunk
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* Lr = reinterpret_cast<T*>(smem_raw);         // [NB][LP]
    T* Li = Lr + NB * LP;
    T* zr = Li + NB * LP;                           // [NB][MAX_RHS]
    T* zi = zr + NB * MAX_RHS;
    __shared__ int timed_out;
    const int tid = threadIdx.x;
    const int i = tid / TPR, jq = tid % TPR;  // row within the block, RHS phase
    if (tid == 0) timed_out = 0;
    // cp.async of an NB x NB tile (row-major, stride ld) into Lr/Li
    auto issue_tile = [&](const T* gr, const T* gi, size_t ldg) {
        for (int idx = tid; idx < NB * (NB / CH); idx += NT) {
            int rr = idx / (NB / CH), cc = (idx % (NB / CH)) * CH;
            unsigned dr = (unsigned)__cvta_generic_to_shared(Lr + rr * LP + cc);
            unsigned di = (unsigned)__cvta_generic_to_shared(Li + rr * LP + cc);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dr), "l"(gr + rr * ldg + cc) : "memory");
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(di), "l"(gi + rr * ldg + cc) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    for (int round = blockIdx.x; round < nblk; round += gridDim.x) {
        const int b = which == 0 ? round : nblk - 1 - round;
        const size_t row = (size_t)b * NB + i;
        T ar_[JPT], ai_[JPT];
#pragma unroll
        for (int u = 0; u < JPT; ++u) {
            int j = jq + u * TPR;
            ar_[u] = j < R ? Yin[2 * (row * R + j)] : (T)0;
            ai_[u] = j < R ? Yin[2 * (row * R + j) + 1] : (T)0;
        }
        const int cnt = which == 0 ? b : nblk - 1 - b;
        for (int t = 0; t < cnt; ++t) {
            const int c = which == 0 ? t : nblk - 1 - t;
            const size_t goff = (size_t)b * NB * A.ld + (size_t)c * NB;
            issue_tile(A.re + goff, A.im + goff, A.ld);   // overlaps with the wait below
            if (tid == 0) {
                int v = 0;
                long it = 0;
                for (;;) {
                    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(ready + c) : "memory");
                    if (v >= epoch || timed_out) break;
                    if (++it > (1L << 26)) { timed_out = 1; atomicOr(gflags, FLAG_TIMEOUT); break; }
                }
                __threadfence();
            }
            __syncthreads();
            for (int idx = tid; idx < NB * R; idx += NT) {
                size_t o = 2 * (((size_t)c * NB) * R + idx);
                int k = idx / R, j = idx % R;
                zr[k * MAX_RHS + j] = __ldcg(Xout + o);
                zi[k * MAX_RHS + j] = __ldcg(Xout + o + 1);
            }
            asm volatile("cp.async.wait_all;" ::: "memory");
            __syncthreads();
            const T* lr = Lr + i * LP;
            const T* li = Li + i * LP;
#pragma unroll 4
            for (int k = 0; k < NB; ++k) {
                T mr = lr[k], mi = li[k];
#pragma unroll
                for (int u = 0; u < JPT; ++u) {
                    int j = jq + u * TPR;
                    if (j < R) {
                        T vr = zr[k * MAX_RHS + j], vi = zi[k * MAX_RHS + j];
                        ar_[u] -= mr * vr - mi * vi;
                        ai_[u] -= mr * vi + mi * vr;
                    }
                }
            }
            __syncthreads();
        }
        if (which == 1) {
            // x_b = D_bb^-1 z_b
            const size_t ioff = (size_t)b * NB * NB;
            issue_tile(invr + ioff, invi + ioff, NB);
#pragma unroll
            for (int u = 0; u < JPT; ++u) {
                int j = jq + u * TPR;
                if (j < R) { zr[i * MAX_RHS + j] = ar_[u]; zi[i * MAX_RHS + j] = ai_[u]; }
            }
            asm volatile("cp.async.wait_all;" ::: "memory");
            __syncthreads();
#pragma unroll
            for (int u = 0; u < JPT; ++u) { ar_[u] = 0; ai_[u] = 0; }
            const T* mrow = Lr + i * LP;
            const T* mirow = Li + i * LP;
#pragma unroll 4
            for (int k = 0; k < NB; ++k) {
                T mr = mrow[k], mi = mirow[k];
#pragma unroll
                for (int u = 0; u < JPT; ++u) {
                    int j = jq + u * TPR;
                    if (j < R) {
                        T vr = zr[k * MAX_RHS + j], vi = zi[k * MAX_RHS + j];
                        ar_[u] += mr * vr - mi * vi;
                        ai_[u] += mr * vi + mi * vr;
                    }
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int u = 0; u < JPT; ++u) {
            int j = jq + u * TPR;
            if (j < R) {
                Xout[2 * (row * R + j)] = ar_[u];
                Xout[2 * (row * R + j) + 1] = ai_[u];
            }
        }
        __syncthreads();  // all stores of the block, then one fence + release store of its flag
        if (tid == 0) {
            __threadfence();
            asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(ready + b), "r"(epoch) : "memory");
        }
    }
}

template <typename T, int NB, int TPR>
static int trsv_coop(cudaStream_t st, int n, CMat<T> A, const T* invr, const T* invi, int which, int R,
                     const T* Y, T* X, int* ready, int epoch, int* flags) {
    const int nblk = n / NB;
    int dev = 0, nsm = 0, per_sm = 0;
    constexpr int LP = NB + 16 / (int)sizeof(T);
    const size_t smem = sizeof(T) * (2 * (size_t)NB * LP + 2 * (size_t)NB * MAX_RHS);
    cudaFuncSetAttribute(k_trsv_coop<T, NB, TPR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_coop<T, NB, TPR>, NB * TPR, smem);
    int grid = std::min(nblk, std::max(1, per_sm) * nsm);
    void* args[] = {(void*)&nblk, (void*)&R, (void*)&A, (void*)&invr, (void*)&invi, (void*)&which, (void*)&Y,
                    (void*)&X, (void*)&ready, (void*)&epoch, (void*)&flags};
    ++g_launches;
    ++t_launches;
    return cudaLaunchCooperativeKernel((void*)k_trsv_coop<T, NB, TPR>, dim3(grid), dim3(NB * TPR), args, smem, st) ==
                   cudaSuccess
               ? 0
               : 1;
}

// ---------------------------------------------------------------------------
// FP32 block triangular solves of the pair-folded factors (lu_pair_fold).  Both are
// chains over super-blocks of 256 rows whose diagonal blocks are the identity:
//   which = 0 (forward, L''):   y_b = v_b - sum_{c<b} L''_bc y_c
//   which = 1 (backward, U''):  z_b = v_b - sum_{c>b} U''_bc z_c
// k_pair_apply then applies P^-1 (resp. Q^-1), one independent 128 x 128 product per
// pair, and the backward solve ends with the block-diagonal D^-1 (k_dinv_apply), so
// nothing on either chain waits for a block inverse.  The last super-block has 128 rows
// when n / 128 is odd.
// A super-block is shared by 32 CTAs of 8 rows (sub-blocks), so the product on the
// critical path (one 8 x 256 tile against the newest super-block of x) is small.
// Thread (i, s) = (tid % 8, tid / 8) owns row i of the sub-block and the 8 columns s*8..
// of every tile; the tile is prefetched into registers one dependency ahead, and the
// super-blocks of x are staged in shared memory by cp.async, double-buffered: while a
// CTA multiplies one tile, the next is already in flight whenever its producer has
// published it.  The 32 column slices are summed once at the end (warp shuffles, then
// shared memory).  Yin and Xout may be the same array: a CTA reads its own rows of Yin
// before it writes them, and other super-blocks' rows of Xout only after their flags.
// xflag[u] (u = sub-block) is raised to `epoch` when the rows of u are in memory; one
// warp polls the 32 flags of a super-block at once.  Waits give up at a 2 s deadline
// (FLAG_TIMEOUT).
// Scheduling needs no co-residency (plain launch, one CTA per sub-block): each CTA
// draws a ticket when it starts and tickets map to sub-blocks in dependency order, so
// a CTA waits only on sub-blocks of CTAs that started before it.  The lowest unfinished
// ticket therefore always progresses, whatever else runs on the GPU.  The CTA that
// draws the last ticket resets the counter.  Three CTAs fit on an SM (80 registers): a
// chain that shares the GPU with a persistent assembly kernel keeps more CTAs resident.
constexpr int TS_NB = 256, TS_RW = 8, TS_SB = TS_NB / TS_RW, TS_THREADS = 256, TS_SL = TS_THREADS / TS_RW,
              TS_KC = TS_NB / TS_SL, TS_WARPS = TS_THREADS / 32;
// k_pair_apply and k_dinv_apply: 128-row blocks, 8 CTAs of 16 rows, 16 column slices of 8
constexpr int DA_NB = 128, DA_RW = 16, DA_SB = DA_NB / DA_RW, DA_SL = TS_THREADS / DA_RW, DA_KC = DA_NB / DA_SL;
static_assert(TS_KC == 8 && DA_KC == 8 && TS_SB == 32, "rows are read 8 floats at a time; one warp polls a super-block");

__device__ __forceinline__ unsigned long long ts_now() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void ts_wait(const int* f, int epoch, unsigned long long deadline, int& dead,
                                        int* gflags) {
    if (dead) return;
    // the timer is read once per 256 polls: a %globaltimer read costs far more than a poll
    for (int i = 1;; ++i) {
        int v;
        asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(f) : "memory");
        if (v >= epoch) return;
        if ((i & 255) == 0 && ts_now() > deadline) { dead = 1; atomicOr(gflags, FLAG_TIMEOUT); return; }
    }
}

__device__ __forceinline__ bool ts_ready(const int* f, int epoch) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(f) : "memory");
    return v >= epoch;
}

__device__ __forceinline__ void ld_row8(const float* __restrict__ gr, const float* __restrict__ gi, float* r,
                                        float* im) {
#pragma unroll
    for (int v = 0; v < 2; ++v) {
        float4 a = __ldg(reinterpret_cast<const float4*>(gr) + v);
        float4 b = __ldg(reinterpret_cast<const float4*>(gi) + v);
        r[4 * v] = a.x; r[4 * v + 1] = a.y; r[4 * v + 2] = a.z; r[4 * v + 3] = a.w;
        im[4 * v] = b.x; im[4 * v + 1] = b.y; im[4 * v + 2] = b.z; im[4 * v + 3] = b.w;
    }
}

// Floats of one staging buffer: a rows x R complex block in its global layout, plus RC
// complex of zero padding (rows are read RC wide), rounded to 16 bytes.
__host__ __device__ constexpr int ts_zstride(int rows, int R, int RC) { return ((2 * (rows * R + RC)) + 3) & ~3; }

template <int RC>
__global__ void __launch_bounds__(TS_THREADS, 3) k_trsv_tk(int n, int R, CMat<float> A, int which,
                                                        float* Yin, float* Xout, int* xflag, int* ticket,
                                                        int epoch, int* gflags, int wait_skew,
                                                        unsigned long long wait_ns) {
    extern __shared__ __align__(16) float ts_smem[];
    __shared__ int s_ticket, s_go;
    const int zs = ts_zstride(TS_NB, R, RC);
    float* zb = ts_smem;                             // [2][zs]
    float* red = zb + 2 * zs;                        // [TS_WARPS][TS_RW][RC] complex interleaved
    float* ybase = red + TS_WARPS * TS_RW * RC * 2;  // [TS_RW][R] complex: this sub-block's rows of Yin
    const int tid = threadIdx.x, lane = tid % TS_RW, s = tid / TS_RW, wl = tid & 31;
    const int nsub = n / TS_RW, nsb = (n + TS_NB - 1) / TS_NB;
    // wait_skew > 0 (failure-detection tests only) makes every wait ask for a flag value
    // nothing publishes, so each wait runs into its deadline (wait_ns from the CTA's start)
    const unsigned long long deadline = ts_now() + wait_ns;
    const int want = epoch + wait_skew;
    int dead = 0;
    if (tid == 0) {
        const int t = atomicAdd(ticket, 1);
        if (t == (int)gridDim.x - 1) atomicExch(ticket, 0);  // every ticket of this launch is drawn
        s_ticket = t;
    }
    for (int idx = 2 * TS_NB * R + tid; idx < zs; idx += blockDim.x) { zb[idx] = 0.f; zb[zs + idx] = 0.f; }
    __syncthreads();
    const int tk = s_ticket;
    const int u = which == 0 ? tk : nsub - 1 - tk;
    const int b = u / TS_SB;
    const size_t row0 = (size_t)u * TS_RW;
    const int cnt = which == 0 ? b : nsb - 1 - b;
    auto cidx = [&](int t) { return which == 0 ? t : nsb - 1 - t; };
    auto width = [&](int c) { return min(TS_NB, n - c * TS_NB); };
    // the sub-block's rows of Yin are static during the launch: fetch them now, off the
    // critical path of the final reduction
    for (int idx = tid; idx < TS_RW * R; idx += blockDim.x)
        reinterpret_cast<float2*>(ybase)[idx] = reinterpret_cast<const float2*>(Yin)[row0 * R + idx];
    // stage the width(c) x R block of x at super-block c into buffer buf, 16 bytes per cp.async
    auto issue_copy = [&](int c, int buf) {
        const float* src = Xout + (size_t)c * TS_NB * R * 2;
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(zb + buf * zs);
        const int chunks = width(c) * R / 2;
        for (int i = tid; i < chunks; i += blockDim.x)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + 16 * i), "l"(src + 4 * i)
                         : "memory");
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    // every sub-block of super-block c is published: one flag per lane of warp 0
    auto probe = [&](int c) {
        const int k = wl, subs = width(c) / TS_RW;
        const bool ok = k >= subs || ts_ready(xflag + c * TS_SB + k, want);
        return __all_sync(0xffffffffu, ok);
    };
    auto wait_block = [&](int c) {
        if (tid < width(c) / TS_RW) ts_wait(xflag + c * TS_SB + tid, want, deadline, dead, gflags);
    };
    float ar[RC], ai[RC];
#pragma unroll
    for (int j = 0; j < RC; ++j) { ar[j] = 0.f; ai[j] = 0.f; }
    float cr[TS_KC], ci[TS_KC], nr[TS_KC], ni[TS_KC];
    // row lane of this sub-block, columns s*8.. of super-block c (only where c is that wide)
    auto load_tile = [&](int t, float* r, float* im) {
        const int c = cidx(t);
        if (s * TS_KC < width(c)) {
            const size_t off = (row0 + lane) * A.ld + (size_t)c * TS_NB + s * TS_KC;
            ld_row8(A.re + off, A.im + off, r, im);
        }
    };
    // acc -= tile * z (z: a staged super-block)
    auto mac = [&](const float* z, int c) {
        if (s * TS_KC >= width(c)) return;
#pragma unroll
        for (int kk = 0; kk < TS_KC; ++kk) {
            const float lr = -cr[kk], li = -ci[kk];
            const float2* zk = reinterpret_cast<const float2*>(z) + (size_t)(s * TS_KC + kk) * R;
#pragma unroll
            for (int j = 0; j < RC; ++j) {  // columns j >= R read padding or the next row: never stored
                const float2 v = zk[j];
                ar[j] = fmaf(lr, v.x, fmaf(-li, v.y, ar[j]));
                ai[j] = fmaf(lr, v.y, fmaf(li, v.x, ai[j]));
            }
        }
    };
    if (cnt > 0) {
        load_tile(0, cr, ci);
        wait_block(cidx(0));
        __syncthreads();
        issue_copy(cidx(0), 0);
    }
    for (int t = 0; t < cnt; ++t) {
        if (t + 1 < cnt) load_tile(t + 1, nr, ni);
        // start the next super-block's copy now if its producers are done
        bool early = false;
        if (t + 1 < cnt) {
            if (tid < 32) {
                const bool ok = probe(cidx(t + 1));
                if (tid == 0) s_go = ok ? 1 : 0;
            }
            __syncthreads();
            early = s_go != 0;
            if (early) issue_copy(cidx(t + 1), (t + 1) & 1);
        }
        if (early) asm volatile("cp.async.wait_group 1;" ::: "memory");
        else asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();
        mac(zb + (t & 1) * zs, cidx(t));
        __syncthreads();  // buffer t & 1 is refilled for tile t + 2
        if (t + 1 < cnt && !early) {
            wait_block(cidx(t + 1));
            __syncthreads();
            issue_copy(cidx(t + 1), (t + 1) & 1);
        }
#pragma unroll
        for (int kk = 0; kk < TS_KC; ++kk) { cr[kk] = nr[kk]; ci[kk] = ni[kk]; }
    }
    // sum the column slices: the four slices of a warp by shuffles (lanes l, l+8, l+16,
    // l+24 hold row l % 8), then the eight warps through shared memory: out = y + sum
#pragma unroll
    for (int j = 0; j < RC; ++j) {
        ar[j] += __shfl_xor_sync(0xffffffffu, ar[j], 8);
        ai[j] += __shfl_xor_sync(0xffffffffu, ai[j], 8);
        ar[j] += __shfl_xor_sync(0xffffffffu, ar[j], 16);
        ai[j] += __shfl_xor_sync(0xffffffffu, ai[j], 16);
    }
    if (wl < TS_RW) {
        const int w = tid >> 5;
#pragma unroll
        for (int j = 0; j < RC; ++j)
            *reinterpret_cast<float2*>(red + ((w * TS_RW + wl) * RC + j) * 2) = make_float2(ar[j], ai[j]);
    }
    __syncthreads();
    for (int idx = tid; idx < TS_RW * R; idx += blockDim.x) {
        const int i = idx / R, j = idx % R;
        float2 o = reinterpret_cast<const float2*>(ybase)[idx];
#pragma unroll
        for (int w = 0; w < TS_WARPS; ++w) {
            const float2 v = *reinterpret_cast<const float2*>(red + ((w * TS_RW + i) * RC + j) * 2);
            o.x += v.x;
            o.y += v.y;
        }
        reinterpret_cast<float2*>(Xout)[(row0 + i) * R + j] = o;
    }
    // the CTA barrier orders every thread's stores before thread 0's release store of
    // the flag, and release is cumulative: a consumer that acquires the flag sees them
    __syncthreads();
    if (tid == 0) asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(xflag + u), "r"(epoch) : "memory");
}

// The 128-row block products after a chain: CTA (pair or block, 16-row group q),
// thread (i, s) = (tid % 16, tid / 16) multiplies row q*16 + i of a 128 x 128 matrix,
// columns s*8.., against a staged 128 x R block; the 16 column slices are summed
// through shared memory.
template <int RC>
struct BlockRowProduct {
    float ar[RC], ai[RC];
    __device__ void run(const float* __restrict__ mr, const float* __restrict__ mi, const float* zb, float* red,
                        int R, int lane, int s) {
        float cr[DA_KC], ci[DA_KC];
        ld_row8(mr, mi, cr, ci);
        __syncthreads();  // the staged block is complete
#pragma unroll
        for (int j = 0; j < RC; ++j) { ar[j] = 0.f; ai[j] = 0.f; }
#pragma unroll
        for (int kk = 0; kk < DA_KC; ++kk) {
            const float2* zk = reinterpret_cast<const float2*>(zb) + (size_t)(s * DA_KC + kk) * R;
#pragma unroll
            for (int j = 0; j < RC; ++j) {  // columns j >= R read padding or the next row: never stored
                const float2 v = zk[j];
                ar[j] = fmaf(cr[kk], v.x, fmaf(-ci[kk], v.y, ar[j]));
                ai[j] = fmaf(cr[kk], v.y, fmaf(ci[kk], v.x, ai[j]));
            }
        }
#pragma unroll
        for (int j = 0; j < RC; ++j)
            *reinterpret_cast<float2*>(red + ((s * DA_RW + lane) * RC + j) * 2) = make_float2(ar[j], ai[j]);
        __syncthreads();
    }
};

__device__ __forceinline__ void stage_block(const float* __restrict__ src, float* zb, int R, int zs) {
    const float4* s4 = reinterpret_cast<const float4*>(src);
    for (int i = threadIdx.x; i < DA_NB * R / 2; i += blockDim.x) reinterpret_cast<float4*>(zb)[i] = __ldg(s4 + i);
    for (int idx = 2 * DA_NB * R + threadIdx.x; idx < zs; idx += blockDim.x) zb[idx] = 0.f;
}

// The pair products of the folded factors, in place (one 128 x 128 product per pair):
//   which = 0:  x_{2p+1} -= L_{2p+1,2p} x_{2p}               (x = P^-1 y)
//   which = 1:  x_{2p}   -= (U D^-1)_{2p,2p+1} x_{2p+1}      (x = Q^-1 z)
// The pair blocks are in A (the fold keeps them).  A CTA writes rows of its target block
// only and reads the source block, which no CTA of the launch writes.
template <int RC>
__global__ void __launch_bounds__(TS_THREADS) k_pair_apply(int R, CMat<float> A, int which, float* X) {
    extern __shared__ __align__(16) float pa_smem[];
    const int zs = ts_zstride(DA_NB, R, RC);
    float* zb = pa_smem;  // the 128 x R complex source block, then RC complex of zeros
    float* red = zb + zs; // [DA_SL][DA_RW][RC] complex interleaved
    const int tid = threadIdx.x, lane = tid % DA_RW, s = tid / DA_RW;
    const int p = blockIdx.x / DA_SB, q = blockIdx.x % DA_SB;
    const int tgt = which == 0 ? 2 * p + 1 : 2 * p, src = which == 0 ? 2 * p : 2 * p + 1;
    stage_block(X + (size_t)src * DA_NB * R * 2, zb, R, zs);
    const size_t row0 = (size_t)tgt * DA_NB + q * DA_RW;
    const size_t off = (row0 + lane) * A.ld + (size_t)src * DA_NB + s * DA_KC;
    BlockRowProduct<RC> prod;
    prod.run(A.re + off, A.im + off, zb, red, R, lane, s);
    for (int idx = tid; idx < DA_RW * R; idx += blockDim.x) {
        const int i = idx / R, j = idx % R;
        float2 o = reinterpret_cast<const float2*>(X)[(row0 + i) * R + j];
#pragma unroll
        for (int w = 0; w < DA_SL; ++w) {
            const float2 v = *reinterpret_cast<const float2*>(red + ((w * DA_RW + i) * RC + j) * 2);
            o.x -= v.x;
            o.y -= v.y;
        }
        reinterpret_cast<float2*>(X)[(row0 + i) * R + j] = o;
    }
}

// x_b = D_b^-1 z_b for every 128-row block b.  Z and X must not overlap.
template <int RC>
__global__ void __launch_bounds__(TS_THREADS) k_dinv_apply(int R, const float* __restrict__ invr,
                                                           const float* __restrict__ invi,
                                                           const float* __restrict__ Z, float* __restrict__ X) {
    extern __shared__ __align__(16) float da_smem[];
    const int zs = ts_zstride(DA_NB, R, RC);
    float* zb = da_smem;  // the 128 x R complex block of z, then RC complex of zeros
    float* red = zb + zs; // [DA_SL][DA_RW][RC] complex interleaved
    const int tid = threadIdx.x, lane = tid % DA_RW, s = tid / DA_RW;
    const int b = blockIdx.x / DA_SB, q = blockIdx.x % DA_SB;
    const size_t row0 = (size_t)b * DA_NB + q * DA_RW;
    stage_block(Z + (size_t)b * DA_NB * R * 2, zb, R, zs);
    const size_t off = (size_t)b * DA_NB * DA_NB + (size_t)(q * DA_RW + lane) * DA_NB + s * DA_KC;
    BlockRowProduct<RC> prod;
    prod.run(invr + off, invi + off, zb, red, R, lane, s);
    for (int idx = tid; idx < DA_RW * R; idx += blockDim.x) {
        const int i = idx / R, j = idx % R;
        float2 o = make_float2(0.f, 0.f);
#pragma unroll
        for (int w = 0; w < DA_SL; ++w) {
            const float2 v = *reinterpret_cast<const float2*>(red + ((w * DA_RW + i) * RC + j) * 2);
            o.x += v.x;
            o.y += v.y;
        }
        reinterpret_cast<float2*>(X)[(row0 + i) * R + j] = o;
    }
}

// Forward chain, P^-1, backward chain (in place over the forward's output), Q^-1 and
// the block-diagonal D^-1, for one column count RC >= R.
template <int RC>
static int trsv_tk_launch(cudaStream_t st, int n, CMat<float> A, const float* invr, const float* invi, int R,
                          float* X, float* tmp, int* xflag, int* ticket, int epoch, int* flags, int skew,
                          unsigned long long wait_ns) {
    const int nsub = n / TS_RW, np = n / 256, nblk = n / DA_NB;
    const size_t smem =
        sizeof(float) * (2 * (size_t)ts_zstride(TS_NB, R, RC) + TS_WARPS * TS_RW * RC * 2 + TS_RW * 2 * R);
    const size_t smem_d = sizeof(float) * ((size_t)ts_zstride(DA_NB, R, RC) + DA_SL * DA_RW * RC * 2);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(k_trsv_tk<RC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (smem_d > 48 * 1024) {
        cudaFuncSetAttribute(k_dinv_apply<RC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_d);
        cudaFuncSetAttribute(k_pair_apply<RC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_d);
    }
    BEM_LAUNCH(k_trsv_tk<RC><<<nsub, TS_THREADS, smem, st>>>(n, R, A, 0, X, tmp, xflag, ticket, epoch, flags, skew,
                                                              wait_ns));
    if (np > 0) BEM_LAUNCH(k_pair_apply<RC><<<np * DA_SB, TS_THREADS, smem_d, st>>>(R, A, 0, tmp));
    BEM_LAUNCH(k_trsv_tk<RC><<<nsub, TS_THREADS, smem, st>>>(n, R, A, 1, tmp, tmp, xflag, ticket, epoch + 1,
                                                              flags, skew, wait_ns));
    if (np > 0) BEM_LAUNCH(k_pair_apply<RC><<<np * DA_SB, TS_THREADS, smem_d, st>>>(R, A, 1, tmp));
    BEM_LAUNCH(k_dinv_apply<RC><<<nblk * DA_SB, TS_THREADS, smem_d, st>>>(R, invr, invi, tmp, X));
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 1;
}

static int trsv_tk(cudaStream_t st, int n, CMat<float> A, const float* invr, const float* invi, int R, float* X,
                   float* tmp, int* xflag, int* ticket, int epoch, int* flags, int sk, unsigned long long wns) {
    switch ((R + 1) / 2) {
        case 1: return trsv_tk_launch<2>(st, n, A, invr, invi, R, X, tmp, xflag, ticket, epoch, flags, sk, wns);
        case 2: return trsv_tk_launch<4>(st, n, A, invr, invi, R, X, tmp, xflag, ticket, epoch, flags, sk, wns);
        case 3: return trsv_tk_launch<6>(st, n, A, invr, invi, R, X, tmp, xflag, ticket, epoch, flags, sk, wns);
        case 4: return trsv_tk_launch<8>(st, n, A, invr, invi, R, X, tmp, xflag, ticket, epoch, flags, sk, wns);
        case 5: return trsv_tk_launch<10>(st, n, A, invr, invi, R, X, tmp, xflag, ticket, epoch, flags, sk, wns);
        case 6: return trsv_tk_launch<12>(st, n, A, invr, invi, R, X, tmp, xflag, ticket, epoch, flags, sk, wns);
        case 7: return trsv_tk_launch<14>(st, n, A, invr, invi, R, X, tmp, xflag, ticket, epoch, flags, sk, wns);
        case 8: return trsv_tk_launch<16>(st, n, A, invr, invi, R, X, tmp, xflag, ticket, epoch, flags, sk, wns);
        default: return 1;
    }
}

// The solve needs an n x R scratch; it lives right after X (caller allocates 2 n R).
// ready: n/nb ints, zero at allocation; epoch: strictly increasing per call (2 used per call).
int lu_solve_f64(cudaStream_t st, int n, CMat<double> A, const double* invr, const double* invi, int R, double* X,
                 int* ready, int epoch, int* flags) {
    double* tmp = X + (size_t)2 * n * R;
    if (trsv_coop<double, 64, 8>(st, n, A, invr, invi, 0, R, X, tmp, ready, epoch, flags)) return 1;
    return trsv_coop<double, 64, 8>(st, n, A, invr, invi, 1, R, tmp, X, ready, epoch + 1, flags);
}
int lu_solve_f32(cudaStream_t st, int n, CMat<float> A, const float* invr, const float* invi, int R, float* X,
                 int* ready, int epoch, int* flags, int wait_skew, unsigned long long wait_ns) {
    // ready holds n / TS_RW flags (one per 8-row sub-block) and a ticket counter, zero
    // between launches.  A is in the pair-folded form of lu_pair_fold, D^-1 in invr / invi.
    float* tmp = X + (size_t)2 * n * R;
    int* xflag = ready;
    int* ticket = ready + n / TS_RW;
    // Solves of several contexts may run at once on one GPU: a CTA waits only on
    // sub-blocks of lower tickets of its own launch, which are already running.
    return trsv_tk(st, n, A, invr, invi, R, X, tmp, xflag, ticket, epoch, flags, wait_skew, wait_ns);
}

// ---------------------------------------------------------------------------
// ---------------------------------------------------------------------------
// P = M X for an N x N row-major matrix M (real, or complex planar when Mi is
// given) and an N x R complex block X: a skinny, HBM-bound product.  Phase 1:
// CTA (row tile of 64, column chunk of 512) stages its X chunk in shared
// memory (planar per column, so lanes read consecutive words) and writes
// partial sums for its 64 rows; each element of M is read once.  Phase 2 sums
// the chunks: out = beta * base + alpha * P  (base may alias out).
constexpr int MX_ROWS = 64, MX_COLS = 512;

template <bool CPLX>
__global__ void __launch_bounds__(256) k_matx_partial(int N, int ld, const double* __restrict__ Mr,
                                                      const double* __restrict__ Mi, int R, int j0,
                                                      const double* __restrict__ X, int xstride,
                                                      double* __restrict__ part) {
    extern __shared__ double xs[];  // [2][R][MX_COLS]
    const int rt = blockIdx.x, ct = blockIdx.y;
    const int s0 = ct * MX_COLS;
    const int ns = min(MX_COLS, N - s0);
    for (int idx = threadIdx.x; idx < R * MX_COLS; idx += blockDim.x) {
        int j = idx / MX_COLS, k = idx % MX_COLS;
        double vr = 0, vi = 0;
        if (k < ns) {
            const double* x = X + 2 * ((size_t)(s0 + k) * xstride + j0 + j);
            vr = x[0]; vi = x[1];
        }
        xs[(size_t)j * MX_COLS + k] = vr;
        xs[(size_t)(R + j) * MX_COLS + k] = vi;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int rr = warp; rr < MX_ROWS; rr += 8) {
        const int r = rt * MX_ROWS + rr;
        if (r >= N) break;
        double ar[MAX_RHS], ai[MAX_RHS];
#pragma unroll
        for (int j = 0; j < MAX_RHS; ++j) { ar[j] = 0; ai[j] = 0; }
        const double* mr = Mr + (size_t)r * ld + s0;
        const double* mi = CPLX ? Mi + (size_t)r * ld + s0 : nullptr;
        for (int k = lane; k < ns; k += 32) {
            double a = mr[k];
            double b = CPLX ? mi[k] : 0.0;
#pragma unroll
            for (int j = 0; j < MAX_RHS; ++j) {
                if (j < R) {
                    double xr = xs[(size_t)j * MX_COLS + k], xi = xs[(size_t)(R + j) * MX_COLS + k];
                    ar[j] = fma(a, xr, ar[j]);
                    ai[j] = fma(a, xi, ai[j]);
                    if (CPLX) {
                        ar[j] = fma(-b, xi, ar[j]);
                        ai[j] = fma(b, xr, ai[j]);
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < MAX_RHS; ++j) {
            if (j < R) {
                double vr = ar[j], vi = ai[j];
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    vr += __shfl_xor_sync(0xffffffffu, vr, off);
                    vi += __shfl_xor_sync(0xffffffffu, vi, off);
                }
                if (lane == 0) {
                    double* p = part + 2 * (((size_t)ct * N + r) * R + j);
                    p[0] = vr;
                    p[1] = vi;
                }
            }
        }
    }
}

// out[r][j0 + j] = beta * base[r][j0 + j] + alpha * sum_c part[c][r][j]   (stride ostride)
__global__ void k_matx_reduce(int N, int R, int nchunk, const double* __restrict__ part, double alpha, double beta,
                              const double* base, double* out, int j0, int ostride) {
    size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (idx >= (size_t)N * R) return;
    int r = (int)(idx / R), j = (int)(idx % R);
    double sr = 0, si = 0;
    for (int c = 0; c < nchunk; ++c) {
        const double* p = part + 2 * (((size_t)c * N + r) * R + j);
        sr += p[0];
        si += p[1];
    }
    size_t o = 2 * ((size_t)r * ostride + j0 + j);
    double br = 0, bi = 0;
    if (beta != 0.0) { br = base[o]; bi = base[o + 1]; }
    out[o] = beta * br + alpha * sr;
    out[o + 1] = beta * bi + alpha * si;
}

// ---------------------------------------------------------------------------
// Double-float products M X for a real N x N matrix held as float pairs
// (m = mhi + mlo) and a complex N x R block X.  GB300's FP64 rate is 1/64 of its
// FP32 rate, so the refinement residual (M = Re D) and the static right-hand
// side (M = the Rankine source matrix) are formed with float pairs:
// x = xhi + xlo; each product as p + e with e exact from an FMA, sums with
// Knuth's two-sum compensation.  One thread per matrix row, so the X chunk is a
// shared-memory broadcast and no cross-lane reduction is needed; each thread's
// pair goes to FP64 once per 256-column chunk and the chunks are summed by
// k_matx_reduce.
constexpr int MXD_ROWS = 128, MXD_COLS = 256;

__global__ void k_split_df(int N, int R, const double* __restrict__ X, int xstride, int j0,
                           float4* __restrict__ Xdf) {
    const size_t n = (size_t)N * R;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / R, j = i % R;
        const double re = X[2 * (r * xstride + j0 + j)], im = X[2 * (r * xstride + j0 + j) + 1];
        const float rh = (float)re, ih = (float)im;
        Xdf[i] = make_float4(rh, (float)(re - (double)rh), ih, (float)(im - (double)ih));
    }
}

__global__ void k_split_mat_df(size_t n, const double* __restrict__ M, float* __restrict__ hi, float* __restrict__ lo) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double v = M[i];
        const float h = (float)v;
        hi[i] = h;
        lo[i] = (float)(v - (double)h);
    }
}

struct DF { float s, c; };
__device__ __forceinline__ void df_mac(DF& acc, float dh, float dl, float xh, float xl) {
    float p = dh * xh;
    float e = fmaf(dh, xh, -p);
    e = fmaf(dh, xl, fmaf(dl, xh, e));
    float t = acc.s + p;
    float z = t - acc.s;
    acc.c += ((acc.s - (t - z)) + (p - z)) + e;
    acc.s = t;
}

template <int RR>
__global__ void __launch_bounds__(MXD_ROWS) k_matx_df(int N, int ld, const float* __restrict__ Mhi,
                                                      const float* __restrict__ Mlo,
                                                      const float4* __restrict__ Xdf, double* __restrict__ part) {
    extern __shared__ float4 xs4[];  // [MXD_COLS][RR]
    const int ct = blockIdx.y;
    const int s0 = ct * MXD_COLS;
    const int ns = min(MXD_COLS, N - s0);
    for (int idx = threadIdx.x; idx < RR * MXD_COLS; idx += blockDim.x) {
        const int k = idx / RR, j = idx % RR;
        xs4[idx] = k < ns ? Xdf[(size_t)(s0 + k) * RR + j] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    const int r = blockIdx.x * MXD_ROWS + threadIdx.x;
    if (r >= N) return;
    DF ar[RR], ai[RR];
#pragma unroll
    for (int j = 0; j < RR; ++j) { ar[j] = DF{0.f, 0.f}; ai[j] = DF{0.f, 0.f}; }
    const float* hrow = Mhi + (size_t)r * ld + s0;
    const float* lrow = Mlo + (size_t)r * ld + s0;
    const int n8 = ns & ~7;
    for (int k = 0; k < n8; k += 8) {
        const float4 h0 = __ldg(reinterpret_cast<const float4*>(hrow + k));
        const float4 h1 = __ldg(reinterpret_cast<const float4*>(hrow + k + 4));
        const float4 l0 = __ldg(reinterpret_cast<const float4*>(lrow + k));
        const float4 l1 = __ldg(reinterpret_cast<const float4*>(lrow + k + 4));
        const float dh[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
        const float dl[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
            const float4* xk = xs4 + (k + kk) * RR;
#pragma unroll
            for (int j = 0; j < RR; ++j) {
                const float4 x = xk[j];
                df_mac(ar[j], dh[kk], dl[kk], x.x, x.y);
                df_mac(ai[j], dh[kk], dl[kk], x.z, x.w);
            }
        }
    }
    for (int k = n8; k < ns; ++k) {
        const float dh = hrow[k], dl = lrow[k];
#pragma unroll
        for (int j = 0; j < RR; ++j) {
            const float4 x = xs4[k * RR + j];
            df_mac(ar[j], dh, dl, x.x, x.y);
            df_mac(ai[j], dh, dl, x.z, x.w);
        }
    }
#pragma unroll
    for (int j = 0; j < RR; ++j) {
        double* p = part + 2 * (((size_t)ct * N + r) * RR + j);
        p[0] = (double)ar[j].s + (double)ar[j].c;
        p[1] = (double)ai[j].s + (double)ai[j].c;
    }
}

__device__ __forceinline__ void df_add(DF& acc, float v) {
    const float t = acc.s + v;
    const float z = t - acc.s;
    acc.c += (acc.s - (t - z)) + (v - z);
    acc.s = t;
}

// The same product from the high words of the matrix and of X only, for a residual that
// needs about 1e-7 relative accuracy (the first refinement sweep, whose residual is about
// 1e-3 of the right-hand side; later sweeps correct what this one leaves): FP32 products
// summed in FP32 over runs of 32 columns, each run added into a float pair.  A thread
// takes two rows (r, r + 128), so each staged x word (the high words of re and im, 8
// bytes) feeds four FMAs; a tenth of the instructions of k_matx_df, half its matrix bytes.
template <int RR>
__global__ void __launch_bounds__(MXD_ROWS) k_matx_f32(int N, int ld, const float* __restrict__ Mhi,
                                                       const float4* __restrict__ Xdf, double* __restrict__ part) {
    extern __shared__ float2 xs2[];  // [MXD_COLS][RR]
    const int ct = blockIdx.y;
    const int s0 = ct * MXD_COLS;
    const int ns = min(MXD_COLS, N - s0);
    for (int idx = threadIdx.x; idx < RR * MXD_COLS; idx += blockDim.x) {
        const int k = idx / RR, j = idx % RR;
        float2 v = make_float2(0.f, 0.f);
        if (k < ns) {
            const float4 x = Xdf[(size_t)(s0 + k) * RR + j];
            v = make_float2(x.x, x.z);
        }
        xs2[idx] = v;
    }
    __syncthreads();
    const int r0 = blockIdx.x * 2 * MXD_ROWS + threadIdx.x, r1 = r0 + MXD_ROWS;
    if (r0 >= N) return;
    const bool two = r1 < N;
    DF a0r[RR], a0i[RR], a1r[RR], a1i[RR];
#pragma unroll
    for (int j = 0; j < RR; ++j) {
        a0r[j] = DF{0.f, 0.f}; a0i[j] = DF{0.f, 0.f}; a1r[j] = DF{0.f, 0.f}; a1i[j] = DF{0.f, 0.f};
    }
    const float* h0 = Mhi + (size_t)r0 * ld + s0;
    const float* h1 = Mhi + (size_t)(two ? r1 : r0) * ld + s0;
    constexpr int RUN = 32;
    for (int k0 = 0; k0 < ns; k0 += RUN) {
        float s0r[RR], s0i[RR], s1r[RR], s1i[RR];
#pragma unroll
        for (int j = 0; j < RR; ++j) { s0r[j] = 0.f; s0i[j] = 0.f; s1r[j] = 0.f; s1i[j] = 0.f; }
        if (k0 + RUN <= ns) {
#pragma unroll 1
            for (int k = k0; k < k0 + RUN; k += 4) {
                const float4 p = __ldg(reinterpret_cast<const float4*>(h0 + k));
                const float4 q = __ldg(reinterpret_cast<const float4*>(h1 + k));
                const float d0[4] = {p.x, p.y, p.z, p.w}, d1[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const float2* xk = xs2 + (k + kk) * RR;
#pragma unroll
                    for (int j = 0; j < RR; ++j) {
                        const float2 x = xk[j];
                        s0r[j] = fmaf(d0[kk], x.x, s0r[j]);
                        s0i[j] = fmaf(d0[kk], x.y, s0i[j]);
                        s1r[j] = fmaf(d1[kk], x.x, s1r[j]);
                        s1i[j] = fmaf(d1[kk], x.y, s1i[j]);
                    }
                }
            }
        } else {
            for (int k = k0; k < ns; ++k) {
                const float d0 = h0[k], d1 = h1[k];
#pragma unroll
                for (int j = 0; j < RR; ++j) {
                    const float2 x = xs2[k * RR + j];
                    s0r[j] = fmaf(d0, x.x, s0r[j]);
                    s0i[j] = fmaf(d0, x.y, s0i[j]);
                    s1r[j] = fmaf(d1, x.x, s1r[j]);
                    s1i[j] = fmaf(d1, x.y, s1i[j]);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < RR; ++j) {
            df_add(a0r[j], s0r[j]); df_add(a0i[j], s0i[j]);
            df_add(a1r[j], s1r[j]); df_add(a1i[j], s1i[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < RR; ++j) {
        double* p = part + 2 * (((size_t)ct * N + r0) * RR + j);
        p[0] = (double)a0r[j].s + (double)a0r[j].c;
        p[1] = (double)a0i[j].s + (double)a0i[j].c;
        if (two) {
            double* q = part + 2 * (((size_t)ct * N + r1) * RR + j);
            q[0] = (double)a1r[j].s + (double)a1r[j].c;
            q[1] = (double)a1i[j].s + (double)a1i[j].c;
        }
    }
}

// Per-column max |Rres| and max |Y| (non-negative doubles compare as integers).
__global__ void k_norms(int N, int R, const double* __restrict__ Rres, const double* __restrict__ Y,
                        unsigned long long* nrm) {
    double rn[MAX_RHS], yn[MAX_RHS];
#pragma unroll
    for (int j = 0; j < MAX_RHS; ++j) { rn[j] = 0; yn[j] = 0; }
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
#pragma unroll
        for (int j = 0; j < MAX_RHS; ++j) {
            if (j < R) {
                size_t o = 2 * ((size_t)r * R + j);
                double e = sqrt(Rres[o] * Rres[o] + Rres[o + 1] * Rres[o + 1]);
                if (!isfinite(e)) e = 1.0e300;
                rn[j] = fmax(rn[j], e);
                yn[j] = fmax(yn[j], sqrt(Y[o] * Y[o] + Y[o + 1] * Y[o + 1]));
            }
        }
    }
#pragma unroll
    for (int j = 0; j < MAX_RHS; ++j) {
        if (j < R) {
            double a = rn[j], b = yn[j];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                a = fmax(a, __shfl_xor_sync(0xffffffffu, a, off));
                b = fmax(b, __shfl_xor_sync(0xffffffffu, b, off));
            }
            if ((threadIdx.x & 31) == 0) {
                atomicMax(nrm + j, (unsigned long long)__double_as_longlong(a));
                atomicMax(nrm + R + j, (unsigned long long)__double_as_longlong(b));
            }
        }
    }
}

__global__ void k_to_f32(size_t n, const double* __restrict__ s, float* __restrict__ d) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        d[i] = (float)s[i];
}
__global__ void k_add_f32(size_t n, const float* __restrict__ s, double* __restrict__ d) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        d[i] += (double)s[i];
}
__global__ void k_pad_rhs(int N, int Np, int R, double* X) {
    size_t total = (size_t)(Np - N) * R * 2;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
        X[(size_t)N * R * 2 + i] = 0.0;
}

size_t matx_part_doubles(int N, int R) {
    return (size_t)2 * ((N + std::min(MX_COLS, MXD_COLS) - 1) / std::min(MX_COLS, MXD_COLS)) * N * R;
}

void launch_matx(cudaStream_t st, int N, int ld, const double* Mr, const double* Mi, int R, int j0, const double* X,
                 int xstride, double* part, double alpha, double beta, const double* base, double* out,
                 int ostride) {
    dim3 grd((N + MX_ROWS - 1) / MX_ROWS, (N + MX_COLS - 1) / MX_COLS);
    size_t smem = sizeof(double) * 2 * R * MX_COLS;
    if (smem > 48 * 1024) {
        cudaFuncSetAttribute(k_matx_partial<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_matx_partial<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    if (Mi) BEM_LAUNCH(k_matx_partial<true><<<grd, 256, smem, st>>>(N, ld, Mr, Mi, R, j0, X, xstride, part));
    else BEM_LAUNCH(k_matx_partial<false><<<grd, 256, smem, st>>>(N, ld, Mr, Mi, R, j0, X, xstride, part));
    size_t tot = (size_t)N * R;
    BEM_LAUNCH(k_matx_reduce<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(N, R, (int)grd.y, part, alpha, beta,
                                                                             base, out, j0, ostride));
}

template <int RR>
static void matx_df_rr(cudaStream_t st, int N, int ld, const float* Mhi, const float* Mlo, const float4* Xdf,
                       double* part) {
    dim3 grd((N + MXD_ROWS - 1) / MXD_ROWS, (N + MXD_COLS - 1) / MXD_COLS);
    const size_t smem = sizeof(float4) * RR * MXD_COLS;
    if (!Mlo) {
        const size_t smem2 = sizeof(float2) * RR * MXD_COLS;
        const dim3 grd2((N + 2 * MXD_ROWS - 1) / (2 * MXD_ROWS), (N + MXD_COLS - 1) / MXD_COLS);
        if (smem2 > 48 * 1024)
            cudaFuncSetAttribute(k_matx_f32<RR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
        BEM_LAUNCH(k_matx_f32<RR><<<grd2, MXD_ROWS, smem2, st>>>(N, ld, Mhi, Xdf, part));
        return;
    }
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_matx_df<RR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    BEM_LAUNCH(k_matx_df<RR><<<grd, MXD_ROWS, smem, st>>>(N, ld, Mhi, Mlo, Xdf, part));
}

void launch_matx_df(cudaStream_t st, int N, int ld, const float* Mhi, const float* Mlo, int R, const double* X,
                    int xstride, int j0, float4* Xdf, double* part, double alpha, double beta, const double* base,
                    double* out, int ostride) {
    BEM_LAUNCH(k_split_df<<<256, 256, 0, st>>>(N, R, X, xstride, j0, Xdf));
    switch (R) {
        case 1: matx_df_rr<1>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 2: matx_df_rr<2>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 3: matx_df_rr<3>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 4: matx_df_rr<4>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 5: matx_df_rr<5>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 6: matx_df_rr<6>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 7: matx_df_rr<7>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 8: matx_df_rr<8>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 9: matx_df_rr<9>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 10: matx_df_rr<10>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 11: matx_df_rr<11>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 12: matx_df_rr<12>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 13: matx_df_rr<13>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 14: matx_df_rr<14>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        case 15: matx_df_rr<15>(st, N, ld, Mhi, Mlo, Xdf, part); break;
        default: matx_df_rr<16>(st, N, ld, Mhi, Mlo, Xdf, part); break;
    }
    const size_t tot = (size_t)N * R;
    BEM_LAUNCH(k_matx_reduce<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(
        N, R, (N + MXD_COLS - 1) / MXD_COLS, part, alpha, beta, base, out, j0, ostride));
}

void launch_split_df(cudaStream_t st, int N, int R, const double* X, int xstride, int j0, float4* Xdf) {
    BEM_LAUNCH(k_split_df<<<256, 256, 0, st>>>(N, R, X, xstride, j0, Xdf));
}

void launch_split_mat_df(cudaStream_t st, size_t n, const double* M, float* hi, float* lo) {
    BEM_LAUNCH(k_split_mat_df<<<1024, 256, 0, st>>>(n, M, hi, lo));
}

void launch_norms(cudaStream_t st, int N, int R, const double* Rres, const double* Y, unsigned long long* nrm) {
    BEM_LAUNCH(k_norms<<<152, 256, 0, st>>>(N, R, Rres, Y, nrm));
}
void launch_to_f32(cudaStream_t st, size_t n, const double* src, float* dst) {
    BEM_LAUNCH(k_to_f32<<<1024, 256, 0, st>>>(n, src, dst));
}
void launch_add_f32(cudaStream_t st, size_t n, const float* src, double* dst) {
    BEM_LAUNCH(k_add_f32<<<1024, 256, 0, st>>>(n, src, dst));
}
void launch_pad_rhs(cudaStream_t st, int N, int Np, int R, double* X) {
    if (Np > N) BEM_LAUNCH(k_pad_rhs<<<256, 256, 0, st>>>(N, Np, R, X));
}

}  // namespace bem
