// bem_internal.h -- declarations shared by the host runtime and the kernels.
#pragma once
#include <atomic>
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

struct bem_mlp;

namespace bem {

// Count of kernel launches issued by this library (all contexts).
extern std::atomic<unsigned long long> g_launches;  // kernel launches (all threads)
extern thread_local unsigned long long t_launches;  // kernel launches of this host thread
#define BEM_LAUNCH(...) (++::bem::g_launches, ++::bem::t_launches, __VA_ARGS__)

constexpr int RK_STRIDE = 32;   // doubles per Rankine panel record
constexpr int MAX_RHS = 16;     // 6 radiation + up to 10 headings
constexpr int MAX_BETA = MAX_RHS - 6;
constexpr int LD_ALIGN = 128;   // matrix leading dimension / padded order

// Sticky device status bits (one int per context, read back after a solve).
enum DevFlag : int {
    FLAG_PIVOT = 1,      // a multiplier |l_ik| > 1: partial pivoting would exchange rows
    FLAG_ZERO_PIVOT = 2, // a zero (or non-finite) pivot
    FLAG_NONFINITE = 4,  // non-finite residual
    FLAG_TIMEOUT = 8,    // a bounded device-side wait expired (kernel abandoned its tile)
    FLAG_GROWTH = 16,    // a multiplier |l_ik| > 16 (element growth a solve should not accept)
};

#ifdef __CUDACC__
// Round-to-nearest TF32 value of x (10-bit mantissa, the low 13 bits cleared).  The
// tensor cores truncate FP32 operands; operands rounded here carry unbiased errors.
__device__ __forceinline__ float tf32_rn(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
#endif

constexpr int WAVE_SM_SLOTS = 256;  // per-SM admission counters of the persistent wave kernel (>= %nsmid)
constexpr int WAVE_SPLIT = 4;       // source ranges per receiver row (work items of the persistent wave kernel)
constexpr int WAVE_ALWAYS = 16;     // CTAs of each wave launch admitted wherever they land

struct WaveArgs {
    int N, ld, R, mode;   // mode 0: assemble D and S*B; 1: raw ws/wd (N x N interleaved)
    double K;
    const double* xr;     // collocation points [3][N]
    const double* gq;     // mirrored-panel Gauss data [7][4][N]: x, y, z, w, nx, ny, nz
    const int* nq;        // Gauss points per panel (3 or 4)
    const double* RD;     // d + dr           [N][ld]
    const double* RSR;    // -sr * 2 n_z(S)   [N][ld]
    const double* Bm;     // RHS block B      [N][R] complex interleaved
    double* Y;            // S * B accumulator [N][R] complex interleaved (+=)
    double* D64r; double* D64i;   // [ld][ld]
    float* D32r; float* D32i;     // [ld][ld] or null
    double* ws_out; double* wd_out;
    // mixed mode only
    const float* xr32;    // collocation points, hi/lo split: [6][N] (xh, yh, zh, xl, yl, zl)
    const float* gq32;    // Gauss data [10][4][N]: xh, yh, zh, w, nx, ny, nz, xl, yl, zl
    const float4* gq32v;  // the same as [4][3][N] float4: (xh, yh, zh, w), (nx, ny, nz, xl), (yl, zl, 0, 0)
    float* Dhi; float* Dlo;   // Re D as a float pair hi + lo (~48-bit) for the refinement residual [N][ld]
    const float* Bm32;        // B as floats [N][R] complex interleaved
    const float* RDhi; const float* RDlo;    // RD as float pairs [N][ld]
    const float* RSRhi; const float* RSRlo;  // RSR as float pairs [N][ld]
    // persistent mixed kernel: work items (row x source range) are drawn from *row_ctr (zero at
    // launch); a CTA stays only if its SM id is >= reserve and fewer than per_sm of its CTAs are
    // on that SM (sm_ctr[smid], zero at launch; sm_ctr[WAVE_SM_SLOTS] counts arrivals), so a
    // concurrent LU keeps SMs for its own CTAs
    int* row_ctr;
    int* sm_ctr;
    int reserve, per_sm;
    int split;            // source ranges per receiver row (work items); 0: WAVE_SPLIT
    // FP32 constants of the mixed kernel, computed on the host so that no FP64 instruction
    // (slow on this GPU) can be rematerialised inside its inner loop: K = kh + kl,
    // c1 = K / (4 pi), c2 = K^2 / (4 pi), live = (K != 0)
    float kh, kl, c1f, c2f;
    int live;
};
void set_wave_f32_constants(WaveArgs& a);

// The surrogate form of the mixed assembly (k_wave_surrogate): far-field pairs inside the
// network's domain take G and dG/dh from the tensor-core network, the rest (pairs nearer
// than `near` panel diameters, out-of-domain pairs and a seeded sample of far pairs, the
// judge) from the FP32 closed form.  Re ws goes to ws32 ([N][ld]); the host adds -ws32 B
// to the right-hand sides.  stats (zeroed by the caller): [0] Gauss points by the network,
// [1] by the closed form, [2] judged pairs, [3] largest judged error |surrogate - closed
// form| / envelope as float bits.
struct SurArgs {
    const uint8_t* img;       // operand image and FP32 tail of the network (mlp_tc_build_image)
    const float* fw;
    float in_shift[2], in_scale[2], out_shift[6], out_scale[6];
    float kr_min, kr_max, kz_min;  // the domain in K R and K Z
    float near2;              // (near-field distance in panel diameters)^2
    const float* pdiam;       // panel diameters [N]
    unsigned judge_mod;       // a far pair is judged if hash(row, column, seed) % judge_mod == 0
    unsigned judge_seed;
    float* ws32;
    unsigned long long* stats;
    int* gflags;
};
// Launches k_wave_surrogate on the persistent-assembly counters of a (a.mode 0 or 1); nonzero
// if the launch failed.
int launch_wave_surrogate(cudaStream_t st, const WaveArgs& a, const SurArgs& sa);

cudaError_t upload_poly_constants(int device);
void launch_rankine(cudaStream_t st, int N, int ld, const double* rec, const double* xr, const double* rn, int mode,
                    double* o0, double* o1, double* o2, double* o3);
void launch_wave(cudaStream_t st, const WaveArgs& a, bool fp32);
// Folds the dipole influence of W trailing-wake strips into H (N x N, leading dimension ld):
// H[r][te_up[w]] += D_w(x_r), H[r][te_lo[w]] -= D_w(x_r) (Kutta condition).
void launch_wake_fold(cudaStream_t st, int N, int ld, int W, const double* rec_w, const double* xr, const int* te_up,
                      const int* te_lo, double* H);
// Exterior outputs after a solve (X = [Phi_J | Phi_S], N x (6 + NB) complex):
// free-surface elevation at NW points wp ([3][NW]) and Kochin functions at NK angles;
// out: [NW or NK][6 + NB] complex interleaved.
// Sources are the first nsrc panels (the hull; a.N is the panel-array stride).
void launch_fs_elevation(cudaStream_t st, const WaveArgs& a, int nsrc, int NW, const double* wp, const double* rec,
                         const double* rn, double Omega, int NB, const double* Nk, const double* dphiI,
                         const double* X, double* out);
void launch_kochin(cudaStream_t st, int N, int nsrc, int NK, int NB, double K, const double* cen, const double* nrm,
                   const double* area, const double* Nk, const double* dphiI, const double* X, double* out);
// Plane-wave factors of the imaginary wave influence (M angles, stored as float
// pairs) and the product out += i * scale * Re-part operator applied to Z, in
// double-float arithmetic (k_influence.cu).  Zdf: Z split by launch_split_df;
// T: scratch of 4 M R doubles.
void launch_pw_build(cudaStream_t st, int N, int M, double K, const double* xr, const double* gq, const int* nq,
                     float4* E, float4* V, float4* W);
void launch_pw_correct(cudaStream_t st, int N, int M, int R, double scale, const float4* P, const float4* E,
                       const float4* Zdf, double* T, double* out);
// Xdf[r][j] = X[r][j0 + j] (complex, row stride xstride) split into float pairs.
void launch_split_df(cudaStream_t st, int N, int R, const double* X, int xstride, int j0, float4* Xdf);
void launch_pad_identity(cudaStream_t st, int N, int ld, double* D64r, double* D64i, float* D32r, float* D32i);
void launch_incident(cudaStream_t st, int N, int NB, int R, const double* betas, double K, double Omega,
                     const double* cen, const double* nrm, const double* area, double* phiI, double* dphiI,
                     double* Bm);
// Blocks of the hull integrations (launch_post); their partial sums need
// 2 * post_blocks(N) * (36 + 12 NB) doubles.
int post_blocks(int N);
void launch_post(cudaStream_t st, int N, int NB, int R, const double* X, const double* Nk, const double* area,
                 const double* phiI, const double* dphiI, double* part, double* out);
void launch_havelock(cudaStream_t st, int n, const double* x, const double* y, const double* v, double* out,
                     bool fp32);

// ---- dense LU / solves (k_lu.cu, k_tc_gemm.cu) ------------------------------
// A planar complex matrix view.
template <typename T> struct CMat {
    T* re;
    T* im;
    int ld;
};

struct LUWork;  // opaque workspace (host_api.cpp)

// Blocked LU without row exchanges of the n x n (n % nb == 0) planar matrix;
// diagonal-block inverses go to inv (re/im, [n/nb][2][nb][nb]: L^-1 then U^-1).
int lu_factor_f64(cudaStream_t st, int n, CMat<double> A, double* invr, double* invi, double* wl, double* wu,
                  int* flags);
// LU with partial pivoting (k_lu_piv.cu; Eigen's rule: the first row of largest |a_ij|), in
// place, pivots in piv (n ints), FLAG_ZERO_PIVOT on a zero pivot; the solve exchanges X's rows
// (n x R complex interleaved) and substitutes in place.  Nonzero if a launch failed.
int lu_piv_factor_f64(cudaStream_t st, int n, CMat<double> A, int* piv, int* flags);
int lu_piv_solve_f64(cudaStream_t st, int n, CMat<double> A, const int* piv, int R, double* X);
// Lookahead schedule for the tensor-core LU: the panel of step k+1 (diagonal-block
// inverse, W21, U12^T) runs on `panel` (a higher-priority stream) while the main
// stream applies the rest of step k's trailing update on all but `reserve_sms` SMs.
struct LuStreams {
    cudaStream_t panel;
    cudaEvent_t ev_panel, ev_cross, ev_rest;
    cudaStream_t ucol;      // U-column transforms (U D^-1) behind the panel chain
    cudaEvent_t ev_ucol;
    int reserve_sms;
    int rest_tiles;         // tiles per trailing-update CTA when reserve_sms == 0
    cudaEvent_t* timeline;  // optional, 6 timing events per block step (see lu_factor_f32_lookahead)
    int cluster_inverse;    // CTAs per block inverse: 2, 4 or 8 (a cluster, k_inv128c), 1: one CTA
    int ucol_own;           // 1: U-column transforms on `ucol`, 0: on `panel` after each W21
    int ucol_ctas;          // CTAs per U-column transform (0: one per tile)
    cudaStream_t panel_tail;  // optional: W21 / transpose tiles beyond the first, off the inverse chain
    cudaEvent_t ev_head, ev_t0;
    int block_inverse;      // cluster inverse: 0 one pivot at a time (k_inv128c), 1 eight at a time
                            // (k_inv128b), 2 eight at a time with the next pivot block ahead (k_inv128l)
    cudaStream_t rest;      // paired schedule: trailing updates of two steps at a time
    cudaEvent_t ev_panel2, ev_cross2;
    float* pair_t;          // 4 (n / 256) 128 128 floats: transposed pair blocks of the pair fold
    int pdl;                // 1: each block inverse is launched as a programmatic dependent of the
                            // corner update before it (its CTAs start while the update finishes)
};
// wl2: two [2][n][128] buffers (4 n 128 floats); wut2: the same plus the transposed
// diagonal-block inverses, [n/128][2][128][128] (4 n 128 + 256 n floats).  The
// factorization leaves L as W blocks below the diagonal, the diagonal-block
// inverses in inv, and above the diagonal U D^-1 (each column block right-multiplied
// by the inverse of its diagonal block); then the pair fold (lu_pair_fold) puts both
// factors in the form lu_solve_f32 uses.
int lu_factor_f32_lookahead(cudaStream_t st, const LuStreams& ls, int n, CMat<float> A, float* invr, float* invi,
                            float* wl2, float* wut2, int* flags);
// Paired schedule (two elimination steps per pass over the trailing matrix); needs
// ls.panel_tail, ls.rest and ls.ucol_own.  wl4: 8 n 128 floats; wut4: 8 n 128 + 256 n.
int lu_factor_f32_paired(cudaStream_t st, const LuStreams& ls, int n, CMat<float> A, float* invr, float* invi,
                         float* wl4, float* wut4, int* flags);
// Forward/back substitution with the factors: X (n x R, interleaved complex) in place,
// with an n x R scratch right after X.  ready: zeroed at allocation, n/64 ints for the
// FP64 solve, n/8 + 1 for the FP32 one (sub-block flags and a ticket counter); epoch
// strictly increasing across calls on the same ready array (each call uses epoch and
// epoch + 1).  The FP32 solve expects the pair-folded factors of lu_pair_fold.
// Returns nonzero if a launch failed.
int lu_solve_f64(cudaStream_t st, int n, CMat<double> A, const double* invr, const double* invi, int R, double* X,
                 int* ready, int epoch, int* flags);
// wait_skew / wait_ns: the chain's waits ask for epoch + wait_skew and give up wait_ns
// after a CTA starts (FLAG_TIMEOUT); wait_skew > 0 is for failure-detection tests only.
int lu_solve_f32(cudaStream_t st, int n, CMat<float> A, const float* invr, const float* invi, int R, float* X,
                 int* ready, int epoch, int* flags, int wait_skew = 0, unsigned long long wait_ns = 2000000000ull);
// out[:, j0:j0+R] = beta * base[:, j0:j0+R] + alpha * M X[:, j0:j0+R] for an N x N
// row-major matrix M (real if Mi is null, else planar complex), X, base, out
// N x stride complex interleaved.  part: scratch of matx_part_doubles(N, R) doubles.
size_t matx_part_doubles(int N, int R);
void launch_matx(cudaStream_t st, int N, int ld, const double* Mr, const double* Mi, int R, int j0, const double* X,
                 int xstride, double* part, double alpha, double beta, const double* base, double* out,
                 int ostride);
// Same contract as launch_matx for a real matrix stored as float pairs
// (M = Mhi + Mlo), in double-float arithmetic (products exact to ~2^-48,
// compensated sums); the selected columns of X are split into float pairs first
// (Xdf: N x R float4 scratch).  Mlo = null: FP32 products of the high words, summed
// in runs of 32 into float pairs (about 1e-7 relative; for the first refinement sweep).
void launch_matx_df(cudaStream_t st, int N, int ld, const float* Mhi, const float* Mlo, int R, const double* X,
                    int xstride, int j0, float4* Xdf, double* part, double alpha, double beta, const double* base,
                    double* out, int ostride);
// hi[i] = (float)M[i], lo[i] = (float)(M[i] - hi[i]) for n doubles.
void launch_split_mat_df(cudaStream_t st, size_t n, const double* M, float* hi, float* lo);
// nrm[j] = max_r |Rres[r][j]|, nrm[R + j] = max_r |Y[r][j]| as ordered bit patterns (zero them first).
void launch_norms(cudaStream_t st, int N, int R, const double* Rres, const double* Y, unsigned long long* nrm);
// Flexible-GMRES vector kernels (k_gmres.cu).  Vectors are Np x R complex blocks
// (interleaved, R columns); a set of nvec vectors lies vstride doubles apart.
//   gm_dots:    h[v][r] = sum_n conj(V_v[n][r]) w[n][r]   (part: gm_part_doubles(Np, nvec))
//   gm_combine: out = beta out + sign sum_v c[v][r] V_v
//   gm_scale:   out = w / sqrt(Re nrm2[r]) per column (0 for a vanishing norm)
size_t gm_part_doubles(int Np, int nvec);
void launch_gm_dots(cudaStream_t st, int Np, int R, int nvec, const double* V, size_t vstride, const double* w,
                    double* part, double* h);
void launch_gm_combine(cudaStream_t st, int Np, int R, int nvec, const double* V, size_t vstride, const double* c,
                       double sign, double beta, double* out);
void launch_gm_scale(cudaStream_t st, int Np, int R, const double* w, const double* nrm2, double* out);
void launch_f32_to_f64(cudaStream_t st, size_t n, const float* src, double* dst);
void launch_to_f32(cudaStream_t st, size_t n, const double* src, float* dst);
void launch_add_f32(cudaStream_t st, size_t n, const float* src, double* dst);
void launch_pad_rhs(cudaStream_t st, int N, int Np, int R, double* X);
// Device-side state of one frequency's classic refinement when its sweeps repeat inside a
// graph (conditional while node): sweeps done, outcome, the slot's device flags as the
// last test saw them (the LU's and the solves'), last residual (max over the right-hand
// sides of |r|_inf / |y|_inf), the previous sweep's and the previous full-accuracy
// residual, and the last full-to-full contraction.  Zero it before the first sweep.
enum { REFINE_RUNNING = 0, REFINE_CONVERGED = 1, REFINE_FAILED = 2, REFINE_STALLED = 3, REFINE_TIMEOUT = 4 };
struct RefineState {
    int iters, status, flags, pad;
    double resid, prev, prev_full, contraction;
};
// One sweep's convergence test (k_gmres.cu): reads the norms of launch_norms and the
// solve's flags, updates the state and sets h to 1 while the loop should go on.
void launch_refine_step(cudaStream_t st, int R, const unsigned long long* nrm, const int* flags, double tol,
                        int max_iter, int coarse_first, int gmres_switch, RefineState* state,
                        cudaGraphConditionalHandle h);

// Tensor-core inference of the Green-function surrogate network (k_mlp_tc.cu).
// mlp_tc_build_image: the operand image (mlp_tc_image_bytes() bytes) and FP32 tail
// (mlp_tc_param_floats() floats) from the FP32 master parameters of k_mlp.cu.
// mlp_tc_forward: y (n x 6) = network(x (n x 2)), normalised values; nonzero if the
// launch failed.
int mlp_tc_image_bytes();
int mlp_tc_param_floats();
void mlp_tc_build_image(cudaStream_t st, const float* w, uint8_t* img, float* fw);
int mlp_tc_forward(cudaStream_t st, int n, const float* x, float* y, const uint8_t* img, const float* fw, int* flags);

// The network of a bem_mlp as the assembly uses it: operand image, FP32 tail and the
// input / output normalisation (built for the current weights; synchronises the network's
// stream).  Returns nonzero (message in bem_mlp_last_error) if that fails.
struct MlpTcRef {
    const uint8_t* img;
    const float* fw;
    double in_shift[2], in_scale[2], out_shift[6], out_scale[6];
    int device;
};
int mlp_tc_ref(struct ::bem_mlp* m, MlpTcRef* out);

int tc_gemm_supported(int device);
// Measured FP32 FMA throughput of the device (TFLOP/s, 2 flops per FMA), or < 0 on failure.
double ffma_peak_tflops(int device);
// Sets the message returned by bem_last_error(NULL).
void set_static_error(const char* msg);
// One k_tc_update launch in tile mode `mode` on host data (bem_tc_probe); 0 on
// success, -1 with a message in err otherwise.
int tc_probe(int device, int mode, int n, float* C, const float* Wa, const float* Ua, const float* Wb,
             const float* Ub, const float* T, float* Wout, char* err, int err_len);

}  // namespace bem
