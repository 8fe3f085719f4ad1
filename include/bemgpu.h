/*
 * bemgpu.h -- C ABI of the GB300-native frequency-domain panel-method solver.
 *
 * This is the drop-in boundary for the reference's hydrodynamic path
 * (ZeppSav/BEMUse):
 *   - the Boundary mesh generators           (src/Boundary/*.cpp),
 *   - Hydrodynamic_Radiation_Solver           (src/Solver/Hydrodynamic_Solver.{h,cpp}),
 *     behind the virtual BEMUse::Solver API   (src/Solver/Solver_Base.h:39-153),
 *   - the Green-function kernels              (src/Kernels.cpp).
 * Plain pointers and sizes only; all arrays are caller-owned host memory
 * unless stated.  Every call returns a bem_status; bem_last_error() gives the
 * message.  Nothing here aborts the process.
 *
 * Frequency convention: bem_solve takes the internal angular frequency Omega
 * (rad/s).  The reference's Set_Real(Frequency) stores Frequency and computes
 * Omega = Frequency / (2 pi) (Hydrodynamic_Solver.cpp:405); a caller porting
 * Set_Real code passes Frequency / (2 pi).
 */
#ifndef BEMGPU_H
#define BEMGPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    BEM_OK = 0,
    BEM_ERR_ARG = 1,         /* invalid argument (null pointer, bad size, bad mesh) */
    BEM_ERR_CUDA = 2,        /* CUDA runtime error (message holds the CUDA error string) */
    BEM_ERR_STATE = 3,       /* call out of order (e.g. bem_solve before bem_setup) */
    BEM_ERR_NUMERIC = 4,     /* non-finite values, a multiplier |l_ik| > 1 (row exchange needed),
                                or refinement that did not reach its tolerance */
    BEM_ERR_NOMEM = 5,       /* device allocation failed */
    BEM_ERR_UNSUPPORTED = 6  /* feature or device not supported (e.g. no sm_103 GPU) */
} bem_status;

/* Precision modes of bem_solve. */
typedef enum {
    BEM_PLAIN_FP64 = 0, /* FP64 wave assembly, FP64 LU, FP64 solves (the reference's arithmetic) */
    BEM_MIXED = 1       /* FP32 wave assembly into an FP64 operator, TF32 tensor-core LU,
                           FP64 iterative refinement to rel. residual <= refine_tol */
} bem_precision;

typedef struct bem_ctx bem_ctx;

/* A panel mesh.  Nodes are given in the frame of their component; element e of
 * component c has global vertex positions nodes[...] + comp_origin[3c..3c+2]
 * (the translation-only CoordSys of Triple_Spar.cpp:60-67).  elems holds four
 * node indices per element; elems[4e+3] = -1 marks a triangle.  Element order
 * is the panel order of the linear system.  The optional aux mesh is the
 * interior waterplane used for hydrostatics (Hydrodynamic_Solver.cpp:353-367). */
typedef struct {
    int n_nodes;
    const double* nodes;        /* n_nodes x 3 */
    int n_elems;
    const int* elems;           /* n_elems x 4 */
    int n_comp;                 /* >= 1; 0 means one component at the origin */
    const int* comp_first;      /* n_comp + 1 element offsets (may be NULL if n_comp == 0) */
    const double* comp_origin;  /* n_comp x 3 (may be NULL if n_comp == 0) */
} bem_mesh;

/* Mass properties (Boundary_Base.h:149-156).  If mass_matrix / stiffness are
 * non-NULL they are used as given (Hydrodynamic_Solver.cpp:305-309, 346-350);
 * otherwise M and C follow Calculate_Mass_Matrix / Calculate_Hydrostatic_
 * Stiffness_Matrix (:300-397) from mass (0 -> Volume * 1025), cog, gyration
 * radii and the aux waterplane mesh. */
typedef struct {
    double mass;
    double cog[3];
    double gyration[9];          /* row-major 3x3 radii of gyration */
    const double* mass_matrix;   /* optional 6x6 row-major */
    const double* stiffness;     /* optional 6x6 row-major */
    const bem_mesh* aux;         /* optional interior waterplane mesh */
} bem_body_props;

/* Per-frequency outputs; every pointer may be NULL to skip that output.
 * Layouts (f = frequency index, nb = number of headings):
 *   A, B            [f][6][6] row-major (A = Re(AM*Phi_J), B = Im(AM*Phi_J),
 *                   per unit density; Hydrodynamic_Solver.cpp:463-465)
 *   FK, SC, F, RAO  [f][6][nb] complex, interleaved re,im
 *   refine_iters    [f] refinement sweeps used (0 for BEM_PLAIN_FP64)
 *   residual        [f] final max relative residual ||b - D x|| / ||b|| over RHS
 *   phi_rad         N x 6 complex (radiation potentials Phi_J), last frequency
 *   phi_scat        N x nb complex (scattering potentials Phi_S), last frequency
 *   fs_rad          [f][nw][6] complex  ExtRadMat, free-surface elevation of the
 *                   radiation problems at the bem_set_wave_points points
 *                   (Hydrodynamic_Solver.cpp:498-505)
 *   fs_diff         [f][nw][nb] complex ExtDiffMat
 *   kochin_rad      [f][nk][6] complex  KochinRad (:492-494) at theta_i = (i + 1/2) 2 pi / nk
 *   kochin_diff     [f][nk][nb] complex KochinDiff
 * The last four exist for the hydrodynamic solve only; a caller that zero-fills
 * the struct (or initialises only the first ten members) skips them. */
typedef struct {
    double* A;
    double* B;
    double* FK;
    double* SC;
    double* F;
    double* RAO;
    int* refine_iters;
    double* residual;
    double* phi_rad;
    double* phi_scat;
    double* fs_rad;
    double* fs_diff;
    double* kochin_rad;
    double* kochin_diff;
} bem_result;

/* Body and environment data for the result files (host only). */
typedef struct {
    int n_beta;
    const double* betas;   /* headings [rad] */
    double rho;            /* the solver's Density parameter */
    double gravity;        /* the solver's Gravity parameter (printed in .mmx) */
    double M[36];          /* mass matrix, row-major (bem_get_body_matrices) */
    double C[36];          /* hydrostatic stiffness, row-major */
    double volume;         /* displaced volume */
    double cob[3];         /* centre of buoyancy */
    double cog[3];         /* centre of gravity */
    /* optional exterior outputs (zero-filled = none): Kochin angles of
     * bem_result.kochin_rad/diff, and the wave points (n_wave x 3 row-major) of
     * bem_result.fs_rad; they add _KochinRad.bem, _KochinDiff.bem,
     * _WaveElPos.bem and .6r (Hydrodynamic_Solver_IO.cpp:488-500, 589-645). */
    int n_kochin;
    int n_wave;
    const double* wave_points;
} bem_wamit_info;

/* The .bem summary file (Generate_Output_File_BEMUse / Update_Output_File_BEMUse,
 * Hydrodynamic_Solver_IO.cpp:107-426): environment, headings, grid and geometry
 * summary, M and C, then per frequency Omega, period 1 / (2 pi Omega),
 * wavenumber, the A/B table and the Froude-Krylov and excitation tables
 * (|F| / g and phase).  The reference's Setup also writes a block for its
 * Frequency = -1 solve; a caller who wants that block passes omega = -1 / (2 pi)
 * first.  Host only. */
typedef struct {
    const bem_wamit_info* w;   /* headings, M, C, volume, centres */
    int n_nodes, n_elems, n_aux_elems;
    double surface_area;
    double mass;
    const char* file_info;     /* Boundary::FileInfo line (NULL = empty) */
} bem_summary_info;
bem_status bem_write_bem(const char* prefix, const bem_summary_info* info, int n_freq, const double* omega,
                         const bem_result* r);

/* ---- mesh generators (host only; no device needed) ------------------------ */

/* Half_Cylinder (Volume_of_Revolution.cpp:167-199, 12-41, 92-130): radius R,
 * draft, na azimuthal, nr radial (bottom), nv vertical panels, nrfs interior
 * waterplane rings (0 = none), cosine spacing flag (PiCosFac, Boundary_Base.h:39). */
int bem_mesh_cylinder_sizes(int na, int nr, int nv, int nrfs, int* n_nodes, int* n_elems, int* n_aux_nodes,
                            int* n_aux_elems);
int bem_mesh_cylinder(double radius, double draft, int na, int nr, int nv, int nrfs, int cosine, double* nodes,
                      int* elems, double* aux_nodes, int* aux_elems);

/* Barge (Barge.cpp:12-204): length, width, draft; nx, ny, nz panels; five faces. */
int bem_mesh_barge_sizes(int nx, int ny, int nz, int* n_nodes, int* n_elems, int* n_aux_nodes, int* n_aux_elems);
int bem_mesh_barge(double length, double width, double draft, int nx, int ny, int nz, int cosine, double* nodes,
                   int* elems, double* aux_nodes, int* aux_elems);

/* Rectangular wing of a symmetric NACA 00xx section (chord, span, thickness
 * ratio), nc panels around the section (even; half-cosine spacing on both
 * surfaces when cosine != 0), ns spanwise strips, open tips, normals into the
 * wing.  The steady-flow workload's geometry; the reference's Wing class
 * (Wing.cpp:28-109) builds a different (elliptic, Karman-Trefftz) wing. */
int bem_mesh_wing_sizes(int nc, int ns, int* n_nodes, int* n_elems);
int bem_mesh_wing(double chord, double span, double thickness, int nc, int ns, int cosine, double* nodes,
                  int* elems);

/* ---- solver context (Hydrodynamic_Radiation_Solver) ------------------------ */

/* Creates a context on CUDA device `device` (replaces `new Hydrodynamic_Radiation_Solver`). */
bem_status bem_create(bem_ctx** ctx, int device);
/* Frees every device buffer of the context (replaces `delete Solver`). */
void bem_destroy(bem_ctx* ctx);
/* Message of the last failing call on this context (static storage if ctx is NULL). */
const char* bem_last_error(const bem_ctx* ctx);

/* Set_Parameters (Hydrodynamic_Solver.cpp:11-27): density `Density`, gravity
 * `Gravity` (used by the hydrostatics only, as in the reference; the wave
 * number uses g = 9.81, :409) and the headings `WaveAngle` in radians. */
bem_status bem_set_params(bem_ctx* ctx, double density, double gravity, int n_beta, const double* betas);

/* Setup(Boundary*) (Hydrodynamic_Solver.cpp:269-298): panel geometry, mirror
 * panels, collocation points and the frequency-independent Rankine influence
 * matrices (computed on the GPU in FP64).  props may be NULL. */
bem_status bem_setup(bem_ctx* ctx, const bem_mesh* mesh, const bem_body_props* props);

/* Set_Real + Solve (Hydrodynamic_Solver.cpp:400-487) for n_freq angular
 * frequencies in one call.  refine_tol <= 0 selects the default 1e-12.  With
 * BEM_MIXED and n_freq >= 2 the frequencies run as a pipeline on the context's
 * streams (the assembly of one frequency, the LUs of the next one or two and the
 * refinement of the one before them side by side; the tuning keys asm_overlap and
 * lu_overlap select it); results are those of solving the frequencies one at a
 * time.  n_freq = 0 returns at once. */
bem_status bem_solve(bem_ctx* ctx, int n_freq, const double* omega, int precision, double refine_tol,
                     bem_result* out);

/* Panel count N and heading count of the current setup. */
bem_status bem_get_sizes(const bem_ctx* ctx, int* n_panels, int* n_beta);

/* Mass and stiffness matrices used for the RAO (6x6 row-major each), and
 * {volume, xb, yb, zb} (Boundary_Base.cpp:177-224). */
bem_status bem_get_body_matrices(const bem_ctx* ctx, double* mass_matrix, double* stiffness, double* vol_cob);

/* ---- steady potential flow (Aerodynamic_Solver, constant panels) ---------- */

/* Aerodynamic_Solver::Setup (Aerodynamic_Solver.cpp:126-146) with constant
 * panels: collocation points c + 1e-5 n and the Rankine influence matrices
 * G (source) and H (dipole) of the body panels (:42-58), on the GPU in FP64.
 * Replaces any hydrodynamic setup of the context. */
bem_status bem_aero_setup(bem_ctx* ctx, const bem_mesh* mesh);

/* Set_External_BC + Solve_Steady (:150-180): BC_i = V_i . n_i, X = H^-1 (G BC).
 * vel: 3 doubles (uniform onset flow) if n_vel == 1, else 3 per panel (n_vel = N).
 * X (N): perturbation potential at the panels; BC (N) may be NULL. */
bem_status bem_aero_solve(bem_ctx* ctx, int n_vel, const double* vel, int precision, double refine_tol, double* X,
                          double* BC);

/* ---- steady flow with a trailing wake (no reference counterpart) ------------
 * The reference's constant-panel steady solve has no wake, no Kutta condition and no
 * pressure (Aerodynamic_Solver.cpp:169-180); these define them for lifting bodies.
 * bem_aero_set_wake: n_wake flat constant-doublet wake strips (quads: n_wake x 4 x 3
 * vertices, normal from the vertex order as for body panels) whose strengths are the
 * Kutta jumps X[te_upper[w]] - X[te_lower[w]]; the next bem_aero_setup adds each
 * strip's dipole influence to H's column te_upper[w] and subtracts it from column
 * te_lower[w] (on the GPU).  n_wake = 0 removes the wake.
 * bem_mesh_wing_wake: the wake of bem_mesh_wing's wing: one strip per panel column from
 * the trailing edge (x = chord, z = 0) to length chords downstream, normal -z, Kutta pair
 * (upper trailing-edge panel j nc + nc - 1, lower j nc).
 * bem_aero_surface: surface pressure of a solution X for a uniform onset flow vel (3):
 * V = U - (U . n) n + grad X, the least-squares surface gradient over each panel's edge
 * neighbours that face the same side (n_i . n_j > 0); cp = 1 - |V|^2 / |U|^2 (N values,
 * may be NULL); coeffs (may be NULL) = {CFx, CFy, CFz, CL, CD} with CF = sum cp n A / s_ref
 * (n into the body), CL along the unit normal to U in the x-z plane, CD along U.  Host only. */
bem_status bem_aero_set_wake(bem_ctx* ctx, int n_wake, const double* quads, const int* te_upper,
                             const int* te_lower);
int bem_mesh_wing_wake(double chord, double span, int nc, int ns, double length, double* quads, int* te_upper,
                       int* te_lower);
bem_status bem_aero_surface(bem_ctx* ctx, const double* X, const double* vel, double s_ref, double* cp,
                            double* coeffs);

/* ---- influence matrices (Prepare_Linear_System / _Wave_Terms) -------------- */

/* Copies the Rankine kernel values of the current setup to host, N x N
 * row-major (row = receiver, column = source): s, d for the body panels and
 * sr, dr for the mirrored panels (Hydrodynamic_Solver.cpp:103-109 stores
 * SSrc = -s, SSrcRefl = -sr, DSrc = d, DSrcRefl = dr).  Any pointer may be NULL. */
bem_status bem_get_rankine(bem_ctx* ctx, double* s, double* sr, double* d, double* dr);

/* Wave-term influence matrices at wave number K (Hydrodynamic_Solver.cpp:193-202
 * without the Rankine K-term): ws, wd as N x N complex interleaved, computed in
 * FP64 (precision = BEM_PLAIN_FP64) or FP32 (BEM_MIXED). */
bem_status bem_wave_matrices(bem_ctx* ctx, double K, int precision, double* ws, double* wd);

/* ---- Green function (Kernels.cpp) ------------------------------------------ */

/* HavelockGF (Kernels.cpp:342-412) at n nondimensional points (x, y, v) on
 * device `device`; out = n x 8 doubles: Re/Im of G, dG/dx, dG/dy, dG/dz.
 * precision: BEM_PLAIN_FP64 or BEM_MIXED (FP32 arithmetic). */
bem_status bem_havelock(int device, int n, const double* x, const double* y, const double* v, int precision,
                        double* out);

/* ---- dense complex solve ----------------------------------------------------- */

/* Solves A X = B for complex A (n x n) and B (n x nrhs), both row-major
 * interleaved, with the GPU LU of `precision` (refined to refine_tol in
 * BEM_MIXED).  X overwrites B.  Replaces Eigen::PartialPivLU<CMatrix>
 * compute/solve (Hydrodynamic_Solver.cpp:430, 438, 446).  The fast path is the
 * blocked LU without row exchanges; when it meets a multiplier |l_ik| > 1 or a zero
 * pivot (or, in BEM_MIXED, its refinement does not converge), the matrix is factored
 * again in FP64 with partial pivoting (Eigen's rule: the first row of largest
 * |a_ij|) and solved directly; refine_iters is then 0 and residual is computed on
 * the host.  BEM_ERR_NUMERIC only for a singular matrix.  The call uses the
 * context's solver buffers and discards any previous bem_setup. */
bem_status bem_dense_solve(bem_ctx* ctx, int n, const double* A, int nrhs, double* B, int precision,
                           double refine_tol, int* refine_iters, double* residual);

/* Accumulated device time (ms) of bem_solve stages since the last reset:
 * [0] incident wave + static RHS, [1] wave assembly, [2] LU factorization,
 * [3] solves and refinement, [4] hull integrals, [5] frequency-solves counted.
 * reset != 0 zeroes the counters after reading. */
bem_status bem_stage_times(bem_ctx* ctx, double* out6, int reset);

/* Device time of the wave-assembly kernel alone (CUDA events on the solve stream
 * around its launch): out4[0] milliseconds summed over launches, [1] launches,
 * [2] panel pairs per launch (N^2), [3] reserved.  reset != 0 zeroes after reading. */
bem_status bem_kernel_times(bem_ctx* ctx, double* out4, int reset);

/* Tuning knobs (defaults are the measured best on GB300):
 *   "lu_reserve_sms"  > 0: SMs the lookahead LU keeps free of its persistent trailing
 *                     update for the panel chain (inverse, W21, transpose; default 32);
 *                     0: the trailing update runs as short-lived CTAs that hand SMs to
 *                     the higher-priority panel stream as they retire.
 *   "lu_rest_tiles"   tiles per such short-lived CTA (default 4).
 *   "lu_cluster_inverse" CTAs per diagonal-block inverse: 2, 4 or 8 (a thread-block
 *                     cluster, rows split between the CTAs; default 8) or 1 (one CTA).
 *   "lu_ucol_stream"  1: the U D^-1 transform of each finished column block (the
 *                     backward solve's operator) runs on its own stream (default),
 *                     0: on the panel stream behind each W21.
 *   "lu_ucol_ctas"    CTAs of each such transform (0 = one per 128 x 128 tile).
 *   "lu_pair_update"  1: the trailing updates of two elimination steps are applied in
 *                     one pass over the trailing matrix (K = 256; default), 0: one step
 *                     per pass.
 *   "refine_gmres"    refinement of the mixed path, all stopping at the same residual
 *                     test: 0 classic x <- x + LU^-1 (y - D x); 1 flexible GMRES
 *                     (restart 16) with the TF32 factors as preconditioner, which never
 *                     needs more preconditioner solves; 2 (default) classic sweeps while
 *                     each reduces the residual more than 20x, then GMRES from there.
 *   "refine_coarse_first" 1 (default): when the previous solve of the context reduced
 *                     its residual by less than 3e-4 per sweep, the residual of the first
 *                     classic sweep (about 1e-3 of y) is formed from the FP32 high words of
 *                     Re D (about 1e-7 relative), the later ones in double-float; the sweep
 *                     count stays the same at such contraction, and convergence is only
 *                     accepted on a double-float residual.  0: every residual double-float.
 *   "refine_graph"    1: the classic sweeps of each frequency repeat inside a CUDA graph
 *                     (a conditional while node) and their convergence test runs on the
 *                     device, with the same decisions as the host loop (the same sweeps,
 *                     the switch to GMRES, the same failures); 0 (default): the host reads
 *                     each sweep's residual norms (faster inside the frequency pipeline,
 *                     where the loop's kernels would lose the refinement's stream priority).
 *   "lu_block_inverse" 1: the cluster inverse eliminates 8 pivots per synchronisation,
 *                     2 (default): the same with the next panel's pivot block inverted
 *                     by a dedicated warp beside each rank-8 update, 0: one pivot per
 *                     synchronisation.
 *   "lu_split_panel"  1: only the first tile of each panel's W21 and U transpose runs on
 *                     the inverse chain, the rest on a second panel stream (default);
 *                     0: the whole panel on the panel stream.
 *   "lu_pdl"          1: each block inverse of the tensor-core LU, and the first W21 tile
 *                     after it, start as programmatic dependents of the kernel before them
 *                     (default); 0: ordinary launches.
 *   "asm_overlap"     pipelined mixed solves: 1 = the next frequency's wave assembly
 *                     runs beside this frequency's LU and solves (default), 0 = beside
 *                     the solves only.
 *   "lu_overlap"      with asm_overlap = 1: 1 = the LU of frequency f + 1 runs beside the
 *                     refinement of f (its own stream; each frequency slot keeps its own
 *                     block inverses, flags and LU workspaces; three slots), 2 or 3 = the
 *                     LUs of f + 1 .. f + 2 (3) may also run at once on as many streams
 *                     (four or five slots; 2 is the default), 0 = LU and refinement of one
 *                     frequency after the other on one stream.
 *   "asm_reserve_sms" SMs (lowest SM ids) the persistent assembly kernel leaves to the
 *                     LU and the refinement when it overlaps them (default 56).
 *   "asm_ctas_per_sm" assembly CTAs admitted per SM then (1..3, default 3).
 *   "solve_priority"  stream priority of the refinement beside the LU: 0 = highest
 *                     (default), 1 = that of the LU's main stream, 2 = the lowest.
 *   "asm_split"       work items per receiver row of the persistent assembly kernel
 *                     (1..64, default 4; finer items measured slower).
 *   "refine_max_solves" preconditioner solves the mixed path's refinement may use
 *                     (default 60); when they run out bem_solve returns BEM_ERR_NUMERIC.
 *   "test_wait_skew", "test_wait_ms"  failure-detection tests only: with skew 1 every
 *                     wait of the triangular-solve chain asks for a flag value that nothing
 *                     publishes and gives up after test_wait_ms (default 2000) milliseconds;
 *                     bem_solve then returns BEM_ERR_CUDA ("device-side wait ... expired")
 *                     and the context stays usable once the skew is set back to 0. */
bem_status bem_set_tuning(bem_ctx* ctx, const char* key, double value);

/* Autotuner of the pipelined mixed solve: times bem_solve (BEM_MIXED, outputs skipped)
 * on the n_freq >= 2 sample frequencies for each of a small grid of the schedule knobs
 * above (the current setting; assembly reserves of 40, 48 and 64 SMs with
 * lu_overlap = 2, of 40 and 48 with lu_overlap = 3, of 56 with lu_overlap = 1), every
 * setting twice in alternation, and keeps the fastest on the context.  ms_per_freq
 * (optional) receives its time per frequency; report (optional, report_len bytes) one
 * line per setting, the chosen one marked '*'.  Needs bem_setup.  The project's
 * replacement for hand-picked launch shapes: the best split of the GPU between the
 * overlapping assembly and the LU varies between GPUs of one pool. */
bem_status bem_autotune(bem_ctx* ctx, int n_freq, const double* omega, double* ms_per_freq, char* report,
                        int report_len);

/* Timeline of the tensor-core LU's lookahead schedule (tracing aid).  enable = 1
 * turns recording on (events at every block step of later mixed factorizations),
 * 0 turns it off, -1 leaves it unchanged.  out receives, for the first
 * factorization of the last bem_solve call (in a pipelined call it runs beside the
 * next frequency's assembly), up to max_steps rows of 6 times in ms from its first event:
 * cross update of step k started / done (main stream), inverse of block k+1 done,
 * W21 done, panel k+1 ready (panel stream), rest of step k's update done.
 * *steps = rows available. */
bem_status bem_lu_timeline(bem_ctx* ctx, int enable, int max_steps, double* out, int* steps);

/* ---- many bodies --------------------------------------------------------------
 * Solves n_bodies independent bodies at the same frequencies: for each body the
 * Setup + per-frequency Solve sequence of the reference's console loop
 * (BEMUser_Console.cpp:242-262).  n_workers host threads (0: 8), each with its own
 * context on `device`, run bodies concurrently, largest first.  props may be NULL
 * (default mass properties).  results[b] receives body b's outputs as bem_solve
 * fills them; *seconds (may be NULL) the wall time.  The first failure is
 * returned (message in bem_last_error(NULL)); a worker that meets a failure
 * stops, the others finish their bodies. */
bem_status bem_batch_solve(int device, int n_bodies, const bem_mesh* meshes, const bem_body_props* props,
                           double density, double gravity, int n_beta, const double* betas, int n_freq,
                           const double* omega, int precision, double tol, int n_workers, bem_result* results,
                           double* seconds);

/* ---- MLP surrogate of the wave Green function (k_mlp.cu) -------------------
 * Inputs (log10 KR, KZ), 4 hidden layers of width 128 with SiLU, 6 outputs:
 * Re/Im of G, dG/dR, dG/dZ of HavelockGF (Kernels.cpp:342-412; dG/dZ = G there).
 * BF16 weights (FP32 master copy), FP32 accumulation, Adam on the MSE of the
 * normalised outputs; forward and backward kernels are this library's own.
 * Parameters are ordered W0 (128x2), b0, W1 (128x128), b1, ..., W4 (6x128), b4,
 * W row-major [out][in].  Host arrays throughout: x is n x 2, y is n x 6. */
typedef struct bem_mlp bem_mlp;
int bem_mlp_num_params(void);
bem_status bem_mlp_create(bem_mlp** out, int device, unsigned long long seed);
void bem_mlp_destroy(bem_mlp* m);
const char* bem_mlp_last_error(const bem_mlp* m);
/* x_n = (x - in_shift) / in_scale, y_n = (y - out_shift) / out_scale (2 and 6 entries). */
bem_status bem_mlp_set_normalization(bem_mlp* m, const double* in_shift, const double* in_scale,
                                     const double* out_shift, const double* out_scale);
bem_status bem_mlp_get_params(bem_mlp* m, double* w);
bem_status bem_mlp_set_params(bem_mlp* m, const double* w);
bem_status bem_mlp_eval(bem_mlp* m, int n, const double* x, double* y);
/* Loss (MSE of normalised outputs) and its gradient with respect to the parameters on one batch. */
bem_status bem_mlp_grad(bem_mlp* m, int n, const double* x, const double* y, double* grad, double* loss);
bem_status bem_mlp_train(bem_mlp* m, int n, const double* x, const double* y, int epochs, int batch, double lr,
                         unsigned long long seed, double* loss_per_epoch);
/* The surrogate form of the mixed assembly (no reference counterpart; the learned
 * stand-in for HavelockGF, Kernels.cpp:342-412, in FreeSurface_Wave_Kernel,
 * Panel.cpp:601-636).  With mode != 0 the mixed path's wave assembly takes G and
 * dG/dh of far-field pairs inside the network's domain from network m (its
 * tensor-core forward, fused into the assembly kernel), scaled back by the envelope
 * the network is trained on (bemuse_gb300.HavelockSurrogate.envelope); near pairs
 * (a mirrored Gauss point closer than domain[3] panel diameters), pairs outside
 * KR in [domain[0], domain[1]] or KZ >= domain[2] and a seeded fraction
 * judge_fraction of the far pairs (the judge) use the FP32 closed form.  The judged
 * error is max |network - closed form| / envelope over the judged Gauss points.
 *   mode 0  off (the closed form everywhere).
 *   mode 1  strict: every frequency whose judged error exceeds judge_tol is solved
 *           again with the closed form and its results replaced, so the results keep
 *           the mixed path's accuracy whenever the network is not good enough.
 *   mode 2  accept: the network's values are kept (the judged pairs use the closed form).
 * The imaginary parts of the operator and of the right-hand sides keep their exact
 * plane-wave form; the network's imaginary parts reach only the FP32 copy of D that
 * is factorised.  domain may be NULL for {1e-3, 20, -40, 3}.  m must stay alive
 * while the context uses it and be on the context's device.  BEM_MIXED only. */
bem_status bem_set_surrogate(bem_ctx* ctx, bem_mlp* m, int mode, double judge_tol, double judge_fraction,
                             const double* domain);
/* Totals of the surrogate form since the last reset: [0] Gauss points evaluated by the
 * network, [1] by the closed form, [2] judged pairs, [3] largest judged error,
 * [4] frequencies solved again by the strict mode, [5] frequencies assembled with the
 * surrogate, [6] reserved.  reset != 0 zeroes them after reading. */
bem_status bem_surrogate_stats(bem_ctx* ctx, double* out7, int reset);

/* Forward pass on the tensor cores (tcgen05 kind::f16: BF16 weights and activations,
 * FP32 accumulation in TMEM, SiLU as x/2 (1 + tanh(x/2)) with the hardware tanh):
 * the inference form the assembly uses.  It differs from bem_mlp_eval (FP32
 * activations) by the BF16 rounding of the activations (about 1e-3 relative).
 * Needs an sm_103 GPU (BEM_ERR_UNSUPPORTED otherwise). */
bem_status bem_mlp_eval_tc(bem_mlp* m, int n, const double* x, double* y);
/* Throughput of the tensor-core forward pass (evaluations per second of device time). */
bem_status bem_mlp_throughput_tc(bem_mlp* m, int n, double* mlp_evals_per_s);
/* Forward-pass throughput (evaluations per second of device time) on n resident samples. */
bem_status bem_mlp_throughput(bem_mlp* m, int n, double* mlp_evals_per_s);
/* Throughput of the closed-form HavelockGF kernel (evaluations per second of device
 * time) on n resident points; precision as for bem_havelock. */
bem_status bem_havelock_throughput(int device, int n, int precision, double* evals_per_s);

/* ---- exterior outputs (Hydrodynamic_Solver.cpp:205-266, 489-505, 598-642) ----
 * bem_set_wave_points: the exterior free-surface points (x, y, z), n x 3
 * row-major, at which bem_solve evaluates ExtRadMat / ExtDiffMat when the
 * result asks for fs_rad / fs_diff (the reference's Wave_Nodes, e.g. the
 * Barge free-surface grid of Barge.cpp:125-140).  n = 0 clears them.
 * bem_set_kochin: NKochin, the number of Kochin angles (default 36,
 * Hydrodynamic_Solver.h:119).  The reference's Kochin matrices read an
 * uninitialised value (Hydrodynamic_Solver.cpp:626-627); this library computes
 * E = exp(K z + i K (x cos t + y sin t)) at the panel centroids. */
bem_status bem_set_wave_points(bem_ctx* ctx, int n, const double* xyz);

/* Irregular-frequency removal, the IFR parameter (Hydrodynamic_Solver.cpp:17,
 * 45-55, 406): with enable != 0 the next bem_setup appends the interior
 * free-surface panels of bem_body_props.aux (and their mirror images) to the
 * system after the hull panels, so bem_solve solves for hull + lid unknowns
 * and integrates forces over the hull; a zero frequency is solved at
 * Omega = 1e-3.  bem_get_sizes still reports the hull panel count.  Set before
 * bem_setup. */
bem_status bem_set_ifr(bem_ctx* ctx, int enable);
bem_status bem_set_kochin(bem_ctx* ctx, int n_kochin);

/* ---- mesh import --------------------------------------------------------------
 * Reads the mesh files the reference imports, with the reference readers'
 * rules: GDF (GDF_Geometry, GDF_Geo.cpp:12-103), MAR (NEMOH; MAR_Geometry,
 * MAR_Geo.cpp:12-96), ASCII STL (STL_Geometry, STL_Geo.cpp:12-94: positions x
 * 100, corners stored C3 C2 C1) and PNL (HAMS; PNL_Geometry, PNL_Geo.cpp:17-129).
 * BEM_MESH_AUTO picks the reader from ".gdf" / ".mar" / ".stl" / ".pnl" in
 * the path, as the console does (BEMUser_Console.cpp:40-42).  Elements follow
 * the bem_mesh convention (four 0-based node indices, -1 for a triangle's
 * fourth).  Call with nodes == NULL or elems == NULL for the sizes, then with
 * arrays of *n_nodes x 3 doubles and *n_elems x 4 ints.  A malformed line (the
 * reference's std::stod / std::stoi throw) or a panel naming a missing node
 * returns BEM_ERR_ARG, with the reason in bem_read_mesh_error().  Host only. */
enum { BEM_MESH_AUTO = 0, BEM_MESH_GDF = 1, BEM_MESH_MAR = 2, BEM_MESH_STL = 3, BEM_MESH_PNL = 4 };
bem_status bem_read_mesh(const char* path, int format, int* n_nodes, double* nodes, int* n_elems, int* elems);
const char* bem_read_mesh_error(void);

/* ---- result files ----------------------------------------------------------
 * Writes <prefix>.1 .2 .2fk .2sc .4 .hst .mmx in the WAMIT formats of
 * Generate_Output_File_WAMIT / Update_Output_File_WAMIT
 * (Hydrodynamic_Solver_IO.cpp:430-646) for the frequencies omega[0..n_freq) and
 * the results r of bem_solve (A, B, FK, SC, F, RAO; NULL blocks are skipped).
 * The frequency column is the reference's input Frequency = 2 pi Omega; forces
 * are divided by g = 9.81; .hst holds C / (rho g), .mmx holds M / rho.  Omega = 0
 * writes added mass only.  Host only; no device needed. */
bem_status bem_write_wamit(const char* prefix, const bem_wamit_info* info, int n_freq, const double* omega,
                           const bem_result* r);

/* ---- dense complex solve that allocates nothing --------------------------------
 * This entry point has no counterpart in the reference.  It is the FP64 solve of
 * bem_dense_solve (same kernels, same results) for callers that cannot call
 * cudaMalloc: code inside an application that hands all device memory to its own
 * pool allocator, or a loop where cudaMalloc's implicit device-wide
 * synchronization and latency are not acceptable.  It calls no cudaMalloc,
 * cudaFree or allocating library routine; every buffer it needs lives in one
 * fixed file-scope device array (10.9 MB, for n <= BEM_NOALLOC_MAX_N), which
 * every GPU that loads the library holds until the process exits.
 *   - Orders n > BEM_NOALLOC_MAX_N or nrhs outside [1, 16] are rejected with
 *     BEM_ERR_ARG and a message.
 *   - The first call on a device looks up the array's device address (with that
 *     device current); make that first call before any stream capture.  With
 *     lazy module loading (CUDA_MODULE_LOADING=LAZY, the default) that first
 *     call is also when the driver loads this code and reserves the array, so it
 *     can fail with BEM_ERR_CUDA if a pool allocator has already taken all device
 *     memory: make the first call before the pool reserves its memory, or run
 *     with CUDA_MODULE_LOADING=EAGER.  Later calls allocate nothing.
 *   - The address is kept per device for the life of the process; calls after a
 *     cudaDeviceReset of that device are not supported.
 *   - All calls share the one array: calls that overlap on the GPU (other host
 *     threads, other streams) race and corrupt each other's results.
 *   - Work runs on the legacy default stream; the call returns when X is on the host.
 * A is n x n and B is n x nrhs, row-major interleaved complex host arrays; X
 * overwrites B.  Errors: bem_last_error(NULL). */
#define BEM_NOALLOC_MAX_N 512
bem_status bem_dense_solve_noalloc(int device, int n, const double* A, int nrhs, double* B);

/* Number of kernel launches this library has issued since it was loaded. */
unsigned long long bem_launch_count(void);

/* Diagnostic with no reference counterpart: one launch of the tensor-core
 * (tcgen05, TF32) product kernel of the LU in one of its tile modes, on caller
 * data, so that its arithmetic can be checked against an exact product.  All
 * arrays are planar complex FP32 host arrays (the real plane, then the
 * imaginary plane); operands should hold TF32 values (the tensor cores ignore
 * the low 13 mantissa bits).  C is n x n (row-major, n a multiple of 256 in
 * [512, 8192]) and is updated in place; Wa, Ua, Wb, Ub are n x 128; T is
 * 128 x 128 (modes 3, 4) or (n / 256) x 128 x 128 (modes 5, 6).
 *   0  C[128:, 128:] -= Wa[0:n-128] Ua[0:n-128]^T                       (trailing update)
 *   1  C[128:, 128:] -= Wa Ua^T + Wb Ub^T over the same rows, K = 256  (two steps per pass)
 *   2  mode 1 on the L of width 2 only (tile columns 0-1, then tile rows 0-1), without
 *      its first tile                                                  (cross update)
 *   3  W = C[128:, 0:128] T^T, stored rounded to TF32 into Wout rows 0.. and over
 *      C[128:, 0:128]                                                  (W21 = A21 D^-1)
 *   4  C[0:n-128, n-128:] <- C[0:n-128, n-128:] T^T, rounded to TF32    (U D^-1)
 *   5  for each 128-block pair p: C_{r,2p} -= C_{r,2p+1} T_p^T, block rows r >= 2p+2  (L fold)
 *   6  for each pair p: C_{r,2p+1} -= C_{r,2p} T_p^T, block rows r < 2p              (U fold)
 * Errors: BEM_ERR_ARG with the reason in bem_last_error(NULL). */
bem_status bem_tc_probe(int device, int mode, int n, float* C, const float* Wa, const float* Ua, const float* Wb,
                        const float* Ub, const float* T, float* Wout);

/* Measured FP32 throughput of `device` in TFLOP/s (an FMA loop timed with CUDA
 * events, 2 flops per FMA): the roofline denominator of the FP32-bound wave
 * assembly.  No reference counterpart. */
bem_status bem_fp32_peak(int device, double* tflops);

/* Device time (ms, CUDA events, best of two after a warm-up) of cuSOLVER's complex LU
 * with partial pivoting (cusolverDnZgetrf) of a dense n x n complex matrix (seeded,
 * entries of size 0.2 / sqrt(n) plus 0.5 on the diagonal): the library figure beside the
 * plain FP64 path's own LU.  Measurement only; cuSOLVER is opened at run time and its
 * absence returns BEM_ERR_UNSUPPORTED.  No reference counterpart. */
bem_status bem_cusolver_zgetrf_ms(int device, int n, double* ms);

/* Library version string. */
const char* bem_version(void);

#ifdef __cplusplus
}
#endif
#endif /* BEMGPU_H */
