/* C ABI of the GB300-native (sm_103a) Galerkin hot path of VortexPanel.jl: libvortexpanel_gpu.so.
 *
 * Plain pointers and sizes only. Host arrays are caller-owned and read or written during the call; the assembled
 * system and its factorization stay resident on the GPU behind opaque handles until freed. Indices are 0-based,
 * matrices row-major unless stated. Every entry point returns a vp_status; vp_last_error() gives the message of the
 * last failure on a context. One CUDA stream per context; calls are synchronous at the boundary. A context is not
 * safe for concurrent use from several threads; separate contexts are independent.
 *
 * Reference interfaces replaced (paths within the VortexPanel.jl project):
 *   vp_assemble        <- Assembly.assemble(g, dm, els, σ, V∞; opts, wake)       src/assembly/assemble.jl:377-447
 *   vp_factorize       <- Assembly.factorize_galerkin(dm, A; W)                    src/assembly/solve.jl:81-87
 *   vp_solve           <- Assembly.solve_galerkin(F::GalerkinFactorization, b)     src/assembly/solve.jl:95-99
 *   vp_solve_system    <- Assembly.solve_galerkin(dm, A, b; W)                     src/assembly/solve.jl:51-59
 */
#ifndef VORTEXPANEL_GPU_H
#define VORTEXPANEL_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    VP_OK = 0,
    VP_ERR_ARG = 1,        /* invalid argument or option (ArgumentError / DimensionMismatch in the reference) */
    VP_ERR_DEGENERATE = 2, /* degenerate triangle (SourceTriangle's ArgumentError, source_triangle.jl:21) */
    VP_ERR_SINGULAR = 3,   /* zero pivot in the LU (LAPACK SingularException) */
    VP_ERR_NOCONV = 4,     /* iterative refinement did not converge */
    VP_ERR_TIMEOUT = 5,    /* a bounded device-side wait gave up */
    VP_ERR_CUDA = 6,       /* CUDA runtime or cuBLAS failure */
    VP_ERR_NOMEM = 7       /* device allocation failed */
} vp_status;

typedef enum {
    VP_FP64 = 0,  /* every integral, the LU and the solve in FP64 */
    VP_MIXED = 1  /* FP32 far/near tiers, FP64 touching tiers; FP32-class LU refined in FP64 */
} vp_precision;

typedef struct vp_ctx vp_ctx;
typedef struct vp_system vp_system; /* the assembled A (nslot x (nslot + nwake)) and b, on the GPU */
typedef struct vp_factor vp_factor; /* the LU of the bordered system, on the GPU */

/* AssemblyOptions (src/assembly/assemble.jl:26-41); test: 0 hat, 1 onering, 2 dual */
typedef struct {
    int test;
    double far_ratio;
    int far_points;
    int near_points;
    double near_ratio;
    int near_depth;
    int touch_levels;
    double touch_ratio;
    int touch_order;
    double corner_angle;
    double contact_rel;
    double kernel_far;
    int precision; /* vp_precision */
} vp_assembly_options;

/* The reference's stats: pairs and quadrature points per tier (self, edge, vertex, contact, near, far) */
typedef struct {
    long long pairs[6];
    long long points[6];
    double time_ms;
    long long points_fp64; /* points evaluated in FP64 (all of them with VP_FP64) */
} vp_assembly_stats;

/* Fill the reference's default AssemblyOptions (FP64). */
void vp_default_options(vp_assembly_options* opts);

/* A context on CUDA device `device`: its stream, cuBLAS handle and workspaces. */
int vp_ctx_create(int device, vp_ctx** out);
void vp_ctx_destroy(vp_ctx* ctx);
const char* vp_last_error(const vp_ctx* ctx);

/* assemble (src/assembly/assemble.jl:377-447).
 *   x (nnode x 3), tris (ntri x 3), corner_slot (ntri x 3), touch_pairs (ntouch x 2, triangle pairs that get the
 *   deeper near rule), sigma (ntri), vinf (3).
 *   Wake (may be absent: nwnode = 0): wx (nwnode x 3), wtris (nwtri x 3, wake node indices), fil (nfil x 2).
 * On success *out holds A (nslot x (nslot + nwnode)) and b (nslot) on the GPU; stats may be NULL. */
int vp_assemble(vp_ctx* ctx, const vp_assembly_options* opts, int nnode, const double* x, int ntri, const int* tris,
                const int* corner_slot, int nslot, int ntouch, const int* touch_pairs, const double* sigma,
                const double* vinf, int nwnode, const double* wx, int nwtri, const int* wtris, int nfil,
                const int* fil, vp_system** out, vp_assembly_stats* stats);

/* Test triangles per tile of the far tier's kernel (the tile each CTA holds in shared memory against a 128-source
 * tile), per precision: 1, 2 or 4 in VP_FP64 (default 4), 2, 4 or 8 in VP_MIXED (default 8). The autotuner
 * (vortexpanel_gpu/autotune.py) picks it per mesh size from a measured sweep. No counterpart in the reference. */
int vp_set_far_tile(vp_ctx* ctx, int precision, int tile);
/* The current far tile of a precision (0 for a bad argument). */
int vp_get_far_tile(const vp_ctx* ctx, int precision);

/* One system of a batch: the arguments of vp_assemble for one body with its wake. */
typedef struct {
    int nnode;
    const double* x;
    int ntri;
    const int* tris;
    const int* corner_slot;
    int nslot;
    int ntouch;
    const int* touch_pairs;
    const double* sigma;
    const double* vinf;
    int nwnode;
    const double* wx;
    int nwtri;
    const int* wtris;
    int nfil;
    const int* fil;
} vp_assembly_input;

/* assemble (src/assembly/assemble.jl:377-447) of nsys independent systems of uneven sizes in shared launches: the far
 * tier one launch per colour of test tiles over every system, the near tier's lanes and the rest kernels one launch
 * per colour of test triangles over every system, and the self, touching and contact pairs of all of them in one
 * persistent launch. Every system's A and b are those vp_assemble gives it, bit for bit. One options set and
 * precision for the whole batch. out[k] receives system k; stats (nsys entries) may be NULL. No counterpart in the
 * reference, which assembles one body at a time. */
int vp_assemble_batch(vp_ctx* ctx, const vp_assembly_options* opts, int nsys, const vp_assembly_input* in,
                      vp_system** out, vp_assembly_stats* stats);

/* Rows and columns of the assembled A. */
int vp_system_shape(const vp_system* sys, int* nrows, int* ncols);
/* Copy A (row-major, nrows x ncols) and/or b (nrows) to the host; either pointer may be NULL. */
int vp_system_download(vp_ctx* ctx, const vp_system* sys, double* A, double* b);
/* Copy rows [r0, r1) of A (row-major, (r1 - r0) x ncols) and/or of b to the host; either pointer may be NULL. */
int vp_system_download_rows(vp_ctx* ctx, const vp_system* sys, int r0, int r1, double* A, double* b);
void vp_system_free(vp_system* sys);

/* factorize_galerkin (src/assembly/solve.jl:81-87): the bordered system (solve.jl:15-38) of the reduction
 * C' A [C; W] (src/dofmap/system.jl:141-145), one border row per body, factored by a blocked LU with partial
 * pivoting on the GPU (precision: vp_precision).
 *   C: CSR (nslot x nq): C_rowptr (nslot + 1), C_col, C_val.  W: CSR (nwake x nq) of the wake rows, or nwake = 0.
 *   nbody bodies; q_body (nq, 1-based body of every unknown, 0 for none); slot_area, slot_body (nslot, 1-based).
 * *cond receives the 1-norm condition estimate of the bordered matrix (may be NULL). */
int vp_factorize(vp_ctx* ctx, const vp_system* sys, int precision, int nq, const int* C_rowptr, const int* C_col,
                 const double* C_val, int nwake, const int* W_rowptr, const int* W_col, const double* W_val,
                 int nbody, const int* q_body, const double* slot_area, const int* slot_body, vp_factor** out,
                 double* cond);

/* solve_galerkin(F, b) (src/assembly/solve.jl:95-99) for nrhs right hand sides over the slots:
 *   b (nslot x nrhs, column-major), q (nq x nrhs, column-major), lambda (nbody x nrhs, column-major; may be NULL).
 * With VP_MIXED factors the solution is refined to FP64 accuracy with FP64 residuals of the bordered matrix. */
int vp_solve(vp_ctx* ctx, const vp_factor* F, int nrhs, const double* b, double* q, double* lambda);

/* solve_galerkin(dm, A, b; W) (src/assembly/solve.jl:51-59) for the system's own b: q (nq), lambda (nbody),
 * residual = |M x - rhs| / |rhs| of the bordered system (any output may be NULL). */
int vp_solve_system(vp_ctx* ctx, const vp_factor* F, const vp_system* sys, double* q, double* lambda,
                    double* residual);

/* Adjoint (no counterpart in the reference, which differentiates with ForwardDiff duals): the transposed bordered
 * solve M' [xi; eta] = [g; 0] with the same factors, for nrhs right hand sides g (nq x nrhs, column-major); xi (nq x
 * nrhs) out. VP_MIXED factors are refined with FP64 residuals of M'. */
int vp_solve_transposed(vp_ctx* ctx, const vp_factor* F, int nrhs, const double* g, double* xi);

/* Adjoint pair derivatives (no counterpart in the reference): for the inputs of vp_assemble, nadj (1 or 2) vectors
 * of row values nu (nslot x nadj, column-major) and column values mu (nslot + nwnode), the derivatives of
 * F_k = nu_k' (A(x) mu - b(x)) with respect to the body nodes (grad_x, nnode x 3 per vector), the wake nodes
 * (grad_wx, nwnode x 3 per vector) and the angle of attack (dalpha, nadj), with sigma = -vinf·n differentiated as such
 * and dvinf = d vinf / d alpha. The quadrature of every pair is the assembly's; the vectors share one evaluation of
 * every point. stats may be NULL. For J(x, q) with M q = r: dJ/dx = dJ/dx|_q - dF/dx with nu = C xi,
 * mu = [C q; W q], xi from vp_solve_transposed with g = dJ/dq. The outputs are the same bit for bit from call to call
 * on the same inputs (the sums over pairs are exact integer sums of once-rounded terms, whatever their order). */
int vp_adjoint(vp_ctx* ctx, const vp_assembly_options* opts, int nnode, const double* x, int ntri, const int* tris,
               const int* corner_slot, int nslot, int ntouch, const int* touch_pairs, const double* sigma,
               const double* vinf, int nwnode, const double* wx, int nwtri, const int* wtris, int nfil, const int* fil,
               int nadj, const double* nu, const double* mu, const double* dvinf, double* grad_x, double* grad_wx,
               double* dalpha, vp_assembly_stats* stats);

/* Instrumentation (no counterpart in the reference, which only times with @elapsed): device milliseconds per phase
 * since the last reset, measured with CUDA events on the context's stream, in the order setup, classify, far, near
 * (near tier and the adding of the pair blocks), reduce, lu, cond, solve, adjoint setup, adjoint far, adjoint near
 * (near tier, filaments, freestream), adjoint solve, free wake, near pairs (the touching and contact pairs of the
 * assembly), adjoint pairs (those of the adjoint), the free wake simulation's explicit right hand side and its
 * velocities (n entries at most), and the number of this library's kernel launches. */
int vp_phase_times(vp_ctx* ctx, double* ms, int n, long long* launches, int reset);
/* Instrumentation (no counterpart in the reference): bytes copied host->device and device->host by the library. */
int vp_transfer_bytes(vp_ctx* ctx, long long* h2d, long long* d2h, int reset);

/* Diagnostics (no counterpart in the reference): the device kernels at n points, one thread per point.
 *   mode 0: w (3 per point), the unit source velocity of triangle tri (9 per point) at x (3 per point), with the
 *           far-field switch kernel_far and the in-plane side (source_triangle.jl:134-138);
 *   mode 1: s = w·m (m: 3 per point) and its derivatives with respect to x and the triangle's corners (1 + 3 + 9);
 *   mode 2: the filament from tri[0:3] to tri[3:6] with end weights ca = tri[6], cb = tri[7]: s = ca va·m + cb vb·m
 *           (segment.jl:15-25) and its derivatives with respect to x and the two ends (1 + 3 + 6).
 * precision VP_FP64 or VP_MIXED (the FP32 kernels, without the FP64 guard); any other value returns VP_ERR_ARG. */
int vp_eval_points(vp_ctx* ctx, int mode, int precision, int n, const double* tri, const double* x, const double* m,
                   int side, double kernel_far, double* out);

/* No counterpart in the reference. vp_eval_points with no device allocation, for callers that cannot allocate device
 * memory while they run: a host that keeps the device's memory in a pool of its own (Julia's CUDA.jl, a framework's
 * caching allocator) and leaves little outside it, or a stepping loop that cannot afford cudaMalloc/cudaFree, which
 * synchronise the device. Inputs and outputs are staged through a fixed device array of VP_STATIC_POINTS_MAX points
 * (about 0.45 MB, held by every device that loads the library until the process exits); n above that returns
 * VP_ERR_ARG, and so does a precision other than VP_FP64 or VP_MIXED. The array's address is looked up on the first
 * call for each device, which must come before any stream capture on that device, and again on the first call after
 * the device's CUDA context has changed (a cudaDeviceReset). The caller's current device is restored on return.
 * Calls that overlap in time on one device share the array and race: serialise them. */
#define VP_STATIC_POINTS_MAX 2048
int vp_eval_points_static(vp_ctx* ctx, int mode, int precision, int n, const double* tri, const double* x,
                          const double* m, int side, double kernel_far, double* out);

/* Free wake (src/freewake/step.jl, src/assembly/explicit.jl). Blobs are given as 7 doubles each: x (3), alpha (3),
 * core delta. precision VP_FP64, or VP_MIXED for FP32 arithmetic with FP64 accumulation.
 *   vp_blob_velocities  <- FreeWake.blob_velocities(blobs, X)                         src/freewake/step.jl:176-187
 *                          the Rosenhead-Moore sum (src/kernels/blob.jl:21-25) of every blob at every point X.
 *   vp_body_velocity    <- Post.body_velocity(els, sigma, gamma, xs; kernel_far)       src/post/Post.jl:92-112
 *                          sigma_s w_s + gamma_s x w_s of every triangle (corners 9, sigma 1, gamma 3 each) at X.
 *   vp_explicit_rhs     <- Assembly.explicit_rhs(els, dm, ExplicitSources(...); opts) src/assembly/explicit.jl:31-85
 *                          -int psi_i n.u dA of known sheets (corners 9, corner doublets 3 each), filaments (ends 6,
 *                          end circulations 2 each) and particles, one value per slot (rhs, nslot). */
int vp_blob_velocities(vp_ctx* ctx, int precision, int nblob, const double* blobs, int npts, const double* X,
                       double* U);
int vp_body_velocity(vp_ctx* ctx, int precision, int ntri, const double* corners, const double* sigma,
                     const double* gamma, double kernel_far, int npts, const double* X, double* U);
int vp_explicit_rhs(vp_ctx* ctx, const vp_assembly_options* opts, int nnode, const double* x, int ntri,
                    const int* tris, const int* corner_slot, int nslot, int nsheet, const double* sheet_x,
                    const double* sheet_mu, int nseg, const double* seg_x, const double* seg_gamma, int nblob,
                    const double* blobs, double* rhs);

/* consistency (src/assembly/solve.jl:111-115): the quadrature diagnostics of the assembled system in terms of
 * A Cf, Cf = [C; W] (C: CSR nslot x nq; W: CSR nwake x nq of the wake rows, nwake = 0 without wake columns):
 * out[0] = max |row sum| / |A Cf|_inf, out[1] = max |column sum| / |A Cf|_inf, out[2] = |sum b| / sum |b|.
 * FP64 on the GPU, summed in a fixed order. */
int vp_consistency(vp_ctx* ctx, const vp_system* sys, int nq, const int* C_rowptr, const int* C_col,
                   const double* C_val, int nwake, const int* W_rowptr, const int* W_col, const double* W_val,
                   double* out);

/* The gradient route's surface loads in FP64 on the GPU:
 *   gradient_velocity (src/post/Post.jl:72-73): u = V - (V.n)n + grad mu on every triangle (u: ntri x 3, may be NULL);
 *   pressure_coefficient (Post.jl:82-84): cp = 1 - (|u|^2 + 2 dmu/dt)/|V|^2 with dmu/dt the mean of the corners'
 *     slot values of dmudt (nslot; NULL for steady flow) (cp: ntri, may be NULL);
 *   pressure_force (src/post/forces.jl:11-20): F = -sum cp A n and M = sum (c - origin) x (-cp A n) (3 each; origin may
 *     be NULL for 0).
 * corners: ntri x 9; corner_slot: ntri x 3; mu: nslot. */
int vp_surface_loads(vp_ctx* ctx, int ntri, const double* corners, const int* corner_slot, int nslot,
                     const double* mu, const double* dmudt, const double* vinf, const double* origin, double* u,
                     double* cp, double* F, double* M);
/* pressure_force(els, cp; origin) (src/post/forces.jl:11-20) of a given cp (ntri), FP64 on the GPU. */
int vp_pressure_force(vp_ctx* ctx, int ntri, const double* corners, const double* cp, const double* origin, double* F,
                      double* M);
/* kutta_joukowski_force and trefftz_drag (src/post/forces.jl:34-39,53-81) of the doublets mu_w (nte) at the wake's
 * trailing edge nodes te_x (nte x 3), along nline lines (line_ptr: nline + 1 offsets into line_nodes, 0-based node
 * indices; line_closed: nline flags): F_kj (3) and D_trefftz (1), in units of q∞. FP64 on the GPU. */
int vp_wake_loads(vp_ctx* ctx, int nte, const double* te_x, int nline, const int* line_ptr, const int* line_nodes,
                  const int* line_closed, const double* mu_w, const double* vinf, double* F_kj, double* D_trefftz);

/* The free wake as a simulation resident on the GPU: FreeWakeSim(g, dm, V∞; opts, assembly), step!(sim), run!(sim, n)
 * (src/freewake/step.jl:8-58,113-146,205-216) over the state of src/freewake/state.jl:132-147 (node rows newest first
 * with their shed doublets, mu_line, particles with their merge tags and the strips' merge batches). The host resolves
 * FreeWakeOptions (state.jl:25-48: te_len, max_rows, merge_rows, the core rule, delete_beyond), builds the trailing
 * edge panel (te_panel), assembles the body with it and factors the bordered matrix (vp_assemble, vp_factorize); the
 * set-up hands those and the DOF map to the simulation. A step allocates nothing: the particle arrays hold
 * particle_capacity particles and grow (a reallocation) only when a step could overflow them. */
typedef struct vp_freewake vp_freewake;

typedef struct {
    /* FreeWakeOptions, resolved: the time step; free panel rows kept before the oldest is converted (max_rows); the
     * CoreRule (state.jl:64-92: core_mode 0 auto, 1 scaled, 2 the fixed radius core_value; overlap, core_factor and
     * core_floor); advection 0 free, 1 freestream; particles with x.V/|V| above delete_limit are removed
     * (delete_beyond spans past the trailing edge; +inf keeps all) */
    double dt;
    int keep_rows;
    int core_mode;
    double overlap, core_factor, core_floor, core_value;
    int advection;
    double delete_limit;
    vp_assembly_options assembly; /* the explicit right hand side's tiers and the precision of the step */
    /* the body (vp_assemble's inputs), its bordered factorization with the trailing edge panel and that system's b */
    int nnode;
    const double* x;
    int ntri;
    const int* tris;
    const int* corner_slot;
    int nslot;
    const double* sigma;
    const double* vinf;
    const vp_factor* factor;
    const double* b0;
    /* the DOF map: C (CSR nslot x nq) gives mu = C q, K (CSR nte x nq) the trailing edge doublets mu_w = K q */
    int nq;
    const int* C_rowptr;
    const int* C_col;
    const double* C_val;
    int nte;
    const int* K_rowptr;
    const int* K_col;
    const double* K_val;
    /* the wake's trailing edge nodes (nte x 3) and lines (as in vp_wake_loads), for Kutta-Joukowski */
    const double* te_x;
    int nline;
    const int* line_ptr;
    const int* line_nodes;
    const int* line_closed;
    /* Topology (state.jl:99-121): strips (nstrip x 2 trailing edge nodes), the first and last nodes of open lines */
    int nstrip;
    const int* strips;
    int nfirst;
    const int* first_nodes;
    int nlast;
    const int* last_nodes;
    /* the trailing edge panel: its downstream edge (nte x 3, where new rows are shed), and as a rigid wake its nodes
     * (npw x 3) with the trailing edge node of each (pw_te), triangles (npt x 3) and filaments (npf x 2) */
    const double* edge;
    int npw;
    const double* pw_x;
    const int* pw_te;
    int npt;
    const int* pt_tris;
    int npf;
    const int* pf;
    const int* merge;      /* merge_rows per strip (nstrip), or NULL for no merging */
    int particle_capacity; /* particles held before the first reallocation */
} vp_freewake_setup;

/* step!'s record (step.jl:137-139): forces in units of q∞ */
typedef struct {
    int n;
    double t;
    double F_pressure[3], M_pressure[3], F_kj[3], F_impulse[3], Omega[3], I[3];
    int rows, particles;
    double lambda, umax;
} vp_freewake_record;

typedef struct {
    int n;            /* steps taken */
    double t;         /* simulated time */
    int nrows;        /* node rows (free panel rows + 1; 0 before the first step) */
    int nparticles;
    int conversions;
    double I_prev[3]; /* the last step's impulse (the next F_impulse's backward difference) */
} vp_freewake_counts;

int vp_freewake_create(vp_ctx* ctx, const vp_freewake_setup* setup, vp_freewake** out);
/* step!(sim) (step.jl:113-146); rec may be NULL. */
int vp_freewake_step(vp_freewake* fw, vp_freewake_record* rec);
int vp_freewake_info(const vp_freewake* fw, vp_freewake_counts* counts);
/* The state to host arrays (any pointer may be NULL): rows_x (nrows x nte x 3, newest first), rows_mu (nrows x
 * nte), mu_line (nte), particles (nparticles x 7: x, alpha, delta), tag, group (nparticles), batch_rows,
 * batch_length, batch_width (nstrip), and the last step's mu (nslot), mu_w (nte) and cp (ntri). */
int vp_freewake_get_state(const vp_freewake* fw, double* rows_x, double* rows_mu, double* mu_line, double* particles,
                          int* tag, signed char* group, int* batch_rows, double* batch_length, double* batch_width,
                          double* mu, double* mu_w, double* cp);
/* Restore a state taken by vp_freewake_get_state from a simulation of the same body and options (a checkpoint). */
int vp_freewake_set_state(vp_freewake* fw, const vp_freewake_counts* counts, const double* rows_x,
                          const double* rows_mu, const double* mu_line, const double* particles, const int* tag,
                          const signed char* group, const int* batch_rows, const double* batch_length,
                          const double* batch_width, const double* mu, const double* mu_w, const double* cp);
void vp_freewake_free(vp_freewake* fw);

/* Diagnostics (no counterpart in the reference): C -= A B for FP32 column-major host arrays A (m x k, lda), B (k x n,
 * ldb), C (m x n, ldc) through the tensor-core GEMM of the mixed-precision LU's trailing updates (each operand split
 * into three bf16 pieces, six tcgen05 products accumulated in FP32). */
int vp_gemm_sub_f32(vp_ctx* ctx, int m, int n, int k, const float* A, int lda, const float* B, int ldb, float* C,
                    int ldc);

/* Condition estimate and size of a factorization. */
int vp_factor_info(const vp_factor* F, int* n, double* cond);
void vp_factor_free(vp_factor* F);

#ifdef __cplusplus
}
#endif
#endif /* VORTEXPANEL_GPU_H */
