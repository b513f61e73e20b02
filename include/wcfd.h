/*
 * wcfd.h -- C ABI of libwcfd.so, the GB300 (sm_103a) kernels of the collocated
 * finite-volume SIMPLE/PISO step.
 *
 * Conventions
 *   - Every pointer in the structs below is a DEVICE pointer owned by the caller
 *     (in the Python layer: torch tensors).  The library allocates no device memory
 *     on any path declared here except where an entry point says so.
 *   - Every call is asynchronous on the given cudaStream_t (passed as void*; NULL =
 *     legacy default stream) and returns an int status (WCFD_OK = 0).
 *   - Solver outcomes (iteration count, final residual, breakdown, barrier timeout)
 *     are written to a caller-owned device wcfd_solve_stats record; reading it is
 *     the caller's synchronisation point.
 *   - Floating point: fields, geometry and matrices are fp32; Krylov dot products and
 *     residual norms are accumulated in fp64.
 *   - No exception crosses the ABI.  One host thread per case at a time.
 *
 * The reference (warp_cfd, NVIDIA Warp) has no C ABI: its operator API is the Python
 * package.  Each entry point below names the reference function/kernel it replaces
 * (path:line within the warp_cfd project).
 */
#ifndef WCFD_H
#define WCFD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
#define WCFD_OK                  0
#define WCFD_ERR_ARGUMENT        1  /* null pointer, bad size or flag              */
#define WCFD_ERR_CUDA            2  /* a CUDA runtime call failed (see last_error)  */
#define WCFD_KRYLOV_BREAKDOWN    3  /* a Krylov denominator became exactly zero     */
#define WCFD_NOT_CONVERGED       4  /* maxiter reached (informational, as in warp)  */
#define WCFD_BARRIER_TIMEOUT     5  /* a grid barrier wait gave up (bounded spin)   */
#define WCFD_ERR_TOO_LARGE       6  /* size beyond what the entry point supports    */

/* field mask bits: u, v, w, p (columns 0..3 of cell_values) */
#define WCFD_U 1u
#define WCFD_V 2u
#define WCFD_W 4u
#define WCFD_P 8u
#define WCFD_ALL 15u

/* ------------------------------------------------------------------ mesh (SoA)
 * K faces, C cells, B boundary faces, F local face slots per cell (uniform cell type),
 * W = max internal faces of any cell (width of the slot-major off-diagonal storage).
 * Face ids and their order are the reference's (unique sorted node tuples).
 */
typedef struct wcfd_mesh {
    int32_t n_cells;          /* C */
    int32_t n_faces;          /* K */
    int32_t n_bfaces;         /* B */
    int32_t faces_per_cell;   /* F (<= 6) */
    int32_t ell_width;        /* W (<= F) */
    int32_t pad_;
    const int32_t* face_owner;    /* [K]   owner cell (lower id)                      */
    const int32_t* face_nbr;      /* [K]   neighbour cell, -1 on boundary faces       */
    const int32_t* face_brow;     /* [K]   row in the boundary tables, -1 internal    */
    const float*   face_interp;   /* [K*4] skew vector r_f - (psi r_P + (1-psi) r_N), psi */
    const float*   face_normal;   /* [K*4] owner's outward unit normal, area          */
    const float*   face_gdiff;    /* [K]   area/|d| (internal; x|n1| when corrected), area/|r_Pf| (boundary) */
    const float*   face_rpf;      /* [K]   |r_P->f| (owner centroid to face centroid) */
    const float*   cell_slot;     /* [F*C*4] slot-major: A n_cf / V (3), bits of the signed face id
                                     (k for the owner side, ~k for the neighbour side;
                                     INT32_MIN with a zero vector: a null slot of a cell
                                     with fewer faces than F in a mixed mesh) */
    const float*   cell_volume;   /* [C]                                               */
    const int32_t* ell_col;       /* [W*C] slot-major neighbour column; padding = own row */
    const int32_t* boundary_face; /* [B]   face id of each boundary row               */
    const float*   face_dvec;     /* [K*4] owner->neighbour centroid vector d (internal faces)
                                     and 0; read only by the opt-in explicit internal terms
                                     (wcfd_params.explicit_terms), may be NULL otherwise */
    const int16_t* ell_dcol;      /* [W*C] ell_col - row as int16, when every |ell_col - row|
                                     <= 32767 (e.g. a structured numbering), else NULL: the
                                     grid-cooperative CG then streams 2 bytes per slot
                                     instead of 4 (the same columns, the same bits) */
} wcfd_mesh;

/* boundary tables, one row per boundary face, columns u,v,w,p */
typedef struct wcfd_bc {
    const uint8_t* type;   /* [B*4] 1 = fixed value, 2 = fixed normal gradient */
    const float*   value;  /* [B*4]                                             */
} wcfd_bc;

/* the model's field state (the reference's FVM arrays, model.py:167-171) */
typedef struct wcfd_state {
    float* cell_values;     /* [C*4]   u,v,w,p                      */
    float* cell_gradients;  /* [C*4*3]                               */
    float* face_values;     /* [K*4]                                 */
    float* face_gradients;  /* [K*4]   only boundary rows are used   */
    float* mass_fluxes;     /* [K]                                   */
} wcfd_state;

/* scalar or 3-component system on the mesh pattern: diagonal + W off-diagonals per row
 * (slot-major, column = mesh.ell_col).  For the momentum system the off-diagonals are
 * shared by u, v, w and diag/rhs are interleaved [C*3] (row 3c+o, as the reference's
 * interleaved BSR rows D*i+o, equation_kernels.py:10-38). */
typedef struct wcfd_system {
    float* diag;     /* [C] or [C*3] */
    float* off;      /* [W*C]        */
    float* rhs;      /* [C] or [C*3] */
    int32_t ncomp;   /* 1 or 3       */
    int32_t pad_;
} wcfd_system;

#define WCFD_MAX_BLOCKS 2048
#define WCFD_BARRIER_WORDS (WCFD_MAX_BLOCKS + 4)

/* Krylov workspace (caller-allocated, see wcfd_krylov_workspace_floats) */
typedef struct wcfd_krylov_ws {
    float*    vec;        /* wcfd_krylov_workspace_floats(C, ncomp) floats            */
    double*   partials;   /* 8 * WCFD_MAX_BLOCKS doubles (reduction partials), 16-byte aligned */
    double*   results;    /* unused, may be NULL                                      */
    uint32_t* barrier;    /* WCFD_BARRIER_WORDS words: [WCFD_MAX_BLOCKS] the error word,
                             [WCFD_MAX_BLOCKS + 2] the grid barrier's arrival counter
                             (the rest unused); every solve call zeroes them first   */
} wcfd_krylov_ws;

typedef struct wcfd_solve_stats {
    int32_t iterations;
    int32_t status;            /* WCFD_OK, WCFD_NOT_CONVERGED, WCFD_KRYLOV_BREAKDOWN, WCFD_BARRIER_TIMEOUT */
    double  residual;          /* ||b - A x||_2 at exit (fp64)                              */
    double  initial_residual;  /* ||b - A x0||_2 at entry: the outer iteration's residual   */
    double  rhs_norm;          /* ||b||_2                                                   */
} wcfd_solve_stats;

/* per-case scalars of one SIMPLE iteration / PISO step */
typedef struct wcfd_params {
    float   nu;             /* kinematic viscosity mu/rho (incompressible.py:89) */
    float   rho;            /* density                                           */
    float   u_relax;        /* implicit momentum relaxation; <= 0 = none          */
    float   p_relax;        /* explicit p relaxation; <= 0 = replace              */
    float   dt;             /* PISO time step                                     */
    float   ref_value;      /* reference pressure value                           */
    int32_t ref_cell;       /* reference pressure cell, -1 = none                 */
    int32_t steady;         /* 1 = SIMPLE (steady), 0 = PISO (ddt term)           */
    int32_t n_inner;        /* pressure correctors                                */
    int32_t n_ortho;        /* non-orthogonal correctors                          */
    int32_t maxiter;        /* Krylov cap (500 in the reference)                  */
    int32_t skew;           /* skew correction in face interpolation (1)          */
    double  atol_u;         /* momentum BiCGSTAB absolute tolerance               */
    double  atol_p;         /* pressure CG absolute tolerance                     */
    int32_t p_refine;       /* fp64 iterative-refinement sweeps of the pressure solve; 0 = off */
    int32_t rhie_chow;      /* 1 = Rhie-Chow convecting flux (opt-in; the reference's path is 0) */
    double  p_refine_rtol;  /* relative tolerance of each sweep's fp32 CG correction solve */
    double  rtol_u;         /* momentum stop also at ||r|| <= rtol_u ||r_0||; 0 = atol only (the reference) */
    double  rtol_p;         /* pressure stop also at ||r|| <= rtol_p ||r_0||; 0 = atol only (the reference) */
    int32_t explicit_terms; /* opt-in internal-face explicit weights in the RHS (the reference
                               drops them): bit0 convection (skew correction), bit1 with
                               the upwindLinear term, bit2 the non-orthogonal diffusion
                               part (momentum and pressure); 0 = the reference          */
    int32_t convection;     /* implicit convection weights of the momentum system: 0 upwind
                               (incompressible.py:35; also upwindLinear, whose internal
                               explicit part the reference drops), 1 central difference
                               (convection.py:43-91 with interpolation 'central difference') */
} wcfd_params;

/* a full case: everything one SIMPLE iteration touches */
typedef struct wcfd_case {
    wcfd_mesh      mesh;
    wcfd_bc        bc;
    wcfd_state     state;
    wcfd_system    mom;        /* ncomp 3 */
    wcfd_system    pres;       /* ncomp 1 */
    float*         hbya;       /* [C*3] HbyA (incompressible.py:43), momentum x0/out */
    float*         p_x;        /* [C]   pressure solution / warm start (equation.py:68-71) */
    float*         rua;        /* [C]   rUA = V/(a_P rho)                             */
    float*         rua_faces;  /* [K]                                                */
    float*         div;        /* [C]   div of the mass flux                          */
    double*        p_x64;      /* [C]   fp64 pressure solution (p_refine > 0 only)       */
    float*         p_work;     /* [2C+4] refinement residual, correction, sweep count (p_refine > 0) */
    wcfd_krylov_ws ws_u;       /* momentum workspace (ncomp 3)                        */
    wcfd_krylov_ws ws_p;       /* pressure workspace (ncomp 1)                        */
    wcfd_solve_stats* stats;   /* [2]: [0] momentum, [1] pressure (last corrector)    */
    wcfd_params    prm;
    void* const*   events;     /* optional host array of 4 cudaEvent_t recorded before/after the
                                  momentum solve and before/after the last pressure solve; NULL = none */
} wcfd_case;

/* ------------------------------------------------------------------ info */
int         wcfd_version(void);
const char* wcfd_last_error(void);

/* Self-check of the grid barrier the grid-cooperative Krylov kernels use (no reference
 * counterpart): `phases` barriers of two sums over a full cooperative grid, every block
 * checking the sums against their closed form.  skip_block >= 0 makes that block return
 * before its first arrival, so the others' bounded waits run out (a failure made without a
 * fault).  Synchronizes the stream.  result (host): [0] the kernel's error word (WCFD_OK or
 * WCFD_BARRIER_TIMEOUT), [1] 1 if a block received wrong sums, [2] blocks in the grid. */
int wcfd_grid_barrier_check(int32_t skip_block, int32_t phases, int32_t* result, void* stream);
/* floats of wcfd_krylov_ws.vec needed for a C-row system with ncomp components */
int64_t     wcfd_krylov_workspace_floats(int32_t n_cells, int32_t ncomp);

/* ------------------------------------------------------------------ field operators */
/* FVM.set_boundary_conditions (model.py:206-208, conditions.py:5-19): fixed values onto
 * face_values, fixed gradients onto face_gradients, for every field of every boundary face. */
int wcfd_set_boundary_conditions(const wcfd_mesh* m, wcfd_bc bc, wcfd_state s, void* stream);

/* FVM.face_interpolation (model.py:210-229; interpolation_kernels.py:5-54,
 * interpolation_functions.py:5-28, skewness_functions.py:6-19) for the fields in `mask`:
 * linear, or upwind on the current mass flux when `upwind`, plus the skew correction when
 * `skew`, on internal faces; phi_P + |r_Pf| g on fixed-gradient boundary faces. */
int wcfd_face_interpolation(const wcfd_mesh* m, wcfd_bc bc, wcfd_state s, uint32_t mask,
                            int32_t skew, int32_t upwind, void* stream);

/* The three above fused in one face pass: flags bit0 = set boundary conditions first,
 * bit1 = mass flux from the new face values, bit2 = skew correction, bit3 = upwind. */
int wcfd_face_pass_flags(const wcfd_mesh* m, wcfd_bc bc, wcfd_state s, uint32_t mask,
                         uint32_t flags, void* stream);

/* FVM.calculate_mass_flux (model.py:264-266, model_kernels.py:45-60):
 * mdot = (u_f, v_f, w_f) . n_owner A. */
int wcfd_calculate_mass_flux(const wcfd_mesh* m, wcfd_state s, void* stream);

/* FVM.calculate_gradients (model.py:232-239, model_kernels.py:71-90): Green-Gauss gradient
 * of the fields in `mask`; every other field's gradient is set to zero, as the reference's
 * cell_gradients.zero_() does.  Atomic-free (one thread per cell). */
int wcfd_calculate_gradients(const wcfd_mesh* m, wcfd_state s, uint32_t mask, void* stream);

/* FVM.divFlux (model.py:269-275, model_kernels.py:26-34): div[c] = sum of +-mdot. */
int wcfd_div_flux(const wcfd_mesh* m, const float* mass_fluxes, float* div, void* stream);

/* interpolate_cell_value_to_face (solver_kernels.py:21-36): psi-weighted for internal
 * faces, owner value on boundary faces. */
int wcfd_cell_to_face(const wcfd_mesh* m, const float* cell, float* face, void* stream);

/* ------------------------------------------------------------------ assembly */
/* Momentum system of one SIMPLE iteration / PISO predictor, in one cell-parallel pass:
 * ConvectionTerm upwind (convection.py:43-91), DiffusionTerm with scalar nu
 * (diffusion.py:113-198), DdtTerm when !steady (ddt.py:24-32), explicit -grad(p) V / rho
 * (grad.py:20-29, incompressible.py:107), Equation.form_system (equation.py:99-125,
 * equation_kernels.py:52-122), implicit relaxation (equation_kernels.py:128-152) and
 * rUA = V/(a_P[u] rho) (solver_kernels.py:6-16).  No atomics: each cell writes its row. */
int wcfd_assemble_momentum(const wcfd_case* c, void* stream);

/* Pressure system: DiffusionTerm('p', nu = rUA_f) + div(HbyA) on the RHS + reference
 * row (incompressible.py:132-140, equation_kernels.py:155-175). */
int wcfd_assemble_pressure(const wcfd_case* c, void* stream);

/* rUA = V / (a_P rho) from the 3C interleaved momentum diagonal (calculate_rUA,
 * solver_kernels.py:6-16). */
int wcfd_rua(const wcfd_mesh* m, const float* diag3, float rho, float* rua, void* stream);
/* HbyA += rUA grad p, 3C interleaved rows (get_HbyA, solver_kernels.py:38-43). */
int wcfd_hbya_add(int32_t n_cells, const float* pgrad3, const float* rua, float* hbya, void* stream);

/* Implicit relaxation of an assembled system (Equation.relax, equation.py:173-182;
 * equation_kernels.py:128-152): b += (1 - alpha)/alpha d phi and d /= alpha on every
 * diagonal entry, phi the row's field in the C x 4 cell values (fields field0 ..
 * field0 + ncomp - 1).  alpha in (0, 1]. */
int wcfd_relax(const wcfd_mesh* m, wcfd_system A, const float* cell_values, int32_t field0, float alpha,
               void* stream);
/* Row `row` of a scalar system becomes the identity with rhs = value (Equation.replace_row,
 * equation.py:185-194; equation_kernels.py:155-175). */
int wcfd_replace_row(const wcfd_mesh* m, wcfd_system A, int32_t row, float value, void* stream);

/* y = A x on the mesh pattern (warp.sparse.bsr_mv; model.py:287). */
int wcfd_spmv(const wcfd_mesh* m, wcfd_system A, const float* x, float* y, void* stream);

/* ------------------------------------------------------------------ Krylov solves
 * Persistent cooperative kernels (one launch per solve, bounded grid barriers, fp64
 * reductions).  Replace warp.optim.linear.cg / bicgstab with the diagonal preconditioner
 * (Equation.solve_Axb, equation.py:195-200).  Stop: ||r||_2 <= atol before an iteration,
 * or maxiter. */
int wcfd_cg(const wcfd_mesh* m, wcfd_system A, float* x, wcfd_krylov_ws ws, double atol,
            int32_t maxiter, wcfd_solve_stats* stats, void* stream);
/* fp64 iterative refinement of a scalar solve (the precision form of the pressure solve):
 * x64 (fp64, warm start in, result out; x32 receives its fp32 copy).  Each of `sweeps`
 * sweeps computes r = b - A x64 in fp64, solves A d = r with the fp32 CG (wcfd_cg's
 * kernels) down to ||r_d|| <= inner_rtol ||r|| or maxiter, and adds d to x64.  work holds
 * 2 C + 4 floats.  `stats` (device memory) describes the correction solves: iterations is
 * their total over the sweeps, the other fields describe the last sweep's solve (its
 * initial_residual is ||b - A x64||, fp32-rounded, before that sweep). */
int wcfd_cg_refine(const wcfd_mesh* m, wcfd_system A, double* x64, float* x32, float* work, wcfd_krylov_ws ws,
                   int32_t sweeps, double inner_rtol, int32_t maxiter, wcfd_solve_stats* stats, void* stream);

/* Which CG kernel wcfd_cg runs: 0 = automatic (the cluster-resident kernel when the system
 * fits in the shared memory of one cluster of up to 16 CTAs, else the grid-cooperative
 * kernel), 1 = always grid-cooperative, 2 = cluster-resident when it fits, 3 = as 2 with
 * the single-reduction (Chronopoulos-Gear) arrangement of CG where it fits (up to 2048
 * rows per CTA): one cluster all-reduce per iteration instead of two, about 17% faster on
 * a 32,000-row system, the same iterates as textbook CG up to rounding (which, on
 * ill-conditioned systems, moves the solution at an absolute stop by ~1e-4 relative).
 * Process-wide. */
int wcfd_set_krylov_path(int32_t path);
int wcfd_bicgstab(const wcfd_mesh* m, wcfd_system A, float* x, wcfd_krylov_ws ws, double atol,
                  int32_t maxiter, wcfd_solve_stats* stats, void* stream);
/* wcfd_cg (method 0) or wcfd_bicgstab (method 1) with an added relative stop: the solve
 * ends at ||r||_2 <= max(atol, rtol ||r_0||_2).  rtol = 0 is exactly wcfd_cg / wcfd_bicgstab.
 * The reference stops on atol alone; the relative stop lets a steady outer iteration ask
 * for solves whose accuracy follows its own residual (the serving form uses it). */
int wcfd_krylov_solve(const wcfd_mesh* m, wcfd_system A, float* x, wcfd_krylov_ws ws, int32_t method,
                      double atol, double rtol, int32_t maxiter, wcfd_solve_stats* stats, void* stream);

/* Allocation-free variant of wcfd_cg (no counterpart in the reference).  For callers that
 * hold their input and output device arrays but cannot allocate device workspace (device
 * memory budgeted at start-up, plugins that may not allocate): the Krylov workspace is a
 * fixed array inside the library, sized for at most WCFD_NOALLOC_MAX_CELLS rows (about
 * 3.1 MiB, held by every GPU that loads the library until exit); larger systems return
 * WCFD_ERR_TOO_LARGE.  A call made outside stream capture looks the array's device
 * address up (again, so a device reset is picked up); a call on a stream being captured
 * uses the address remembered from the last uncaptured call on that device, so the first
 * call on a device, and the first after a device reset, must come before any capture.
 * The call allocates nothing.  All calls share the array, so calls that overlap on the
 * GPU race; results are those of wcfd_cg. */
#define WCFD_NOALLOC_MAX_CELLS 131072
int wcfd_cg_noalloc(const wcfd_mesh* m, wcfd_system A, float* x, double atol, int32_t maxiter,
                    wcfd_solve_stats* stats, void* stream);

/* ------------------------------------------------------------------ Term / Equation API
 * The reference's terms form weight arrays on the device and Equation adds them into its
 * matrix (warp_cfd/FV/terms/*.py, FV/kernels/equation_kernels.py:52-122).  Layouts as the
 * reference's: face-based weights [C][F][n][3] (owner coefficient, neighbour coefficient,
 * explicit part of cell c's side of the face in slot f), cell-based [C][n][2] (diagonal,
 * explicit part), explicit grad weights [C*3].  Every entry is written by one thread
 * (the cell's side of the face), so no atomics; all pointers are DEVICE pointers. */
typedef struct wcfd_term_fields {
    int32_t n;          /* fields of the term, 1..3 */
    int32_t index[3];   /* their columns of cell_values (u v w p = 0 1 2 3) */
} wcfd_term_fields;

/* ConvectionTerm.calculate_weights (terms/convection.py:43-91): scheme 0 upwind, 1 central
 * difference, 2 upwindLinear (Implicit_Schemes/convectionScheme.py:3-88), skew correction
 * in the explicit part as the reference's term always applies it. */
int wcfd_convection_weights(const wcfd_mesh* m, wcfd_state s, wcfd_term_fields f, int32_t scheme, float* weights,
                            void* stream);
/* DiffusionTerm.calculate_weights (terms/diffusion.py:113-198): viscosity nu, or one value
 * per face in nu_faces (device, K) when not NULL; corrected = the non-orthogonal scheme
 * (laplacianScheme.py:39-67); bc_mode 0 = the boundary table, 1 = every boundary face a
 * fixed normal gradient bc_value (the term's von_neumann / dirchlet options). */
int wcfd_diffusion_weights(const wcfd_mesh* m, wcfd_bc bc, wcfd_state s, wcfd_term_fields f, float nu,
                           const float* nu_faces, int32_t corrected, int32_t bc_mode, float bc_value, float* weights,
                           void* stream);
/* DdtTerm.calculate_weights, backward Euler (terms/ddt.py:24-32) */
int wcfd_ddt_weights(const wcfd_mesh* m, wcfd_state s, wcfd_term_fields f, float dt, float* weights, void* stream);
/* GradTerm.calculate_weights (terms/grad.py:20-29): grad(field) V, rows 3c + d */
int wcfd_grad_weights(const wcfd_mesh* m, wcfd_state s, int32_t field, float* weights, void* stream);

/* one implicit term of an assembly: its device weights and its (assigned) scale */
typedef struct wcfd_term {
    const float* weights;
    float        scale;
    int32_t      cell_based;   /* 1: [C][n][2] weights, 0: [C][F][n][3] */
} wcfd_term;
#define WCFD_MAX_TERMS 8
/* Equation.form_system (terms/equation.py:99-125) over any list of implicit terms (host
 * array of n_terms <= WCFD_MAX_TERMS): the system (ncomp = the terms' field count) is
 * overwritten with the sum of the terms, cell-parallel and atomic-free; explicit weights
 * of internal faces do not reach the RHS, as in the reference (Q1).  The off-diagonals are
 * stored once for all components: they are taken from component 0 (every scheme's
 * neighbour coefficient is the same for all fields). */
int wcfd_assemble_terms(const wcfd_mesh* m, wcfd_system A, const wcfd_term* terms, int32_t n_terms, void* stream);
/* Equation.add_RHS (terms/equation.py:167-168): rhs[i] += scale arr[i], i < n (device) */
int wcfd_add_rhs(float* rhs, const float* arr, float scale, int64_t n, void* stream);

/* ------------------------------------------------------------------ fused steps */
/* One steady SIMPLE outer iteration (incompressible.py:95-156 with steady_state=True),
 * or one PISO time step (NUM_OUTER_LOOPS = 1, steady_state=False), as a fixed sequence of
 * fused kernels on `stream`; capturable in a CUDA graph. */
int wcfd_simple_iteration(const wcfd_case* c, void* stream);

/* ------------------------------------------------------------------ convergence monitor
 * The residual norms of FVM.check_convergence (model.py:278-316, criteria of
 * Convergence.py:53-61) in one fused device pass: out (9 DEVICE doubles) receives
 * ||A x - b||_2 for the three momentum components (A: the momentum system, ncomp 3;
 * x: 3C interleaved velocity), ||b||_2 of each component, ||div||_1, ||rUA grad p||_inf
 * (cell_gradients C x 4 x 3, rua C) and ||p||_inf.  div, cell_gradients/rua and p may be
 * NULL (their norms are then 0).  scratch: wcfd_convergence_scratch_floats() floats of
 * device memory.  Two launches; the sums are float-float and reproducible. */
int64_t wcfd_convergence_scratch_floats(void);
int wcfd_convergence_norms(const wcfd_mesh* m, wcfd_system A, const float* x, const float* div,
                           const float* cell_gradients, const float* rua, const float* p, float* scratch,
                           double* out, void* stream);

/* ------------------------------------------------------------------ batched form
 * Many cases in one launch per kernel: `cases` is a DEVICE array of wcfd_case (a case
 * table; each entry points at that case's own arrays).  Field and assembly kernels run
 * over (case, face/cell) grids; each case's momentum BiCGSTAB and pressure CG run on one
 * thread-block cluster of `cluster_size` CTAs (the CG out of the cluster's shared memory).
 * Every case of a batch must have the same faces_per_cell and ell_width; loop counts are
 * the batch's.  Per-case outcomes go to each case's stats[0..1]. */
typedef struct wcfd_batch_dims {
    int32_t max_cells;       /* largest n_cells in the table           */
    int32_t max_faces;       /* largest n_faces in the table           */
    int32_t faces_per_cell;  /* common to every case                   */
    int32_t ell_width;       /* common to every case                   */
    int32_t n_inner;         /* pressure correctors                    */
    int32_t n_ortho;         /* non-orthogonal correctors              */
    int32_t cluster_size;    /* CTAs per case for the solves; 0 = pick */
    int32_t field_block;     /* threads per block of the field/assembly kernels: 0 = 256,
                                else 64..512 in steps of 32 (the result does not depend
                                on it: those kernels compute each face or cell alone)  */
    int32_t explicit_terms;  /* OR of the cases' wcfd_params.explicit_terms: non-zero
                                selects the assembly kernels with those terms compiled in */
    int32_t p_refine;        /* fp64 iterative-refinement sweeps of every case's pressure
                                solve (each: residual in fp64 from p_x64, a correction CG to
                                the case's p_refine_rtol, p_x64 += correction); 0 = the
                                plain solve.  Every case then needs p_x64 and p_work. */
    int32_t cg_variant;      /* 0 = textbook Jacobi CG (the reference's arithmetic); 1 = the
                                single-reduction (Chronopoulos-Gear) arrangement: one cluster
                                all-reduce and one cluster barrier per iteration instead of two
                                all-reduces, the same iterates up to rounding */
} wcfd_batch_dims;

/* Cluster size wcfd_batch_simple_iteration would pick for these dims (0 = no cluster
 * configuration fits: max_cells too large for the cluster-resident CG).  It prefers at most
 * 2048 rows per CTA (lower latency per case). */
int wcfd_batch_cluster_size(const wcfd_batch_dims* dims);
/* Most rows per CTA the cluster-resident CG holds on the current device for this
 * off-diagonal width (a cluster of cs CTAs takes cases of up to cs times as many cells;
 * the fewest CTAs per case give the most cases in flight). */
int wcfd_batch_max_rows(int32_t ell_width);
/* Set up, on the current device, everything a batched step with these dims needs before
 * its first launch (the cluster kernels' launch attributes), so that the step can be
 * captured into a CUDA graph without a first-use host call inside the capture. */
int wcfd_batch_prepare(const wcfd_batch_dims* dims);

/* One SIMPLE outer iteration (or PISO step) of every case in the table
 * (incompressible.py:95-156 for each case). */
int wcfd_batch_simple_iteration(const wcfd_case* cases, int32_t n_cases, const wcfd_batch_dims* dims,
                                void* stream);
/* Message of the last failed batched call on this thread. */
const char* wcfd_batch_last_error(void);

/* ---------------------------------------------------------------- mesh pass on the device
 * The preprocessing of warp_cfd/preprocess/mesh.py:64-302 (Mesh.get_faces and
 * Mesh.get_mesh_properties) for large meshes: face matching and geometry on the GPU, the
 * topology bit-identical to the host pass (faces numbered triangles first, then quads,
 * each set in lexicographic order of the sorted node ids; owner = lower cell id).  Cells of
 * mixed types (hexahedra, wedges, tetrahedra) are allowed; slots past a cell's own faces are
 * null (face id -1, zero geometry). */
typedef struct wcfd_mesh_cells {
    int32_t n_cells;          /* C                                                       */
    int32_t n_points;         /* P                                                       */
    int32_t faces_per_cell;   /* F: the largest face count of the cell types present     */
    int32_t tri_slots;        /* the largest number of triangular faces of one cell (0: none) */
    int32_t quad_slots;       /* the largest number of quadrilateral faces of one cell   */
    int32_t pad_;
    const double*  points;    /* [P*3]                                                   */
    const int32_t* cells;     /* [C*8] node ids in VTK order, -1 past the cell's nodes   */
    const int32_t* cell_type; /* [C] VTK type: 10 tetra, 12 hexahedron, 13 wedge          */
} wcfd_mesh_cells;

typedef struct wcfd_mesh_faces {  /* device outputs; K = n_faces[0] + n_faces[1] */
    int32_t* cell_faces;      /* [C*F] face id per (cell, slot); -1 on null slots        */
    int32_t* unique_faces;    /* [K*node_width] sorted node ids, -1 padded (faces.unique_faces) */
    int32_t* face_nodes;      /* [K] nodes per face (faces.num_nodes)                    */
    int32_t* face_cells;      /* [K*2] owner, neighbour (-1 on boundary faces)           */
    int32_t* face_slots;      /* [K*2] the face's slot in the owner, neighbour (-1)       */
    double*  centroid;        /* [C*3] node mean                                          */
    double*  volume;          /* [C]   divergence theorem over the fan-triangulated faces */
    double*  area;            /* [C*F] fan-triangulated area (mesh.py:161-183)            */
    double*  normal;          /* [C*F*3] outward unit normal                              */
    double*  to_face;         /* [C*F*3] cell centroid -> face centroid                    */
    double*  face_centroid;   /* [K*3] node mean                                          */
    int32_t  node_width;      /* 4 when the mesh has quads, else 3                        */
    int32_t  pad_;
} wcfd_mesh_faces;

/* Device workspace the two calls below need (0 on a bad argument). */
size_t wcfd_mesh_workspace_bytes(const wcfd_mesh_cells* m);
/* Match faces: keys, per-node buckets, counts.  Synchronizes the stream and returns the
 * number of triangular and of quadrilateral faces in n_faces[0..1] (host memory). */
int wcfd_mesh_match_faces(const wcfd_mesh_cells* m, void* workspace, size_t workspace_bytes, int32_t* n_faces,
                          void* stream);
/* Write the topology and geometry of a matched mesh into caller-allocated arrays. */
int wcfd_mesh_emit(const wcfd_mesh_cells* m, void* workspace, size_t workspace_bytes, const int32_t* n_faces,
                   const wcfd_mesh_faces* out, void* stream);
/* Message of the last failed mesh call on this thread. */
const char* wcfd_mesh_last_error(void);

/* Bounds and consistency check of a device geometry's index arrays (no reference
 * counterpart; the stand-in for a sanitizer on the gathers): face owner / neighbour in
 * range, boundary rows in range, every non-null cell slot naming a face that has the cell
 * on that side, every off-diagonal column in range.  Each index is read only after the
 * bounds it is used under were checked.  Synchronizes the stream; counts (host, 5 ints)
 * receive the violations per kind; WCFD_ERR_ARGUMENT (and wcfd_mesh_last_error) if any. */
int wcfd_check_mesh(const wcfd_mesh* m, int32_t* counts, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* WCFD_H */
